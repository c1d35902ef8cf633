// ma_amg.cu -- aggregation multigrid preconditioner for the Newton linear solve.
//
// The Newton system of solve_laplacian_matrix (include/MA/optimal_transport.hpp:41-87)
// is the Hessian H (a weighted graph Laplacian of the Laguerre-cell adjacency) with
// its last row and column removed.  The reference factorises it (SimplicialLLT);
// here conjugate gradients are preconditioned by one V-cycle of an aggregation
// multigrid built on the device at every Newton step:
//
//   * the fine level is H copied into Morton order (the order of the site index),
//     so that neighbouring rows are close in memory;
//   * every level is aggregated by strength, in two pairwise passes (pairwise
//     aggregation, Notay 2010): each pass matches every row with its strongest
//     neighbour (largest -a_ij) by handshakes -- a row and its strongest free
//     neighbour pair up when each is the other's choice, over four rounds -- and a
//     row left alone joins the pair of its strongest matched neighbour (one such
//     row per pair).  The second pass pairs the first pass's aggregates on their
//     Galerkin matrix, so an aggregate holds up to nine rows (about 4.6 on the
//     Hessians of the 100,000-site workload).  Every choice is a deterministic
//     function of the matrix (ties go to the lower index; claims by atomicMin), and
//     the aggregates are numbered in the order of their first row.  A level whose
//     matching stalls (fewer than 1.5 rows per aggregate) is grouped by four
//     consecutive rows instead;
//   * the coarse matrices are Galerkin products P^T A P with the piecewise-constant
//     prolongation P: a coarse entry (I, J) is the sum of the fine entries (i, j)
//     with i in I and j in J.  Each coarse row is assembled by one warp from the
//     aggregate's member rows, its duplicates summed in a fixed order (reproducible
//     results);
//   * smoothing is damped Jacobi (one sweep before, one after), the coarse
//     correction is scaled by kCoarseScale (piecewise-constant prolongation
//     underestimates the smooth error), and the coarsest level (at most kCoarsest
//     nodes) is solved with its dense inverse;
//   * the whole preconditioned CG -- every level of every V-cycle -- runs in one
//     cooperative kernel with grid barriers between the phases; no host round trip
//     per iteration.
// Rows that are inactive (the gauge row n-1 and empty cells: zero diagonal) belong
// to no aggregate and are held at zero on every level.
#include <cooperative_groups.h>

#include <cfloat>

#include <algorithm>

#include "ma_runtime.h"

namespace cg = cooperative_groups;

namespace ma {

constexpr int kMatchRounds = 4;     // handshake rounds of a pairwise pass
constexpr int kAggGroup = 4;        // rows per aggregate where the matching stalls
constexpr int kCoarsest = 64;       // dense solve at or below this many nodes
constexpr int kRowCap = 512;        // gathered entries of one coarse row
constexpr int kRowWarps = 4;        // coarse rows per block in the setup
constexpr double kOmega = 0.8;  // Jacobi damping (|1 - omega lambda| <= 0.6 on D^-1 H's [0, 2])
constexpr double kCoarseScale = 1.5;
constexpr float kOmegaF = (float)kOmega;  // the preconditioner's FP32 arithmetic
constexpr float kCoarseScaleF = (float)kCoarseScale;

// ---------------------------------------------------------------------------
// setup: coarse rows
// ---------------------------------------------------------------------------
struct CoarseSrc {
    const int* mp;     // members of aggregate I: mem[mp[I] .. mp[I+1])
    const int* mem;
    const int* map;    // fine node -> aggregate (-1: inactive)
    const int* rp;     // fine CSR
    const int* ci;
    const double* va;
};

// One warp per coarse row: gather the member rows' entries in active columns, mapped
// to aggregates, keep the first occurrence of each aggregate, sum its duplicates in
// gather order, and place it by rank of its column.  FILL = false counts the
// distinct columns into cnt[I]; FILL = true writes them at rp[I].
struct RowScratch {  // one warp's gather space
    int col[kRowCap];
    double val[kRowCap];
    unsigned char lead[kRowCap];
};

template <bool FILL>
__device__ void coarse_row(const CoarseSrc& s, int I, int lane, RowScratch& w, int* cnt, const int* rp, int* ci,
                           double* va, int* overflow)
{
    int* col = w.col;
    double* val = w.val;
    unsigned char* lead = w.lead;
    __syncwarp();  // the warp's previous row is done with the scratch
    int E = 0;
    bool over = false;
    // the members' row ranges at once (one member per lane), then their entries in
    // member order, 32 at a time
    const int M = s.mp[I + 1] - s.mp[I];
    for (int m0 = 0; m0 < M && !over; m0 += 32) {
        const int mm = min(32, M - m0);
        int rb = 0, len = 0;
        if (lane < mm) {
            const int i = s.mem[s.mp[I] + m0 + lane];
            rb = s.rp[i];
            len = s.rp[i + 1] - rb;
        }
        int off = len;
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, off, d);
            if (lane >= d) off += y;
        }
        const int tot = __shfl_sync(0xffffffffu, off, 31);
        off -= len;
        for (int b = 0; b < tot; b += 32) {
            const int t = b + lane;
            int who = 0;
            for (int m = 1; m < mm; m++)
                if (t >= __shfl_sync(0xffffffffu, off, m)) who = m;
            const int kb = __shfl_sync(0xffffffffu, rb, who), ko = __shfl_sync(0xffffffffu, off, who);
            int c = -1;
            double v = 0.0;
            if (t < tot) {
                const int k = kb + (t - ko);
                c = s.map[s.ci[k]];
                v = s.va[k];
            }
            const unsigned bal = __ballot_sync(0xffffffffu, c >= 0);
            const int pos = E + __popc(bal & ((1u << lane) - 1u));
            if (c >= 0 && pos < kRowCap) {
                col[pos] = c;
                val[pos] = v;
            }
            E += __popc(bal);
            if (E > kRowCap) {
                over = true;
                break;
            }
        }
    }
    if (over) {
        if (lane == 0) {
            atomicExch(overflow, 1);
            if (!FILL) cnt[I] = 0;
        }
        return;
    }
    __syncwarp();
    int nlead = 0;
    for (int e = lane; e < E; e += 32) {
        const int c = col[e];
        bool first = true;
        for (int f = 0; f < e; f++)
            if (col[f] == c) {
                first = false;
                break;
            }
        lead[e] = first ? 1 : 0;
        nlead += first ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) nlead += __shfl_xor_sync(0xffffffffu, nlead, o);
    if (!FILL) {
        if (lane == 0) cnt[I] = nlead;
        return;
    }
    __syncwarp();
    const int base = rp[I];
    for (int e = lane; e < E; e += 32) {
        if (!lead[e]) continue;
        const int c = col[e];
        double sum = 0.0;
        int rank = 0;
        for (int f = 0; f < E; f++) {
            if (col[f] == c && f >= e) sum += val[f];
            if (lead[f] && col[f] < c) rank++;
        }
        ci[base + rank] = c;
        va[base + rank] = sum;
    }
}

// ---------------------------------------------------------------------------
// setup: pairwise aggregation, one cooperative launch per level
// ---------------------------------------------------------------------------
struct LevelCsr {
    int n;
    const int* rp;
    const int* ci;
    const double* va;
    const double* dinv;  // 0: inactive row
};

constexpr int kSetupThreads = 32 * kRowWarps;

struct SetupArgs {
    LevelCsr A;  // the level to aggregate
    // scratch, n + 2 entries each (rp1: n + 2, ci1 / va1: the level's entries)
    int *mate, *best, *claim, *flag, *id, *join, *agg1, *agg2, *mp1, *mem1, *fill, *cnt;
    int* rp1;
    int* ci1;
    double* va1;
    double* dinv1;
    int* part;    // one int per block
    int* counts;  // [0] first-pass aggregates, [1] second-pass aggregates, [2] the level's aggregates
    // outputs: the level's aggregates and the next level's matrix
    int *agg, *mp, *mem;
    int* rp;
    int* ci;
    double* va;
    double* dinv;
    int* overflow;
    int reuse;  // keep agg / mp / mem (nc aggregates) and rebuild only the next level's matrix
    int nc;
};

// the strongest active neighbour (largest -a_ij > 0) of free active row i among the
// free rows (MATCHED = false) or the matched rows (MATCHED = true); ties to the
// lower index; -1 if there is none or row i is not free
template <bool MATCHED>
__device__ int strongest(const LevelCsr& A, const int* mate, int i)
{
    int b = -1;
    if (A.dinv[i] != 0.0 && mate[i] < 0) {
        double sb = 0.0;
        for (int k = A.rp[i]; k < A.rp[i + 1]; k++) {
            const int j = A.ci[k];
            if (j == i || A.dinv[j] == 0.0 || (mate[j] >= 0) != MATCHED) continue;
            const double v = -A.va[k];
            if (v > sb || (v == sb && b >= 0 && j < b)) {
                sb = v;
                b = j;
            }
        }
    }
    return b;
}

// exclusive block-wide scan of v (kSetupThreads threads); *total gets the sum
__device__ __forceinline__ int block_scan(int v, int* sh, int* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    int before = 0, all = 0;
    for (int q = 0; q < kSetupThreads / 32; q++) {
        if (q < wid) before += sh[q];
        all += sh[q];
    }
    __syncthreads();
    *total = all;
    return before + x - v;
}

// exclusive scan of in[0, n) into out[0, n] (out[n] = total) by the whole grid: each
// block scans a contiguous chunk after the totals of the chunks before it
__device__ void grid_scan(cg::grid_group& grid, const int* in, int* out, int n, int* part, int* sh)
{
    const int nb = gridDim.x, chunk = (n + nb - 1) / nb;
    const int b0 = min(n, blockIdx.x * chunk), b1 = min(n, b0 + chunk);
    int t = 0;
    for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) t += in[i];
    int tot;
    block_scan(t, sh, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
    grid.sync();
    int off = 0;
    for (int q = threadIdx.x; q < blockIdx.x; q += blockDim.x) off += part[q];
    block_scan(off, sh, &off);
    for (int base = b0; base < b1; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < b1 ? in[i] : 0;
        int tile;
        const int ex = block_scan(v, sh, &tile);
        if (i < b1) out[i] = off + ex;
        off += tile;
    }
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) out[n] = off;
    grid.sync();
}

// One pairwise pass over A: kMatchRounds handshake rounds (a row and its strongest
// free neighbour pair up when each is the other's choice), then every row left alone
// bids for the pair of its strongest matched neighbour and the lowest bidder joins
// it; leaders (the lower row of a pair, or a row that stays alone) are numbered in
// row order.  agg[i] = aggregate of row i (-1: inactive), *count = aggregates.
__device__ void pair_pass(cg::grid_group& grid, const LevelCsr& A, const SetupArgs& a, int* agg, int* count, int* sh)
{
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (int i = tid; i < A.n; i += stride) {
        a.mate[i] = -1;
        a.claim[i] = INT_MAX;
    }
    grid.sync();
    for (int r = 0; r < kMatchRounds; r++) {
        for (int i = tid; i < A.n; i += stride) a.best[i] = strongest<false>(A, a.mate, i);
        grid.sync();
        for (int i = tid; i < A.n; i += stride) {
            const int j = a.best[i];
            if (j >= 0 && a.best[j] == i) a.mate[i] = j;
        }
        grid.sync();
    }
    for (int i = tid; i < A.n; i += stride) a.best[i] = strongest<true>(A, a.mate, i);
    grid.sync();
    for (int i = tid; i < A.n; i += stride) {
        const int j = a.best[i];
        if (j >= 0) atomicMin(&a.claim[min(j, a.mate[j])], i);
    }
    grid.sync();
    for (int i = tid; i < A.n; i += stride) {
        int f = 0, jn = -1;
        if (A.dinv[i] != 0.0) {
            const int m = a.mate[i];
            if (m >= 0) {
                f = i < m;
            } else {
                const int j = a.best[i];
                const int p = j >= 0 ? min(j, a.mate[j]) : -1;
                if (p >= 0 && a.claim[p] == i)
                    jn = p;
                else
                    f = 1;
            }
        }
        a.flag[i] = f;
        a.join[i] = jn;
    }
    grid.sync();
    grid_scan(grid, a.flag, a.id, A.n, a.part, sh);
    for (int i = tid; i < A.n; i += stride) {
        int g = -1;
        if (A.dinv[i] != 0.0) {
            const int m = a.mate[i];
            g = m >= 0 ? a.id[min(i, m)] : (a.join[i] >= 0 ? a.id[a.join[i]] : a.id[i]);
        }
        agg[i] = g;
    }
    if (tid == 0) *count = a.id[A.n];
    grid.sync();
}

// member lists of nc aggregates of n rows, each sorted by row
__device__ void member_lists(cg::grid_group& grid, const int* agg, int n, int nc, int* mp, int* mem,
                             const SetupArgs& a, int* sh)
{
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (int I = tid; I < nc; I += stride) {
        a.cnt[I] = 0;
        a.fill[I] = 0;
    }
    grid.sync();
    for (int i = tid; i < n; i += stride)
        if (agg[i] >= 0) atomicAdd(&a.cnt[agg[i]], 1);
    grid.sync();
    grid_scan(grid, a.cnt, mp, nc, a.part, sh);
    for (int i = tid; i < n; i += stride)
        if (agg[i] >= 0) mem[mp[agg[i]] + atomicAdd(&a.fill[agg[i]], 1)] = i;
    grid.sync();
    for (int I = tid; I < nc; I += stride)
        for (int q = mp[I] + 1; q < mp[I + 1]; q++) {
            const int v = mem[q];
            int r = q - 1;
            while (r >= mp[I] && mem[r] > v) {
                mem[r + 1] = mem[r];
                r--;
            }
            mem[r + 1] = v;
        }
    grid.sync();
}

__device__ __forceinline__ double level_dinv(const int* rp, const int* ci, const double* va, int i)
{
    double d = 0.0;
    for (int k = rp[i]; k < rp[i + 1]; k++)
        if (ci[k] == i) d = va[k];
    return d > 0.0 ? 1.0 / d : 0.0;
}

// the Galerkin matrix of nc aggregates (warp per coarse row: count, place, fill) and
// its inverse diagonal (0 for rows without a positive diagonal)
__device__ void galerkin(cg::grid_group& grid, const LevelCsr& A, const int* mp, const int* mem, const int* map,
                         int nc, int* rp, int* ci, double* va, double* dinv, const SetupArgs& a, RowScratch* sw,
                         int* sh)
{
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kRowWarps + wib, nw = gridDim.x * kRowWarps;
    const CoarseSrc src{mp, mem, map, A.rp, A.ci, A.va};
    for (int I = gw; I < nc; I += nw) coarse_row<false>(src, I, lane, sw[wib], a.cnt, nullptr, nullptr, nullptr, a.overflow);
    grid.sync();
    grid_scan(grid, a.cnt, rp, nc, a.part, sh);
    for (int I = gw; I < nc; I += nw) coarse_row<true>(src, I, lane, sw[wib], a.cnt, rp, ci, va, a.overflow);
    grid.sync();
    for (int I = tid; I < nc; I += stride) dinv[I] = level_dinv(rp, ci, va, I);
    grid.sync();
}

// One level: a pairwise pass over A, the Galerkin matrix of its pairs, a second
// pairwise pass over that, the two composed; where a pass leaves more than 2/3 of the
// rows (the matching stalls), groups of kAggGroup consecutive rows instead.  Then the
// member lists and the next level's matrix.  With `reuse`, the aggregates of the
// previous call stay and only the next level's matrix is rebuilt.  Every branch is
// grid-uniform.
__global__ void __launch_bounds__(kSetupThreads) k_level_setup(SetupArgs a)
{
    cg::grid_group grid = cg::this_grid();
    __shared__ RowScratch sw[kRowWarps];
    __shared__ int sh[kSetupThreads / 32];
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    const int n = a.A.n;
    if (a.reuse) {
        galerkin(grid, a.A, a.mp, a.mem, a.agg, a.nc, a.rp, a.ci, a.va, a.dinv, a, sw, sh);
        if (tid == 0) a.counts[2] = a.nc;
        return;
    }
    pair_pass(grid, a.A, a, a.agg1, &a.counts[0], sh);
    const int n1 = *(volatile const int*)&a.counts[0];
    int nc = 0;
    if (n1 > 0 && 3 * n1 < 2 * n) {
        member_lists(grid, a.agg1, n, n1, a.mp1, a.mem1, a, sh);
        galerkin(grid, a.A, a.mp1, a.mem1, a.agg1, n1, a.rp1, a.ci1, a.va1, a.dinv1, a, sw, sh);
        const LevelCsr L1{n1, a.rp1, a.ci1, a.va1, a.dinv1};
        pair_pass(grid, L1, a, a.agg2, &a.counts[1], sh);
        nc = *(volatile const int*)&a.counts[1];
        for (int i = tid; i < n; i += stride) a.agg[i] = a.agg1[i] >= 0 ? a.agg2[a.agg1[i]] : -1;
    }
    if (!(nc > 0 && 3 * nc < 2 * n)) {
        nc = (n + kAggGroup - 1) / kAggGroup;
        for (int i = tid; i < n; i += stride) a.agg[i] = a.A.dinv[i] != 0.0 ? i / kAggGroup : -1;
    }
    grid.sync();
    member_lists(grid, a.agg, n, nc, a.mp, a.mem, a, sh);
    galerkin(grid, a.A, a.mp, a.mem, a.agg, nc, a.rp, a.ci, a.va, a.dinv, a, sw, sh);
    if (tid == 0) a.counts[2] = nc;
}

// dense inverse of the coarsest level (n <= kCoarsest, SPD on its active rows;
// inactive rows become identity rows), Gauss-Jordan in place, one block
__global__ void __launch_bounds__(256) k_dense_inverse(const int* rp, const int* ci, const double* va,
                                                       const double* dinv, int n, double* inv)
{
    __shared__ double a[kCoarsest][kCoarsest + 1];
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) a[t / n][t % n] = 0.0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (dinv[i] == 0.0) {
            a[i][i] = 1.0;
            continue;
        }
        for (int k = rp[i]; k < rp[i + 1]; k++)
            if (dinv[ci[k]] != 0.0) a[i][ci[k]] = va[k];
    }
    __syncthreads();
    __shared__ double fcol[kCoarsest];
    for (int k = 0; k < n; k++) {
        const double p = 1.0 / a[k][k];
        // the multipliers of column k, read before any row changes
        for (int i = threadIdx.x; i < n; i += blockDim.x) fcol[i] = a[i][k];
        __syncthreads();
        // row k scaled (with the pivot position replaced by 1 first)
        for (int j = threadIdx.x; j < n; j += blockDim.x) a[k][j] = (j == k ? 1.0 : a[k][j]) * p;
        __syncthreads();
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
            const int i = t / n, j = t % n;
            if (i == k) continue;
            const double f = fcol[i];
            if (j == k)
                a[i][j] = -f * a[k][k];
            else
                a[i][j] -= f * a[k][j];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int i = t / n, j = t % n;
        inv[t] = (dinv[i] == 0.0 || dinv[j] == 0.0) ? 0.0 : a[i][j];
    }
}

// the fine level in Morton order: row k is H's row perm[k], columns renumbered
__global__ void k_inv_perm(const int* perm, int n, int* inv)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) inv[perm[k]] = k;
}

__global__ void k_fine_count(const int* rp, const int* perm, int n, int* cnt)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) cnt[k] = rp[perm[k] + 1] - rp[perm[k]];
}

// entries of row k, and its inverse diagonal (0 for the gauge row n-1 and for
// empty rows)
__global__ void k_fine_fill(const int* rp, const int* ci, const double* va, const int* perm, const int* inv, int n,
                            const int* rpm, int* cim, double* vam, double* dinv)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = perm[k];
    const int k0 = rp[i], k1 = rp[i + 1], base = rpm[k];
    double d = 0.0;
    for (int e = k0; e < k1; e++) {
        const int j = ci[e];
        if (j == i) d = va[e];
        cim[base + e - k0] = inv[j];
        vam[base + e - k0] = va[e];
    }
    dinv[k] = (i == n - 1 || !(d > 0.0)) ? 0.0 : 1.0 / d;
}

// An FP64 value for the preconditioner's FP32 arithmetic: nonzero stays nonzero (a
// row's diagonal inverse marks it active) and the range saturates at FLT_MAX.
__host__ __device__ __forceinline__ float to_f32(double v)
{
    float f = (float)v;
    if (f == 0.0f && v != 0.0) f = v > 0.0 ? FLT_MIN : -FLT_MIN;
    return fminf(fmaxf(f, -FLT_MAX), FLT_MAX);
}

// sliced ELL of the Morton-ordered fine level: 32 x (longest row of the slice)
// entries per slice of 32 rows
__global__ void k_sell_width(const int* rp, int n, int* cnt)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int len = k < n ? rp[k + 1] - rp[k] : 0;
    for (int o = 16; o > 0; o >>= 1) len = max(len, __shfl_xor_sync(0xffffffffu, len, o));
    if ((k & 31) == 0 && k < n) cnt[k >> 5] = 32 * len;
}

__global__ void k_sell_fill(const int* rp, const int* ci, const double* va, int n, const int* sp, int* eci,
                            double* eva, float* eva32)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int b0 = sp[k >> 5] + (k & 31), w = (sp[(k >> 5) + 1] - sp[k >> 5]) >> 5;
    const int k0 = rp[k], len = rp[k + 1] - k0;
    for (int e = 0; e < w; e++) {
        eci[b0 + 32 * e] = e < len ? ci[k0 + e] : k;
        eva[b0 + 32 * e] = e < len ? va[k0 + e] : 0.0;
        eva32[b0 + 32 * e] = e < len ? to_f32(va[k0 + e]) : 0.0f;
    }
}

// ---------------------------------------------------------------------------
// the multigrid PCG kernel
// ---------------------------------------------------------------------------
// Level l >= 1 keeps the restricted residual b_l and the post-smoothed correction
// xp_l; the pre-smoothed correction omega D^-1 b_l is recomputed where needed.  The
// fine level runs one thread per row; a coarse level gives each row a team of
// T = 1 .. 32 adjacent lanes (sized so that the grid covers the level), the lanes
// striding over the row's entries and summing by shuffles, so that the small levels
// are not a chain of dependent loads in a few threads.  An aggregate's members are
// listed (mem[mp[J] .. mp[J+1])); agg maps a row to its aggregate.  The
// preconditioner computes in FP32, on FP32 copies of the levels' matrices (GB300
// issues FP64 at 1/64 of its FP32 rate, and the per-SM FP64 issue bounded these
// phases; the V-cycle's rounding lies far below its approximation error), while the
// CG recurrences, the product A p and the dot products stay FP64, so that the
// residual the iteration reaches is an FP64 residual.  Grid barriers
// per CG iteration: 2 (nlev - 2) + 4 without the block-local coarse cycle below,
// 2 (c - 1) + 5 with it.
constexpr int kAmgMaxLevels = 16;
constexpr int kAmgMaxThreads = 1024;  // the PCG block size is chosen at launch, up to this

struct AmgLevelDev {
    int n;
    const int* rp;
    const int* ci;
    const double* va;    // the setup's FP64 matrix
    const double* dinv;
    float* va32;         // its FP32 copy for the preconditioner (written by the PCG kernel)
    float* dinv32;
    float* b;   // restricted residual
    float* xp;  // post-smoothed correction
    float* y;   // pre-smoothed plus prolonged correction (levels 1 .. nlev-3)
    int tr;      // team size restricting this level into the next
    int tp;      // team size prolonging into this level
    const int* agg;  // row -> node of the next level (-1: inactive)
    const int* mp;   // members of node J of the next level: mem[mp[J] .. mp[J+1])
    const int* mem;
    // level 0 only: the same matrix as sliced ELL, slices of 32 rows stored
    // entry-major (entry e of row 32 s + r at sp[s] + 32 e + r), padded with
    // zero entries pointing at the row itself
    const int* sp;
    const int* eci;
    const double* eva;
    const float* eva32;
};

struct AmgPcgArgs {
    int nlev;  // levels 0 .. nlev-1; nlev-1 is solved densely
    AmgLevelDev L[kAmgMaxLevels];  // level 0: H in Morton order
    const int* perm;  // Morton position -> row of H
    const double* cinv;
    const double* b;  // right-hand side, rows of H (component n-1 ignored)
    double* x;        // solution, rows of H
    // work vectors in Morton order
    double* xs;
    double* r0;  // residual, double-buffered
    double* r1;
    double* z;
    double* p;
    double* q;
    float* ys;     // the fine level's pre-smoothed plus prolonged correction (levels >= 3)
    float* r32a;   // FP32 copies of the residual (double-buffered like r0/r1) and of q,
    float* r32b;   // which the preconditioner reads
    float* q32;
    float* s32;    // the fine residual of the pre-smoothed correction
    double* part;  // 3 * gridDim.x partial sums
    double* out;   // [iterations, |r|, |b|]
    double rtol;
    int maxiter;
    const int* overflow;  // set by the setup: fall back to Jacobi
    int tail_bytes;       // dynamic shared memory of a block, for the block-local coarse cycle
};

__device__ __forceinline__ double amg_block_sum(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
        sh[32] = s;
    }
    __syncthreads();
    const double s = sh[32];
    __syncthreads();
    return s;
}

__device__ __forceinline__ double amg_grid_total(const double* part, int nb, double* sh)
{
    double v = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) v += part[k];
    return amg_block_sum(v, sh);
}

// sum over lanes xor-adjacent below `width` (bitwise identical on all of them)
__device__ __forceinline__ float team_sum(float v, int width)
{
    for (int o = width >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// inclusive sum of v over the lanes of a team of T (lanes below t included)
__device__ __forceinline__ int team_scan(int v, int t, int T)
{
    for (int d = 1; d < T; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, d, T);
        if (t >= d) v += y;
    }
    return v;
}

// Loop over rows [0, nrows) with teams of T lanes: calls fn(row, lane_in_team)
// with row < nrows, or row = -1 for lanes without a row in this pass (they still
// take part in the team's shuffles).  Warp-uniform trip count.  LOCAL: the teams of
// this block alone (the block-local coarse cycle), else those of the whole grid.
template <bool LOCAL, class Fn>
__device__ __forceinline__ void team_rows(int nrows, int T, Fn&& fn)
{
    const int tid = LOCAL ? (int)threadIdx.x : (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int nteams = (LOCAL ? (int)blockDim.x : (int)(gridDim.x * blockDim.x)) / T;
    const int lane = threadIdx.x & 31;
    const int wteam0 = (tid >> 5) * (32 / T);  // first team of this warp
    for (int base = wteam0; base < nrows; base += nteams) {
        const int row = base + lane / T;
        fn(row < nrows ? row : -1, lane & (T - 1));
    }
}

// b_{l+1} from level l >= 1: the residual of the pre-smoothed correction summed
// over each aggregate, b_{l+1}[J] = sum_{I in J} b_l[I] - omega sum over the
// member rows' entries a_IK D_K^-1 b_l[K]
template <bool LOCAL>
__device__ __forceinline__ void restrict_level(const AmgLevelDev* L, int l, int tail)
{
    const AmgLevelDev& A = L[l];
    const AmgLevelDev& C = L[l + 1];
    const int T = A.tr;
    team_rows<LOCAL>(C.n, T, [&](int J, int t) {
        // the members' rows at once (member q on team lane q), then their entries in
        // member order, T at a time
        // every loop bound is a maximum over the warp (teams of one warp share it)
        const int q0 = J >= 0 ? A.mp[J] : 0, M = J >= 0 ? A.mp[J + 1] - q0 : 0;
        const int Mmax = __reduce_max_sync(0xffffffffu, M);
        float s = 0.0f;
        for (int m0 = 0; m0 < Mmax; m0 += T) {
            const int mm = max(0, min(T, M - m0));
            int rb = 0, len = 0;
            if (t < mm) {
                const int I = A.mem[q0 + m0 + t];
                s += A.b[I];
                rb = A.rp[I];
                len = A.rp[I + 1] - rb;
            }
            int off = team_scan(len, t, T);
            const int tot = __shfl_sync(0xffffffffu, off, T - 1, T);
            off -= len;
            const int mw = __reduce_max_sync(0xffffffffu, mm);
            const int totw = __reduce_max_sync(0xffffffffu, tot);
            for (int b = 0; b < totw; b += T) {
                const int e = b + t;
                int who = 0;
                for (int m = 1; m < mw; m++)
                    if (e >= __shfl_sync(0xffffffffu, off, m, T)) who = m;
                const int kb = __shfl_sync(0xffffffffu, rb, who, T), ko = __shfl_sync(0xffffffffu, off, who, T);
                if (e < tot && J >= 0) {
                    const int k = kb + (e - ko);
                    const int K = A.ci[k];
                    s -= A.va32[k] * (kOmegaF * A.dinv32[K] * A.b[K]);
                }
            }
        }
        s = team_sum(s, T);
        if (J >= 0 && t == 0) {
            C.b[J] = C.dinv32[J] != 0.0f ? s : 0.0f;
            if (C.y && l + 1 != tail - 1) C.y[J] = C.dinv32[J] != 0.0f ? kOmegaF * C.dinv32[J] * s : 0.0f;
        }
    });
}

// b_1 from the fine level: the fine residuals of the pre-smoothed correction (in s)
// summed over each aggregate
__device__ __forceinline__ void restrict_fine(const AmgPcgArgs& a, const float* s_fine, int tail)
{
    const AmgLevelDev& F = a.L[0];
    const AmgLevelDev& C = a.L[1];
    const int T = F.tr;
    team_rows<false>(C.n, T, [&](int J, int t) {
        float s = 0.0f;
        if (J >= 0)
            for (int q = F.mp[J] + t; q < F.mp[J + 1]; q += T) s += s_fine[F.mem[q]];
        s = team_sum(s, T);
        if (J >= 0 && t == 0) {
            C.b[J] = C.dinv32[J] != 0.0f ? s : 0.0f;
            if (C.y && tail != 2) C.y[J] = C.dinv32[J] != 0.0f ? kOmegaF * C.dinv32[J] * s : 0.0f;
        }
    });
}

// the coarsest level's solution cinv b, computed into shared memory (xc) before the
// phase that prolongs it, by every block or by the block of the block-local cycle;
// cinv itself stays in shared memory (sinv) for the whole kernel.  Thread r < n
// forms row r, its b[k] from shared memory.
__device__ __forceinline__ void coarsest_solve(const AmgLevelDev& C, float* xc, const float* sinv, float* sb)
{
    for (int k = threadIdx.x; k < C.n; k += blockDim.x) sb[k] = C.b[k];
    __syncthreads();
    for (int r = threadIdx.x; r < C.n; r += blockDim.x) {
        float v = 0.0f;
        for (int k = 0; k < C.n; k++) v += sinv[k * C.n + r] * sb[k];
        xc[r] = v;
    }
    __syncthreads();
}

// the coarse correction of aggregate J of level l, i.e. node J of level l+1
__device__ __forceinline__ float coarse_corr(const AmgLevelDev* L, int nlev, int l, int J, const float* xc)
{
    if (J < 0) return 0.0f;  // a row in no aggregate
    return (l + 2 < nlev) ? L[l + 1].xp[J] : xc[J];
}

// xp_l for level l >= 1: pre-smoothed plus scaled coarse correction, then one
// damped Jacobi sweep
template <bool LOCAL>
__device__ __forceinline__ void prolong_level(const AmgLevelDev* L, int nlev, int l, int tail, float* ys,
                                              float* xc, const float* sinv, float* sb)
{
    const AmgLevelDev& A = L[l];
    const int T = A.tp;
    // level tail - 1 keeps no y: its prolongation recomputes the terms from b and the
    // corrections of level tail (the same values), which the block-local cycle
    // leaves in global memory, so that the cycle scatters nothing into level tail - 1
    const bool has_y = A.y != nullptr && l != tail - 1;
    if (l + 2 == nlev) coarsest_solve(L[nlev - 1], xc, sinv, sb);
    team_rows<LOCAL>(A.n, T, [&](int I, int t) {
        float s = 0.0f, yI = 0.0f, dI = 0.0f;
        if (I >= 0) {
            dI = A.dinv32[I];
            if (dI != 0.0f) {
                if (has_y) {
                    // y complete since the prolongation of level l + 1: one gather
                    for (int k = A.rp[I] + t; k < A.rp[I + 1]; k += T) s -= A.va32[k] * A.y[A.ci[k]];
                    yI = A.y[I];
                } else {
                    for (int k = A.rp[I] + t; k < A.rp[I + 1]; k += T) {
                        const int K = A.ci[k];
                        const float dK = A.dinv32[K];
                        const float yK = dK != 0.0f ? kOmegaF * dK * A.b[K] +
                                                          kCoarseScaleF * coarse_corr(L, nlev, l, A.agg[K], xc)
                                                    : 0.0f;
                        s -= A.va32[k] * yK;
                    }
                    yI = kOmegaF * dI * A.b[I] + kCoarseScaleF * coarse_corr(L, nlev, l, A.agg[I], xc);
                }
            }
        }
        s = team_sum(s, T);
        const float xI = dI != 0.0f ? yI + kOmegaF * dI * (A.b[I] + s) : 0.0f;
        if (I >= 0 && t == 0) A.xp[I] = xI;
        if (I >= 0 && l != tail) {
            // the rows of aggregate I one level down take their share of the correction now
            const AmgLevelDev& D = L[l - 1];
            float* yd = l == 1 ? ys : D.y;
            for (int q = D.mp[I] + t; q < D.mp[I + 1]; q += T) yd[D.mem[q]] += kCoarseScaleF * xI;
        }
    });
}

// The block-local coarse cycle.  Levels c .. nlev-1 of the hierarchy, when they fit the
// dynamic shared memory of a block, are copied there once per launch, and each
// iteration block 0 alone restricts through them, solves the coarsest level and
// prolongs back to level c with block barriers, while the other blocks wait at one
// grid barrier: the small levels cost shared-memory latencies instead of a grid
// barrier and a chain of L2 loads each.  The arithmetic is that of the grid-wide
// phases, term for term.  Per level, in this order, each array padded to 16 bytes:
// va32, dinv32, b, [xp for l > c], [y where the level keeps one], rp, ci, agg, mem, mp;
// the coarsest level holds b and dinv.  Level c's xp stays in global memory, where
// the prolongation of level c - 1 reads it per entry (level c - 1 keeps no y, so the
// cycle writes nothing else), and level c - 1's aggregates stay there too.
constexpr int kTailMaxRows = 2048;  // a larger level is faster on the whole grid

__host__ __device__ __forceinline__ size_t tail_pad(size_t b) { return (b + 15) & ~(size_t)15; }

__host__ __device__ __forceinline__ size_t tail_level_bytes(int l, int c, int nlev, int n, int nnz, int nnext)
{
    const size_t vn = tail_pad(4 * (size_t)n);
    if (l == nlev - 1) return 2 * vn;
    size_t s = tail_pad(4 * (size_t)nnz) + 2 * vn;
    if (l > c) s += vn;
    if (l + 3 <= nlev) s += vn;
    s += tail_pad(4 * (size_t)(n + 1)) + tail_pad(4 * (size_t)nnz) + 2 * tail_pad(4 * (size_t)n) +
         tail_pad(4 * (size_t)(nnext + 1));
    return s;
}

// the first level c >= 1 of the block-local cycle, 0 for none; every block finds the
// same from the same sizes
__device__ __forceinline__ int tail_level(const AmgPcgArgs& a)
{
    int best = 0;
    if (a.tail_bytes <= 0) return 0;
    for (int c = a.nlev - 2; c >= 1; c--) {
        if (a.L[c].n > kTailMaxRows) break;
        size_t tot = 0;
        for (int l = c; l < a.nlev; l++) {
            const int n = a.L[l].n;
            const bool last = l == a.nlev - 1;
            tot += tail_level_bytes(l, c, a.nlev, n, last ? 0 : a.L[l].rp[n], last ? 0 : a.L[l + 1].n);
        }
        if (tot > (size_t)a.tail_bytes) break;
        best = c;
    }
    return best;
}

// lanes per row for a level cycled through by one block
__device__ __forceinline__ int local_team(int rows)
{
    int t = 1;
    while (t < 32 && rows * t * 2 <= (int)blockDim.x) t <<= 1;
    return t;
}

// block 0: the level table of the cycle (levels below c as they are, levels c and
// up in shared memory) and the copies of their matrices and aggregates
__device__ __forceinline__ void tail_setup(const AmgPcgArgs& a, int c, AmgLevelDev* tl, unsigned char* sm)
{
    if (threadIdx.x == 0) {
        for (int l = 0; l < a.nlev; l++) tl[l] = a.L[l];
        size_t off = 0;
        auto take = [&](size_t bytes) {
            unsigned char* q = sm + off;
            off += tail_pad(bytes);
            return q;
        };
        for (int l = c; l < a.nlev; l++) {
            AmgLevelDev& T = tl[l];
            const int n = T.n;
            if (l == a.nlev - 1) {
                T.b = (float*)take(4 * (size_t)n);
                T.dinv32 = (float*)take(4 * (size_t)n);
                continue;
            }
            const int nnz = a.L[l].rp[n], nn = a.L[l + 1].n;
            T.va32 = (float*)take(4 * (size_t)nnz);
            T.dinv32 = (float*)take(4 * (size_t)n);
            T.b = (float*)take(4 * (size_t)n);
            if (l > c) T.xp = (float*)take(4 * (size_t)n);
            if (l + 3 <= a.nlev) T.y = (float*)take(4 * (size_t)n);
            T.rp = (const int*)take(4 * (size_t)(n + 1));
            T.ci = (const int*)take(4 * (size_t)nnz);
            T.agg = (const int*)take(4 * (size_t)n);
            T.mem = (const int*)take(4 * (size_t)n);
            T.mp = (const int*)take(4 * (size_t)(nn + 1));
            T.tr = local_team(nn);
            T.tp = local_team(n);
        }
    }
    __syncthreads();
    for (int l = c; l < a.nlev; l++) {
        const AmgLevelDev& G = a.L[l];
        const AmgLevelDev& T = tl[l];
        const int n = G.n;
        for (int k = threadIdx.x; k < n; k += blockDim.x) T.dinv32[k] = G.dinv32[k];
        if (l == a.nlev - 1) continue;
        const int nnz = G.rp[n], nn = a.L[l + 1].n;
        for (int k = threadIdx.x; k < nnz; k += blockDim.x) {
            T.va32[k] = G.va32[k];
            const_cast<int*>(T.ci)[k] = G.ci[k];
        }
        for (int k = threadIdx.x; k <= n; k += blockDim.x) const_cast<int*>(T.rp)[k] = G.rp[k];
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const_cast<int*>(T.agg)[k] = G.agg[k];
            const_cast<int*>(T.mem)[k] = G.mem[k];
        }
        for (int k = threadIdx.x; k <= nn; k += blockDim.x) const_cast<int*>(T.mp)[k] = G.mp[k];
    }
    __syncthreads();
}

// block 0, each iteration: level c's restricted residual (and y) in, level c's
// correction out
__device__ __forceinline__ void tail_cycle(const AmgPcgArgs& a, int c, const AmgLevelDev* tl, float* xc,
                                           const float* sinv, float* sb)
{
    {
        const AmgLevelDev& T = tl[c];
        const AmgLevelDev& G = a.L[c];
        for (int k = threadIdx.x; k < T.n; k += blockDim.x) {
            T.b[k] = G.b[k];
            if (T.y) T.y[k] = G.y[k];
        }
    }
    __syncthreads();
    for (int l = c; l + 1 < a.nlev; l++) {
        restrict_level<true>(tl, l, c);
        __syncthreads();
    }
    for (int l = a.nlev - 2; l >= c; l--) {
        prolong_level<true>(tl, a.nlev, l, c, a.ys, xc, sinv, sb);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kAmgMaxThreads, 1) k_pcg_amg(const __grid_constant__ AmgPcgArgs a)
{
    cg::grid_group grid = cg::this_grid();
    extern __shared__ __align__(16) unsigned char tail_sm[];
    __shared__ double sh[40];
    __shared__ float xc[kCoarsest];
    __shared__ float sb[kCoarsest];
    __shared__ float sinv[kCoarsest * kCoarsest];  // the coarsest inverse, transposed
    __shared__ AmgLevelDev tl[kAmgMaxLevels];        // the block-local cycle's levels
    __shared__ int s_tail;
    const int nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    const AmgLevelDev& F = a.L[0];
    const int n = F.n;
    const bool jacobi = *a.overflow != 0;
    // three partial-sum regions, one per reduction of an iteration (rr, rz, pq):
    // a region is rewritten only after every block has passed the barrier that
    // follows its last read
    double* part_rr = a.part;
    double* part_rz = a.part + nb;
    double* part_pq = a.part + 2 * nb;
    double* rc = a.r0;  // current residual
    double* rn = a.r1;  // next residual
    float* rc32 = a.r32a;
    float* rn32 = a.r32b;

    if (threadIdx.x == 0) s_tail = jacobi ? 0 : tail_level(a);
    __syncthreads();
    const int tail = s_tail;  // first level of the block-local cycle, 0: none
    if (!jacobi && (tail == 0 || blockIdx.x == 0)) {  // the coarsest inverse, transposed
        const int cn = a.L[a.nlev - 1].n;
        for (int t = threadIdx.x; t < cn * cn; t += blockDim.x) sinv[(t % cn) * cn + t / cn] = (float)a.cinv[t];
    }
    if (!jacobi) {
        // the FP32 copies of the coarse levels' matrices
        for (int l = 1; l < a.nlev; l++) {
            const AmgLevelDev& A = a.L[l];
            const int nnz = A.rp[A.n];
            for (int k = tid; k < nnz; k += stride) A.va32[k] = to_f32(A.va[k]);
            for (int k = tid; k < A.n; k += stride) A.dinv32[k] = to_f32(A.dinv[k]);
        }
    }
    // x = 0, p = q = 0, r = b (active rows); the first pass below is a CG update
    // with alpha = 0
    for (int k = tid; k < n; k += stride) {
        a.xs[k] = 0.0;
        a.p[k] = 0.0;
        a.q[k] = 0.0;
        const double r = F.dinv[k] != 0.0 ? a.b[a.perm[k]] : 0.0;
        rc[k] = r;
        if (!jacobi) {
            F.dinv32[k] = to_f32(F.dinv[k]);
            rc32[k] = (float)r;
            a.q32[k] = 0.0f;
        }
    }
    grid.sync();
    if (tail > 0 && blockIdx.x == 0) tail_setup(a, tail, tl, tail_sm);
    double alpha = 0.0, rz = 0.0, rr = 0.0, bnorm = 0.0, tol = 0.0;
    int it = 0;
    for (;;) {
        // ---- x += alpha p, r -= alpha q (FP64), and in FP32 the fine residual of the
        // pre-smoothed correction, the neighbours' new residuals formed from the FP32
        // copies of r and q --------------------------------------------------------
        {
            double l_rr = 0.0;
            const float alpha32 = (float)alpha;
            for (int k = tid; k < n; k += stride) {
                const double rk = rc[k] - alpha * a.q[k];
                a.xs[k] += alpha * a.p[k];
                rn[k] = rk;
                l_rr += rk * rk;
                if (!jacobi) {
                    const float rk32 = (float)rk;
                    const float dk = F.dinv32[k];
                    rn32[k] = rk32;
                    a.ys[k] = dk != 0.0f ? kOmegaF * dk * rk32 : 0.0f;
                    float s = 0.0f;
                    if (dk != 0.0f) {
                        s = rk32;
                        const int b0 = F.sp[k >> 5] + (k & 31), w = (F.sp[(k >> 5) + 1] - F.sp[k >> 5]) >> 5;
#pragma unroll 4
                        for (int e = 0; e < w; e++) {
                            const int j = F.eci[b0 + 32 * e];
                            s -= F.eva32[b0 + 32 * e] * (kOmegaF * F.dinv32[j] * (rc32[j] - alpha32 * a.q32[j]));
                        }
                    }
                    a.s32[k] = s;
                }
            }
            const double t = amg_block_sum(l_rr, sh);
            if (threadIdx.x == 0) part_rr[blockIdx.x] = t;
        }
        grid.sync();
        {
            double* t = rc;
            rc = rn;
            rn = t;
            float* t32 = rc32;
            rc32 = rn32;
            rn32 = t32;
        }
        rr = amg_grid_total(part_rr, nb, sh);
        if (it == 0) {
            bnorm = sqrt(rr);
            tol = a.rtol * bnorm;
        }
        if (it >= a.maxiter || !(sqrt(rr) > tol)) break;
        // ---- z = M r -------------------------------------------------------------
        double l_rz = 0.0;
        if (jacobi) {
            for (int k = tid; k < n; k += stride) {
                const double zk = F.dinv[k] * rc[k];
                a.z[k] = zk;
                l_rz += zk * rc[k];
            }
        } else {
            restrict_fine(a, a.s32, tail);
            grid.sync();
            const int lr = tail > 0 ? tail : a.nlev - 1;  // grid-wide restrictions below lr
            for (int l = 1; l < lr; l++) {
                restrict_level<false>(a.L, l, tail);
                grid.sync();
            }
            if (tail > 0) {
                if (blockIdx.x == 0) tail_cycle(a, tail, tl, xc, sinv, sb);
                grid.sync();
            }
            for (int l = (tail > 0 ? tail - 1 : a.nlev - 2); l >= 1; l--) {
                prolong_level<false>(a.L, a.nlev, l, tail, a.ys, xc, sinv, sb);
                grid.sync();
            }
            if (a.nlev == 2) coarsest_solve(a.L[1], xc, sinv, sb);
            if (a.nlev > 2 && tail != 1) {
                // y, complete since the level-1 prolongation: one gather per entry
                for (int k = tid; k < n; k += stride) {
                    const float dk = F.dinv32[k];
                    float zk = 0.0f;
                    if (dk != 0.0f) {
                        float s = rc32[k];
                        const int b0 = F.sp[k >> 5] + (k & 31), w = (F.sp[(k >> 5) + 1] - F.sp[k >> 5]) >> 5;
#pragma unroll 4
                        for (int e = 0; e < w; e++) s -= F.eva32[b0 + 32 * e] * a.ys[F.eci[b0 + 32 * e]];
                        zk = a.ys[k] + kOmegaF * dk * s;
                    }
                    const double zd = (double)zk;
                    a.z[k] = zd;
                    l_rz += zd * rc[k];
                }
            } else {
                // two levels, or level 1 in the block-local cycle: the corrections of
                // level 1 (xc, or xp of level 1) gathered per entry
                for (int k = tid; k < n; k += stride) {
                    const float dk = F.dinv32[k];
                    float zk = 0.0f;
                    if (dk != 0.0f) {
                        const float yk =
                            kOmegaF * dk * rc32[k] + kCoarseScaleF * coarse_corr(a.L, a.nlev, 0, F.agg[k], xc);
                        float s = rc32[k];
                        const int b0 = F.sp[k >> 5] + (k & 31), w = (F.sp[(k >> 5) + 1] - F.sp[k >> 5]) >> 5;
#pragma unroll 4
                        for (int e = 0; e < w; e++) {
                            const int j = F.eci[b0 + 32 * e];
                            const float dj = F.dinv32[j];
                            const float yj = dj != 0.0f ? kOmegaF * dj * rc32[j] +
                                                              kCoarseScaleF * coarse_corr(a.L, a.nlev, 0, F.agg[j], xc)
                                                        : 0.0f;
                            s -= F.eva32[b0 + 32 * e] * yj;
                        }
                        zk = yk + kOmegaF * dk * s;
                    }
                    const double zd = (double)zk;
                    a.z[k] = zd;
                    l_rz += zd * rc[k];
                }
            }
        }
        {
            const double t = amg_block_sum(l_rz, sh);
            if (threadIdx.x == 0) part_rz[blockIdx.x] = t;
        }
        grid.sync();
        const double rz_new = amg_grid_total(part_rz, nb, sh);
        if (!(rz_new > 0.0)) break;
        const double beta = it == 0 ? 0.0 : rz_new / rz;
        rz = rz_new;
        // ---- p = z + beta p, q = A p (= A z + beta q) ------------------------------
        double l_pq = 0.0;
        for (int k = tid; k < n; k += stride) {
            double w = 0.0;
            if (F.dinv[k] != 0.0) {
                const int b0 = F.sp[k >> 5] + (k & 31), wd = (F.sp[(k >> 5) + 1] - F.sp[k >> 5]) >> 5;
#pragma unroll 4
                for (int e = 0; e < wd; e++) w += F.eva[b0 + 32 * e] * a.z[F.eci[b0 + 32 * e]];
            }
            const double pk = a.z[k] + beta * a.p[k];
            const double qk = w + beta * a.q[k];
            a.p[k] = pk;
            a.q[k] = qk;
            if (!jacobi) a.q32[k] = (float)qk;
            l_pq += pk * qk;
        }
        {
            const double t = amg_block_sum(l_pq, sh);
            if (threadIdx.x == 0) part_pq[blockIdx.x] = t;
        }
        grid.sync();
        const double pq = amg_grid_total(part_pq, nb, sh);
        if (!(pq > 0.0)) break;
        alpha = rz / pq;
        it++;
    }
    // the solution back in the rows of H
    for (int k = tid; k < n; k += stride) a.x[a.perm[k]] = a.xs[k];
    if (tid == 0) {
        a.out[0] = (double)it;
        a.out[1] = sqrt(rr);
        a.out[2] = bnorm;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int amg_levels(int n) { return n > kCoarsest ? 2 : 1; }

// Build the hierarchy for the Hessian in c->rowptr/col/val (n rows) and run the
// preconditioned CG.  Matrices of level l >= 1 never have more rows or entries than
// the fine one, so every level is sized by the fine level.
ma_status amg_pcg_solve(Ctx* c, int n, const double* b, double* x, double rtol, int maxiter, int reuse, int* iters,
                        double* relres)
{
    cudaStream_t s = c->stream;
    if (n <= kCoarsest) return MA_ERR_INVALID_ARGUMENT;
    Amg& G = c->amg;
    const size_t nnz = (size_t)(c->nnz > 0 ? c->nnz : 1);
    MA_CUDA(c, c->cg_r.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_z.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_p.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_q.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_dinv.ensure(sizeof(double) * n));
    MA_CUDA(c, c->cg_scal.ensure(sizeof(double) * 8));
    MA_CUDA(c, G.r1.ensure(sizeof(double) * n));
    MA_CUDA(c, G.xs.ensure(sizeof(double) * n));
    MA_CUDA(c, G.inv.ensure(sizeof(int) * n));
    MA_CUDA(c, G.cnt.ensure(sizeof(int) * (n + 2)));
    MA_CUDA(c, G.rp0.ensure(sizeof(int) * (n + 1)));
    MA_CUDA(c, G.ci0.ensure(sizeof(int) * nnz));
    MA_CUDA(c, G.va0.ensure(sizeof(double) * nnz));
    MA_CUDA(c, G.flag.ensure(sizeof(int) * 4));
    for (DevBuf* d : {&G.mate, &G.best, &G.claim, &G.mflag, &G.join, &G.agg1, &G.agg2, &G.mem1})
        MA_CUDA(c, d->ensure(sizeof(int) * (n + 1)));
    for (DevBuf* d : {&G.mid, &G.mp1, &G.mfill, &G.rp1}) MA_CUDA(c, d->ensure(sizeof(int) * (n + 2)));
    MA_CUDA(c, G.ci1.ensure(sizeof(int) * nnz));
    MA_CUDA(c, G.va1.ensure(sizeof(double) * nnz));
    MA_CUDA(c, G.dinv1.ensure(sizeof(double) * n));
    MA_CUDA(c, G.counts.ensure(sizeof(int) * 4));
    MA_CUDA(c, cudaMemsetAsync(G.flag.p, 0, sizeof(int) * 4, s));
    const int* perm = c->perm.as<int>();
    const unsigned g1 = (unsigned)((n + 255) / 256);
    ProfScope setup_scope(c, &c->profile.amg_setup_ms, nullptr);
    k_inv_perm<<<g1, 256, 0, s>>>(perm, n, G.inv.as<int>());
    k_fine_count<<<g1, 256, 0, s>>>(c->rowptr.as<int>(), perm, n, G.cnt.as<int>());
    launch_scan(G.cnt.as<int>(), G.rp0.as<int>(), n, c->scan_scratch.as<int>(), s);
    k_fine_fill<<<g1, 256, 0, s>>>(c->rowptr.as<int>(), c->col.as<int>(), c->val.as<double>(), perm,
                                   G.inv.as<int>(), n, G.rp0.as<int>(), G.ci0.as<int>(), G.va0.as<double>(),
                                   c->cg_dinv.as<double>());
    const int nslice = (n + 31) / 32;
    size_t ell_cap = nnz + 32 * (size_t)nslice * 8;  // grown below if a slice is wider
    MA_CUDA(c, G.sp.ensure(sizeof(int) * (nslice + 1)));
    k_sell_width<<<(unsigned)((nslice * 32 + 255) / 256), 256, 0, s>>>(G.rp0.as<int>(), n, G.cnt.as<int>());
    launch_scan(G.cnt.as<int>(), G.sp.as<int>(), nslice, c->scan_scratch.as<int>(), s);
    {
        int total = 0;
        MA_CUDA(c, cudaMemcpyAsync(&total, G.sp.as<int>() + nslice, sizeof(int), cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, ctx_sync(c));
        if ((size_t)total > ell_cap) ell_cap = (size_t)total;
    }
    MA_CUDA(c, G.eci.ensure(sizeof(int) * ell_cap));
    MA_CUDA(c, G.eva.ensure(sizeof(double) * ell_cap));
    MA_CUDA(c, G.eva32.ensure(sizeof(float) * ell_cap));
    k_sell_fill<<<g1, 256, 0, s>>>(G.rp0.as<int>(), G.ci0.as<int>(), G.va0.as<double>(), n, G.sp.as<int>(),
                                   G.eci.as<int>(), G.eva.as<double>(), G.eva32.as<float>());
    c->launches += 9;
    for (DevBuf* d : {&G.dinv32, &G.r32a, &G.r32b, &G.q32, &G.s32}) MA_CUDA(c, d->ensure(sizeof(float) * n));

    AmgPcgArgs a{};
    {
        AmgLevelDev& F = a.L[0];
        F.n = n;
        F.rp = G.rp0.as<int>();
        F.ci = G.ci0.as<int>();
        F.va = G.va0.as<double>();
        F.dinv = c->cg_dinv.as<double>();
        F.dinv32 = G.dinv32.as<float>();
        F.tr = F.tp = 1;
        F.sp = G.sp.as<int>();
        F.eci = G.eci.as<int>();
        F.eva = G.eva.as<double>();
        F.eva32 = G.eva32.as<float>();
    }
    // the level setup's cooperative grid: co-resident blocks, at most one row per thread
    int setup_max = 0, sms = 0;
    {
        int per_sm = 0;
        MA_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_level_setup, kSetupThreads, 0));
        MA_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
        setup_max = std::max(1, per_sm * sms / std::max(1, c->grid_share));
    }
    MA_CUDA(c, G.part.ensure(sizeof(int) * (size_t)setup_max));
    // the aggregates of the last hierarchy serve again for the same site index
    const bool keep = reuse && G.agg_epoch == c->index_epoch && G.agg_nlev >= 2 && G.agg_n[0] == n;
    if (!keep) G.agg_epoch = -1;  // the level buffers are about to change
    int nlev = 1;
    while (keep ? nlev < G.agg_nlev : (a.L[nlev - 1].n > kCoarsest && nlev < kAmgMaxLevels)) {
        const int l = nlev - 1;
        AmgLevelDev& A = a.L[l];
        AmgBuf& B = G.lev[l];  // this level's aggregates
        MA_CUDA(c, B.agg.ensure(sizeof(int) * (A.n + 1)));
        MA_CUDA(c, B.mem.ensure(sizeof(int) * (A.n + 1)));
        MA_CUDA(c, B.mp.ensure(sizeof(int) * (A.n + 2)));
        AmgBuf& Cb = G.lev[l + 1];  // the next level's matrix, sized by this level
        MA_CUDA(c, Cb.rp.ensure(sizeof(int) * (A.n + 2)));
        MA_CUDA(c, Cb.ci.ensure(sizeof(int) * nnz));
        MA_CUDA(c, Cb.va.ensure(sizeof(double) * nnz));
        MA_CUDA(c, Cb.dinv.ensure(sizeof(double) * A.n));
        MA_CUDA(c, Cb.b.ensure(sizeof(float) * A.n));
        MA_CUDA(c, Cb.xp.ensure(sizeof(float) * A.n));
        MA_CUDA(c, Cb.va32.ensure(sizeof(float) * nnz));
        MA_CUDA(c, Cb.dinv32.ensure(sizeof(float) * A.n));
        SetupArgs sa;
        sa.A = LevelCsr{A.n, A.rp, A.ci, A.va, A.dinv};
        sa.mate = G.mate.as<int>();
        sa.best = G.best.as<int>();
        sa.claim = G.claim.as<int>();
        sa.flag = G.mflag.as<int>();
        sa.id = G.mid.as<int>();
        sa.join = G.join.as<int>();
        sa.agg1 = G.agg1.as<int>();
        sa.agg2 = G.agg2.as<int>();
        sa.mp1 = G.mp1.as<int>();
        sa.mem1 = G.mem1.as<int>();
        sa.fill = G.mfill.as<int>();
        sa.cnt = G.cnt.as<int>();
        sa.rp1 = G.rp1.as<int>();
        sa.ci1 = G.ci1.as<int>();
        sa.va1 = G.va1.as<double>();
        sa.dinv1 = G.dinv1.as<double>();
        sa.part = G.part.as<int>();
        sa.counts = G.counts.as<int>();
        sa.agg = B.agg.as<int>();
        sa.mp = B.mp.as<int>();
        sa.mem = B.mem.as<int>();
        sa.rp = Cb.rp.as<int>();
        sa.ci = Cb.ci.as<int>();
        sa.va = Cb.va.as<double>();
        sa.dinv = Cb.dinv.as<double>();
        sa.overflow = G.flag.as<int>();
        sa.reuse = keep ? 1 : 0;
        sa.nc = keep ? G.agg_n[l + 1] : 0;
        // a thread per row for the matching; when only the Galerkin matrix is rebuilt, a
        // warp per coarse row instead (its grid has four barriers, not ~50)
        const int rows_blocks = (A.n + kSetupThreads - 1) / kSetupThreads;
        const int gal_blocks = keep ? (G.agg_n[l + 1] + kRowWarps - 1) / kRowWarps : 0;
        const int nbs = std::max(1, std::min(setup_max, std::max(rows_blocks, gal_blocks)));
        void* sargs[] = {&sa};
        MA_CUDA(c, cudaLaunchCooperativeKernel((void*)k_level_setup, dim3(nbs), dim3(kSetupThreads), sargs, 0, s));
        c->launches += 1;
        int nc = sa.nc;
        if (!keep) {  // the next level's size decides the next iteration
            MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 7, G.counts.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
            MA_CUDA(c, ctx_sync(c));
            nc = c->hinfo[7];
        }
        A.agg = B.agg.as<int>();
        A.mp = B.mp.as<int>();
        A.mem = B.mem.as<int>();
        {
            AmgLevelDev& C = a.L[l + 1];
            C = AmgLevelDev{};
            C.n = nc;
            C.rp = Cb.rp.as<int>();
            C.ci = Cb.ci.as<int>();
            C.va = Cb.va.as<double>();
            C.dinv = Cb.dinv.as<double>();
            C.va32 = Cb.va32.as<float>();
            C.dinv32 = Cb.dinv32.as<float>();
            C.b = Cb.b.as<float>();
            C.xp = Cb.xp.as<float>();
            C.tr = C.tp = 1;
        }
        nlev++;
    }
    if (a.L[nlev - 1].n > kCoarsest) {
        G.agg_epoch = -1;
        return fail(c, MA_ERR_CAPACITY, "multigrid coarsest level too large");
    }
    a.nlev = nlev;
    for (int l = 1; l + 3 <= nlev; l++) {  // levels whose corrections are materialised
        MA_CUDA(c, G.lev[l].y.ensure(sizeof(float) * (size_t)a.L[l].n));
        a.L[l].y = G.lev[l].y.as<float>();
    }
    if (!keep) {
        G.agg_epoch = c->index_epoch;
        G.agg_nlev = nlev;
        for (int l = 0; l < nlev; l++) G.agg_n[l] = a.L[l].n;
    }
    const AmgLevelDev& C = a.L[nlev - 1];
    MA_CUDA(c, G.cinv.ensure(sizeof(double) * kCoarsest * kCoarsest));
    k_dense_inverse<<<1, 256, 0, s>>>(C.rp, C.ci, C.va, C.dinv, C.n, G.cinv.as<double>());
    c->launches += 1;
    setup_scope.end();
    c->profile.amg_levels = nlev;

    // the co-resident grid: kWideBlocksPerSm blocks of kWideThreads per SM, the rest of
    // the SM's shared memory split between them for the block-local coarse cycle
    // (512 x 2 measured faster than 1024 x 1 and 256 x 4 on 100,000 sites); a batch
    // worker, which shares the GPU with the other workers' kernels, launches blocks of
    // kShareThreads, up to kShareBlocksPerSm of them on an SM, and a cycle sized to match
    constexpr int kWideThreads = 512, kWideBlocksPerSm = 2;
    constexpr int kShareThreads = 256, kShareBlocksPerSm = 4;
    const bool shared_gpu = c->grid_share > 1;
    const int bthreads = shared_gpu ? kShareThreads : kWideThreads;
    const int bps = shared_gpu ? kShareBlocksPerSm : kWideBlocksPerSm;
    int max_blocks = 0, dyn = 0;
    {
        int per_sm = 0, sms = 0, sm_bytes = 0, optin = 0;
        cudaFuncAttributes fa;
        MA_CUDA(c, cudaFuncGetAttributes(&fa, k_pcg_amg));
        MA_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
        MA_CUDA(c, cudaDeviceGetAttribute(&sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device));
        MA_CUDA(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
        // each resident block also takes 1 KB that the system reserves
        dyn = sm_bytes / bps - 1024 - (int)fa.sharedSizeBytes;
        dyn = std::min(dyn, optin - (int)fa.sharedSizeBytes);
        dyn = std::max(0, dyn) & ~15;
        // the attribute at the largest size any launch asks for, so that contexts with
        // different launch shapes never race on it
        MA_CUDA(c, cudaFuncSetAttribute(k_pcg_amg, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        std::max(0, optin - (int)fa.sharedSizeBytes)));
        MA_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_amg, bthreads, dyn));
        if (per_sm < 1) return fail(c, MA_ERR_CUDA, "the multigrid PCG kernel does not fit an SM");
        max_blocks = std::min(per_sm, bps) * sms;
        // a batch worker leaves the rest of the GPU to the other workers' problems
        if (shared_gpu) max_blocks = std::max(1, max_blocks / c->grid_share);
    }
    int want = (n + bthreads / 4 - 1) / (bthreads / 4);
    int nb = want < max_blocks ? want : max_blocks;
    if (nb < 1) nb = 1;
    MA_CUDA(c, c->cg_part.ensure(sizeof(double) * 3 * nb));
    // lanes per coarse row: enough teams to cover the level with the launched grid
    const int threads = nb * bthreads;
    auto team = [&](int rows) {
        int t = 1;
        while (t < 32 && (int64_t)rows * t * 2 <= threads) t <<= 1;
        return t;
    };
    a.L[0].tr = team(a.L[1].n);
    for (int l = 1; l < nlev; l++) {
        a.L[l].tp = team(a.L[l].n);
        if (l + 1 < nlev) a.L[l].tr = team(a.L[l + 1].n);
    }
    a.perm = perm;
    a.cinv = G.cinv.as<double>();
    a.b = b;
    a.x = x;
    a.xs = G.xs.as<double>();
    a.r0 = c->cg_r.as<double>();
    a.r1 = G.r1.as<double>();
    a.z = c->cg_z.as<double>();
    a.p = c->cg_p.as<double>();
    a.q = c->cg_q.as<double>();
    MA_CUDA(c, G.ys.ensure(sizeof(float) * n));
    a.ys = G.ys.as<float>();
    a.r32a = G.r32a.as<float>();
    a.r32b = G.r32b.as<float>();
    a.q32 = G.q32.as<float>();
    a.s32 = G.s32.as<float>();
    a.part = c->cg_part.as<double>();
    a.out = c->cg_scal.as<double>();
    a.rtol = rtol;
    a.maxiter = maxiter;
    a.overflow = G.flag.as<int>();
    a.tail_bytes = dyn;
    void* args[] = {&a};
    {
        ProfScope ps(c, &c->profile.pcg_ms, &c->profile.pcg_launches);
        MA_CUDA(c, cudaLaunchCooperativeKernel((void*)k_pcg_amg, dim3(nb), dim3(bthreads), args, (size_t)dyn, s));
    }
    c->launches += 1;
    MA_CUDA(c, cudaMemcpyAsync(c->hstat + 8, c->cg_scal.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 6, G.flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, ctx_sync(c));
    if (iters) *iters = (int)c->hstat[8];
    c->profile.pcg_iters += (int64_t)c->hstat[8];
    if (c->hinfo[6]) c->profile.amg_fallbacks++;
    if (relres) *relres = c->hstat[10] > 0 ? c->hstat[9] / c->hstat[10] : 0.0;
    return MA_OK;
}

}  // namespace ma
