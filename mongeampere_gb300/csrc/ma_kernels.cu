// ma_kernels.cu -- device kernels of the Laguerre-cell engine.
//
//  K0  bounding box of the sites, weight refresh of the sorted sites, scans.
//  (the cell kernels themselves are in ma_cells.cu)
//  K3  deterministic reductions (value, total mass, min mass, residual norms).
//  K4  CSR compaction of the per-row staging.
#include <cfloat>

#include "ma_internal.h"

namespace ma {

// ---------------------------------------------------------------------------
// ordered keys: unsigned order == double order
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long dkey(double d)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k)
{
    unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

template <class Op>
__device__ __forceinline__ unsigned long long block_reduce_key(unsigned long long v, Op op)
{
    __shared__ unsigned long long sh[32];
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    if (wid == 0) {
        v = (lane < nw) ? sh[lane] : sh[0];
        for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

struct KMin {
    __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a < b ? a : b; }
};
struct KMax {
    __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const { return a > b ? a : b; }
};

// keys: [min x, max x, min y, max y, max w] (caller initialises mins to ~0, maxes to 0)
__global__ void k_bbox(const double* x, const double* y, const double* w, int n, unsigned long long* keys)
{
    unsigned long long mnx = ~0ull, mxx = 0, mny = ~0ull, mxy = 0, mxw = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned long long kx = dkey(x[i]), ky = dkey(y[i]);
        mnx = min(mnx, kx);
        mxx = max(mxx, kx);
        mny = min(mny, ky);
        mxy = max(mxy, ky);
        if (w) mxw = max(mxw, dkey(w[i]));
    }
    mnx = block_reduce_key(mnx, KMin());
    mxx = block_reduce_key(mxx, KMax());
    mny = block_reduce_key(mny, KMin());
    mxy = block_reduce_key(mxy, KMax());
    mxw = block_reduce_key(mxw, KMax());
    if (threadIdx.x == 0) {
        atomicMin(&keys[0], mnx);
        atomicMax(&keys[1], mxx);
        atomicMin(&keys[2], mny);
        atomicMax(&keys[3], mxy);
        if (w) atomicMax(&keys[4], mxw);
    }
}

void launch_bbox(const double* x, const double* y, const double* w, int n, unsigned long long* keys,
                 cudaStream_t s)
{
    int b = 256, g = (n + b - 1) / b;
    if (g > 1216) g = 1216;
    if (g < 1) g = 1;
    k_bbox<<<g, b, 0, s>>>(x, y, w, n, keys);
}

__global__ void k_key_to_double(const unsigned long long* key, double* out, int count)
{
    int i = threadIdx.x;
    if (i < count) out[i] = dkey_inv(key[i]);
}

void launch_key_to_double(const unsigned long long* key, double* out, int count, cudaStream_t s)
{
    k_key_to_double<<<1, 32, 0, s>>>(key, out, count);
}

__global__ void k_update_weights(const double* w, const int* perm, int n, SiteD* sites)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    sites[k].w = w[perm[k]];
}

void launch_update_weights(const double* w, const int* perm, int n, SiteD* sites, cudaStream_t s)
{
    k_update_weights<<<(n + 255) / 256, 256, 0, s>>>(w, perm, n, sites);
}

// ---------------------------------------------------------------------------
// exclusive scan
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_scan_tile(const int* in, int* out, int n, int* sums)
{
    __shared__ int sh[kScanThreads];
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int tsum = 0;
    for (int j = 0; j < kScanItems; j++) {
        int idx = base + j;
        v[j] = (idx < n) ? in[idx] : 0;
        tsum += v[j];
    }
    sh[threadIdx.x] = tsum;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
        int t = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    int run = sh[threadIdx.x] - tsum;
    for (int j = 0; j < kScanItems; j++) {
        int idx = base + j;
        if (idx < n) out[idx] = run;
        run += v[j];
    }
    if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void k_scan_add(int* out, int n, const int* sums)
{
    int base = blockIdx.x * kScanTile;
    int add = sums[blockIdx.x];
    for (int j = threadIdx.x; j < kScanTile; j += blockDim.x) {
        int idx = base + j;
        if (idx < n) out[idx] += add;
    }
}

__global__ void k_scan_total(const int* in, int* out, int n)
{
    // out[n] = out[n-1] + in[n-1]
    out[n] = (n > 0) ? out[n - 1] + in[n - 1] : 0;
}

size_t scan_scratch_ints(int n)
{
    size_t tot = 0;
    int m = n;
    while (true) {
        int nb = (m + kScanTile - 1) / kScanTile;
        tot += 2 * (size_t)nb + 1;  // block sums + their scan (nb + 1)
        if (nb <= 1) break;
        m = nb;
    }
    return tot + 16;
}

static void scan_rec(const int* in, int* out, int n, int* scratch, cudaStream_t s)
{
    int nb = (n + kScanTile - 1) / kScanTile;
    if (nb < 1) nb = 1;
    int* sums = scratch;
    k_scan_tile<<<nb, kScanThreads, 0, s>>>(in, out, n, sums);
    if (nb > 1) {
        int* sums_scanned = scratch + nb;
        // the scanned sums (exclusive) into sums_scanned[0..nb]
        scan_rec(sums, sums_scanned, nb, scratch + 2 * nb + 1, s);
        k_scan_add<<<nb, 256, 0, s>>>(out, n, sums_scanned);
    }
}

void launch_scan(const int* in, int* out, int n, int* scratch, cudaStream_t s)
{
    if (n > 0) scan_rec(in, out, n, scratch, s);
    k_scan_total<<<1, 1, 0, s>>>(in, out, n);
}

// ---------------------------------------------------------------------------
// K4: CSR compaction
// ---------------------------------------------------------------------------
__global__ void k_csr_compact(int n, const int* rowptr, const int* rowcnt, const int* st_col, const double* st_val,
                              int scap, const int* big_index, const int* big_col, const double* big_val, int big_cap,
                              int* col, double* val)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = rowcnt[i], o = rowptr[i];
    int b = big_index[i];
    const int* sc = b >= 0 ? big_col + (size_t)b * big_cap : st_col + (size_t)i * scap;
    const double* sv = b >= 0 ? big_val + (size_t)b * big_cap : st_val + (size_t)i * scap;
    for (int j = 0; j < c; j++) {
        col[o + j] = sc[j];
        val[o + j] = sv[j];
    }
}

void launch_csr_compact(int n, const int* rowptr, const int* rowcnt, const int* st_col, const double* st_val,
                        int scap, const int* big_index, const int* big_col, const double* big_val, int big_cap,
                        int* col, double* val, cudaStream_t s)
{
    k_csr_compact<<<(n + 255) / 256, 256, 0, s>>>(n, rowptr, rowcnt, st_col, st_val, scap, big_index, big_col,
                                                  big_val, big_cap, col, val);
}

// ---------------------------------------------------------------------------
// K3: deterministic statistics
// ---------------------------------------------------------------------------
constexpr int kStatThreads = 256;
constexpr int kStatItems = 8;

int stats_blocks(int n)
{
    int per = kStatThreads * kStatItems;
    int b = (n + per - 1) / per;
    return b < 1 ? 1 : b;
}

struct Stat5 {
    double f, sm, mn, sq, mr;
};

__device__ __forceinline__ Stat5 st_comb(Stat5 a, Stat5 b)
{
    return Stat5{a.f + b.f, a.sm + b.sm, fmin(a.mn, b.mn), a.sq + b.sq, fmax(a.mr, b.mr)};
}

__device__ Stat5 block_reduce_stat(Stat5 v)
{
    __shared__ double sh[5][kStatThreads];
    sh[0][threadIdx.x] = v.f;
    sh[1][threadIdx.x] = v.sm;
    sh[2][threadIdx.x] = v.mn;
    sh[3][threadIdx.x] = v.sq;
    sh[4][threadIdx.x] = v.mr;
    __syncthreads();
    for (int off = kStatThreads / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            int o = threadIdx.x + off;
            sh[0][threadIdx.x] += sh[0][o];
            sh[1][threadIdx.x] += sh[1][o];
            sh[2][threadIdx.x] = fmin(sh[2][threadIdx.x], sh[2][o]);
            sh[3][threadIdx.x] += sh[3][o];
            sh[4][threadIdx.x] = fmax(sh[4][threadIdx.x], sh[4][o]);
        }
        __syncthreads();
    }
    Stat5 r{sh[0][0], sh[1][0], sh[2][0], sh[3][0], sh[4][0]};
    __syncthreads();
    return r;
}

__global__ void k_stats(const double* mass, const double* vpart, const double* nu, const double* w, int n,
                        double* partial)
{
    Stat5 acc{0.0, 0.0, INFINITY, 0.0, 0.0};
    int base = blockIdx.x * kStatThreads * kStatItems;
    for (int j = 0; j < kStatItems; j++) {
        int i = base + j * kStatThreads + threadIdx.x;
        if (i < n) {
            double m = mass[i];
            double f = vpart[i];
            Stat5 e{f, m, m, 0.0, 0.0};
            if (nu) {
                double r = m - nu[i];
                e.f = f - nu[i] * w[i];
                e.sq = r * r;
                e.mr = fabs(r) / nu[i];
            }
            acc = st_comb(acc, e);
        }
    }
    Stat5 r = block_reduce_stat(acc);
    if (threadIdx.x == 0) {
        int nb = gridDim.x;
        partial[blockIdx.x] = r.f;
        partial[nb + blockIdx.x] = r.sm;
        partial[2 * nb + blockIdx.x] = r.mn;
        partial[3 * nb + blockIdx.x] = r.sq;
        partial[4 * nb + blockIdx.x] = r.mr;
    }
}

__global__ void k_stats_final(const double* partial, int nb, double* out)
{
    Stat5 acc{0.0, 0.0, INFINITY, 0.0, 0.0};
    for (int b = threadIdx.x; b < nb; b += kStatThreads)
        acc = st_comb(acc, Stat5{partial[b], partial[nb + b], partial[2 * nb + b], partial[3 * nb + b],
                                 partial[4 * nb + b]});
    Stat5 r = block_reduce_stat(acc);
    if (threadIdx.x == 0) {
        out[0] = r.f;
        out[1] = r.sm;
        out[2] = r.mn;
        out[3] = sqrt(r.sq);
        out[4] = r.mr;
    }
}

void launch_stats(const double* mass, const double* vpart, const double* nu, const double* w, int n,
                  double* partial, int nblocks, double* out, cudaStream_t s)
{
    k_stats<<<nblocks, kStatThreads, 0, s>>>(mass, vpart, nu, w, n, partial);
    k_stats_final<<<1, kStatThreads, 0, s>>>(partial, nblocks, out);
}

}  // namespace ma
