// ma_kernels.cu -- device kernels of the Laguerre-cell engine.
//
//  K0  site grid: bounding box, cell keys, counting sort (scan + scatter), a
//      per-cell index sort that makes the order deterministic, and the gather of
//      (x, y, w) into cell order.
//  K1+K2  one thread per site: Laguerre cell by clipping against sites of the
//      grid in rings around it until the security radius certifies the cell,
//      then the cell's intersection with every mesh triangle it touches, with
//      closed-form FP64 integrals and the Hessian row.
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
// mesh visitors: enumerate the triangles that may meet a box
// ---------------------------------------------------------------------------

// largest i in [0, n-2] with g[i] <= x (clamped)
__device__ __forceinline__ int find_square(const double* g, int n, double x)
{
    if (!(x > g[0])) return 0;
    if (x >= g[n - 1]) return n - 2;
    int lo = 0, hi = n - 2;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (g[mid] <= x)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

struct GridVisitor {
    MeshGridDev m;
    template <class Fn>
    __device__ __forceinline__ void visit(const Owner& o, double bx0, double by0, double bx1, double by1,
                                          Fn&& fn) const
    {
        if (bx1 < m.gx[0] || bx0 > m.gx[m.nx - 1] || by1 < m.gy[0] || by0 > m.gy[m.ny - 1]) return;
        int i0 = find_square(m.gx, m.nx, bx0), i1 = find_square(m.gx, m.nx, bx1);
        int j0 = find_square(m.gy, m.ny, by0), j1 = find_square(m.gy, m.ny, by1);
        Fixed T;
        T.n = 3;
        for (int j = j0; j <= j1; j++) {
            double Y0 = m.gy[j], Y1 = m.gy[j + 1], ihy = m.ihy[j];
            const double* row0 = m.val + (size_t)j * m.nx;
            const double* row1 = row0 + m.nx;
            for (int i = i0; i <= i1; i++) {
                double X0 = m.gx[i], X1 = m.gx[i + 1], ihx = m.ihx[i];
                double v00 = row0[i], v10 = row0[i + 1], v01 = row1[i], v11 = row1[i + 1];
                // lower triangle (i,j), (i+1,j), (i+1,j+1)
                set_fixed(T, 0, X0, Y0, o);
                set_fixed(T, 1, X1, Y0, o);
                set_fixed(T, 2, X1, Y1, o);
                {
                    double gx = (v10 - v00) * ihx, gy = (v11 - v10) * ihy;
                    double c0 = v00 - gx * T.rx[0] - gy * T.ry[0];
                    fn(T, c0, gx, gy);
                }
                // upper triangle (i,j), (i+1,j+1), (i,j+1)
                set_fixed(T, 1, X1, Y1, o);
                set_fixed(T, 2, X0, Y1, o);
                {
                    double gx = (v11 - v01) * ihx, gy = (v01 - v00) * ihy;
                    double c0 = v00 - gx * T.rx[0] - gy * T.ry[0];
                    fn(T, c0, gx, gy);
                }
            }
        }
    }
};

struct TriVisitor {
    MeshTriDev m;
    template <class Fn>
    __device__ __forceinline__ void visit(const Owner& o, double bx0, double by0, double bx1, double by1,
                                          Fn&& fn) const
    {
        int cx0 = (int)floor((bx0 - m.bx0) / m.bcw), cx1 = (int)floor((bx1 - m.bx0) / m.bcw);
        int cy0 = (int)floor((by0 - m.by0) / m.bch), cy1 = (int)floor((by1 - m.by0) / m.bch);
        if (cx1 < 0 || cy1 < 0 || cx0 >= m.bnx || cy0 >= m.bny) return;
        cx0 = max(cx0, 0);
        cy0 = max(cy0, 0);
        cx1 = min(cx1, m.bnx - 1);
        cy1 = min(cy1, m.bny - 1);
        Fixed T;
        T.n = 3;
        for (int by = cy0; by <= cy1; by++) {
            for (int bx = cx0; bx <= cx1; bx++) {
                int b = by * m.bnx + bx;
                for (int q = m.bin_start[b]; q < m.bin_start[b + 1]; q++) {
                    int t = m.bin_tri[q];
                    int4 r = m.tbin[t];
                    // visit each triangle once: from the first bin shared with the box
                    if (bx != max(r.x, cx0) || by != max(r.y, cy0)) continue;
                    int a0 = m.tri[3 * t], a1 = m.tri[3 * t + 1], a2 = m.tri[3 * t + 2];
                    set_fixed(T, 0, m.vx[a0], m.vy[a0], o);
                    set_fixed(T, 1, m.vx[a1], m.vy[a1], o);
                    set_fixed(T, 2, m.vx[a2], m.vy[a2], o);
                    double l0 = m.lin[3 * t], gx = m.lin[3 * t + 1], gy = m.lin[3 * t + 2];
                    double c0 = l0 - gx * T.rx[0] - gy * T.ry[0];
                    fn(T, c0, gx, gy);
                }
            }
        }
    }
};

// ---------------------------------------------------------------------------
// K1 + K2: one Laguerre cell per thread
// ---------------------------------------------------------------------------

// per-site workspace: a local variable in the main kernel, a slice of global
// scratch in the large-capacity kernel
template <int CAP>
struct Work {
    Slot slots[CAP];
    Poly<CAP> PA, PB;
    double hv[CAP];
    Nb64 nb[CAP];
    int map[CAP];
    int cols[CAP];
    double vals[CAP];
};

template <int CAP>
__device__ __forceinline__ void compact_slots(Poly<CAP>& P, Slot* slots, int* map, int& ns)
{
    Bits<CAP> used;
    used.clear();
    for (int e = 0; e < P.n; e++)
        if (P.lab[e] >= 0) used.set(P.lab[e]);
    int m = 0;
    for (int s = 0; s < ns; s++) {
        if (used.get(s)) {
            map[s] = m;
            if (m != s) slots[m] = slots[s];
            m++;
        } else {
            map[s] = -1;
        }
    }
    for (int e = 0; e < P.n; e++)
        if (P.lab[e] >= 0) P.lab[e] = map[P.lab[e]];
    ns = m;
}

// Can no site of internal node nd cut polygon P?  With phi_j >= alpha + beta.x_j
// over the node and the node's box [c - h, c + h]:
//   pi_ij(p) / 2 = p.(x_j - x_i) + phi_i - phi_j
//              <= (p - beta).(c - x_i) + |p_x - beta_x| h_x + |p_y - beta_y| h_y - K,
//   K = alpha + beta.x_i - phi_i,
// convex in p, so it suffices that it is negative at every vertex of P.  FP64
// node terms, FP32 per-vertex loop with a bound on every rounding and on the
// vertex radii.
template <int CAP>
__device__ __forceinline__ bool node_harmless(const Poly<CAP>& P, const Owner& o, double phi_o, const double4 bx,
                                              const double4 ab)
{
    if (!(ab.x > -INFINITY)) return false;
    double ex = o.x - ab.y, ey = o.y - ab.z;
    double cx = 0.5 * (bx.x + bx.z) - o.x, cy = 0.5 * (bx.y + bx.w) - o.y;
    double hx = 0.5 * (bx.z - bx.x), hy = 0.5 * (bx.w - bx.y);
    double t1 = ab.y * o.x, t2 = ab.z * o.y;
    double K = ab.x + t1 + t2 - phi_o;
    double kerr = 1e-15 * (fabs(ab.x) + fabs(t1) + fabs(t2) + fabs(phi_o));
    double cerr = 1e-15 * (fabs(bx.x) + fabs(bx.z) + fabs(bx.y) + fabs(bx.w) + fabs(o.x) + fabs(o.y));
    float fex = (float)ex, fey = (float)ey, fcx = (float)cx, fcy = (float)cy;
    float fhx = (float)hx * 1.000001f + 1e-38f, fhy = (float)hy * 1.000001f + 1e-38f;
    float fK = (float)K, fke = (float)kerr * 1.0001f, fce = (float)cerr * 1.0001f;
    float L = fabsf(fcx) + fabsf(fcy) + fhx + fhy;
    float e0 = 1.2e-7f * (fabsf(fex) + fabsf(fey));
    for (int v = 0; v < P.n; v++) {
        float qx = fex + P.ux[v], qy = fey + P.uy[v];
        float T = qx * fcx + qy * fcy + fabsf(qx) * fhx + fabsf(qy) * fhy - fK;
        float S = fabsf(qx * fcx) + fabsf(qy * fcy) + fabsf(qx) * fhx + fabsf(qy) * fhy + fabsf(fK);
        float err = 1e-6f * S + (P.ur[v] + e0) * L * 1.0001f + fke + (fabsf(qx) + fabsf(qy)) * fce + 1e-36f;
        if (!(T + err < 0.0f)) return false;
    }
    return true;
}

template <int CAP, bool MOM, class Mesh>
__device__ void process_site(const CellArgs& A, const Mesh& M, int k, Work<CAP>& W, int big_slot)
{
    const SiteD S = A.sites[k];
    const int gi = A.perm[k];
    Owner o{S.x, S.y, S.w, k};
    uint32_t st = 0;
    bool overflow = false;
    bool empty = false;

    Slot* slots = W.slots;
    int ns = 0;
    Poly<CAP>* P = &W.PA;
    Poly<CAP>* Q = &W.PB;

    Fixed box;
    box.n = 4;
    set_fixed(box, 0, A.X0, A.Y0, o);
    set_fixed(box, 1, A.X1, A.Y0, o);
    set_fixed(box, 2, A.X1, A.Y1, o);
    set_fixed(box, 3, A.X0, A.Y1, o);
    P->n = 4;
    for (int e = 0; e < 4; e++) {
        P->lab[e] = -1 - e;
        P->ux[e] = box.ux[e];
        P->uy[e] = box.uy[e];
        P->ur[e] = box.ur[e];
    }
    if (!(isfinite(S.x) && isfinite(S.y) && isfinite(S.w))) {
        st |= ST_BAD_INPUT;
        empty = true;
    }

    // ---------------- cell stage: branch and bound over the site tree ----------------
    {
        const SiteTree& T = A.tree;
        const double phi_o = 0.5 * (S.x * S.x + S.y * S.y - S.w);
        const float ox = (float)S.x, oy = (float)S.y;
        constexpr int kStack = 80;
        constexpr int kBucket = 8;
        int stack[kStack];
        int sp = 0;
        if (T.n >= 2 && !empty) stack[sp++] = 0;
        auto visit = [&](int q) -> bool {  // clip by sorted site q; false when the cell became empty
            if (q == k) return true;
            const SiteD C = A.sites[q];
            if (C.x == S.x && C.y == S.y) {
                // coincident sites: the larger weight, then the lower index, keeps the cell
                int gj = A.perm[q];
                if (C.w > S.w || (C.w == S.w && gj < gi)) return false;
                return true;
            }
            if (ns == CAP) {
                compact_slots(*P, slots, W.map, ns);
                if (ns == CAP) {
                    overflow = true;
                    return true;
                }
            }
            slots[ns] = make_slot(q, C, o);
            if (clip_poly(*P, *Q, ns, slots, box, o, A.sites, st, overflow)) {
                if (overflow) return true;
                Poly<CAP>* t = P;
                P = Q;
                Q = t;
                ns++;
                if (P->n == 0) return false;
            }
            return true;
        };
        auto dist2 = [&](int c) -> float {
            if (c < 0) {
                float2 p = T.posf[c & 0x7fffffff];
                float dx = p.x - ox, dy = p.y - oy;
                return dx * dx + dy * dy;
            }
            float4 b = T.boxf[c];
            float dx = fmaxf(fmaxf(b.x - ox, ox - b.z), 0.0f), dy = fmaxf(fmaxf(b.y - oy, oy - b.w), 0.0f);
            return dx * dx + dy * dy;
        };
        while (sp > 0 && !empty && !overflow) {
            int nd = stack[--sp];
            if (nd < 0) {
                if (!visit(nd & 0x7fffffff)) empty = true;
                continue;
            }
            int2 rg = T.range[nd];
            bool contains = rg.x <= k && k <= rg.y;
            if (!contains && node_harmless(*P, o, phi_o, T.box[nd], T.ab[nd])) continue;
            if (rg.y - rg.x < kBucket) {
                for (int q = rg.x; q <= rg.y && !empty && !overflow; q++)
                    if (!visit(q)) empty = true;
                continue;
            }
            int2 ch = T.child[nd];
            if (sp > kStack - 2) {
                overflow = true;
                break;
            }
            // nearer child on top
            if (dist2(ch.x) <= dist2(ch.y)) {
                stack[sp++] = ch.y;
                stack[sp++] = ch.x;
            } else {
                stack[sp++] = ch.x;
                stack[sp++] = ch.y;
            }
        }
        if (empty) P->n = 0;
    }

    if (overflow) {
        if (A.redo) {
            int p = atomicAdd(A.nredo, 1);
            A.redo[p] = k;
        }
        atomicOr(A.status, ST_POLY_OVERFLOW);
        return;
    }

    Acc acc{0, 0, 0, 0, 0, 0, 0};
    double* hv = W.hv;
    Nb64* nb = W.nb;
    Bits<CAP> touched;
    touched.clear();
    int m = 0;
    if (!empty && P->n > 0) {
        compact_slots(*P, slots, W.map, ns);
        m = ns;
        for (int s = 0; s < m; s++) {
            nb[s] = make_nb64(A.sites[slots[s].site], o);
            hv[s] = 0.0;
        }
        // cell bounding box (absolute, conservative)
        float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
        for (int e = 0; e < P->n; e++) {
            float r = P->ur[e] * 1.0001f;
            mnx = fminf(mnx, P->ux[e] - r);
            mxx = fmaxf(mxx, P->ux[e] + r);
            mny = fminf(mny, P->uy[e] - r);
            mxy = fmaxf(mxy, P->uy[e] + r);
        }
        double sx = fmax(fabs((double)mnx), fabs((double)mxx)), sy = fmax(fabs((double)mny), fabs((double)mxy));
        double bx0 = S.x + (double)mnx - 1e-6 * sx - 1e-300, bx1 = S.x + (double)mxx + 1e-6 * sx + 1e-300;
        double by0 = S.y + (double)mny - 1e-6 * sy - 1e-300, by1 = S.y + (double)mxy + 1e-6 * sy + 1e-300;
        if (!(mxx - mnx < INFINITY && mxy - mny < INFINITY)) {
            bx0 = A.X0;
            bx1 = A.X1;
            by0 = A.Y0;
            by1 = A.Y1;
        }

        // ---------------- triangle stage ----------------
        Poly<CAP>* Wp = P;
        Poly<CAP>* Vp = Q;
        M.visit(o, bx0, by0, bx1, by1, [&](const Fixed& T, double c0, double gx, double gy) {
            if (overflow) return;
            Wp->n = 3;
            for (int e = 0; e < 3; e++) {
                Wp->lab[e] = -1 - e;
                Wp->ux[e] = T.ux[e];
                Wp->uy[e] = T.uy[e];
                Wp->ur[e] = T.ur[e];
            }
            for (int s = 0; s < m; s++) {
                if (clip_poly(*Wp, *Vp, s, slots, T, o, A.sites, st, overflow)) {
                    if (overflow) return;
                    Poly<CAP>* t = Wp;
                    Wp = Vp;
                    Vp = t;
                    if (Wp->n == 0) return;
                }
            }
            integrate_piece<CAP, MOM>(*Wp, nb, T, c0, gx, gy, acc, hv, touched);
        });
        if (overflow) {
            if (A.redo) {
                int p = atomicAdd(A.nredo, 1);
                A.redo[p] = k;
            }
            atomicOr(A.status, ST_POLY_OVERFLOW);
            return;
        }
    }

    // ---------------- outputs ----------------
    A.mass[gi] = acc.mass;
    A.vpart[gi] = S.w * acc.mass - acc.second;
    if (MOM && A.mom) {
        double* mo = A.mom + 6 * (size_t)gi;
        mo[0] = acc.mass;
        mo[1] = acc.m1x + S.x * acc.mass;
        mo[2] = acc.m1y + S.y * acc.mass;
        mo[3] = 0.0;
        mo[4] = 0.0;
        mo[5] = 0.0;
    }
    if (A.rowcnt) {
        // off-diagonal entries sorted by original index, diagonal in place
        int* cols = W.cols;
        double* vals = W.vals;
        int cnt = 0;
        double diag = 0.0;
        for (int s = 0; s < m; s++) {
            if (!touched.get(s)) continue;
            double d2 = nb[s].dx * nb[s].dx + nb[s].dy * nb[s].dy;
            double v = -hv[s] / (2.0 * d2);
            diag -= v;
            int c = A.perm[slots[s].site];
            int j = cnt - 1;
            while (j >= 0 && cols[j] > c) {
                cols[j + 1] = cols[j];
                vals[j + 1] = vals[j];
                j--;
            }
            cols[j + 1] = c;
            vals[j + 1] = v;
            cnt++;
        }
        int total = cnt > 0 ? cnt + 1 : 0;
        A.rowcnt[gi] = total;
        int* oc;
        double* ov;
        if (big_slot >= 0) {
            // large rows go to the side buffer of the large-capacity pass
            oc = A.big_col + (size_t)big_slot * A.big_cap;
            ov = A.big_val + (size_t)big_slot * A.big_cap;
            A.big_index[gi] = big_slot;
        } else {
            oc = A.st_col + (size_t)gi * A.scap;
            ov = A.st_val + (size_t)gi * A.scap;
        }
        if (total > 0) {
            int w = 0;
            bool placed = false;
            for (int j = 0; j < cnt; j++) {
                if (!placed && cols[j] > gi) {
                    oc[w] = gi;
                    ov[w] = diag;
                    w++;
                    placed = true;
                }
                oc[w] = cols[j];
                ov[w] = vals[j];
                w++;
            }
            if (!placed) {
                oc[w] = gi;
                ov[w] = diag;
            }
        }
    }
    if (st) atomicOr(A.status, st);
}

constexpr int kCapSmall = 48;
constexpr int kCapLarge = 256;

template <int CAP, bool MOM, class Mesh>
__global__ void __launch_bounds__(128) k_cells_small(CellArgs A, Mesh M)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.n) return;
    Work<CAP> W;
    process_site<CAP, MOM>(A, M, t, W, -1);
}

// the sites listed in A.work, each with a workspace in global scratch
template <int CAP, bool MOM, class Mesh>
__global__ void __launch_bounds__(64) k_cells_large(CellArgs A, Mesh M)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.nwork) return;
    Work<CAP>* W = reinterpret_cast<Work<CAP>*>(A.scratch) + t;
    process_site<CAP, MOM>(A, M, A.work[t], *W, t);
}

size_t large_work_bytes() { return sizeof(Work<kCapLarge>); }
int large_row_cap() { return kCapLarge + 1; }
int small_row_cap() { return kCapSmall + 1; }

template <class Mesh>
static void launch_cells_any(const CellArgs& a, const Mesh& v, int cap_kind, bool mom, cudaStream_t s)
{
    if (cap_kind == 0) {
        if (a.n <= 0) return;
        int b = 128, g = (a.n + b - 1) / b;
        if (mom)
            k_cells_small<kCapSmall, true><<<g, b, 0, s>>>(a, v);
        else
            k_cells_small<kCapSmall, false><<<g, b, 0, s>>>(a, v);
    } else {
        if (a.nwork <= 0) return;
        int b = 64, g = (a.nwork + b - 1) / b;
        if (mom)
            k_cells_large<kCapLarge, true><<<g, b, 0, s>>>(a, v);
        else
            k_cells_large<kCapLarge, false><<<g, b, 0, s>>>(a, v);
    }
}

void launch_cells_grid(const CellArgs& a, const MeshGridDev& m, int cap_kind, bool mom, cudaStream_t s)
{
    launch_cells_any(a, GridVisitor{m}, cap_kind, mom, s);
}

void launch_cells_tri(const CellArgs& a, const MeshTriDev& m, int cap_kind, bool mom, cudaStream_t s)
{
    launch_cells_any(a, TriVisitor{m}, cap_kind, mom, s);
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
