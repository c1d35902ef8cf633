// ma_index.cu -- the site index: a binary radix tree over Morton-sorted sites.
//
//  * keys: 20-bit x 20-bit Morton code of the site position over the bounding box,
//    shifted left by 24 bits and or-ed with the site index (unique keys);
//  * an LSD radix sort of the 64-bit keys (8 passes of 8 bits, stable block-local
//    ranking with warp match);
//  * the radix tree of Karras ("Maximizing parallelism in the construction of
//    BVHs, octrees and k-d trees", HPG 2012): internal node i covers a contiguous
//    range of sorted sites, split where the key prefix changes;
//  * bottom-up passes: node bounding boxes (once per set of positions) and, for
//    every evaluation, an affine lower bound of the dual potential
//        phi_j = (|x_j|^2 - w_j) / 2  >=  alpha + beta . x_j   for all j in the node,
//    which lets the cell kernel discard a whole subtree: no site of the node can
//    cut a polygon C of site i when, for every vertex p of C,
//        (p - beta).(c - x_i) + |p_x - beta_x| h_x + |p_y - beta_y| h_y
//            < alpha + beta . x_i - phi_i
//    (c, h: centre and half extents of the node's box).  beta is the least-squares
//    slope of phi over the node, so the bound stays tight when the weights carry a
//    large affine part (cells displaced far from their sites).
#include "ma_internal.h"

namespace ma {

// read a value another thread published before its fence (bypass stale L1 lines)
__device__ __forceinline__ double4 load_published(const double4* p)
{
    const volatile double* q = (const volatile double*)p;
    return make_double4(q[0], q[1], q[2], q[3]);
}

__device__ __forceinline__ uint64_t spread20(uint32_t v)
{
    uint64_t x = v & 0xFFFFFu;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

__global__ void k_morton(const double* x, const double* y, int n, double x0, double y0, double sx, double sy,
                         uint64_t* keys)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double fx = (x[i] - x0) * sx, fy = (y[i] - y0) * sy;
    uint32_t qx = (uint32_t)fmin(fmax(fx, 0.0), 1048575.0);
    uint32_t qy = (uint32_t)fmin(fmax(fy, 0.0), 1048575.0);
    uint64_t code = spread20(qx) | (spread20(qy) << 1);
    keys[i] = (code << 24) | (uint64_t)i;
}

// ---------------------------------------------------------------------------
// LSD radix sort, 8 bits per pass
// ---------------------------------------------------------------------------
constexpr int kSortThreads = 256;

__global__ void k_radix_hist(const uint64_t* keys, int n, int shift, int* hist)
{
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int i = blockIdx.x * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(int)((keys[i] >> shift) & 255u)], 1);
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_radix_scatter(const uint64_t* in, uint64_t* out, int n, int shift, const int* offs)
{
    __shared__ int wc[kSortThreads / 32][256];
    for (int j = threadIdx.x; j < (kSortThreads / 32) * 256; j += kSortThreads) (&wc[0][0])[j] = 0;
    __syncthreads();
    int i = blockIdx.x * kSortThreads + threadIdx.x;
    bool valid = i < n;
    uint64_t key = valid ? in[i] : 0;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int d = valid ? (int)((key >> shift) & 255u) : 256 + lane;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wc[warp][d] = __popc(peers);
    __syncthreads();
    if (!valid) return;
    int before = 0;
    for (int w = 0; w < warp; w++) before += wc[w][d];
    out[offs[d * gridDim.x + blockIdx.x] + before + rank] = key;
}

// ---------------------------------------------------------------------------
// radix tree (Karras 2012)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int prefix_len(const uint64_t* k, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    return __clzll(k[i] ^ k[j]);
}

__global__ void k_tree(const uint64_t* keys, int n, int2* child, int2* range, int* parent, int* leaf_parent)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    if (i == 0) parent[0] = -1;
    int dir = (prefix_len(keys, n, i, i + 1) - prefix_len(keys, n, i, i - 1)) > 0 ? 1 : -1;
    int dmin = prefix_len(keys, n, i, i - dir);
    int lmax = 2;
    while (prefix_len(keys, n, i, i + lmax * dir) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (prefix_len(keys, n, i, i + (l + t) * dir) > dmin) l += t;
    int j = i + l * dir;
    int dnode = prefix_len(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (prefix_len(keys, n, i, i + (s + t) * dir) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * dir + (dir < 0 ? -1 : 0);
    int lo = min(i, j), hi = max(i, j);
    int left = (lo == gamma) ? (int)(0x80000000u | (unsigned)gamma) : gamma;
    int right = (hi == gamma + 1) ? (int)(0x80000000u | (unsigned)(gamma + 1)) : gamma + 1;
    child[i] = make_int2(left, right);
    range[i] = make_int2(lo, hi);
    if (left >= 0)
        parent[left] = i;
    else
        leaf_parent[gamma] = i;
    if (right >= 0)
        parent[right] = i;
    else
        leaf_parent[gamma + 1] = i;
}

// ---------------------------------------------------------------------------
// bottom-up passes (the second thread to reach a node computes it)
// ---------------------------------------------------------------------------
__global__ void k_tree_boxes(const SiteD* sites, int n, const int2* child, const int* parent, const int* leaf_parent,
                             int* flag, double4* box, float4* boxf)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int nd = leaf_parent[k];
    while (nd >= 0) {
        __threadfence();
        if (atomicAdd(&flag[nd], 1) == 0) return;
        __threadfence();
        int2 c = child[nd];
        double4 b;
        b.x = INFINITY;
        b.y = INFINITY;
        b.z = -INFINITY;
        b.w = -INFINITY;
        int cs[2] = {c.x, c.y};
        for (int q = 0; q < 2; q++) {
            double4 cb;
            if (cs[q] < 0) {
                SiteD s = sites[cs[q] & 0x7fffffff];
                cb = make_double4(s.x, s.y, s.x, s.y);
            } else {
                cb = load_published(&box[cs[q]]);
            }
            b.x = fmin(b.x, cb.x);
            b.y = fmin(b.y, cb.y);
            b.z = fmax(b.z, cb.z);
            b.w = fmax(b.w, cb.w);
        }
        box[nd] = b;
        // single-precision copy, rounded outwards (traversal order and the pruning test)
        boxf[nd] = make_float4(__double2float_rd(b.x), __double2float_rd(b.y), __double2float_ru(b.z),
                               __double2float_ru(b.w));
        nd = parent[nd];
    }
}

// moments for the least-squares slope of phi: count, mean x, mean y, Sxx, Sxy, Syy,
// mean phi, Sxphi, Syphi (centred sums, merged with Chan's update).  FP32: the slope
// only has to fit, the offset alpha below is exact for whatever slope is chosen.
struct Mom {
    float c, mx, my, sxx, sxy, syy, mf, sxf, syf;
};

__device__ __forceinline__ Mom mom_leaf(const SiteD& s)
{
    const float x = (float)s.x, y = (float)s.y;
    return Mom{1.0f, x, y, 0.0f, 0.0f, 0.0f, 0.5f * (x * x + y * y - (float)s.w), 0.0f, 0.0f};
}

__device__ __forceinline__ Mom mom_merge(const Mom& a, const Mom& b)
{
    Mom r;
    r.c = a.c + b.c;
    const float rb = b.c / r.c;
    const float dx = b.mx - a.mx, dy = b.my - a.my, df = b.mf - a.mf;
    const float w = a.c * b.c / r.c;
    r.mx = a.mx + dx * rb;
    r.my = a.my + dy * rb;
    r.mf = a.mf + df * rb;
    r.sxx = a.sxx + b.sxx + w * dx * dx;
    r.sxy = a.sxy + b.sxy + w * dx * dy;
    r.syy = a.syy + b.syy + w * dy * dy;
    r.sxf = a.sxf + b.sxf + w * dx * df;
    r.syf = a.syf + b.syf + w * dy * df;
    return r;
}

__device__ __forceinline__ double phi_of(const SiteD& s) { return 0.5 * (s.x * s.x + s.y * s.y - s.w); }

// phi_j - beta . x_j for one site, rounded down
__device__ __forceinline__ double site_alpha(const SiteD& s, double bx, double by)
{
    double v = phi_of(s) - (bx * s.x + by * s.y);
    return v - 1e-15 * (s.x * s.x + s.y * s.y + fabs(s.w) + fabs(bx * s.x) + fabs(by * s.y));
}

// Nodes of fewer than this many sites take the exact offset alpha = min over their
// sites of phi_j - beta . x_j; larger ones combine their children's bounds, which
// adds the spread of the child's slope over the child's box.  Propagated through
// every level that spread compounds to several squared site spacings and lets an
// order of magnitude more sites through the pruning test; above this size the
// nodes are far enough from the cells that test them for it not to matter.
constexpr int kExactAlpha = 64;

__device__ __forceinline__ bool small_node(const int2* range, int nd) { return range[nd].y - range[nd].x < kExactAlpha; }

// doubles as unsigned keys in the same order (for atomicMin)
__device__ __forceinline__ unsigned long long ord_key(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double ord_val(unsigned long long k)
{
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// pass 1, bottom-up (the second thread to reach a node computes it): moments and the
// least-squares slope beta of every internal node; the exact-offset slots of the
// small nodes set to +infinity
__global__ void k_tree_slopes(const SiteD* sites, int n, const int2* child, const int2* range, const int* parent,
                              const int* leaf_parent, int* flag, Mom* mom, unsigned long long* amin, double4* ab)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int nd = leaf_parent[k];
    while (nd >= 0) {
        __threadfence();
        if (atomicAdd(&flag[nd], 1) == 0) return;
        __threadfence();
        const int2 c = child[nd];
        Mom m[2];
        const int cs[2] = {c.x, c.y};
        for (int q = 0; q < 2; q++) {
            if (cs[q] < 0) {
                m[q] = mom_leaf(sites[cs[q] & 0x7fffffff]);
            } else {
                const volatile Mom* vm = (const volatile Mom*)&mom[cs[q]];
                m[q] = Mom{vm->c, vm->mx, vm->my, vm->sxx, vm->sxy, vm->syy, vm->mf, vm->sxf, vm->syf};
            }
        }
        const Mom r = mom_merge(m[0], m[1]);
        mom[nd] = r;
        // least-squares slope; the centroid (slope of |x|^2/2) when the fit is degenerate
        const float det = r.sxx * r.syy - r.sxy * r.sxy;
        float bx = r.mx, by = r.my;
        if (r.c >= 3.0f && det > 1e-6f * (r.sxx * r.syy) && det > 0.0f) {
            bx = (r.syy * r.sxf - r.sxy * r.syf) / det;
            by = (r.sxx * r.syf - r.sxy * r.sxf) / det;
        }
        if (!(isfinite(bx) && isfinite(by))) {
            bx = r.mx;
            by = r.my;
        }
        ab[nd] = make_double4(-INFINITY, (double)bx, (double)by, 0.0);
        amin[nd] = ord_key(INFINITY);
        nd = parent[nd];
    }
}

// pass 2, one thread per site: its term phi_j - beta . x_j in every small ancestor's
// minimum (exact FP64, every lane busy)
__global__ void k_tree_small_alpha(const SiteD* sites, int n, const int2* range, const int* parent,
                                   const int* leaf_parent, const double4* ab, unsigned long long* amin)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const SiteD s = sites[k];
    for (int nd = leaf_parent[k]; nd >= 0 && small_node(range, nd); nd = parent[nd]) {
        double v = site_alpha(s, ab[nd].y, ab[nd].z);
        if (!(v == v)) v = -INFINITY;  // never prune a node whose bound is not finite
        atomicMin(&amin[nd], ord_key(v));
    }
}

// alpha bound contributed by one child for the parent's slope beta: a site's own
// term, a small node's exact offset, or a large node's bound widened over its box
__device__ __forceinline__ double child_alpha(int c, const SiteD* sites, const int2* range, const double4* box,
                                              const double4* ab, const unsigned long long* amin, double bx, double by)
{
    if (c < 0) return site_alpha(sites[c & 0x7fffffff], bx, by);
    double4 a = load_published(&ab[c]);
    if (small_node(range, c)) a.x = ord_val(amin[c]);
    if (!(a.x < INFINITY)) return INFINITY;
    const double4 b = box[c];
    const double gx = a.y - bx, gy = a.z - by;
    const double mx = fmin(gx * b.x, gx * b.z), my = fmin(gy * b.y, gy * b.w);
    const double v = a.x + mx + my;
    return v - 1e-15 * (fabs(a.x) + fabs(mx) + fabs(my));
}

// the bound about the node's FP32 box centre, for the FP32 node test of the cell stage
__device__ __forceinline__ float4 node_k(double al, double bx, double by, const float4 bf)
{
    if (!(al > -INFINITY)) return make_float4(-INFINITY, 0.0f, 0.0f, 0.0f);
    const double cx = (double)(0.5f * (bf.x + bf.z)), cy = (double)(0.5f * (bf.y + bf.w));
    const double q = 0.5 * (cx * cx + cy * cy);
    const double A = al + bx * cx + by * cy - q;
    const double e = 8e-16 * (fabs(al) + fabs(bx * cx) + fabs(by * cy) + q);
    return make_float4(__double2float_rd(A - e), (float)(bx - cx), (float)(by - cy), 0.0f);
}

// pass 3, one thread per internal node: a small node takes its exact minimum; the
// large nodes are computed bottom-up from their children (the second arrival
// computes a node; a child that is a site or a small node is there from the start)
__global__ void k_tree_large_alpha(const SiteD* sites, int n, const int2* child, const int2* range, const int* parent,
                                   int* flag, const double4* box, const float4* boxf, const unsigned long long* amin,
                                   double4* ab, float4* nk)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n - 1) return;
    if (small_node(range, t)) {
        double a = ord_val(amin[t]);
        if (!(a == a)) a = -INFINITY;
        ab[t].x = a;
        nk[t] = node_k(a, ab[t].y, ab[t].z, boxf[t]);
        return;
    }
    const int2 c0 = child[t];
    const int ready = (c0.x < 0 || small_node(range, c0.x)) + (c0.y < 0 || small_node(range, c0.y));
    if (ready == 0) return;
    int nd = t;
    if (ready == 1) {
        __threadfence();
        if (atomicAdd(&flag[nd], 1) == 0) return;
        __threadfence();
    }
    while (true) {
        const int2 c = child[nd];
        const double4 own = ab[nd];
        double al = fmin(child_alpha(c.x, sites, range, box, ab, amin, own.y, own.z),
                         child_alpha(c.y, sites, range, box, ab, amin, own.y, own.z));
        if (!(al == al)) al = -INFINITY;
        ab[nd].x = al;
        nk[nd] = node_k(al, own.y, own.z, boxf[nd]);
        nd = parent[nd];
        if (nd < 0) return;
        __threadfence();
        if (atomicAdd(&flag[nd], 1) == 0) return;
        __threadfence();
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
void launch_morton(const double* x, const double* y, int n, double x0, double y0, double x1, double y1,
                   uint64_t* keys, cudaStream_t s)
{
    double W = x1 - x0, H = y1 - y0;
    double sx = W > 0 ? 1048576.0 / W : 0.0, sy = H > 0 ? 1048576.0 / H : 0.0;
    k_morton<<<(n + 255) / 256, 256, 0, s>>>(x, y, n, x0, y0, sx, sy, keys);
}

int radix_sort_blocks(int n) { return (n + kSortThreads - 1) / kSortThreads; }

void launch_radix_sort(uint64_t* keys, uint64_t* tmp, int n, int* hist, int* hist_scan, int* scan_scratch,
                       cudaStream_t s)
{
    int nb = radix_sort_blocks(n);
    uint64_t* a = keys;
    uint64_t* b = tmp;
    for (int shift = 0; shift < 64; shift += 8) {
        k_radix_hist<<<nb, kSortThreads, 0, s>>>(a, n, shift, hist);
        launch_scan(hist, hist_scan, 256 * nb, scan_scratch, s);
        k_radix_scatter<<<nb, kSortThreads, 0, s>>>(a, b, n, shift, hist_scan);
        uint64_t* t = a;
        a = b;
        b = t;
    }
    // 8 passes: the result is back in `keys`
}

void launch_tree(const uint64_t* keys, int n, int2* child, int2* range, int* parent, int* leaf_parent,
                 cudaStream_t s)
{
    if (n < 2) return;
    k_tree<<<(n - 1 + 255) / 256, 256, 0, s>>>(keys, n, child, range, parent, leaf_parent);
}

void launch_tree_boxes(const SiteD* sites, int n, const int2* child, const int* parent, const int* leaf_parent,
                       int* flag, double4* box, float4* boxf, cudaStream_t s)
{
    if (n < 2) return;
    cudaMemsetAsync(flag, 0, sizeof(int) * (n - 1), s);
    k_tree_boxes<<<(n + 255) / 256, 256, 0, s>>>(sites, n, child, parent, leaf_parent, flag, box, boxf);
}

__global__ void k_perm_gather(const uint64_t* keys, const double* x, const double* y, const double* w, int n,
                              int* perm, SiteD* sites, float2* posf)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int i = (int)(keys[k] & 0xFFFFFFull);
    perm[k] = i;
    SiteD s;
    s.x = x[i];
    s.y = y[i];
    s.w = w ? w[i] : 0.0;
    s.pad = 0.0;
    sites[k] = s;
    posf[k] = make_float2((float)s.x, (float)s.y);
}

void launch_perm_gather(const uint64_t* keys, const double* x, const double* y, const double* w, int n, int* perm,
                        SiteD* sites, float2* posf, cudaStream_t s)
{
    k_perm_gather<<<(n + 255) / 256, 256, 0, s>>>(keys, x, y, w, n, perm, sites, posf);
}

// per internal node: its moments, then (8-byte aligned) its exact-offset slot
static size_t mom_part(int n) { return (sizeof(Mom) * (size_t)(n > 1 ? n - 1 : 1) + 15) & ~(size_t)15; }
size_t tree_mom_bytes(int n) { return mom_part(n) + sizeof(unsigned long long) * (size_t)(n > 1 ? n - 1 : 1); }

void launch_tree_bounds(const SiteD* sites, int n, const int2* child, const int2* range, const int* parent,
                        const int* leaf_parent, int* flag, const double4* box, const float4* boxf, void* mom,
                        double4* ab, float4* nk, cudaStream_t s)
{
    if (n < 2) return;
    Mom* m = (Mom*)mom;
    unsigned long long* amin = (unsigned long long*)((char*)mom + mom_part(n));
    const unsigned g = (unsigned)((n + 255) / 256);
    cudaMemsetAsync(flag, 0, sizeof(int) * (n - 1), s);
    k_tree_slopes<<<g, 256, 0, s>>>(sites, n, child, range, parent, leaf_parent, flag, m, amin, ab);
    k_tree_small_alpha<<<g, 256, 0, s>>>(sites, n, range, parent, leaf_parent, ab, amin);
    cudaMemsetAsync(flag, 0, sizeof(int) * (n - 1), s);
    k_tree_large_alpha<<<g, 256, 0, s>>>(sites, n, child, range, parent, flag, box, boxf, amin, ab, nk);
}

}  // namespace ma
