// ma_polygon.cu -- every Laguerre cell clipped to one polygon.
//
// MA::voronoi_polygon_intersection (include/MA/voronoi_polygon_intersection.hpp:153-188)
// takes one site v of a Delaunay or regular triangulation and clips a polygon P by the
// radical axis between v and each of its neighbours, with Pgon_intersector (:27-151):
// Sutherland-Hodgman over symbolic vertices (a pair of edges, each a polygon edge or a
// radical axis), inside-tests by Side1 (a polygon corner), Side2 (two radical axes)
// and Side3 (a polygon edge and a radical axis), coordinates by intersecting the two
// edges' supporting lines at the end (:64-69).  The reference's callers run it for
// every site in turn (tests/test_power.cpp:42-49, tests/test_voronoi.cpp:39-46).
//
// Here one call does all sites.  Each site's clip runs in one thread, with the cell
// stage of the evaluation (ma_stage.cuh) started from P instead of the mesh's box:
// the walk over the site tree clips by every site it cannot prove harmless, which
// gives the site's cell in the diagram of all sites, restricted to P -- the reference's
// clip by the triangulation's neighbours gives the same region.  Inside-tests are the
// same symbolic predicates with certified FP32 and FP64 filters and an exact fallback.
// A count pass sizes every polygon, an exclusive scan places them, an emit pass
// recomputes them (the same arithmetic, so the same polygons) and writes FP64 vertices;
// P's own corners are copied exactly.  The first pass holds 48 slots and 16 polygon
// corners per thread in local memory and has no exact fallback; sites that need more
// room or an exact predicate, and every site when P has more than 16 corners, go to a
// second pass with 256 slots, up to 64 corners and the exact predicates, its
// workspaces in global scratch.
#include <algorithm>
#include <cmath>

#include "ma_stage.cuh"
#include "ma_runtime.h"

namespace ma {

constexpr int kPgonFixSmall = 16;   // polygon corners held by the first pass
constexpr int kPgonMax = 64;        // polygon corners at most
constexpr int kPgonCapSmall = 48;   // slots / polygon vertices of the first pass
constexpr int kPgonCapLarge = 256;  //                              of the second pass
constexpr int kPgonLargeThreads = 152 * 64;  // second-pass threads (each with a workspace)

struct PgonArgs {
    CellArgs A;             // sites, permutation, tree; no mesh
    const double* px;       // polygon corners (absolute, device)
    const double* py;
    int k;
    int* cnt;               // count: vertices per site (original order)
    const int* base;        // emit: first vertex per site (original order)
    int64_t* off;           // emit: the same as int64
    double* xy;             // emit: vertices (x, y)
    int* edge;              // emit: edge starting at each vertex
    const int* list;        // second pass: sorted positions, or null for all sites
    int nlist;
    int* redo;              // first pass: sites handed to the second pass
    int* nredo;
    void* scratch;          // second pass: one workspace per thread
    uint32_t* status;
};

template <int CAP, int FC>
struct PgonWork {
    FixedN<FC> fx;
    Slot slots[CAP];
    Poly<CAP> PA, PB;
    int map[CAP];
    Nb64 nb[CAP];
};

// the polygon of sorted site k; false when it does not fit this pass (without EXACT:
// also when a predicate needs the exact fallback)
template <int CAP, int FC, bool EXACT, bool EMIT>
__device__ bool pgon_cell(const PgonArgs& g, int k, PgonWork<CAP, FC>& W)
{
    const CellArgs& A = g.A;
    const SiteD S = A.sites[k];
    const Owner o{S.x, S.y, S.w, k};
    W.fx.n = g.k;
    for (int e = 0; e < g.k; e++) set_fixed(W.fx, e, g.px[e], g.py[e], o);
    Poly<CAP>* P = &W.PA;
    Poly<CAP>* Q = &W.PB;
    const CellOut c = cell_stage<CAP, EXACT>(A, k, S, o, W.fx, W.slots, W.map, P, Q);
    if (c.st & ~ST_NEED_EXACT) atomicOr(g.status, c.st & ~ST_NEED_EXACT);
    if (c.overflow) return false;
    const int gi = A.perm[k];
    const int nv = c.empty ? 0 : P->n;
    if (!EMIT) {
        g.cnt[gi] = nv;
        return true;
    }
    const int64_t b = g.base[gi];
    g.off[gi] = b;
    for (int s = 0; s < c.ns && nv > 0; s++) W.nb[s] = make_nb64(A.sites[W.slots[s].site], o);
    for (int e = 0; e < nv; e++) {
        const int prev = P->lab[e == 0 ? nv - 1 : e - 1], cur = P->lab[e];
        double X, Y;
        if (prev < 0 && cur < 0) {
            X = W.fx.ax[-1 - cur];  // a corner of P, as given
            Y = W.fx.ay[-1 - cur];
        } else {
            vtx64(prev, cur, W.nb, W.fx, X, Y);
            X += S.x;
            Y += S.y;
        }
        g.xy[2 * (b + e)] = X;
        g.xy[2 * (b + e) + 1] = Y;
        g.edge[b + e] = cur >= 0 ? A.perm[W.slots[cur].site] : cur;
    }
    return true;
}

// first pass: one thread per site, workspace in local memory
template <bool EMIT>
__global__ void __launch_bounds__(128) k_polygon_cells(PgonArgs g)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= g.A.n) return;
    PgonWork<kPgonCapSmall, kPgonFixSmall> W;
    if (!pgon_cell<kPgonCapSmall, kPgonFixSmall, false, EMIT>(g, k, W) && !EMIT)
        g.redo[atomicAdd(g.nredo, 1)] = k;
}

// second pass: a fixed number of threads walk the list, workspaces in global scratch
template <bool EMIT>
__global__ void __launch_bounds__(64) k_polygon_cells_large(PgonArgs g)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    auto* W = reinterpret_cast<PgonWork<kPgonCapLarge, kPgonMax>*>(g.scratch) + t;
    for (int i = t; i < g.nlist; i += gridDim.x * blockDim.x) {
        const int k = g.list ? g.list[i] : i;
        if (!pgon_cell<kPgonCapLarge, kPgonMax, true, EMIT>(g, k, *W)) atomicOr(g.status, ST_POLY_OVERFLOW);
    }
}

__global__ void k_pgon_total(const int* base, int n, int64_t* off)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) off[n] = base[n];
}

}  // namespace ma

using namespace ma;

extern "C" {

ma_status ma_polygon_cells(ma_ctx* cp, int64_t n, const double* x, const double* y, const double* w,
                           const double* px, const double* py, int k, ma_mem mem, int64_t* nverts)
{
    Ctx* c = cp;
    if (!c || !x || !y || !px || !py || n < 1 || n >= (int64_t)1 << 24 || k < 3 || k > kPgonMax)
        return MA_ERR_INVALID_ARGUMENT;
    double X0 = px[0], X1 = px[0], Y0 = py[0], Y1 = py[0];
    for (int e = 0; e < k; e++) {
        if (!std::isfinite(px[e]) || !std::isfinite(py[e]))
            return fail(c, MA_ERR_INVALID_ARGUMENT, "non-finite polygon corner");
        X0 = std::min(X0, px[e]);
        X1 = std::max(X1, px[e]);
        Y0 = std::min(Y0, py[e]);
        Y1 = std::max(Y1, py[e]);
    }
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    c->have_pgon = false;
    const int nn = (int)n;
    const double *dx, *dy, *dw;
    ma_status st;
    if ((st = stage_in(c, c->hx, x, n, mem, &dx)) != MA_OK) return st;
    if ((st = stage_in(c, c->hy, y, n, mem, &dy)) != MA_OK) return st;
    if (w) {
        if ((st = stage_in(c, c->hw, w, n, mem, &dw)) != MA_OK) return st;
    } else {  // no weights: the Voronoi diagram
        MA_CUDA(c, c->hw.ensure(sizeof(double) * (size_t)n));
        MA_CUDA(c, cudaMemsetAsync(c->hw.p, 0, sizeof(double) * (size_t)n, s));
        dw = c->hw.as<double>();
    }
    if ((st = build_site_index_box(c, X0, Y0, X1, Y1, nn, dx, dy, dw)) != MA_OK) return st;
    launch_update_weights(dw, c->perm.as<int>(), nn, c->sites.as<SiteD>(), s);
    launch_tree_bounds(c->sites.as<SiteD>(), nn, c->t_child.as<int2>(), c->t_range.as<int2>(),
                       c->t_parent.as<int>(), c->t_leaf_parent.as<int>(), c->t_flag.as<int>(),
                       c->t_box.as<double4>(), c->t_boxf.as<float4>(), c->t_mom.p,
                           c->t_ab.as<double4>(), c->t_nk.as<float4>(), s);
    c->launches += 1 + tree_bounds_launches(nn);

    MA_CUDA(c, c->pg_poly.ensure(sizeof(double) * 2 * kPgonMax));
    MA_CUDA(c, cudaMemcpyAsync(c->pg_poly.p, px, sizeof(double) * k, cudaMemcpyHostToDevice, s));
    MA_CUDA(c, cudaMemcpyAsync(c->pg_poly.as<double>() + kPgonMax, py, sizeof(double) * k, cudaMemcpyHostToDevice,
                               s));
    MA_CUDA(c, c->pg_cnt.ensure(sizeof(int) * ((size_t)n + 1)));
    MA_CUDA(c, c->pg_base.ensure(sizeof(int) * ((size_t)n + 1)));
    MA_CUDA(c, c->pg_off.ensure(sizeof(int64_t) * ((size_t)n + 1)));
    MA_CUDA(c, c->pg_list.ensure(sizeof(int) * (size_t)n));
    MA_CUDA(c, c->status.ensure(sizeof(uint32_t) * 4));
    MA_CUDA(c, c->nredo.ensure(sizeof(int) * 4));
    MA_CUDA(c, c->scan_scratch.ensure(sizeof(int) * scan_scratch_ints(nn)));
    MA_CUDA(c, cudaMemsetAsync(c->status.p, 0, sizeof(uint32_t) * 4, s));
    MA_CUDA(c, cudaMemsetAsync(c->nredo.p, 0, sizeof(int) * 4, s));

    PgonArgs g{};
    CellArgs& a = g.A;
    a.n = nn;
    a.sites = c->sites.as<SiteD>();
    a.perm = c->perm.as<int>();
    a.tree.n = nn;
    a.tree.child = c->t_child.as<int2>();
    a.tree.range = c->t_range.as<int2>();
    a.tree.box = c->t_box.as<double4>();
    a.tree.boxf = c->t_boxf.as<float4>();
    a.tree.ab = c->t_ab.as<double4>();
    a.tree.nk = c->t_nk.as<float4>();
    a.tree.posf = c->posf.as<float2>();
    a.tree.parent = c->t_parent.as<int>();
    a.tree.leaf_parent = c->t_leaf_parent.as<int>();
    a.X0 = X0;
    a.Y0 = Y0;
    a.X1 = X1;
    a.Y1 = Y1;
    a.prev_valid = 0;
    a.abort_flag = nullptr;
    a.counters = nullptr;
    g.px = c->pg_poly.as<double>();
    g.py = c->pg_poly.as<double>() + kPgonMax;
    g.k = k;
    g.cnt = c->pg_cnt.as<int>();
    g.redo = c->pg_list.as<int>();
    g.nredo = c->nredo.as<int>();
    g.status = c->status.as<uint32_t>();

    // count: the first pass (small polygons), then the second pass on what it left
    int nlarge = nn;
    const int* large_list = nullptr;
    if (k <= kPgonFixSmall) {
        k_polygon_cells<false><<<(nn + 127) / 128, 128, 0, s>>>(g);
        c->launches += 1;
        MA_CUDA(c, cudaMemcpyAsync(c->hinfo, c->nredo.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        MA_CUDA(c, cudaStreamSynchronize(s));
        nlarge = c->hinfo[0];
        large_list = c->pg_list.as<int>();
    }
    const int nthreads = std::min(std::max(nlarge, 1), kPgonLargeThreads);
    if (nlarge > 0) {
        MA_CUDA(c, c->pg_work.ensure(sizeof(PgonWork<kPgonCapLarge, kPgonMax>) * (size_t)nthreads));
        g.scratch = c->pg_work.p;
        g.list = large_list;
        g.nlist = nlarge;
        k_polygon_cells_large<false><<<(nthreads + 63) / 64, 64, 0, s>>>(g);
        c->launches += 1;
    }
    MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 1, c->status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaStreamSynchronize(s));
    const uint32_t status = (uint32_t)c->hinfo[1];
    if (status & ST_BAD_INPUT) return fail(c, MA_ERR_INVALID_ARGUMENT, "non-finite site or weight");
    if (status & ST_EXACT_OVERFLOW)
        return fail(c, MA_ERR_EXACT_OVERFLOW, "an exact predicate ran out of expansion capacity");
    if (status & ST_POLY_OVERFLOW)
        return fail(c, MA_ERR_CAPACITY, "a clipped cell needed more than 256 slots or vertices");

    // place, then emit with the same passes
    launch_scan(c->pg_cnt.as<int>(), c->pg_base.as<int>(), nn, c->scan_scratch.as<int>(), s);
    k_pgon_total<<<1, 1, 0, s>>>(c->pg_base.as<int>(), nn, c->pg_off.as<int64_t>());
    MA_CUDA(c, cudaMemcpyAsync(c->hinfo + 2, c->pg_base.as<int>() + nn, sizeof(int), cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaStreamSynchronize(s));
    const int64_t nv = c->hinfo[2];
    MA_CUDA(c, c->pg_xy.ensure(sizeof(double) * 2 * (size_t)(nv + 1)));
    MA_CUDA(c, c->pg_edge.ensure(sizeof(int) * (size_t)(nv + 1)));
    g.base = c->pg_base.as<int>();
    g.off = c->pg_off.as<int64_t>();
    g.xy = c->pg_xy.as<double>();
    g.edge = c->pg_edge.as<int>();
    if (k <= kPgonFixSmall) {
        k_polygon_cells<true><<<(nn + 127) / 128, 128, 0, s>>>(g);
        c->launches += 1;
    }
    if (nlarge > 0) {
        k_polygon_cells_large<true><<<(nthreads + 63) / 64, 64, 0, s>>>(g);
        c->launches += 1;
    }
    c->launches += 3;
    MA_CUDA(c, cudaStreamSynchronize(s));
    MA_CUDA(c, cudaGetLastError());
    c->pg_n = n;
    c->pg_nv = nv;
    c->have_pgon = true;
    if (nverts) *nverts = nv;
    return MA_OK;
}

ma_status ma_polygon_cells_copy(ma_ctx* cp, int64_t* off, double* xy, int32_t* edge, ma_mem mem)
{
    Ctx* c = cp;
    if (!c) return MA_ERR_INVALID_ARGUMENT;
    if (!c->have_pgon) return fail(c, MA_ERR_INVALID_ARGUMENT, "no polygon cells have been computed");
    cudaSetDevice(c->device);
    cudaMemcpyKind kind = mem == MA_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t n = (size_t)c->pg_n, nv = (size_t)c->pg_nv;
    if (off) MA_CUDA(c, cudaMemcpyAsync(off, c->pg_off.p, sizeof(int64_t) * (n + 1), kind, c->stream));
    if (xy && nv) MA_CUDA(c, cudaMemcpyAsync(xy, c->pg_xy.p, sizeof(double) * 2 * nv, kind, c->stream));
    if (edge && nv) MA_CUDA(c, cudaMemcpyAsync(edge, c->pg_edge.p, sizeof(int) * nv, kind, c->stream));
    MA_CUDA(c, cudaStreamSynchronize(c->stream));
    return MA_OK;
}

}  // extern "C"
