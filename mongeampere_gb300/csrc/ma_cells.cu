// ma_cells.cu -- Laguerre cells and their pieces (the hot path of one evaluation).
//
// Reference behaviour: voronoi_triangulation_intersection_raw / Tri_intersector
// (include/MA/voronoi_triangulation_intersection.hpp:42-313) produce every
// non-empty (site, triangle) piece; kantorovich's callback
// (include/MA/kantorovich.hpp:87-136) integrates it.  Here the same pieces are
// produced cell by cell in two kernels:
//
//   stage 1, k_cells_stage1 (one thread per site): branch and bound over the site
//     tree (the walk and the node test are in ma_stage.cuh); Sutherland-Hodgman
//     clips of the mesh's bounding box give the cell and its neighbour list, written
//     out in site order with the cell's bounding box;
//   stage 2, k_pieces (a warp per eight consecutive cells): certified corner tests
//     sort the mesh triangles under the cells' boxes into outside, inside and
//     crossed; the crossed ones are clipped by the half-warps, a vertex per lane; the
//     pieces are listed in shared memory, integrated one per lane in FP64, and the
//     per-cell sums (in a fixed order, so results are reproducible) give the mass,
//     the value part and the Hessian row.
//
// Cells that outgrow the 48 slots of stage 1, or whose pieces need exact arithmetic
// or more than 12 vertices, are redone end to end by k_cells_large, one thread per
// cell with a 256-slot workspace in global scratch.
#include <climits>
#include <type_traits>

#include "ma_internal.h"

namespace ma {

// ---------------------------------------------------------------------------
// mesh access
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

// square (i, j) of the grid mesh, triangle tt (0: (i,j) (i+1,j) (i+1,j+1);
// 1: (i,j) (i+1,j+1) (i,j+1)), owner-relative corners
__device__ __forceinline__ void grid_fixed(const MeshGridDev& m, int i, int j, int tt, const Owner& o, Fixed& T)
{
    const double X0 = m.gx[i], X1 = m.gx[i + 1], Y0 = m.gy[j], Y1 = m.gy[j + 1];
    T.n = 3;
    set_fixed(T, 0, X0, Y0, o);
    if (tt == 0) {
        set_fixed(T, 1, X1, Y0, o);
        set_fixed(T, 2, X1, Y1, o);
    } else {
        set_fixed(T, 1, X1, Y1, o);
        set_fixed(T, 2, X0, Y1, o);
    }
}

// the same with the density on it, rho(u) = c0 + g . u
__device__ __forceinline__ void grid_triangle(const MeshGridDev& m, int i, int j, int tt, const Owner& o, Fixed& T,
                                              double& c0, double& gx, double& gy)
{
    grid_fixed(m, i, j, tt, o, T);
    const double* row0 = m.val + (size_t)j * m.nx;
    const double* row1 = row0 + m.nx;
    const double v00 = row0[i], v10 = row0[i + 1], v01 = row1[i], v11 = row1[i + 1];
    if (tt == 0) {
        gx = (v10 - v00) * m.ihx[i];
        gy = (v11 - v10) * m.ihy[j];
    } else {
        gx = (v11 - v01) * m.ihx[i];
        gy = (v01 - v00) * m.ihy[j];
    }
    c0 = v00 - gx * T.rx[0] - gy * T.ry[0];
}

__device__ __forceinline__ void tri_fixed(const MeshTriDev& m, int t, const Owner& o, Fixed& T)
{
    const int a0 = m.tri[3 * t], a1 = m.tri[3 * t + 1], a2 = m.tri[3 * t + 2];
    T.n = 3;
    set_fixed(T, 0, m.vx[a0], m.vy[a0], o);
    set_fixed(T, 1, m.vx[a1], m.vy[a1], o);
    set_fixed(T, 2, m.vx[a2], m.vy[a2], o);
}

__device__ __forceinline__ void tri_triangle(const MeshTriDev& m, int t, const Owner& o, Fixed& T, double& c0,
                                             double& gx, double& gy)
{
    tri_fixed(m, t, o, T);
    const double l0 = m.lin[3 * t];
    gx = m.lin[3 * t + 1];
    gy = m.lin[3 * t + 2];
    c0 = l0 - gx * T.rx[0] - gy * T.ry[0];
}

// FP32 owner-relative corners of a triangle with their error radii (the values
// set_fixed gives), in registers
struct Corners {
    float ux[3], uy[3], ur[3];
};

__device__ __forceinline__ float corner_radius(float ux, float uy) { return kU32 * fmaxf(fabsf(ux), fabsf(uy)) + 1e-37f; }

__device__ __forceinline__ Corners grid_corners(const MeshGridDev& m, int i, int j, int tt, const Owner& o)
{
    const float x0 = (float)dsub(m.gx[i], o.x), x1 = (float)dsub(m.gx[i + 1], o.x);
    const float y0 = (float)dsub(m.gy[j], o.y), y1 = (float)dsub(m.gy[j + 1], o.y);
    Corners c;
    c.ux[0] = x0;
    c.uy[0] = y0;
    c.ux[1] = x1;
    c.uy[1] = tt == 0 ? y0 : y1;
    c.ux[2] = tt == 0 ? x1 : x0;
    c.uy[2] = y1;
    for (int e = 0; e < 3; e++) c.ur[e] = corner_radius(c.ux[e], c.uy[e]);
    return c;
}

__device__ __forceinline__ Corners tri_corners(const MeshTriDev& m, int t, const Owner& o)
{
    Corners c;
    for (int e = 0; e < 3; e++) {
        const int a = m.tri[3 * t + e];
        c.ux[e] = (float)dsub(m.vx[a], o.x);
        c.uy[e] = (float)dsub(m.vy[a], o.y);
        c.ur[e] = corner_radius(c.ux[e], c.uy[e]);
    }
    return c;
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
        for (int j = j0; j <= j1; j++)
            for (int i = i0; i <= i1; i++)
                for (int tt = 0; tt < 2; tt++) {
                    double c0, gx, gy;
                    grid_triangle(m, i, j, tt, o, T, c0, gx, gy);
                    fn(T, c0, gx, gy, ((j * (m.nx - 1) + i) << 1) | tt);
                }
    }
};

// bin range of a box; false when it misses the mesh
__device__ __forceinline__ bool tri_bins(const MeshTriDev& m, double bx0, double by0, double bx1, double by1,
                                         int& cx0, int& cy0, int& cx1, int& cy1)
{
    cx0 = (int)floor((bx0 - m.bx0) / m.bcw);
    cx1 = (int)floor((bx1 - m.bx0) / m.bcw);
    cy0 = (int)floor((by0 - m.by0) / m.bch);
    cy1 = (int)floor((by1 - m.by0) / m.bch);
    if (cx1 < 0 || cy1 < 0 || cx0 >= m.bnx || cy0 >= m.bny) return false;
    cx0 = max(cx0, 0);
    cy0 = max(cy0, 0);
    cx1 = min(cx1, m.bnx - 1);
    cy1 = min(cy1, m.bny - 1);
    return true;
}

struct TriVisitor {
    MeshTriDev m;
    template <class Fn>
    __device__ __forceinline__ void visit(const Owner& o, double bx0, double by0, double bx1, double by1,
                                          Fn&& fn) const
    {
        int cx0, cy0, cx1, cy1;
        if (!tri_bins(m, bx0, by0, bx1, by1, cx0, cy0, cx1, cy1)) return;
        Fixed T;
        for (int by = cy0; by <= cy1; by++) {
            for (int bx = cx0; bx <= cx1; bx++) {
                int b = by * m.bnx + bx;
                for (int q = m.bin_start[b]; q < m.bin_start[b + 1]; q++) {
                    int t = m.bin_tri[q];
                    int4 r = m.tbin[t];
                    // visit each triangle once: from the first bin shared with the box
                    if (bx != max(r.x, cx0) || by != max(r.y, cy0)) continue;
                    double c0, gx, gy;
                    tri_triangle(m, t, o, T, c0, gx, gy);
                    fn(T, c0, gx, gy, t);
                }
            }
        }
    }
};

}  // namespace ma

#include "ma_stage.cuh"

namespace ma {

// conservative absolute bounding box of polygon P (owner-relative FP32 + radii)
template <int CAP>
__device__ __forceinline__ double4 cell_box(const Poly<CAP>& P, const SiteD& S, const CellArgs& A)
{
    float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    for (int e = 0; e < P.n; e++) {
        float r = P.ur[e] * 1.0001f;
        mnx = fminf(mnx, P.ux[e] - r);
        mxx = fmaxf(mxx, P.ux[e] + r);
        mny = fminf(mny, P.uy[e] - r);
        mxy = fmaxf(mxy, P.uy[e] + r);
    }
    if (!(mxx - mnx < INFINITY && mxy - mny < INFINITY)) return make_double4(A.X0, A.Y0, A.X1, A.Y1);
    double sx = fmax(fabs((double)mnx), fabs((double)mxx)), sy = fmax(fabs((double)mny), fabs((double)mxy));
    return make_double4(S.x + (double)mnx - 1e-6 * sx - 1e-300, S.y + (double)mny - 1e-6 * sy - 1e-300,
                        S.x + (double)mxx + 1e-6 * sx + 1e-300, S.y + (double)mxy + 1e-6 * sy + 1e-300);
}

// ---------------------------------------------------------------------------
// outputs of one site
// ---------------------------------------------------------------------------
template <bool MOM>
__device__ void write_site(const CellArgs& A, int gi, const SiteD& S, const Acc& acc, int m, const Slot* slots,
                           const Nb64* nb, const double* hvtot, const uint64_t* touched_words, int* cols,
                           double* vals, int big_slot)
{
    A.mass[gi] = acc.mass;
    A.vpart[gi] = S.w * acc.mass - acc.second;
    if (MOM && A.mom) {
        double* mo = A.mom + 6 * (size_t)gi;
        double M = acc.mass;
        mo[0] = M;
        mo[1] = acc.m1x + S.x * M;
        mo[2] = acc.m1y + S.y * M;
        // int rho x x^T = int rho u u^T + x_i (int rho u)^T + (int rho u) x_i^T + M x_i x_i^T
        mo[3] = acc.sxx + 2.0 * S.x * acc.m1x + S.x * S.x * M;
        mo[4] = acc.syy + 2.0 * S.y * acc.m1y + S.y * S.y * M;
        mo[5] = acc.sxy + S.x * acc.m1y + S.y * acc.m1x + S.x * S.y * M;
    }
    if (!A.rowcnt) return;
    // off-diagonal entries sorted by original index, diagonal in place
    int cnt = 0;
    double diag = 0.0;
    for (int s = 0; s < m; s++) {
        if (!((touched_words[s >> 6] >> (s & 63)) & 1ull)) continue;
        double d2 = nb[s].dx * nb[s].dx + nb[s].dy * nb[s].dy;
        double v = -hvtot[s] / (2.0 * d2);
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
        oc = A.big_col + (size_t)big_slot * A.big_cap;
        ov = A.big_val + (size_t)big_slot * A.big_cap;
        A.big_index[gi] = big_slot;
    } else {
        oc = A.st_col + (size_t)gi * A.scap;
        ov = A.st_val + (size_t)gi * A.scap;
    }
    if (total == 0) return;
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

__device__ __forceinline__ void write_empty(const CellArgs& A, int gi, bool mom)
{
    A.mass[gi] = 0.0;
    A.vpart[gi] = 0.0;
    if (mom && A.mom)
        for (int q = 0; q < 6; q++) A.mom[6 * (size_t)gi + q] = 0.0;
    if (A.rowcnt) A.rowcnt[gi] = 0;
}

// clip triangle T by slots 0..m-1 and integrate the piece
template <int CAP, bool MOM, bool EXACT>
__device__ __forceinline__ bool piece(const Fixed& T, double c0, double gx, double gy, const Slot* slots,
                                      const Nb64* nb, int m, const Owner& o, const SiteD* sites, Poly<CAP>* Wp,
                                      Poly<CAP>* Vp, Acc& acc, double* hv, Bits<CAP>& touched, uint32_t& st)
{
    bool overflow = false;
    Wp->n = 3;
    for (int e = 0; e < 3; e++) {
        Wp->lab[e] = -1 - e;
        Wp->ux[e] = T.ux[e];
        Wp->uy[e] = T.uy[e];
        Wp->ur[e] = T.ur[e];
    }
    for (int s = 0; s < m; s++) {
        if (clip_poly<CAP, EXACT>(*Wp, *Vp, s, slots, T, o, sites, st, overflow)) {
            if (overflow) return false;
            Poly<CAP>* t = Wp;
            Wp = Vp;
            Vp = t;
            if (Wp->n == 0) return true;
        }
    }
    integrate_piece<CAP, MOM>(*Wp, nb, T, c0, gx, gy, acc, hv, touched);
    return true;
}

// ---------------------------------------------------------------------------
// one thread per cell, workspace in global scratch (large cells)
// ---------------------------------------------------------------------------
template <int CAP, bool MOM, class Mesh>
__device__ void process_site(const CellArgs& A, const Mesh& M, int k, Work<CAP>& W, int big_slot)
{
    const SiteD S = A.sites[k];
    const int gi = A.perm[k];
    Owner o{S.x, S.y, S.w, k};
    Poly<CAP>* P = &W.PA;
    Poly<CAP>* Q = &W.PB;
    CellOut c = cell_stage<CAP, true>(A, k, S, o, domain_box(A, o), W.slots, W.map, P, Q);
    uint32_t st = c.st;
    if (c.overflow) {
        if (A.redo) A.redo[atomicAdd(A.nredo, 1)] = k;
        atomicOr(A.status, ST_POLY_OVERFLOW);
        return;
    }
    Acc acc{0, 0, 0, 0, 0, 0, 0};
    Bits<CAP> touched;
    touched.clear();
    const int m = c.empty ? 0 : c.ns;
    if (!c.empty && P->n > 0) {
        double4 bb = cell_box(*P, S, A);
        // the neighbours by site index, whatever order the walk met them in: the pieces
        // are clipped in slot order, so this keeps their sums independent of the seeds
        for (int s = 1; s < m; s++) {
            const Slot v = W.slots[s];
            int r = s - 1;
            while (r >= 0 && W.slots[r].site > v.site) {
                W.slots[r + 1] = W.slots[r];
                r--;
            }
            W.slots[r + 1] = v;
        }
        for (int s = 0; s < m; s++) {
            W.nb[s] = make_nb64(A.sites[W.slots[s].site], o);
            W.hv[s] = 0.0;
        }
        bool bad = false;
        M.visit(o, bb.x, bb.y, bb.z, bb.w, [&](const Fixed& T, double c0, double gx, double gy, int) {
            if (bad) return;
            if (!piece<CAP, MOM, true>(T, c0, gx, gy, W.slots, W.nb, m, o, A.sites, P, Q, acc, W.hv, touched, st))
                bad = true;
        });
        if (bad) {
            if (A.redo) A.redo[atomicAdd(A.nredo, 1)] = k;
            atomicOr(A.status, ST_POLY_OVERFLOW);
            return;
        }
    }
    write_site<MOM>(A, gi, S, acc, m, W.slots, W.nb, W.hv, touched.w, W.cols, W.vals, big_slot);
    if (st) atomicOr(A.status, st);
}

// The pieces of one cell, one thread per cell with exact predicates (the large-capacity
// pass of ma_pieces: cells beyond stage 1's capacity, or whose clips meet exact ties):
// count them (pc_cnt, pv_cnt) or emit them at the cell's offsets, in the order of the
// warp kernel (triangles in the mesh's order under the cell's box, every triangle
// clipped by the neighbours in site order, vertex e the start of edge e).
template <int CAP, bool EMIT, class Mesh>
__device__ void list_site(const CellArgs& A, const Mesh& M, int k, Work<CAP>& W)
{
    const SiteD S = A.sites[k];
    const int gi = A.perm[k];
    Owner o{S.x, S.y, S.w, k};
    Poly<CAP>* P = &W.PA;
    Poly<CAP>* Q = &W.PB;
    CellOut c = cell_stage<CAP, true>(A, k, S, o, domain_box(A, o), W.slots, W.map, P, Q);
    uint32_t st = c.st;
    bool bad = c.overflow;
    int np = 0, nv = 0;
    int64_t gp = EMIT ? A.pc_base[k] : 0, gv = EMIT ? A.pv_base[k] : 0;
    const int m = c.empty ? 0 : c.ns;
    if (!bad && !c.empty && P->n > 0) {
        const double4 bb = cell_box(*P, S, A);
        for (int s = 1; s < m; s++) {
            const Slot v = W.slots[s];
            int r = s - 1;
            while (r >= 0 && W.slots[r].site > v.site) {
                W.slots[r + 1] = W.slots[r];
                r--;
            }
            W.slots[r + 1] = v;
        }
        for (int s = 0; s < m; s++) W.nb[s] = make_nb64(A.sites[W.slots[s].site], o);
        M.visit(o, bb.x, bb.y, bb.z, bb.w, [&](const Fixed& T, double, double, double, int id) {
            if (bad) return;
            Poly<CAP>* Wp = P;
            Poly<CAP>* Vp = Q;
            Wp->n = 3;
            for (int e = 0; e < 3; e++) {
                Wp->lab[e] = -1 - e;
                Wp->ux[e] = T.ux[e];
                Wp->uy[e] = T.uy[e];
                Wp->ur[e] = T.ur[e];
            }
            bool overflow = false;
            for (int s = 0; s < m && Wp->n > 0; s++) {
                if (clip_poly<CAP, true>(*Wp, *Vp, s, W.slots, T, o, A.sites, st, overflow)) {
                    if (overflow) {
                        bad = true;
                        return;
                    }
                    Poly<CAP>* t = Wp;
                    Wp = Vp;
                    Vp = t;
                }
            }
            const int n = Wp->n;
            if (n == 0) return;
            if (EMIT) {
                A.out_site[gp] = gi;
                A.out_tri[gp] = id;
                A.out_off[gp] = gv;
                for (int e = 0; e < n; e++) {
                    double X, Y;
                    vtx64(Wp->lab[e == 0 ? n - 1 : e - 1], Wp->lab[e], W.nb, T, X, Y);
                    A.out_xy[2 * (gv + e)] = S.x + X;
                    A.out_xy[2 * (gv + e) + 1] = S.y + Y;
                    const int l = Wp->lab[e];
                    A.out_edge[gv + e] = l >= 0 ? A.perm[W.slots[l].site] : l;
                }
            }
            np++;
            nv += n;
            gp++;
            gv += n;
        });
    }
    if (bad) {
        atomicAdd(A.nredo, 1);  // beyond every capacity: the call fails
        atomicOr(A.status, ST_POLY_OVERFLOW);
        return;
    }
    if (!EMIT) {
        A.pc_cnt[k] = np;
        A.pv_cnt[k] = nv;
    }
    st &= ~(uint32_t)ST_NEED_EXACT;
    if (st) atomicOr(A.status, st);
}

// ---------------------------------------------------------------------------
// stage 1: a warp per cell
// ---------------------------------------------------------------------------
// The cell's polygon is held a vertex per lane (its labels, FP32 positions and error
// radii in registers, mirrored in shared memory for the tests that read every vertex);
// the neighbour slots live in shared memory.  Candidate sites are tested 32 at a time
// ("can this site cut the polygon?", certified FP32, every vertex) and the ones that
// may cut are clipped one after another by the whole warp: a side test per vertex, a
// ballot of the vertices outside, a scan of the Sutherland-Hodgman outputs
// (vti.hpp:168-198) and a pass through shared memory.  The candidates are
//   1. the seeds: the previous evaluation's neighbours (same sites, nearby weights),
//      or else the 16 sites around the site in Morton order;
//   2. the site tree, walked in batches of up to 32 nodes from the top of a stack: it
//      starts from the siblings of the site's own root-to-leaf path (every other
//      subtree); a node that no site of can cut the polygon (node_harmless_v) is
//      dropped, a small node's sites become candidates, a larger one is replaced by
//      its two children.
// The cell is exact whatever order the candidates come in (every decision is certified
// or symbolic); the neighbour list is written sorted by site index.
constexpr int kCapLarge = 256;
constexpr int kS1Warps = 4;     // warps per block
constexpr int kS1Stack = 512;   // tree nodes waiting per warp
constexpr int kS1Cand = 128;    // candidate sites of one batch (32 nodes of < 4 sites)
constexpr int kS1Bucket = 4;    // nodes of fewer sites are visited site by site
constexpr int kS1Window = 8;    // Morton-order seeds on either side without a previous list

struct Stage1Warp {
    float pux[32], puy[32], pur[32];  // the polygon, a vertex per lane
    int plab[32];
    Slot slot[kCapSmall];
    int seed[kSeedCap + 1];
    int stack[kS1Stack];
    int cand[kS1Cand];
    Fixed box;
};

__global__ void __launch_bounds__(32 * kS1Warps, 6) k_cells_stage1(CellArgs A)
{
    constexpr unsigned kFull = 0xffffffffu;
    __shared__ Stage1Warp shw[kS1Warps];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Stage1Warp& W = shw[wib];
    const int k = blockIdx.x * kS1Warps + wib;
    if (k >= A.n) return;
    const SiteD S = A.sites[k];
    const Owner o{S.x, S.y, S.w, k};
    const int gi = A.perm[k];
    if (!(isfinite(S.x) && isfinite(S.y) && isfinite(S.w))) {
        if (lane == 0) {
            A.nb_cnt[k] = -1;
            atomicOr(A.status, ST_BAD_INPUT);
            if (A.abort_flag) atomicExch(A.abort_flag, 1);
        }
        return;
    }
    // the mesh's bounding box (domain_box's corners), lanes 0..3
    if (lane < 4) {
        const double bx = (lane == 0 || lane == 3) ? A.X0 : A.X1;
        const double by = lane < 2 ? A.Y0 : A.Y1;
        set_fixed(W.box, lane, bx, by, o);
    }
    if (lane == 0) W.box.n = 4;
    __syncwarp();
    int n = 4;  // polygon vertices
    float vx = 0.0f, vy = 0.0f, vr = 0.0f;
    int vl = 0;
    if (lane < 4) {
        vx = W.box.ux[lane];
        vy = W.box.uy[lane];
        vr = W.box.ur[lane];
        vl = -1 - lane;
        W.pux[lane] = vx;
        W.puy[lane] = vy;
        W.pur[lane] = vr;
        W.plab[lane] = vl;
    }
    const float ox = (float)S.x, oy = (float)S.y;
    const float owh = (float)(0.5 * S.w), oxa = fabsf(ox) + fabsf(oy);
    int ns = 0;  // slots in use
    uint32_t st = 0;
    bool empty = false, overflow = false, aborted = false;
    int popped = 0, tested = 0, pruned = 0, visited = 0, cuts = 0;
    __syncwarp();

    // clip the polygon by slot cs: 0 no vertex outside, 1 clipped, 2 nothing left,
    // 3 beyond capacity or undecided (the cell goes to the large-capacity pass)
    auto clip = [&](int cs) -> int {
        const Slot c = W.slot[cs];
        const bool act = lane < n;
        const int prevlab = __shfl_sync(kFull, vl, lane == 0 ? n - 1 : lane - 1);
        bool vout = false, und = false;
        if (act) {
            const int t = test32(vx, vy, vr, c);
            if (t != 0)
                vout = t > 0;
            else
                vout = !sym_inside<kCapSmall, false>(prevlab, vl, W.slot, W.box, o, A.sites, c.site, st, und);
        }
        if (__any_sync(kFull, und)) {
            st |= ST_NEED_EXACT;
            return 3;
        }
        const unsigned om = __ballot_sync(kFull, act && vout);
        if (om == 0u) return 0;
        if (__popc(om) == n) return 2;
        const int v1 = lane + 1 == n ? 0 : lane + 1;
        const bool in0 = act && !vout, in1 = !((om >> v1) & 1u);
        const int cnt = act ? (in0 ? (in1 ? 1 : 2) : (in1 ? 1 : 0)) : 0;
        int pos = cnt;
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(kFull, pos, d);
            if (lane >= d) pos += y;
        }
        const int m = __shfl_sync(kFull, pos, 31);
        pos -= cnt;
        if (m > 32) return 3;
        __syncwarp();
        if (act) {
            int q = pos;
            if (in0) {
                W.pux[q] = vx;
                W.puy[q] = vy;
                W.pur[q] = vr;
                W.plab[q] = vl;
                q++;
            }
            if (in0 != in1) {
                float nx, ny, nr;
                new_vertex<kCapSmall>(vl, cs, W.slot, W.box, nx, ny, nr);
                W.pux[q] = nx;
                W.puy[q] = ny;
                W.pur[q] = nr;
                W.plab[q] = in0 ? cs : vl;
            }
        }
        __syncwarp();
        n = m;
        if (lane < n) {
            vx = W.pux[lane];
            vy = W.puy[lane];
            vr = W.pur[lane];
            vl = W.plab[lane];
        }
        __syncwarp();
        return 1;
    };

    // keep only the slots the polygon's edges use (compact_slots, a warp at a time)
    auto compact = [&]() {
        const unsigned lo = __reduce_or_sync(kFull, (lane < n && vl >= 0 && vl < 32) ? (1u << vl) : 0u);
        const unsigned hi = __reduce_or_sync(kFull, (lane < n && vl >= 32) ? (1u << (vl - 32)) : 0u);
        const bool u0 = lane < ns && ((lo >> lane) & 1u), u1 = lane + 32 < ns && ((hi >> lane) & 1u);
        Slot a0, a1;
        if (u0) a0 = W.slot[lane];
        if (u1) a1 = W.slot[lane + 32];
        __syncwarp();
        const unsigned below = (1u << lane) - 1u;
        if (u0) W.slot[__popc(lo & below)] = a0;
        if (u1) W.slot[__popc(lo) + __popc(hi & below)] = a1;
        if (lane < n && vl >= 0)
            vl = vl < 32 ? __popc(lo & ((1u << vl) - 1u)) : __popc(lo) + __popc(hi & ((1u << (vl - 32)) - 1u));
        if (lane < n) W.plab[lane] = vl;
        ns = __popc(lo) + __popc(hi);
        __syncwarp();
    };

    // clip by the sites list[0..cnt): 32 at a time, the ones that may cut in list order
    auto try_sites = [&](const int* list, int cnt) {
        for (int c0 = 0; c0 < cnt && !empty && !overflow; c0 += 32) {
            const int j = c0 + lane;
            bool cut = false, kill = false;
            Slot sl;
            int q = j < cnt ? list[j] : -1;
            // a site already clipped against (a seed met again): its radical axis carries
            // polygon vertices, where the side tests would be exactly tied
            for (int t = 0; t < ns && q >= 0; t++)
                if (W.slot[t].site == q) q = -1;
            if (q >= 0) {
                const SiteD C = A.sites[q];
                if (C.x == S.x && C.y == S.y) {
                    // coincident sites: the larger weight, then the lower index, keeps the cell
                    const int gj = A.perm[q];
                    kill = C.w > S.w || (C.w == S.w && gj < gi);
                } else {
                    sl = make_slot(q, C, o);
                    for (int v = 0; v < n && !cut; v++) cut = test32(W.pux[v], W.puy[v], W.pur[v], sl) >= 0;
                }
            }
            if (__any_sync(kFull, kill)) {
                empty = true;
                break;
            }
            unsigned cm = __ballot_sync(kFull, cut);
            visited += __popc(cm);
            while (cm) {
                const int src = __ffs(cm) - 1;
                cm &= cm - 1;
                if (ns == kCapSmall) {
                    compact();
                    if (ns == kCapSmall) {
                        overflow = true;
                        break;
                    }
                }
                if (lane == src) W.slot[ns] = sl;
                __syncwarp();
                const int r = clip(ns);
                if (r == 1) {
                    ns++;
                    cuts++;
                } else if (r == 2) {
                    empty = true;
                    break;
                } else if (r == 3) {
                    overflow = true;
                    break;
                }
            }
        }
    };

    // 1. seeds
    int nseed = 0;
    if (A.prev_valid) {
        const int c = A.nb_cnt[k];
        if (c > 0 && c <= kSeedCap) nseed = c;
    }
    const bool windowed = nseed == 0;
    int wlo = 0, whi = -1;
    int ccount;  // candidates waiting in the list (the seeds first, then W.cand)
    if (windowed) {
        wlo = max(k - kS1Window, 0);
        whi = min(k + kS1Window, A.n - 1);
        for (int q = wlo + lane; q <= whi; q += 32)
            if (q != k) W.seed[q - wlo - (q > k ? 1 : 0)] = q;
        ccount = whi - wlo;  // the window without k
    } else {
        for (int j = lane; j < nseed; j += 32) W.seed[j] = A.nb_lab[(size_t)k * kSeedCap + j];
        ccount = nseed;
    }
    __syncwarp();
    // a window seed is skipped by its range; a previous-list seed is one of the cell's
    // slots (the previous neighbours bound the cell again) and try_sites skips it there
    auto is_seed = [&](int q) -> bool { return windowed && q >= wlo && q <= whi; };

    // 2. the site tree, a batch of up to 32 nodes after each list of candidates
    int sp = -1;  // -1: the walk has not started
    const int* clist = W.seed;
    for (;;) {
        if (ccount) try_sites(clist, ccount);
        if (empty || overflow) break;
        clist = W.cand;
        ccount = 0;
        if (sp < 0) {
            sp = 0;
            if (A.tree.n >= 2) {
                if (lane == 0) {
                    int cur = (int)(0x80000000u | (unsigned)k);
                    int p = A.tree.leaf_parent[k];
                    while (p >= 0 && sp < kS1Stack) {
                        const int2 ch = A.tree.child[p];
                        W.stack[sp++] = ch.x == cur ? ch.y : ch.x;
                        cur = p;
                        p = A.tree.parent[p];
                    }
                    if (p >= 0) sp = -1;
                }
                sp = __shfl_sync(kFull, sp, 0);
                __syncwarp();
                if (sp < 0) {
                    overflow = true;
                    break;
                }
                if (windowed) {
                    // Without a previous list the window leaves the polygon far from the
                    // cell; before the walk, every sibling subtree of the path gives the
                    // sites it holds nearest the site: a lane descends it, taking the child
                    // whose box is nearer each time, down to a leaf or a small node.  The
                    // walk visits these sites again and finds them harmless.
                    int clo = 0, ccnt = 0;
                    if (lane < min(sp, 32)) {
                        int c = W.stack[sp - 1 - lane];
                        for (;;) {
                            if (c < 0) {
                                clo = c & 0x7fffffff;
                                ccnt = 1;
                                break;
                            }
                            const int2 rg = A.tree.range[c];
                            if (rg.y - rg.x < kS1Bucket) {
                                clo = rg.x;
                                ccnt = rg.y - rg.x + 1;
                                break;
                            }
                            const int2 ch = A.tree.child[c];
                            float d0, d1;
                            if (ch.x < 0) {
                                const float2 q = A.tree.posf[ch.x & 0x7fffffff];
                                d0 = (q.x - ox) * (q.x - ox) + (q.y - oy) * (q.y - oy);
                            } else {
                                const float4 b = A.tree.boxf[ch.x];
                                const float dx = fmaxf(fmaxf(b.x - ox, ox - b.z), 0.0f);
                                const float dy = fmaxf(fmaxf(b.y - oy, oy - b.w), 0.0f);
                                d0 = dx * dx + dy * dy;
                            }
                            if (ch.y < 0) {
                                const float2 q = A.tree.posf[ch.y & 0x7fffffff];
                                d1 = (q.x - ox) * (q.x - ox) + (q.y - oy) * (q.y - oy);
                            } else {
                                const float4 b = A.tree.boxf[ch.y];
                                const float dx = fmaxf(fmaxf(b.x - ox, ox - b.z), 0.0f);
                                const float dy = fmaxf(fmaxf(b.y - oy, oy - b.w), 0.0f);
                                d1 = dx * dx + dy * dy;
                            }
                            c = d0 <= d1 ? ch.x : ch.y;
                        }
                    }
                    int cpos = ccnt;
                    for (int d = 1; d < 32; d <<= 1) {
                        const int y = __shfl_up_sync(kFull, cpos, d);
                        if (lane >= d) cpos += y;
                    }
                    ccount = __shfl_sync(kFull, cpos, 31);
                    cpos -= ccnt;
                    for (int q = 0; q < ccnt; q++) W.cand[cpos + q] = clo + q;
                    __syncwarp();
                    continue;
                }
            }
        }
        if (sp == 0) break;
        if (A.abort_flag) {
            const int f = lane == 0 ? *(volatile const int*)A.abort_flag : 0;
            if (__shfl_sync(kFull, f, 0)) {
                aborted = true;
                break;
            }
        }
        const int nb = min(sp, 32);
        sp -= nb;
        const bool have = lane < nb;
        const int nd = have ? W.stack[sp + lane] : 0;
        __syncwarp();
        popped += nb;
        int npush = 0, c0 = 0, c1 = 0, clo = 0, ccnt = 0;
        bool test = false, prune = false;
        if (have) {
            if (nd < 0) {
                clo = nd & 0x7fffffff;
                ccnt = 1;
            } else {
                // every node here lies outside the path to site k
                const int2 rg = A.tree.range[nd];
                const int2 ch = A.tree.child[nd];
                const float4 nbf = A.tree.boxf[nd];
                const float4 nnk = A.tree.nk[nd];
                test = true;
                prune = node_harmless_v(W.pux, W.puy, W.pur, n, ox, oy, owh, oxa, nbf, nnk);
                if (!prune) {
                    if (rg.y - rg.x < kS1Bucket) {
                        clo = rg.x;
                        ccnt = rg.y - rg.x + 1;
                    } else {
                        npush = 2;
                        c0 = ch.x;
                        c1 = ch.y;
                    }
                }
            }
        }
        tested += __popc(__ballot_sync(kFull, test));
        pruned += __popc(__ballot_sync(kFull, prune));
        // children onto the stack
        int pos = npush;
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(kFull, pos, d);
            if (lane >= d) pos += y;
        }
        const int tot = __shfl_sync(kFull, pos, 31);
        pos -= npush;
        if (sp + tot > kS1Stack) {
            overflow = true;
            break;
        }
        if (npush) {
            W.stack[sp + pos] = c1;
            W.stack[sp + pos + 1] = c0;
        }
        sp += tot;
        // the candidate sites, without the seeds already clipped
        unsigned cmask = 0;
        for (int q = 0; q < ccnt; q++)
            if (!is_seed(clo + q)) cmask |= 1u << q;
        const int cn = __popc(cmask);
        int cpos = cn;
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(kFull, cpos, d);
            if (lane >= d) cpos += y;
        }
        ccount = __shfl_sync(kFull, cpos, 31);
        cpos -= cn;
        for (int q = 0; q < ccnt; q++)
            if ((cmask >> q) & 1u) W.cand[cpos++] = clo + q;
        __syncwarp();
    }

    if (aborted) return;
    if (A.counters && lane == 0) {
        atomicAdd(&A.counters[0], (unsigned long long)popped);
        atomicAdd(&A.counters[1], (unsigned long long)tested);
        atomicAdd(&A.counters[2], (unsigned long long)pruned);
        atomicAdd(&A.counters[3], (unsigned long long)visited);
        atomicAdd(&A.counters[4], (unsigned long long)cuts);
    }
    const uint32_t sto = st & ~(uint32_t)ST_NEED_EXACT;
    if (sto && lane == 0) atomicOr(A.status, sto);
    if (empty) {
        if (lane == 0) {
            A.nb_cnt[k] = -1;
            if (A.abort_flag) atomicExch(A.abort_flag, 1);
        }
        return;
    }
    if (overflow) {
        if (lane == 0) {
            A.nb_cnt[k] = -2;  // finished by the large-capacity pass
            A.redo[atomicAdd(A.nredo, 1)] = k;
            atomicOr(A.status, ST_POLY_OVERFLOW);
        }
        return;
    }
    compact();
    if (A.counters && lane == 0) atomicAdd(&A.counters[5], (unsigned long long)ns);
    // the neighbour list by site index (the pieces are clipped in list order, so a
    // fixed order keeps their sums independent of the order of the walk)
    const int s0 = lane < ns ? W.slot[lane].site : INT_MAX;
    const int s1 = lane + 32 < ns ? W.slot[lane + 32].site : INT_MAX;
    int r0 = 0, r1 = 0;
    for (int j = 0; j < 32; j++) {
        const int a = __shfl_sync(kFull, s0, j), b = __shfl_sync(kFull, s1, j);
        r0 += (a < s0) + (b < s0);
        r1 += (a < s1) + (b < s1);
    }
    int* lab = A.nb_lab + (size_t)k * kCapSmall;
    if (lane < ns) lab[r0] = s0;
    if (lane + 32 < ns) lab[r1] = s1;
    // the cell's conservative absolute bounding box (cell_box)
    float mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    if (lane < n) {
        const float r = vr * 1.0001f;
        mnx = vx - r;
        mxx = vx + r;
        mny = vy - r;
        mxy = vy + r;
    }
    for (int d = 16; d > 0; d >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(kFull, mnx, d));
        mny = fminf(mny, __shfl_xor_sync(kFull, mny, d));
        mxx = fmaxf(mxx, __shfl_xor_sync(kFull, mxx, d));
        mxy = fmaxf(mxy, __shfl_xor_sync(kFull, mxy, d));
    }
    if (lane == 0) {
        A.nb_cnt[k] = ns;
        if (!(mxx - mnx < INFINITY && mxy - mny < INFINITY)) {
            A.cell_box[k] = make_double4(A.X0, A.Y0, A.X1, A.Y1);
        } else {
            const double sx = fmax(fabs((double)mnx), fabs((double)mxx)), sy = fmax(fabs((double)mny), fabs((double)mxy));
            A.cell_box[k] = make_double4(S.x + (double)mnx - 1e-6 * sx - 1e-300, S.y + (double)mny - 1e-6 * sy - 1e-300,
                                         S.x + (double)mxx + 1e-6 * sx + 1e-300, S.y + (double)mxy + 1e-6 * sy + 1e-300);
        }
    }
}

// ---------------------------------------------------------------------------
// stage 2: the pieces, batched over the cells of a warp
// ---------------------------------------------------------------------------
// A warp takes kWarpCells consecutive cells (neighbours in Morton order) and works
// in rounds:
//   A  the lanes walk the flat list of (cell, mesh triangle under the cell's box),
//      32 entries at a time, clip each triangle by its cell's neighbours (certified
//      FP32 side tests, FP64 filter) and append every non-empty piece -- cell,
//      triangle, edge labels -- to a list in shared memory, in list order;
//   B  each lane integrates one listed piece in FP64, so the lanes stay busy
//      whatever the sizes of the cells;
//   C  per cell the pieces' integrals and Hessian parts are summed in list order
//      (reproducible), and every cell whose triangles are all done is written out
//      by the whole warp.
// A cell that needs exact arithmetic or more capacity goes to the large pass.
__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

constexpr int kPieceWarps = 2;  // warps per block
constexpr int kWarpCells = 8;   // cells per warp
constexpr int kSlotPool = 96;   // neighbour slots held per warp
constexpr int kList = 64;       // listed pieces per round
constexpr int kPV = 12;         // vertices of a listed piece
constexpr int kClipCap = 16;    // polygon capacity while a triangle is clipped
static_assert(kSlotPool >= kCapSmall, "the pool must hold one full cell");
static_assert(kList >= 64, "a round needs room for one batch of 32 after 32 listed pieces");
static_assert(kCapSmall <= 64, "two Hessian slots per lane");

struct PieceRec {
    int tri;
    int8_t cell, n;
    int8_t lab[kPV];
    int rank, vrank;  // count / emit modes: index of the piece and of its first vertex within the cell
};

struct CellInfo {
    int k;     // sorted site index
    int m;     // neighbour slots (-1 empty cell, -2 left to the large pass)
    int soff;  // first slot in the pool
    int pre;   // first flat triangle entry
    int4 box;  // mesh-specific range of triangles under the cell's box
    int np, nv;  // count / emit modes: pieces and vertices listed so far
    double ax, ay;  // mixed mode: the centre of the cell's box, relative to the site
};

// modes of k_pieces: the evaluation, the evaluation with moments, the adjoint, and
// the two passes that materialise the pieces (count per cell, then emit)
constexpr int kModeEval = 0, kModeMoments = 1, kModeVjp = 2, kModeCount = 3, kModeEmit = 4, kModeMixed = 5,
              kModeVjpMixed = 6;

// phase A's cooperative clip: the polygon being clipped (one vertex per lane) passes
// through here between clip steps; the round's clipped pieces wait here for the list
struct ClipStage {
    float ux[32], uy[32], ur[32];
    int lab[32];
    int8_t res_lab[32][kPV];
    int8_t res_n[32];  // vertices of the clipped piece of each lane's entry; -1: needs the large pass
};

template <int MODE>
struct PieceWarp {
    static constexpr int kAcc =
        MODE == kModeVjp || MODE == kModeVjpMixed || MODE == kModeMixed ? 3 : (MODE == kModeMoments ? 7 : 2);
    ClipStage cs;
    Slot slot[kSlotPool];
    Nb64 nb[kSlotPool];
    float zc[MODE == kModeMixed || MODE == kModeVjpMixed ? kSlotPool : 1];  // mixed: each axis about its cell's anchor
    PieceRec rec[kList];
    double out[kAcc][kList];
    // the Hessian part of each listed piece's edges; FP32 in the mixed evaluation (its
    // edges are FP32 integrals, or FP64 ones that need only 2.5e-4), which leaves room
    // for one more block per SM
    typename std::conditional<MODE == kModeMixed, float, double>::type hvc[kPV][kList];
    CellInfo ci[kWarpCells + 1];
    short epre[kList + 1];  // phase C: first contribution of each of the cell's listed pieces
    signed char lead[64];   // phase C: the lane holding each slot's sum of a batch, or -1
};

// triangles of the grid mesh under a box: squares [i0, i0+nsx) x [j0, j0+nsy),
// two triangles each; triangle id = ((j (nx-1) + i) << 1) | tt
struct GridPieces {
    MeshGridDev m;
    __device__ __forceinline__ int setup(const double4& bb, int4& p) const
    {
        if (bb.z < m.gx[0] || bb.x > m.gx[m.nx - 1] || bb.w < m.gy[0] || bb.y > m.gy[m.ny - 1]) return 0;
        int i0 = find_square(m.gx, m.nx, bb.x), i1 = find_square(m.gx, m.nx, bb.z);
        int j0 = find_square(m.gy, m.ny, bb.y), j1 = find_square(m.gy, m.ny, bb.w);
        p = make_int4(i0, j0, i1 - i0 + 1, j1 - j0 + 1);
        return 2 * p.z * p.w;
    }
    __device__ __forceinline__ int get(const int4& p, int t) const
    {
        int sq = t >> 1;
        int i = p.x + sq % p.z, j = p.y + sq / p.z;
        return ((j * (m.nx - 1) + i) << 1) | (t & 1);
    }
    __device__ __forceinline__ void fixed(int id, const Owner& o, Fixed& T) const
    {
        int sq = id >> 1;
        grid_fixed(m, sq % (m.nx - 1), sq / (m.nx - 1), id & 1, o, T);
    }
    __device__ __forceinline__ Corners corners(int id, const Owner& o) const
    {
        int sq = id >> 1;
        return grid_corners(m, sq % (m.nx - 1), sq / (m.nx - 1), id & 1, o);
    }
    __device__ __forceinline__ void triangle(int id, const Owner& o, Fixed& T, double& c0, double& gx,
                                             double& gy) const
    {
        int sq = id >> 1;
        grid_triangle(m, sq % (m.nx - 1), sq / (m.nx - 1), id & 1, o, T, c0, gx, gy);
    }
    // vertex indices (j nx + i) of the triangle's corners, in the order of grid_fixed
    __device__ __forceinline__ void vertices(int id, int* v) const
    {
        const int sq = id >> 1, i = sq % (m.nx - 1), j = sq / (m.nx - 1);
        const int v00 = j * m.nx + i;
        v[0] = v00;
        v[1] = (id & 1) ? v00 + m.nx + 1 : v00 + 1;
        v[2] = (id & 1) ? v00 + m.nx : v00 + m.nx + 1;
    }
};

// triangles of an explicit mesh under a box: the entries of the box's bins (a row
// of bins is contiguous in the bin lists); a triangle is taken from the first bin
// it shares with the box, its other entries give -1
struct TriPieces {
    MeshTriDev m;
    __device__ __forceinline__ int setup(const double4& bb, int4& p) const
    {
        int cx0, cy0, cx1, cy1;
        if (!tri_bins(m, bb.x, bb.y, bb.z, bb.w, cx0, cy0, cx1, cy1)) return 0;
        p = make_int4(cx0, cy0, cx1, cy1);
        int cnt = 0;
        for (int by = cy0; by <= cy1; by++) cnt += m.bin_start[by * m.bnx + cx1 + 1] - m.bin_start[by * m.bnx + cx0];
        return cnt;
    }
    __device__ __forceinline__ int get(const int4& p, int t) const
    {
        for (int by = p.y; by <= p.w; by++) {
            const int b0 = by * m.bnx + p.x;
            const int q0 = m.bin_start[b0], r = m.bin_start[by * m.bnx + p.z + 1] - q0;
            if (t < r) {
                const int q = q0 + t;
                int bx = p.x;
                while (m.bin_start[by * m.bnx + bx + 1] <= q) bx++;
                const int tri = m.bin_tri[q];
                const int4 tb = m.tbin[tri];
                if (bx != max(tb.x, p.x) || by != max(tb.y, p.y)) return -1;
                return tri;
            }
            t -= r;
        }
        return -1;
    }
    __device__ __forceinline__ void fixed(int id, const Owner& o, Fixed& T) const { tri_fixed(m, id, o, T); }
    __device__ __forceinline__ Corners corners(int id, const Owner& o) const { return tri_corners(m, id, o); }
    __device__ __forceinline__ void triangle(int id, const Owner& o, Fixed& T, double& c0, double& gx,
                                             double& gy) const
    {
        tri_triangle(m, id, o, T, c0, gx, gy);
    }
    __device__ __forceinline__ void vertices(int id, int* v) const
    {
        v[0] = m.tri[3 * id];
        v[1] = m.tri[3 * id + 1];
        v[2] = m.tri[3 * id + 2];
    }
};

// write one finished cell: lane 0 the masses and moments, lane s (and s + 32) the
// Hessian entry of neighbour slot s, placed by rank of its column
template <bool MOM>
__device__ __forceinline__ void finish_cell(const CellArgs& A, const CellInfo& C, const double* run, double h0,
                                            double h1, bool t0, bool t1, const Slot* sl, const Nb64* nb, int lane)
{
    const int gi = A.perm[C.k];
    const SiteD S = A.sites[C.k];
    if (lane == 0) {
        A.mass[gi] = run[0];
        A.vpart[gi] = S.w * run[0] - run[1];
        if (MOM && A.mom) {
            double* mo = A.mom + 6 * (size_t)gi;
            const double M = run[0], m1x = run[2], m1y = run[3];
            mo[0] = M;
            mo[1] = m1x + S.x * M;
            mo[2] = m1y + S.y * M;
            mo[3] = run[4] + 2.0 * S.x * m1x + S.x * S.x * M;
            mo[4] = run[5] + 2.0 * S.y * m1y + S.y * S.y * M;
            mo[5] = run[6] + S.x * m1y + S.y * m1x + S.x * S.y * M;
        }
    }
    if (!A.rowcnt) return;
    const bool a0 = t0 && lane < C.m, a1 = t1 && lane + 32 < C.m;
    int col0 = INT_MAX, col1 = INT_MAX;
    double v0 = 0.0, v1 = 0.0;
    if (a0) {
        const Nb64 d = nb[lane];
        v0 = -h0 / (2.0 * (d.dx * d.dx + d.dy * d.dy));
        col0 = A.perm[sl[lane].site];
    }
    if (a1) {
        const Nb64 d = nb[lane + 32];
        v1 = -h1 / (2.0 * (d.dx * d.dx + d.dy * d.dy));
        col1 = A.perm[sl[lane + 32].site];
    }
    const double diag = -warp_sum(v0 + v1);
    const int cnt = __popc(__ballot_sync(0xffffffffu, a0)) + __popc(__ballot_sync(0xffffffffu, a1));
    const int total = cnt > 0 ? cnt + 1 : 0;
    if (lane == 0) A.rowcnt[gi] = total;
    if (total == 0) return;
    int r0 = gi < col0 ? 1 : 0, r1 = gi < col1 ? 1 : 0, rd = 0;
    for (int j = 0; j < 32; j++) {
        const int c0 = __shfl_sync(0xffffffffu, col0, j), c1 = __shfl_sync(0xffffffffu, col1, j);
        r0 += (c0 < col0) + (c1 < col0);
        r1 += (c0 < col1) + (c1 < col1);
        rd += (c0 < gi) + (c1 < gi);
    }
    int* oc = A.st_col + (size_t)gi * A.scap;
    double* ov = A.st_val + (size_t)gi * A.scap;
    if (a0) {
        oc[r0] = col0;
        ov[r0] = v0;
    }
    if (a1) {
        oc[r1] = col1;
        ov[r1] = v1;
    }
    if (lane == 0) {
        oc[rd] = gi;
        ov[rd] = diag;
    }
}

// the adjoint of one listed piece: its share of g_w and g_x of the owner (the
// radical-axis edge terms of integrate_vjp plus the value's interior terms
// a int rho and 2 a int rho u), and its share of g_rho on the triangle's corners,
//     int_piece (a (w_i - |u|^2) + b_i + e_i . x) lambda_k(x)
// for the barycentric coordinate lambda_k (linear; the integrand is cubic in u)
template <bool F32, class E>
__device__ __forceinline__ void vjp_piece(const CellArgs& A, const E& mesh, const PieceRec& R, int k, int gi,
                                          const SiteD& S, const Slot* sl, const Nb64* nb, const float* zc, double ax,
                                          double ay, const Fixed& T, double c0, double gx, double gy, double& ow,
                                          double& ox, double& oy)
{
    const double a = A.cot_value;
    const double bi = A.cot_mass ? A.cot_mass[gi] : 0.0;
    const double exi = A.cot_mom ? A.cot_mom[2 * (size_t)gi] : 0.0;
    const double eyi = A.cot_mom ? A.cot_mom[2 * (size_t)gi + 1] : 0.0;
    PieceMoments M;
    double gw = 0.0, gpx = 0.0, gpy = 0.0;
    auto lab_of = [&](int e) { return (int)R.lab[e]; };
    auto cot = [&](int slot, double& bj, double& ejx, double& ejy) {
        const int gj = A.perm[sl[slot].site];
        bj = A.cot_mass ? A.cot_mass[gj] : 0.0;
        ejx = A.cot_mom ? A.cot_mom[2 * (size_t)gj] : 0.0;
        ejy = A.cot_mom ? A.cot_mom[2 * (size_t)gj + 1] : 0.0;
    };
    if (F32)
        integrate_vjp32((int)R.n, lab_of, sl, zc, ax, ay, T, c0, gx, gy, S.x, S.y, bi, exi, eyi, cot, M, gw, gpx, gpy);
    else
        integrate_vjp((int)R.n, lab_of, nb, T, c0, gx, gy, S.x, S.y, bi, exi, eyi, cot, M, gw, gpx, gpy);
    const double rho_m = c0 * M.I1 + gx * M.Iux + gy * M.Iuy;
    const double rux = c0 * M.Iux + gx * M.Sxx + gy * M.Sxy, ruy = c0 * M.Iuy + gx * M.Sxy + gy * M.Syy;
    ow = gw + a * rho_m;
    ox = gpx + 2.0 * a * rux;
    oy = gpy + 2.0 * a * ruy;
    if (!A.grad_rho) return;
    int v[3];
    mesh.vertices(R.tri, v);
    const double cp = a * S.w + bi + exi * S.x + eyi * S.y;
    const double s0 = cp * M.I1 + exi * M.Iux + eyi * M.Iuy - a * M.Iq;
    const double sx = cp * M.Iux + M.Sxx * exi + M.Sxy * eyi - a * M.Icx;
    const double sy = cp * M.Iuy + M.Sxy * exi + M.Syy * eyi - a * M.Icy;
    const double A2 = (T.rx[1] - T.rx[0]) * (T.ry[2] - T.ry[0]) - (T.ry[1] - T.ry[0]) * (T.rx[2] - T.rx[0]);
    for (int q = 0; q < 3; q++) {
        const int q1 = q == 2 ? 0 : q + 1, q2 = q == 0 ? 2 : q - 1;
        const double ex = T.rx[q2] - T.rx[q1], ey = T.ry[q2] - T.ry[q1];
        // lambda_q(u) = (e x (u - r_q1)) / A2 = alpha + beta . u
        const double alpha = (ey * T.rx[q1] - ex * T.ry[q1]) / A2;
        const double bx = -ey / A2, by = ex / A2;
        atomicAdd(&A.grad_rho[v[q]], alpha * s0 + bx * sx + by * sy);
    }
}

template <int MODE, class E>
__global__ void __launch_bounds__(32 * kPieceWarps, 7) k_pieces(CellArgs A, E mesh)
{
    constexpr bool MOM = MODE == kModeMoments, VJP = MODE == kModeVjp || MODE == kModeVjpMixed;
    // the mixed modes take the cell's integrals about its anchor (integrate_piece32)
    constexpr bool ANCHOR = MODE == kModeMixed || MODE == kModeVjpMixed;
    constexpr bool LISTING = MODE == kModeCount || MODE == kModeEmit;
    constexpr bool MIXED = MODE == kModeMixed;
    constexpr int kAcc = PieceWarp<MODE>::kAcc;
    constexpr unsigned kFull = 0xffffffffu;
    __shared__ PieceWarp<MODE> shw[kPieceWarps];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    PieceWarp<MODE>& W = shw[wib];
    // the cells: sorted indices kbase .. kbase + 7, or entries of a cell list (the
    // mixed form's cells redone in FP64)
    const int ntot = A.cell_list ? A.ncell_list : A.n;
    auto cell_at = [&](int q) { return A.cell_list ? A.cell_list[q] : q; };
    const int kbase = (blockIdx.x * kPieceWarps + wib) * kWarpCells;
    if (kbase >= ntot) return;
    if (A.abort_flag && *(volatile const int*)A.abort_flag) return;
    const int ncell = min(kWarpCells, ntot - kbase);
    // lane c sets up cell c
    int my_m = -2, my_cnt = 0;
    int4 my_box = make_int4(0, 0, 0, 0);
    double my_ax = 0.0, my_ay = 0.0;
    if (lane < ncell) {
        const int k = cell_at(kbase + lane);
        my_m = A.nb_cnt[k];
        if (my_m == -1) {
            const int gi = A.perm[k];
            if (LISTING) {
                if (MODE == kModeCount) {
                    A.pc_cnt[k] = 0;
                    A.pv_cnt[k] = 0;
                }
            } else if (VJP) {
                A.grad_w[gi] = 0.0;
                A.grad_x[gi] = 0.0;
                A.grad_y[gi] = 0.0;
            } else {
                write_empty(A, gi, MOM);
            }
        }
        if (my_m >= 0) {
            const double4 cb = A.cell_box[k];
            my_cnt = mesh.setup(cb, my_box);
            if (ANCHOR) {
                const SiteD S = A.sites[k];
                my_ax = 0.5 * (cb.x + cb.z) - S.x;
                my_ay = 0.5 * (cb.y + cb.w) - S.y;
            }
        }
    }
    uint32_t st = 0;
    unsigned redo = 0;  // cells of the warp to redo (bit c)
    int mx_np = 0, mx_fa = 0, mx_ne = 0, mx_fe = 0;  // mixed mode: pieces, cells redone in FP64, edges, FP64 edges
    for (int g0 = 0; g0 < ncell;) {
        // a group of cells whose neighbour slots fit in the pool
        int g1 = g0, soff = 0, pre = 0;
        while (g1 < ncell) {
            const int mc = __shfl_sync(kFull, my_m, g1), nc = __shfl_sync(kFull, my_cnt, g1);
            const int4 bx = make_int4(__shfl_sync(kFull, my_box.x, g1), __shfl_sync(kFull, my_box.y, g1),
                                      __shfl_sync(kFull, my_box.z, g1), __shfl_sync(kFull, my_box.w, g1));
            const int used = max(mc, 0);
            if (soff + used > kSlotPool) break;
            const double cax = __shfl_sync(kFull, my_ax, g1), cay = __shfl_sync(kFull, my_ay, g1);
            if (lane == 0) W.ci[g1 - g0] = CellInfo{cell_at(kbase + g1), mc, soff, pre, bx, 0, 0, cax, cay};
            soff += used;
            pre += nc;
            g1++;
        }
        const int ng = g1 - g0, nslot = soff, total = pre;
        if (lane == 0) W.ci[ng].pre = total;  // sentinel
        __syncwarp();
        for (int idx = lane; idx < nslot; idx += 32) {
            int c = 0;
            while (c + 1 < ng && W.ci[c + 1].soff <= idx) c++;
            const CellInfo& C = W.ci[c];
            const int q = A.nb_lab[(size_t)C.k * kCapSmall + (idx - C.soff)];
            const SiteD S = A.sites[C.k];
            const Owner o{S.x, S.y, S.w, C.k};
            const SiteD Q = A.sites[q];
            W.slot[idx] = make_slot(q, Q, o);
            const Nb64 nbq = make_nb64(Q, o);
            W.nb[idx] = nbq;
            // mixed: the radical axis about the cell's anchor, 2 v.d = z - 2 a.d
            if (ANCHOR) W.zc[idx] = (float)(nbq.z - 2.0 * (C.ax * nbq.dx + C.ay * nbq.dy));
        }
        __syncwarp();
        int f = 0;     // next flat entry
        int cfin = 0;  // next cell of the group to finish
        double run[kAcc];
        for (int q = 0; q < kAcc; q++) run[q] = 0.0;
        double h0 = 0.0, h1 = 0.0;
        bool t0 = false, t1 = false;
        for (;;) {
            // A: clip 32 entries at a time while a full batch still fits in the list
            int L = 0;
            while (f < total && L <= kList - 32) {
                const int idx = f + lane;
                int cc = 0, id = -1;
                bool out = true;  // no triangle, or one outside the cell
                uint64_t cut = 0;
                Corners K;
                if (idx < total) {
                    while (W.ci[cc + 1].pre <= idx) cc++;
                    const CellInfo& C = W.ci[cc];
                    id = mesh.get(C.box, idx - C.pre);
                    if (id >= 0) {
                        const SiteD S = A.sites[C.k];
                        const Owner o{S.x, S.y, S.w, C.k};
                        const Slot* sl = W.slot + C.soff;
                        // certified corner tests: a slot with all three corners outside
                        // rejects the triangle; a slot with all three inside contains every
                        // sub-polygon of it and needs no clip
                        K = mesh.corners(id, o);
                        out = false;
                        for (int s = 0; s < C.m; s++) {
                            const Slot cs = sl[s];
                            const int t0 = test32(K.ux[0], K.uy[0], K.ur[0], cs);
                            const int t1 = test32(K.ux[1], K.uy[1], K.ur[1], cs);
                            const int t2 = test32(K.ux[2], K.uy[2], K.ur[2], cs);
                            if (t0 > 0 && t1 > 0 && t2 > 0) {
                                out = true;
                                break;
                            }
                            if (!(t0 < 0 && t1 < 0 && t2 < 0)) cut |= 1ull << s;
                        }
                    }
                }
                // the triangles that some radical axis crosses, clipped two at a time, one
                // per half-warp: lane v of the half holds vertex v, a clip step is a ballot
                // of the vertices outside, an exclusive scan of the Sutherland-Hodgman
                // outputs (vtx_* of ma_cell.cuh for the new vertices) and a pass through
                // the half's part of the stage
                static_assert(kClipCap == 16, "one polygon vertex per lane of a half-warp");
                const int hw = lane >> 4, hl = lane & 15;
                const unsigned hmask = 0xFFFFu << (16 * hw);
                unsigned pend = __ballot_sync(kFull, !out && cut != 0);
                while (pend) {
                    const int s0 = __ffs(pend) - 1;
                    pend &= pend - 1;
                    int s1 = -1;
                    if (pend) {
                        s1 = __ffs(pend) - 1;
                        pend &= pend - 1;
                    }
                    const int src = hw == 0 ? s0 : s1;
                    const int srcq = src < 0 ? s0 : src;
                    const int ecc = __shfl_sync(kFull, cc, srcq), eid = __shfl_sync(kFull, id, srcq);
                    uint64_t ecut = ((uint64_t)__shfl_sync(kFull, (unsigned)(cut >> 32), srcq) << 32) |
                                    (uint64_t)__shfl_sync(kFull, (unsigned)cut, srcq);
                    float cx[3], cy[3], cr[3];
                    for (int e = 0; e < 3; e++) {
                        cx[e] = __shfl_sync(kFull, K.ux[e], srcq);
                        cy[e] = __shfl_sync(kFull, K.uy[e], srcq);
                        cr[e] = __shfl_sync(kFull, K.ur[e], srcq);
                    }
                    const CellInfo& C = W.ci[ecc];
                    const SiteD S = A.sites[C.k];
                    const Owner o{S.x, S.y, S.w, C.k};
                    const Slot* sl = W.slot + C.soff;
                    float* sux = W.cs.ux + 16 * hw;
                    float* suy = W.cs.uy + 16 * hw;
                    float* sur = W.cs.ur + 16 * hw;
                    int* slab = W.cs.lab + 16 * hw;
                    int n = src < 0 ? 0 : 3;
                    float pux = hl == 0 ? cx[0] : (hl == 1 ? cx[1] : cx[2]);
                    float puy = hl == 0 ? cy[0] : (hl == 1 ? cy[1] : cy[2]);
                    float pur = hl == 0 ? cr[0] : (hl == 1 ? cr[1] : cr[2]);
                    int plab = -1 - min(hl, 2);
                    bool ebad = false;
                    while (ecut && n > 0) {
                        const int s = __ffsll((long long)ecut) - 1;
                        ecut &= ecut - 1;
                        const Slot c = sl[s];
                        const bool act = hl < n;
                        const int prevlab = __shfl_sync(hmask, plab, hl == 0 ? n - 1 : hl - 1, 16);
                        bool vout = false, und = false;
                        if (act) {
                            const int t = test32(pux, puy, pur, c);
                            if (t != 0) {
                                vout = t > 0;
                            } else {
                                Fixed T;  // the exact corners, only for an undecided vertex
                                mesh.fixed(eid, o, T);
                                vout = !sym_inside<kClipCap, false>(prevlab, plab, sl, T, o, A.sites, c.site, st, und);
                            }
                        }
                        if (__any_sync(hmask, und)) {
                            // an exact decision is needed: the cell is redone by the exact pass
                            st |= ST_NEED_EXACT;
                            ebad = true;
                            break;
                        }
                        const unsigned om = (__ballot_sync(hmask, act && vout) >> (16 * hw)) & 0xFFFFu;
                        const int nout = __popc(om);
                        if (nout == 0) continue;
                        if (nout == n) {
                            n = 0;
                            break;
                        }
                        const int v1 = hl + 1 == n ? 0 : hl + 1;
                        const bool in0 = act && !vout, in1 = !((om >> v1) & 1u);
                        const int cnt = act ? (in0 ? (in1 ? 1 : 2) : (in1 ? 1 : 0)) : 0;
                        int pos = cnt;
                        for (int d = 1; d < 16; d <<= 1) {
                            const int y = __shfl_up_sync(hmask, pos, d, 16);
                            if (hl >= d) pos += y;
                        }
                        const int m = __shfl_sync(hmask, pos, 15, 16);
                        pos -= cnt;
                        if (m > kClipCap) {
                            ebad = true;
                            break;
                        }
                        if (act) {
                            int q = pos;
                            if (in0) {
                                sux[q] = pux;
                                suy[q] = puy;
                                sur[q] = pur;
                                slab[q] = plab;
                                q++;
                            }
                            if (in0 != in1) {
                                float nx, ny, nr;
                                if (plab < 0) {
                                    const int e = -1 - plab, e1 = e == 2 ? 0 : e + 1;
                                    vtx_seg_bis(pick(cx, e), pick(cy, e), pick(cr, e), pick(cx, e1), pick(cy, e1),
                                                pick(cr, e1), c, nx, ny, nr);
                                } else {
                                    vtx_bis_bis(sl[plab], c, nx, ny, nr);
                                }
                                sux[q] = nx;
                                suy[q] = ny;
                                sur[q] = nr;
                                slab[q] = in0 ? s : plab;
                            }
                        }
                        __syncwarp(hmask);
                        n = m;
                        if (hl < n) {
                            pux = sux[hl];
                            puy = suy[hl];
                            pur = sur[hl];
                            plab = slab[hl];
                        }
                        __syncwarp(hmask);
                    }
                    if (!ebad && n > kPV) ebad = true;
                    if (src >= 0) {
                        if (hl == 0) W.cs.res_n[src] = (int8_t)(ebad ? -1 : n);
                        if (!ebad && hl < n) W.cs.res_lab[src][hl] = (int8_t)plab;
                    }
                    __syncwarp();
                }
                __syncwarp();
                const bool whole = !out && cut == 0;
                const int rn = (!out && cut != 0) ? (int)W.cs.res_n[lane] : 0;
                const bool bad = rn < 0;
                const bool keep = whole || rn > 0;
                redo |= __reduce_or_sync(kFull, bad ? (1u << (g0 + cc)) : 0u);
                const unsigned bal = __ballot_sync(kFull, keep);
                const int pn = whole ? 3 : (keep ? rn : 0);
                if (keep) {
                    PieceRec& R = W.rec[L + __popc(bal & ((1u << lane) - 1u))];
                    R.tri = id;
                    R.cell = (int8_t)cc;
                    R.n = (int8_t)pn;
                    if (whole) {
                        R.lab[0] = -1;
                        R.lab[1] = -2;
                        R.lab[2] = -3;
                    } else {
                        for (int e = 0; e < pn; e++) R.lab[e] = W.cs.res_lab[lane][e];
                    }
                }
                if (LISTING) {
                    // rank of each kept piece within its cell, and the vertices of the
                    // cell's earlier pieces (the lanes of one cell are adjacent)
                    const unsigned same = __match_any_sync(kFull, keep ? cc : -1 - lane);
                    const unsigned before = same & bal & ((1u << lane) - 1u);
                    const int nk = pn;
                    int vpre = 0;
                    for (int j = 0; j < 32; j++) {
                        const int nj = __shfl_sync(kFull, nk, j);
                        if ((before >> j) & 1u) vpre += nj;
                    }
                    if (keep) {
                        PieceRec& R = W.rec[L + __popc(bal & ((1u << lane) - 1u))];
                        R.rank = W.ci[cc].np + __popc(before);
                        R.vrank = W.ci[cc].nv + vpre;
                    }
                    __syncwarp();
                    if (keep && !(same & bal & ~((2u << lane) - 1u))) {
                        W.ci[cc].np += __popc(before) + 1;
                        W.ci[cc].nv += vpre + nk;
                    }
                    __syncwarp();
                }
                L += __popc(bal);
                f += 32;
            }
            f = min(f, total);
            __syncwarp();
            // B: one piece per lane
            for (int p = lane; p < L && MODE != kModeCount; p += 32) {
                const PieceRec& R = W.rec[p];  // read in place: a local copy would sit in local memory
                if (MODE == kModeEmit) {
                    const CellInfo& C = W.ci[R.cell];
                    const SiteD S = A.sites[C.k];
                    const Owner o{S.x, S.y, S.w, C.k};
                    Fixed T;
                    mesh.fixed(R.tri, o, T);
                    const int64_t gp = A.pc_base[C.k] + R.rank, gv = A.pv_base[C.k] + R.vrank;
                    A.out_site[gp] = A.perm[C.k];
                    A.out_tri[gp] = R.tri;
                    A.out_off[gp] = gv;
                    const Slot* sl = W.slot + C.soff;
                    const int n = R.n;
                    for (int e = 0; e < n; e++) {
                        double X, Y;
                        vtx64(R.lab[e == 0 ? n - 1 : e - 1], R.lab[e], W.nb + C.soff, T, X, Y);
                        A.out_xy[2 * (gv + e)] = S.x + X;
                        A.out_xy[2 * (gv + e) + 1] = S.y + Y;
                        const int l = R.lab[e];
                        A.out_edge[gv + e] = l >= 0 ? A.perm[sl[l].site] : l;
                    }
                    continue;
                }
                const CellInfo& C = W.ci[R.cell];
                const SiteD S = A.sites[C.k];
                const Owner o{S.x, S.y, S.w, C.k};
                Fixed T;
                double c0, gx, gy;
                mesh.triangle(R.tri, o, T, c0, gx, gy);
                if (VJP) {
                    double ow, ox, oy;
                    vjp_piece<MODE == kModeVjpMixed>(A, mesh, R, C.k, A.perm[C.k], S, W.slot + C.soff, W.nb + C.soff,
                                                     W.zc + (ANCHOR ? C.soff : 0), C.ax, C.ay, T, c0, gx, gy, ow,
                                                     ox, oy);
                    W.out[0][p] = ow;
                    W.out[1 % kAcc][p] = ox;
                    W.out[2 % kAcc][p] = oy;
                    continue;
                }
                if (MIXED) {
                    // FP32 integrals of the piece; the cell sums below are FP64
                    double pm, ps, pe;
                    integrate_piece32(
                        (int)R.n, [&](int e) { return (int)R.lab[e]; }, W.slot + C.soff, W.nb + C.soff,
                        W.zc + (MIXED ? C.soff : 0), C.ax, C.ay, T, c0, gx, gy, pm, ps, pe,
                        [&](int e, int, double v) { W.hvc[e][p] = v; }, mx_ne, mx_fe);
                    mx_np++;
                    W.out[0][p] = pm;
                    W.out[1][p] = ps;
                    W.out[2 % kAcc][p] = pe;
                    continue;
                }
                Acc acc{0, 0, 0, 0, 0, 0, 0};
                integrate_labels<MOM>(
                    (int)R.n, [&](int e) { return (int)R.lab[e]; }, W.nb + C.soff, T, c0, gx, gy, acc,
                    [&](int e, int, double v) { W.hvc[e][p] = v; }, MOM || A.value != 0);
                W.out[0][p] = acc.mass;
                W.out[1][p] = acc.second;
                if (MOM) {
                    W.out[2 % kAcc][p] = acc.m1x;
                    W.out[3 % kAcc][p] = acc.m1y;
                    W.out[4 % kAcc][p] = acc.sxx;
                    W.out[5 % kAcc][p] = acc.syy;
                    W.out[6 % kAcc][p] = acc.sxy;
                }
            }
            __syncwarp();
            // C: sums per cell in list order; finish the complete cells
            int p0 = 0;
            while (cfin < ng) {
                const CellInfo& C = W.ci[cfin];
                const int cend = W.ci[cfin + 1].pre;
                const bool complete = cend <= f;
                if (!complete && C.pre >= f) break;
                int p1 = p0;
                for (;;) {
                    const int q = p1 + lane;
                    const unsigned b = __ballot_sync(kFull, q < L && W.rec[q].cell == cfin);
                    p1 += __popc(b);
                    if (b != kFull) break;
                }
                for (int q = 0; q < kAcc && !LISTING; q++) {
                    double v = 0.0;
                    for (int p = p0 + lane; p < p1; p += 32) v += W.out[q][p];
                    run[q] += warp_sum(v);
                }
                if (!VJP && !LISTING) {
                    // the Hessian part of every edge (piece p, vertex e) of the cell's listed
                    // pieces, 32 at a time in list order: the lanes with the same slot are
                    // summed in lane order by the lowest of them, and lane l (l + 32) adds
                    // the sums of slot l (l + 32) -- a fixed order, so the rows reproduce
                    int eb = 0;
                    for (int q = p0; q < p1; q += 32) {
                        const int pp = q + lane;
                        const int cnt = pp < p1 ? (int)W.rec[pp].n : 0;
                        int x = cnt;
                        for (int d = 1; d < 32; d <<= 1) {
                            const int y = __shfl_up_sync(kFull, x, d);
                            if (lane >= d) x += y;
                        }
                        if (pp < p1) W.epre[pp - p0] = (short)(eb + x - cnt);
                        eb += __shfl_sync(kFull, x, 31);
                    }
                    if (lane == 0) W.epre[p1 - p0] = (short)eb;
                    W.lead[lane] = -1;
                    W.lead[lane + 32] = -1;
                    __syncwarp();
                    const int np = p1 - p0;
                    for (int t0b = 0; t0b < eb; t0b += 32) {
                        const int t = t0b + lane;
                        int l = -1;
                        double v = 0.0;
                        if (t < eb) {
                            int lo = 0, hi = np - 1;  // the piece: last epre <= t
                            while (lo < hi) {
                                const int mid = (lo + hi + 1) >> 1;
                                if (W.epre[mid] <= t)
                                    lo = mid;
                                else
                                    hi = mid - 1;
                            }
                            const int pq = p0 + lo, e = t - W.epre[lo];
                            l = W.rec[pq].lab[e];
                            if (l >= 0) v = W.hvc[e][pq];
                        }
                        const unsigned grp = __match_any_sync(kFull, l >= 0 ? l : -1 - lane);
                        const bool leader = l >= 0 && (grp & ((1u << lane) - 1u)) == 0u;
                        const int gmax = __reduce_max_sync(kFull, __popc(grp));
                        double gs = 0.0;
                        unsigned rem = grp;
                        for (int r = 0; r < gmax; r++) {
                            const int src = rem ? __ffs(rem) - 1 : lane;
                            rem &= rem - 1;
                            const double vr = __shfl_sync(kFull, v, src);
                            if (leader && r < __popc(grp)) gs += vr;
                        }
                        if (leader) W.lead[l] = (signed char)lane;
                        __syncwarp();
                        const int l0 = W.lead[lane], l1 = W.lead[lane + 32];
                        const double g0v = __shfl_sync(kFull, gs, l0 >= 0 ? l0 : lane);
                        const double g1v = __shfl_sync(kFull, gs, l1 >= 0 ? l1 : lane);
                        if (l0 >= 0) {
                            h0 += g0v;
                            t0 = true;
                        }
                        if (l1 >= 0) {
                            h1 += g1v;
                            t1 = true;
                        }
                        __syncwarp();
                        W.lead[lane] = -1;
                        W.lead[lane + 32] = -1;
                        __syncwarp();
                    }
                }
                p0 = p1;
                if (!complete) break;
                if (C.m >= 0) {
                    // mixed: a cell whose certified FP32 mass error exceeds kMassTol32 of its
                    // mass is redone by the FP64 pieces kernel (its cell list)
                    const bool fp64_redo = MIXED && !((redo >> (g0 + cfin)) & 1u) &&
                                           !(run[2 % kAcc] <= (double)kMassTol32 * fabs(run[0]));
                    if (fp64_redo) {
                        if (lane == 0) {
                            A.redo64[atomicAdd(A.nredo64, 1)] = C.k;
                            mx_fa++;
                        }
                    } else if ((redo >> (g0 + cfin)) & 1u) {
                        if (lane == 0) {
                            A.redo[atomicAdd(A.nredo, 1)] = C.k;
                            atomicOr(A.status, ST_POLY_OVERFLOW);
                        }
                    } else if (LISTING) {
                        if (MODE == kModeCount && lane == 0) {
                            A.pc_cnt[C.k] = C.np;
                            A.pv_cnt[C.k] = C.nv;
                        }
                    } else if (VJP) {
                        if (lane == 0) {
                            const int gi = A.perm[C.k];
                            A.grad_w[gi] = run[0];
                            A.grad_x[gi] = run[1 % kAcc];
                            A.grad_y[gi] = run[2 % kAcc];
                        }
                    } else {
                        finish_cell<MOM>(A, C, run, h0, h1, t0, t1, W.slot + C.soff, W.nb + C.soff, lane);
                    }
                }
                for (int q = 0; q < kAcc; q++) run[q] = 0.0;
                h0 = h1 = 0.0;
                t0 = t1 = false;
                cfin++;
            }
            __syncwarp();
            if (f >= total) break;
        }
        g0 = g1;
    }
    st &= ~(uint32_t)ST_NEED_EXACT;
    if (st) atomicOr(A.status, st);
    if (MIXED && A.counters) {
        const int c0 = __reduce_add_sync(kFull, mx_np), c1 = __reduce_add_sync(kFull, mx_fa);
        const int c2 = __reduce_add_sync(kFull, mx_ne), c3 = __reduce_add_sync(kFull, mx_fe);
        if (lane == 0) {
            atomicAdd(&A.counters[6], (unsigned long long)c0);
            atomicAdd(&A.counters[7], (unsigned long long)c1);
            atomicAdd(&A.counters[8], (unsigned long long)c2);
            atomicAdd(&A.counters[9], (unsigned long long)c3);
        }
    }
}

// ---------------------------------------------------------------------------
// large-capacity pass and launchers
// ---------------------------------------------------------------------------
template <int CAP, bool MOM, class Mesh>
__global__ void __launch_bounds__(64) k_cells_large(CellArgs A, Mesh M)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.nwork) return;
    Work<CAP>* W = reinterpret_cast<Work<CAP>*>(A.scratch) + t;
    process_site<CAP, MOM>(A, M, A.work[t], *W, t);
}

template <bool EMIT, class Mesh>
__global__ void __launch_bounds__(64) k_cells_large_list(CellArgs A, Mesh M)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.nwork) return;
    Work<kCapLarge>* W = reinterpret_cast<Work<kCapLarge>*>(A.scratch) + t;
    list_site<kCapLarge, EMIT>(A, M, A.work[t], *W);
}

__global__ void k_mark_large(const int* work, int nwork, int* nb_cnt)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nwork) nb_cnt[work[t]] = -3;
}

void launch_cells_large_list(const CellArgs& a, const MeshGridDev* g, const MeshTriDev* tm, bool emit, cudaStream_t s)
{
    if (a.nwork <= 0) return;
    const int nb = (a.nwork + 63) / 64;
    if (!emit) k_mark_large<<<(a.nwork + 255) / 256, 256, 0, s>>>(a.work, a.nwork, a.nb_cnt);
    if (g) {
        GridVisitor v{*g};
        if (emit)
            k_cells_large_list<true><<<nb, 64, 0, s>>>(a, v);
        else
            k_cells_large_list<false><<<nb, 64, 0, s>>>(a, v);
    } else {
        TriVisitor v{*tm};
        if (emit)
            k_cells_large_list<true><<<nb, 64, 0, s>>>(a, v);
        else
            k_cells_large_list<false><<<nb, 64, 0, s>>>(a, v);
    }
}

size_t large_work_bytes() { return sizeof(Work<kCapLarge>); }
int large_row_cap() { return kCapLarge + 1; }
int small_row_cap() { return kCapSmall + 1; }
int stage1_cap() { return kCapSmall; }

void launch_cells_stage1(const CellArgs& a, cudaStream_t s)
{
    if (a.n <= 0) return;
    k_cells_stage1<<<(a.n + kS1Warps - 1) / kS1Warps, 32 * kS1Warps, 0, s>>>(a);
}

static unsigned pieces_blocks(int n)
{
    const int warps = (n + kWarpCells - 1) / kWarpCells;
    return (unsigned)((warps + kPieceWarps - 1) / kPieceWarps);
}

void launch_pieces_grid(const CellArgs& a, const MeshGridDev& m, int mode, cudaStream_t s)
{
    if (a.n <= 0 || (a.cell_list && a.ncell_list <= 0)) return;
    const int nc = a.cell_list ? a.ncell_list : a.n;
    GridPieces e{m};
    if (mode == kModeVjp)
        k_pieces<kModeVjp><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeVjpMixed)
        k_pieces<kModeVjpMixed><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeCount)
        k_pieces<kModeCount><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeEmit)
        k_pieces<kModeEmit><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeMixed)
        k_pieces<kModeMixed><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeMoments)
        k_pieces<kModeMoments><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else
        k_pieces<kModeEval><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
}

void launch_pieces_tri(const CellArgs& a, const MeshTriDev& m, int mode, cudaStream_t s)
{
    if (a.n <= 0 || (a.cell_list && a.ncell_list <= 0)) return;
    const int nc = a.cell_list ? a.ncell_list : a.n;
    TriPieces e{m};
    if (mode == kModeVjp)
        k_pieces<kModeVjp><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeVjpMixed)
        k_pieces<kModeVjpMixed><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeCount)
        k_pieces<kModeCount><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeEmit)
        k_pieces<kModeEmit><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeMixed)
        k_pieces<kModeMixed><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else if (mode == kModeMoments)
        k_pieces<kModeMoments><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
    else
        k_pieces<kModeEval><<<pieces_blocks(nc), 32 * kPieceWarps, 0, s>>>(a, e);
}

void launch_cells_large_grid(const CellArgs& a, const MeshGridDev& m, bool mom, cudaStream_t s)
{
    if (a.nwork <= 0) return;
    int g = (a.nwork + 63) / 64;
    GridVisitor v{m};
    if (mom)
        k_cells_large<kCapLarge, true><<<g, 64, 0, s>>>(a, v);
    else
        k_cells_large<kCapLarge, false><<<g, 64, 0, s>>>(a, v);
}

void launch_cells_large_tri(const CellArgs& a, const MeshTriDev& m, bool mom, cudaStream_t s)
{
    if (a.nwork <= 0) return;
    int g = (a.nwork + 63) / 64;
    TriVisitor v{m};
    if (mom)
        k_cells_large<kCapLarge, true><<<g, 64, 0, s>>>(a, v);
    else
        k_cells_large<kCapLarge, false><<<g, 64, 0, s>>>(a, v);
}

}  // namespace ma
