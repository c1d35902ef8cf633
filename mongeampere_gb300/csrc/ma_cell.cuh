// ma_cell.cuh -- one Laguerre cell, clipped and integrated by one thread.
//
// Reference behaviour restated (paths in the MongeAmpere++ tree):
//   include/MA/voronoi_triangulation_intersection.hpp:42-199  symbolic polygon
//       edges (EDGE_T between two mesh points, EDGE_DT on the radical axis of two
//       sites), inside(), and the Sutherland-Hodgman clip by one radical axis;
//   include/MA/predicates.hpp:73-135  Side1 (power distance at a mesh point),
//       Side2 (at the weighted circumcentre of three sites), Side3 (at the
//       crossing of a mesh edge with a radical axis), strict SMALLER = inside;
//   include/MA/kantorovich.hpp:95-135  per-piece integrals and Hessian triplets.
//
// Design:
//   * A polygon is a cyclic list of edge labels.  Vertex k is the start of edge
//     k, i.e. the crossing of edges k-1 and k.  Labels >= 0 name a slot (a site
//     whose radical axis bounds the polygon); labels < 0 name fixed edge -1-e,
//     the segment from fixed point e to fixed point e+1 (box corners in the cell
//     stage, triangle corners in the triangle stage).
//   * Every vertex also carries an FP32 position relative to the owner site and a
//     rigorous per-component error bound.  "Is vertex k strictly closer to the
//     owner than to site c?" is first answered in FP32 with that bound; only
//     when the bound straddles zero is the question re-asked symbolically from
//     the input doubles (Side1/2/3), with an FP64 running-error filter and, when
//     that cannot decide either, exact expansion arithmetic.  The combinatorial
//     result (which edges survive) is therefore exact.
//   * Positions used for integrals are recomputed in FP64 from the labels, so the
//     integrals do not inherit the FP32 positions.
#pragma once

#include "ma_exact.cuh"

namespace ma {

// status bits (per launch, OR-ed into a device word)
enum : uint32_t {
    ST_POLY_OVERFLOW = 1u,   // polygon / slot capacity exceeded: site redone with a larger capacity
    ST_EXACT_OVERFLOW = 2u,  // an exact predicate ran out of expansion capacity
    ST_ROW_OVERFLOW = 4u,    // a Hessian row did not fit its staging slots
    ST_BAD_INPUT = 8u,       // non-finite input
    ST_NEED_EXACT = 16u,     // a predicate needed exact arithmetic (cell redone by the exact pass)
};

struct SiteD {
    double x, y, w, pad;
};

// element e of a small fixed-size array by a chain of selects: a runtime index into a
// local array would place the whole array in local memory
template <class T, int N>
MA_HD T pick(const T (&a)[N], int e)
{
    T v = a[0];
#pragma unroll
    for (int k = 1; k < N; k++) v = e == k ? a[k] : v;
    return v;
}

// A site whose radical axis (with the owner) bounds, or may bound, the polygon.
// d = x_site - x_owner, z = |d|^2 - (w_site - w_owner); the radical axis is
// {u : 2 u.d = z} in owner-relative coordinates u, and u is strictly closer to
// the owner iff 2 u.d - z < 0.
struct Slot {
    int site;          // sorted index
    float dx, dy, z;   // FP32 values
    float ed, ez;      // per-component error bound of (dx, dy); error bound of z
    float d1;          // |dx| + |dy|
};

struct Owner {
    double x, y, w;
    int self;          // sorted index
};

// fixed points of the fixed edges: box corners, triangle corners, or the corners of
// a clipping polygon (FC of them at most)
template <int FC>
struct FixedN {
    static constexpr int kCap = FC;
    int n;
    float ux[FC], uy[FC], ur[FC];  // owner-relative FP32 and per-component error
    double rx[FC], ry[FC];         // owner-relative FP64
    double ax[FC], ay[FC];         // absolute (exact input doubles)
};
using Fixed = FixedN<4>;

template <int CAP>
struct Poly {
    int n;
    int lab[CAP];
    float ux[CAP], uy[CAP], ur[CAP];
};

// fixed-size bit set (one word for the small capacities)
template <int CAP>
struct Bits {
    static constexpr int W = (CAP + 63) / 64;
    uint64_t w[W];
    MA_HD void clear()
    {
        for (int i = 0; i < W; i++) w[i] = 0;
    }
    MA_HD void set(int i) { w[i >> 6] |= 1ull << (i & 63); }
    MA_HD bool get(int i) const { return (w[i >> 6] >> (i & 63)) & 1ull; }
};

MA_HD Slot make_slot(int site, const SiteD& c, const Owner& o)
{
    double dx = dsub(c.x, o.x), dy = dsub(c.y, o.y), dw = dsub(c.w, o.w);
    float fx = (float)dx, fy = (float)dy, fw = (float)dw;
    float ed = kU32 * fmaxf(fabsf(fx), fabsf(fy)) + 1e-37f;
    F X{fx, ed}, Y{fy, ed}, W{fw, kU32 * fabsf(fw) + 1e-37f};
    F Z = f_sub(f_add(f_mul(X, X), f_mul(Y, Y)), W);
    Slot s;
    s.site = site;
    s.dx = fx;
    s.dy = fy;
    s.z = Z.v;
    s.ed = ed;
    s.ez = Z.e;
    s.d1 = fabsf(fx) + fabsf(fy);
    return s;
}

template <class FX>
MA_HD void set_fixed(FX& f, int k, double ax, double ay, const Owner& o)
{
    f.ax[k] = ax;
    f.ay[k] = ay;
    f.rx[k] = dsub(ax, o.x);
    f.ry[k] = dsub(ay, o.y);
    f.ux[k] = (float)f.rx[k];
    f.uy[k] = (float)f.ry[k];
    f.ur[k] = kU32 * fmaxf(fabsf(f.ux[k]), fabsf(f.uy[k])) + 1e-37f;
}

// FP32 certified side test of vertex (ux, uy) +- ur against slot c:
// +1: certainly not inside (2u.d - z > 0), -1: certainly inside, 0: undecided.
MA_HD int test32(float ux, float uy, float ur, const Slot& c)
{
    float val = 2.0f * fmaf(ux, c.dx, uy * c.dy) - c.z;
    float u1 = fabsf(ux) + fabsf(uy);
    float b = 2.0f * ur * c.d1 + 2.0f * (u1 + 2.0f * ur) * c.ed + c.ez +
              4.8e-7f * (2.0f * u1 * c.d1 + fabsf(c.z));
    b = b * 1.0001f + 1e-36f;
    if (val > b) return 1;
    if (val < -b) return -1;
    return 0;
}

// ---------------------------------------------------------------------------
// symbolic predicates on the input doubles (FP64 filter, then exact)
// ---------------------------------------------------------------------------

// pow(E, v) - pow(E, w) with pow(E, p) = |E - p|^2 - p.w  (Side1's quantity)
MA_HD R r_pi(double vx, double vy, double vw, double wx, double wy, double ww, double ex, double ey)
{
    R ax = r_sub(rv(ex), rv(vx)), ay = r_sub(rv(ey), rv(vy));
    R bx = r_sub(rv(ex), rv(wx)), by = r_sub(rv(ey), rv(wy));
    R s = r_sub(r_add(r_mul(ax, ax), r_mul(ay, ay)), r_add(r_mul(bx, bx), r_mul(by, by)));
    return r_add(s, r_sub(rv(ww), rv(vw)));
}

constexpr int kExS = 24;  // capacity of a power-difference expansion
constexpr int kExL = 48;  // capacity of a product expansion

template <int C>
MA_HD void ex_pi(Exp<C>& h, double vx, double vy, double vw, double wx, double wy, double ww, double ex,
                 double ey, bool& ok)
{
    double t[20];
    two_prod(2.0 * ex, wx, t[1], t[0]);
    two_prod(-2.0 * ex, vx, t[3], t[2]);
    two_prod(2.0 * ey, wy, t[5], t[4]);
    two_prod(-2.0 * ey, vy, t[7], t[6]);
    two_prod(vx, vx, t[9], t[8]);
    two_prod(vy, vy, t[11], t[10]);
    two_prod(-wx, wx, t[13], t[12]);
    two_prod(-wy, wy, t[15], t[14]);
    t[16] = -vw;
    t[17] = ww;
    ex_set(h, 0.0);
    for (int k = 0; k < 18 && ok; k++) ex_grow(h, t[k], ok);
    ex_compress(h);
}

template <int CH, int CA, int CB>
MA_HD void ex_mul2(Exp<CH>& h, const Exp<CA>& a, const Exp<CB>& b, bool& ok)
{
    ex_set(h, 0.0);
    for (int j = 0; j < b.n && ok; j++) {
        for (int i = 0; i < a.n && ok; i++) {
            double p, e;
            two_prod(a.c[i], b.c[j], p, e);
            ex_grow(h, e, ok);
            if (ok) ex_grow(h, p, ok);
        }
        ex_compress(h);
    }
}

template <int CH, int CF>
MA_HD void ex_acc(Exp<CH>& h, const Exp<CF>& f, double sgn, bool& ok)
{
    for (int j = 0; j < f.n && ok; j++) ex_grow(h, sgn * f.c[j], ok);
    ex_compress(h);
}

// Side1: is fixed point E strictly closer (power distance) to the owner than to c?
// The filter returns the sign of pi(E, owner, c) when certain, 0 otherwise.
MA_HD int filt_side1(const Owner& o, const SiteD& c, double ex, double ey)
{
    return r_sign(r_pi(o.x, o.y, o.w, c.x, c.y, c.w, ex, ey));
}

MA_HDNI int exact_side1(const Owner& o, const SiteD& c, double ex, double ey, uint32_t& st)
{
    bool ok = true;
    Exp<kExS> h;
    ex_pi(h, o.x, o.y, o.w, c.x, c.y, c.w, ex, ey, ok);
    if (!ok) st |= ST_EXACT_OVERFLOW;
    return ex_sign(h);
}

// Side3: E = segment line (p, q) crossing the radical axis of (owner, u).
// With A = pi(., owner, u), B = pi(., owner, c):
//   pi(E, owner, c) = (A(p) B(q) - A(q) B(p)) / (A(p) - A(q)).
// FP64 filter: +1 / -1 for a certain sign of pi(E, owner, c), 0 when undecided
MA_HD int filt_side3(const Owner& o, const SiteD& u, double px, double py, double qx, double qy, const SiteD& c)
{
    R Ap = r_pi(o.x, o.y, o.w, u.x, u.y, u.w, px, py), Aq = r_pi(o.x, o.y, o.w, u.x, u.y, u.w, qx, qy);
    R Bp = r_pi(o.x, o.y, o.w, c.x, c.y, c.w, px, py), Bq = r_pi(o.x, o.y, o.w, c.x, c.y, c.w, qx, qy);
    int sd = r_sign(r_sub(r_mul(Ap, Bq), r_mul(Aq, Bp)));
    int sn = r_sign(r_sub(Ap, Aq));
    return sd * sn;
}

MA_HDNI int exact_side3(const Owner& o, const SiteD& u, double px, double py, double qx, double qy, const SiteD& c,
                        uint32_t& st)
{
    bool ok = true;
    Exp<kExS> eAp, eAq, eBp, eBq;
    ex_pi(eAp, o.x, o.y, o.w, u.x, u.y, u.w, px, py, ok);
    ex_pi(eAq, o.x, o.y, o.w, u.x, u.y, u.w, qx, qy, ok);
    ex_pi(eBp, o.x, o.y, o.w, c.x, c.y, c.w, px, py, ok);
    ex_pi(eBq, o.x, o.y, o.w, c.x, c.y, c.w, qx, qy, ok);
    Exp<kExL> t1, t2;
    ex_mul2(t1, eAp, eBq, ok);
    ex_mul2(t2, eAq, eBp, ok);
    ex_acc(t1, t2, -1.0, ok);
    int sd = ex_sign(t1);
    Exp<kExL> dn;
    ex_set(dn, 0.0);
    ex_acc(dn, eAp, 1.0, ok);
    ex_acc(dn, eAq, -1.0, ok);
    int sn = ex_sign(dn);
    if (!ok) st |= ST_EXACT_OVERFLOW;
    return sd * sn;  // sn == 0: the radical axis is parallel to the segment, no vertex
}

// Side2: E = weighted circumcentre of (owner, a, b).  Relative to the owner, with
// d_k = x_k - x_o and z_k = |d_k|^2 - (w_k - w_o):
//   pi(E, owner, c) = M / D,  D = d_a x d_b,
//   M = d_c.x (z_a d_b.y - z_b d_a.y) + d_c.y (d_a.x z_b - d_b.x z_a) - z_c D.
MA_HD int filt_side2(const Owner& o, const SiteD& a, const SiteD& b, const SiteD& c)
{
    R dax = r_sub(rv(a.x), rv(o.x)), day = r_sub(rv(a.y), rv(o.y));
    R dbx = r_sub(rv(b.x), rv(o.x)), dby = r_sub(rv(b.y), rv(o.y));
    R dcx = r_sub(rv(c.x), rv(o.x)), dcy = r_sub(rv(c.y), rv(o.y));
    R za = r_sub(r_add(r_mul(dax, dax), r_mul(day, day)), r_sub(rv(a.w), rv(o.w)));
    R zb = r_sub(r_add(r_mul(dbx, dbx), r_mul(dby, dby)), r_sub(rv(b.w), rv(o.w)));
    R zc = r_sub(r_add(r_mul(dcx, dcx), r_mul(dcy, dcy)), r_sub(rv(c.w), rv(o.w)));
    R D = r_sub(r_mul(dax, dby), r_mul(day, dbx));
    R M = r_mul(dcx, r_sub(r_mul(za, dby), r_mul(zb, day)));
    M = r_add(M, r_mul(dcy, r_sub(r_mul(dax, zb), r_mul(dbx, za))));
    M = r_sub(M, r_mul(zc, D));
    return r_sign(M) * r_sign(D);
}

MA_HDNI int exact_side2(const Owner& o, const SiteD& a, const SiteD& b, const SiteD& c, uint32_t& st)
{
    int sm, sd;
    bool ok = true;
    Exp<4> ax, ay, bx, by, cx, cy;
    ex_diff(ax, a.x, o.x);
    ex_diff(ay, a.y, o.y);
    ex_diff(bx, b.x, o.x);
    ex_diff(by, b.y, o.y);
    ex_diff(cx, c.x, o.x);
    ex_diff(cy, c.y, o.y);
    Exp<kExS> Z[3];
    const Exp<4>* px[3] = {&ax, &bx, &cx};
    const Exp<4>* py[3] = {&ay, &by, &cy};
    const SiteD* ps[3] = {&a, &b, &c};
    for (int k = 0; k < 3; k++) {
        Exp<kExS> sq;
        ex_mul2(Z[k], *px[k], *px[k], ok);
        ex_mul2(sq, *py[k], *py[k], ok);
        ex_acc(Z[k], sq, 1.0, ok);
        Exp<4> dw;
        ex_diff(dw, ps[k]->w, o.w);
        ex_acc(Z[k], dw, -1.0, ok);
    }
    Exp<kExS> Dx, t;
    ex_mul2(Dx, ax, by, ok);
    ex_mul2(t, ay, bx, ok);
    ex_acc(Dx, t, -1.0, ok);
    sd = ex_sign(Dx);
    Exp<kExL> Mx, u1, u2, v;
    // za*dby - zb*day
    ex_mul2(u1, Z[0], by, ok);
    ex_mul2(u2, Z[1], ay, ok);
    ex_acc(u1, u2, -1.0, ok);
    ex_mul2(Mx, u1, cx, ok);
    // dax*zb - dbx*za
    ex_mul2(u1, ax, Z[1], ok);
    ex_mul2(u2, bx, Z[0], ok);
    ex_acc(u1, u2, -1.0, ok);
    ex_mul2(v, u1, cy, ok);
    ex_acc(Mx, v, 1.0, ok);
    ex_mul2(v, Z[2], Dx, ok);
    ex_acc(Mx, v, -1.0, ok);
    sm = ex_sign(Mx);
    if (!ok) st |= ST_EXACT_OVERFLOW;
    return sm * sd;  // sd == 0: collinear sites, no weighted circumcentre
}

// Is the vertex between edges `prev` and `cur` strictly closer to the owner than
// to slot c's site?  (Tri_intersector::inside, vti.hpp:129-166.)  Without EXACT an
// undecided filter sets `undecided` (the caller redoes the cell with EXACT).
template <int CAP, bool EXACT, class FX>
MA_HDNI bool sym_inside(int prev, int cur, const Slot* slots, const FX& fx, const Owner& o, const SiteD* sites,
                        int csite, uint32_t& st, bool& undecided)
{
    const SiteD c = sites[csite];
    int s;
    if (prev < 0 && cur < 0) {
        int e = -1 - cur;
        s = filt_side1(o, c, fx.ax[e], fx.ay[e]);
        if (s == 0 && EXACT) s = exact_side1(o, c, fx.ax[e], fx.ay[e], st);
    } else if (prev >= 0 && cur >= 0) {
        const SiteD a = sites[slots[prev].site];
        const SiteD b = sites[slots[cur].site];
        s = filt_side2(o, a, b, c);
        if (s == 0 && EXACT) s = exact_side2(o, a, b, c, st);
    } else {
        int e = (prev < 0) ? -1 - prev : -1 - cur;
        int u = (prev < 0) ? cur : prev;
        int e1 = (e + 1 == fx.n) ? 0 : e + 1;
        const SiteD us = sites[slots[u].site];
        s = filt_side3(o, us, fx.ax[e], fx.ay[e], fx.ax[e1], fx.ay[e1], c);
        if (s == 0 && EXACT) s = exact_side3(o, us, fx.ax[e], fx.ay[e], fx.ax[e1], fx.ay[e1], c, st);
    }
    if (s == 0 && !EXACT) undecided = true;
    return s < 0;
}

// ---------------------------------------------------------------------------
// FP32 vertex construction with error radius
// ---------------------------------------------------------------------------

MA_HD void sanitize(float& ux, float& uy, float& ur)
{
    if (!(ur < INFINITY) || !(fabsf(ux) < INFINITY) || !(fabsf(uy) < INFINITY)) {
        ux = 0.0f;
        uy = 0.0f;
        ur = INFINITY;
    }
}

// crossing of the segment p -> q (owner-relative FP32 points with error radii) with
// the radical axis of slot a
MA_HD void vtx_seg_bis(float pxv, float pyv, float pr, float qxv, float qyv, float qr, const Slot& a, float& ux,
                       float& uy, float& ur)
{
    F px{pxv, pr}, py{pyv, pr};
    F qx{qxv, qr}, qy{qyv, qr};
    F dx{a.dx, a.ed}, dy{a.dy, a.ed}, z{a.z, a.ez};
    F Ap = f_sub(f_scale2(f_add(f_mul(px, dx), f_mul(py, dy))), z);
    F ex = f_sub(qx, px), ey = f_sub(qy, py);
    F den = f_scale2(f_add(f_mul(ex, dx), f_mul(ey, dy)));  // A(q) - A(p)
    F t = f_div(Ap, den);
    t.v = -t.v;
    F X = f_add(px, f_mul(t, ex)), Y = f_add(py, f_mul(t, ey));
    ux = X.v;
    uy = Y.v;
    ur = fmaxf(X.e, Y.e);
    sanitize(ux, uy, ur);
}

// crossing of fixed edge e (fixed point e -> e+1) with the radical axis of slot a
template <class FX>
MA_HD void vtx_fixed_bis(const FX& fx, int e, const Slot& a, float& ux, float& uy, float& ur)
{
    int e1 = (e + 1 == fx.n) ? 0 : e + 1;
    vtx_seg_bis(pick(fx.ux, e), pick(fx.uy, e), pick(fx.ur, e), pick(fx.ux, e1), pick(fx.uy, e1), pick(fx.ur, e1), a,
                ux, uy, ur);
}

// crossing of the radical axes of slots a and b (weighted circumcentre)
MA_HD void vtx_bis_bis(const Slot& a, const Slot& b, float& ux, float& uy, float& ur)
{
    F ax{a.dx, a.ed}, ay{a.dy, a.ed}, az{a.z, a.ez};
    F bx{b.dx, b.ed}, by{b.dy, b.ed}, bz{b.z, b.ez};
    F D = f_scale2(f_sub(f_mul(ax, by), f_mul(ay, bx)));
    F Nx = f_sub(f_mul(az, by), f_mul(bz, ay));
    F Ny = f_sub(f_mul(ax, bz), f_mul(bx, az));
    F X = f_div(Nx, D), Y = f_div(Ny, D);
    ux = X.v;
    uy = Y.v;
    ur = fmaxf(X.e, Y.e);
    sanitize(ux, uy, ur);
}

template <int CAP, class FX>
MA_HD void new_vertex(int edge, int cslot, const Slot* slots, const FX& fx, float& ux, float& uy, float& ur)
{
    if (edge < 0)
        vtx_fixed_bis(fx, -1 - edge, slots[cslot], ux, uy, ur);
    else
        vtx_bis_bis(slots[edge], slots[cslot], ux, uy, ur);
}

// Sutherland-Hodgman clip of P by the half-plane of slot `cs` (vti.hpp:168-198).
// Returns false (and leaves Q untouched) when no vertex lies outside.  Sets
// `overflow` when the result would exceed CAP, or (without EXACT) when a vertex
// needs exact arithmetic.
template <int CAP, bool EXACT, class FX>
MA_HD bool clip_poly(const Poly<CAP>& P, Poly<CAP>& Q, int cs, const Slot* slots, const FX& fx,
                     const Owner& o, const SiteD* sites, uint32_t& st, bool& overflow)
{
    const int n = P.n;
    const Slot c = slots[cs];
    Bits<CAP> outm;
    outm.clear();
    int nout = 0;
    for (int k = 0; k < n; k++) {
        int t = test32(P.ux[k], P.uy[k], P.ur[k], c);
        bool out;
        if (t != 0) {
            out = t > 0;
        } else {
            int prev = P.lab[k == 0 ? n - 1 : k - 1];
            bool undecided = false;
            out = !sym_inside<CAP, EXACT>(prev, P.lab[k], slots, fx, o, sites, c.site, st, undecided);
            if (undecided) {
                // an exact decision is needed: the cell is redone by the exact pass
                st |= ST_NEED_EXACT;
                overflow = true;
                return true;
            }
        }
        if (out) {
            outm.set(k);
            nout++;
        }
    }
    if (nout == 0) return false;
    if (nout == n) {
        Q.n = 0;
        return true;
    }
    int m = 0;
    for (int i = 0; i < n; i++) {
        int i1 = (i + 1 == n) ? 0 : i + 1;
        bool in0 = !outm.get(i), in1 = !outm.get(i1);
        if (in0) {
            if (m >= CAP) { overflow = true; return true; }
            Q.lab[m] = P.lab[i];
            Q.ux[m] = P.ux[i];
            Q.uy[m] = P.uy[i];
            Q.ur[m] = P.ur[i];
            m++;
            if (!in1) {
                if (m >= CAP) { overflow = true; return true; }
                Q.lab[m] = cs;
                new_vertex<CAP>(P.lab[i], cs, slots, fx, Q.ux[m], Q.uy[m], Q.ur[m]);
                m++;
            }
        } else if (in1) {
            if (m >= CAP) { overflow = true; return true; }
            Q.lab[m] = P.lab[i];
            new_vertex<CAP>(P.lab[i], cs, slots, fx, Q.ux[m], Q.uy[m], Q.ur[m]);
            m++;
        }
    }
    Q.n = m;
    return true;
}

// ---------------------------------------------------------------------------
// FP64 piece integration
// ---------------------------------------------------------------------------

// FP64 owner-relative data of a neighbour slot
struct Nb64 {
    double dx, dy, z;
};

MA_HD Nb64 make_nb64(const SiteD& c, const Owner& o)
{
    Nb64 r;
    r.dx = dsub(c.x, o.x);
    r.dy = dsub(c.y, o.y);
    double dw = dsub(c.w, o.w);
    r.z = dfma(r.dx, r.dx, dfma(r.dy, r.dy, -dw));
    return r;
}

// FP64 vertex between edges prev and cur (owner-relative)
template <class FX>
MA_HD void vtx64(int prev, int cur, const Nb64* nb, const FX& fx, double& X, double& Y)
{
    if (prev < 0 && cur < 0) {
        int e = -1 - cur;
        X = pick(fx.rx, e);
        Y = pick(fx.ry, e);
        return;
    }
    if (prev >= 0 && cur >= 0) {
        const Nb64 a = nb[prev], b = nb[cur];
        double D = 2.0 * (a.dx * b.dy - a.dy * b.dx);
        double inv = 1.0 / D;
        X = (a.z * b.dy - b.z * a.dy) * inv;
        Y = (a.dx * b.z - b.dx * a.z) * inv;
        return;
    }
    int e = (prev < 0) ? -1 - prev : -1 - cur;
    const Nb64 a = nb[(prev < 0) ? cur : prev];
    int e1 = (e + 1 == fx.n) ? 0 : e + 1;
    double px = pick(fx.rx, e), py = pick(fx.ry, e);
    double ex = pick(fx.rx, e1) - px, ey = pick(fx.ry, e1) - py;
    double Ap = 2.0 * (px * a.dx + py * a.dy) - a.z;
    double den = 2.0 * (ex * a.dx + ey * a.dy);
    double t = -Ap / den;
    X = px + t * ex;
    Y = py + t * ey;
}

// per-site FP64 accumulators (u = x - x_site)
struct Acc {
    double mass, second;
    double m1x, m1y;         // int rho u
    double sxx, syy, sxy;    // int rho u u^T
};

// Integrate the linear density rho(u) = c0 + gx u.x + gy u.y over the polygon
// (owner-relative coordinates) with the fan from the owner: for an edge a -> b
// and cr = a x b, the triangle (0, a, b) contributes
//   int 1          = cr/2
//   int u          = cr (a + b) / 6
//   int u u^T      = cr/12 (a a^T + b b^T) + cr/24 (a b^T + b a^T)
//   int u |u|^2    = cr/60 [a (3|a|^2 + 2 a.b + |b|^2) + b (|a|^2 + 2 a.b + 3|b|^2)]
//   int u_x^3      = cr/20 (a_x^3 + a_x^2 b_x + a_x b_x^2 + b_x^3)
//   int u_x^2 u_y  = cr/60 (3 a_x^2 a_y + a_x^2 b_y + 2 a_x b_x a_y + 2 a_x b_x b_y + b_x^2 a_y + 3 b_x^2 b_y)
// (monomial integrals over a simplex).  These are exact for the integrands of
// kantorovich.hpp:125-131 and lloyd.hpp:57-62, as are the reference's
// centroid and Albrecht-Collatz rules.  Each DT edge adds |e x d| rho(mid) to
// hv[slot]; the Hessian entry is then -hv / (2 |d|^2) (kantorovich.hpp:110-121:
// length * rho(mid) / (2 |x_i - x_j|), with length = |e x d| / |d|).
// The polygon is given by its edge labels lab(0..n-1); edge(k, slot, v) receives the
// Hessian part v of edge k when that edge lies on the radical axis of `slot`.
// value = false leaves out int rho |u|^2 (acc.second stays 0): a Newton solve's
// evaluations need the value only at its end.
template <bool MOM, class Lab, class Edge>
MA_HD void integrate_labels(int n, const Lab& lab_of, const Nb64* nb, const Fixed& fx, double c0, double gx,
                            double gy, Acc& acc, const Edge& edge, bool value = true)
{
    double x0, y0;
    vtx64(lab_of(n - 1), lab_of(0), nb, fx, x0, y0);
    double ax = x0, ay = y0;
    double m0 = 0, m1x = 0, m1y = 0, q2 = 0, c3x = 0, c3y = 0, sxx = 0, syy = 0, sxy = 0;
    double t30 = 0, t21 = 0, t12 = 0, t03 = 0;
    for (int k = 0; k < n; k++) {
        double bx, by;
        const int lab = lab_of(k);
        if (k + 1 < n)
            vtx64(lab, lab_of(k + 1), nb, fx, bx, by);
        else {
            bx = x0;
            by = y0;
        }
        double cr = ax * by - ay * bx;
        m0 += cr;
        m1x += cr * (ax + bx);
        m1y += cr * (ay + by);
        if (value) {
            double aa = ax * ax + ay * ay, ab = ax * bx + ay * by, bb = bx * bx + by * by;
            q2 += cr * (aa + ab + bb);
            double ka = 3.0 * aa + 2.0 * ab + bb, kb = aa + 2.0 * ab + 3.0 * bb;
            c3x += cr * (ax * ka + bx * kb);
            c3y += cr * (ay * ka + by * kb);
        }
        if (MOM) {
            sxx += cr * (2.0 * (ax * ax + bx * bx) + 2.0 * ax * bx);
            syy += cr * (2.0 * (ay * ay + by * by) + 2.0 * ay * by);
            sxy += cr * (2.0 * (ax * ay + bx * by) + ax * by + bx * ay);
            // third moments over the triangle (0, a, b): int u_x^3, u_x^2 u_y, u_x u_y^2, u_y^3
            t30 += cr * 3.0 * (ax * ax * ax + ax * ax * bx + ax * bx * bx + bx * bx * bx);
            t21 += cr * (3.0 * ax * ax * ay + ax * ax * by + 2.0 * ax * bx * ay + 2.0 * ax * bx * by + bx * bx * ay +
                         3.0 * bx * bx * by);
            t12 += cr * (3.0 * ay * ay * ax + ay * ay * bx + 2.0 * ay * by * ax + 2.0 * ay * by * bx + by * by * ax +
                         3.0 * by * by * bx);
            t03 += cr * 3.0 * (ay * ay * ay + ay * ay * by + ay * by * by + by * by * by);
        }
        if (lab >= 0) {
            const Nb64 d = nb[lab];
            double exv = bx - ax, eyv = by - ay;
            double crs = fabs(exv * d.dy - eyv * d.dx);
            double mx = 0.5 * (ax + bx), my = 0.5 * (ay + by);
            edge(k, lab, crs * (c0 + gx * mx + gy * my));
        }
        ax = bx;
        ay = by;
    }
    // int rho = c0 int 1 + g . int u ; int rho |u|^2 = c0 int |u|^2 + g . int u |u|^2
    double I1 = m0 * 0.5;
    double Iux = m1x * (1.0 / 6.0), Iuy = m1y * (1.0 / 6.0);
    double Iq = q2 * (1.0 / 12.0);
    double Icx = c3x * (1.0 / 60.0), Icy = c3y * (1.0 / 60.0);
    acc.mass += c0 * I1 + gx * Iux + gy * Iuy;
    acc.second += c0 * Iq + gx * Icx + gy * Icy;
    if (MOM) {
        double Sxx = sxx * (1.0 / 24.0), Syy = syy * (1.0 / 24.0), Sxy = sxy * (1.0 / 24.0);
        double T30 = t30 * (1.0 / 60.0), T21 = t21 * (1.0 / 60.0), T12 = t12 * (1.0 / 60.0), T03 = t03 * (1.0 / 60.0);
        acc.m1x += c0 * Iux + gx * Sxx + gy * Sxy;
        acc.m1y += c0 * Iuy + gx * Sxy + gy * Syy;
        acc.sxx += c0 * Sxx + gx * T30 + gy * T21;
        acc.syy += c0 * Syy + gx * T12 + gy * T03;
        acc.sxy += c0 * Sxy + gx * T21 + gy * T12;
    }
}

// ---------------------------------------------------------------------------
// the mixed-precision integrals (FP32)
// ---------------------------------------------------------------------------
// FP32 sum with a running compensation (Neumaier's variant of Kahan summation): the
// rounding error of every addition is carried in c, so the sum's error does not grow
// with the number of terms
struct CompF {
    float s, c;
    MA_HD void add(float x)
    {
        const float t = s + x;
        c += fabsf(s) >= fabsf(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    MA_HD float val() const { return s + c; }
};

// The mixed-precision integrals of one piece.  Every position is taken about an anchor
// a near the cell (the centre of its bounding box, site-relative FP64): a cell can lie
// many cell sizes away from its site, and FP32 positions relative to the site would
// carry errors of 1e-7 of that distance.  The FP64 work is the triangle's corners minus
// the anchor, per piece, and each radical axis's offset about the anchor, once per cell
// and neighbour (zc): the axis {u : 2 u.d = z} becomes {v : 2 v.d = z - 2 a.d}.  The vertices come from the
// certified FP32 constructions (vtx_fixed_bis, vtx_bis_bis: a value and an error radius
// R); the mass's fan sums are compensated, the moments' plain FP32.  The certified radii
// give two bounds:
//   err_mass: the piece's mass moves by at most 1/2 sum over its edges of
//   (R_a + R_b) |e|_1 times the largest density on it; the caller sums these per cell and
//   redoes in FP64 a cell whose total exceeds kMassTol32 (2.4e-4) of its mass;
//   a radical-axis edge is integrated in FP64 (vtx64, site-relative) when 2 (R_a + R_b)
//   exceeds kEdgeTol32 of its length |e|_1: crs = |e x d| = |e| |d| with
//   |e| >= |e|_1 / sqrt 2, so a kept edge is within kEdgeTol32 plus a few FP32 roundings,
//   and every Hessian entry, a sum of edges of one sign, within ~2.5e-4 of the FP64 one.
constexpr float kMassTol32 = 0x1p-12f;
constexpr float kEdgeTol32 = 0x1p-12f;

// a triangle's corners about the anchor (FP32 values and error radii)
struct FixedA {
    int n;
    float ux[3], uy[3], ur[3];
};

// the vertex between edges prev and cur about the anchor, with its error radius
MA_HD void vtx_anchor(int prev, int cur, const Slot* slots, const float* zc, const FixedA& fa, float& X, float& Y,
                      float& R)
{
    auto slot_at = [&](int lab) -> Slot {
        Slot t = slots[lab];
        t.z = zc[lab];
        t.ez = kU32 * fabsf(t.z) + 1e-37f;
        return t;
    };
    if (prev < 0 && cur < 0) {
        const int e = -1 - cur;
        X = pick(fa.ux, e);
        Y = pick(fa.uy, e);
        R = pick(fa.ur, e);
    } else if (prev >= 0 && cur >= 0) {
        vtx_bis_bis(slot_at(prev), slot_at(cur), X, Y, R);
    } else {
        const int e = prev < 0 ? -1 - prev : -1 - cur;
        vtx_fixed_bis(fa, e, slot_at(prev < 0 ? cur : prev), X, Y, R);
    }
}

// the Hessian part of the radical-axis edge from vertex (p0, lab) to (lab, p1) in FP64
MA_HDNI double edge64(int p0, int lab, int p1, const Nb64* nb, const Fixed& fx, double c0, double gx, double gy)
{
    double px, py, qx, qy;
    vtx64(p0, lab, nb, fx, px, py);
    vtx64(lab, p1, nb, fx, qx, qy);
    const Nb64 d = nb[lab];
    const double crs = fabs((qx - px) * d.dy - (qy - py) * d.dx);
    return crs * (c0 + gx * 0.5 * (px + qx) + gy * 0.5 * (py + qy));
}

template <class Lab, class Edge>
MA_HD void integrate_piece32(int n, const Lab& lab_of, const Slot* slots, const Nb64* nb, const float* zc,
                             double ax, double ay,
                             const Fixed& fx, double c0, double gx, double gy, double& mass, double& second,
                             double& err_mass, const Edge& edge, int& nedge, int& fb_edge)
{
    // the triangle's corners about the anchor
    FixedA fa;
    fa.n = fx.n;
#pragma unroll
    for (int e = 0; e < 3; e++) {  // triangles
        fa.ux[e] = (float)(fx.rx[e] - ax);
        fa.uy[e] = (float)(fx.ry[e] - ay);
        fa.ur[e] = kU32 * fmaxf(fabsf(fa.ux[e]), fabsf(fa.uy[e])) + 1e-37f;
    }
    // rho about the anchor: rho(v) = ca + g . v
    const float caf = (float)(c0 + gx * ax + gy * ay), gxf = (float)gx, gyf = (float)gy;
    float x0 = 0.0f, y0 = 0.0f, r0 = 0.0f;
    float vx = 0.0f, vy = 0.0f, vr = 0.0f;
    // the mass's sums compensated; the value part's moments as plain FP32 sums (at most 12
    // terms, each with its own product rounding, which the error bound below counts)
    CompF m0{0, 0}, m1x{0, 0}, m1y{0, 0};
    float q2 = 0.0f, c3x = 0.0f, c3y = 0.0f, sxx = 0.0f, syy = 0.0f, sxy = 0.0f;
    float errA = 0.0f, vmax = 0.0f, acr = 0.0f;
    // vertex k + 1 in iteration k; iteration -1 makes vertex 0 (one copy of the constructions)
    for (int k = -1; k < n; k++) {
        const int lab = k < 0 ? lab_of(n - 1) : lab_of(k);
        float bx, by, br;
        if (k + 1 < n)
            vtx_anchor(lab, lab_of(k + 1), slots, zc, fa, bx, by, br);
        else {
            bx = x0;
            by = y0;
            br = r0;
        }
        if (k < 0) {
            x0 = vx = bx;
            y0 = vy = by;
            r0 = vr = br;
            vmax = fabsf(bx) + fabsf(by) + br;
            continue;
        }
        const float ex = bx - vx, ey = by - vy, e1 = fabsf(ex) + fabsf(ey);
        errA += (vr + br) * e1;
        vmax = fmaxf(vmax, fabsf(bx) + fabsf(by) + br);
        const float cr = vx * by - vy * bx;
        acr += fabsf(vx * by) + fabsf(vy * bx);
        const float aa = vx * vx + vy * vy, ab = vx * bx + vy * by, bb = bx * bx + by * by;
        m0.add(cr);
        m1x.add(cr * (vx + bx));
        m1y.add(cr * (vy + by));
        q2 += cr * (aa + ab + bb);
        const float ka = 3.0f * aa + 2.0f * ab + bb, kb = aa + 2.0f * ab + 3.0f * bb;
        c3x += cr * (vx * ka + bx * kb);
        c3y += cr * (vy * ka + by * kb);
        sxx += cr * (2.0f * (vx * vx + bx * bx) + 2.0f * vx * bx);
        syy += cr * (2.0f * (vy * vy + by * by) + 2.0f * vy * by);
        sxy += cr * (2.0f * (vx * vy + bx * by) + vx * by + bx * vy);
        if (lab >= 0) {
            nedge++;
            if (2.0f * (vr + br) <= kEdgeTol32 * e1) {
                const Slot d = slots[lab];
                const float crs = fabsf(ex * d.dy - ey * d.dx);
                edge(k, lab, (double)(crs * (caf + gxf * 0.5f * (vx + bx) + gyf * 0.5f * (vy + by))));
            } else {
                fb_edge++;
                edge(k, lab, edge64(lab_of(k == 0 ? n - 1 : k - 1), lab, lab_of(k + 1 < n ? k + 1 : 0), nb, fx, c0, gx, gy));
            }
        }
        vx = bx;
        vy = by;
        vr = br;
    }
    const float A2 = m0.val();  // twice the area
    // the vertices' radii, and the FP32 roundings of the products and the sum (a few ulps
    // of the terms' magnitudes, which can exceed the piece's area: slivers)
    err_mass = 0.5 * ((double)errA + 4.0 * (double)kU32 * (double)acr) *
               ((double)fabsf(caf) + ((double)fabsf(gxf) + (double)fabsf(gyf)) * (double)vmax);
    // int rho, int rho v, int rho |v|^2 about the anchor (fan from it, see integrate_labels)
    const float I1 = A2 * 0.5f, Ivx = m1x.val() * (1.0f / 6.0f), Ivy = m1y.val() * (1.0f / 6.0f);
    const float Sxx = sxx * (1.0f / 24.0f), Syy = syy * (1.0f / 24.0f), Sxy = sxy * (1.0f / 24.0f);
    const float rm = caf * I1 + gxf * Ivx + gyf * Ivy;
    const float rvx = caf * Ivx + gxf * Sxx + gyf * Sxy, rvy = caf * Ivy + gxf * Sxy + gyf * Syy;
    const float rq = caf * (q2 * (1.0f / 12.0f)) + gxf * (c3x * (1.0f / 60.0f)) + gyf * (c3y * (1.0f / 60.0f));
    // int rho |u|^2 with u = v + a: int rho |v|^2 + 2 a . int rho v + |a|^2 int rho
    mass = (double)rm;
    second = (double)rq + 2.0 * (ax * (double)rvx + ay * (double)rvy) + (ax * ax + ay * ay) * (double)rm;
}

// ---------------------------------------------------------------------------
// adjoint of one piece
// ---------------------------------------------------------------------------
// Moments of the piece in owner-relative coordinates u = x - x_i (fan from the
// owner, as above): I1 = int 1, Iu = int u, S = int u u^T (xx, yy, xy),
// Iq = int |u|^2, Ic = int u |u|^2.
struct PieceMoments {
    double I1, Iux, Iuy, Sxx, Syy, Sxy, Iq, Icx, Icy;
};

// The cotangent-weighted boundary terms of the piece's radical-axis edges.  An edge
// on the radical axis of neighbour j moves when x_i, x_j, w_i or w_j move; with
// d = x_j - x_i and the line integrals over the edge
//     E0 = int rho / |d|,  Eu = int rho u / |d|,  Euu = int rho u u^T / |d|
// (rho and u are linear along the edge, so Simpson's rule is exact for all three),
// the terms that land on site i are
//     g_w += (b_i - b_j) E0 / 2 + (e_i - e_j) . (x_i E0 + Eu) / 2
//     g_x += (b_i - b_j) Eu + ((e_i - e_j) . x_i) Eu + Euu (e_i - e_j)
// for the cotangents b of the masses and e of the first moments int rho x.  (The
// reference has no adjoint; these are the shape derivatives of its cells, whose
// w-part is the Hessian of kantorovich.hpp:110-121.)  cot(slot) returns the
// neighbour's (b_j, e_jx, e_jy).
template <class Lab, class Cot>
MA_HD void integrate_vjp(int n, const Lab& lab_of, const Nb64* nb, const Fixed& fx, double c0, double gx, double gy,
                         double xi, double yi, double bi, double exi, double eyi, const Cot& cot, PieceMoments& M,
                         double& gw, double& gpx, double& gpy)
{
    double x0, y0;
    vtx64(lab_of(n - 1), lab_of(0), nb, fx, x0, y0);
    double ax = x0, ay = y0;
    double m0 = 0, m1x = 0, m1y = 0, q2 = 0, c3x = 0, c3y = 0, sxx = 0, syy = 0, sxy = 0;
    for (int k = 0; k < n; k++) {
        const int lab = lab_of(k);
        double bx, by;
        if (k + 1 < n)
            vtx64(lab, lab_of(k + 1), nb, fx, bx, by);
        else {
            bx = x0;
            by = y0;
        }
        const double cr = ax * by - ay * bx;
        const double aa = ax * ax + ay * ay, ab = ax * bx + ay * by, bb = bx * bx + by * by;
        m0 += cr;
        m1x += cr * (ax + bx);
        m1y += cr * (ay + by);
        q2 += cr * (aa + ab + bb);
        const double ka = 3.0 * aa + 2.0 * ab + bb, kb = aa + 2.0 * ab + 3.0 * bb;
        c3x += cr * (ax * ka + bx * kb);
        c3y += cr * (ay * ka + by * kb);
        sxx += cr * (2.0 * (ax * ax + bx * bx) + 2.0 * ax * bx);
        syy += cr * (2.0 * (ay * ay + by * by) + 2.0 * ay * by);
        sxy += cr * (2.0 * (ax * ay + bx * by) + ax * by + bx * ay);
        if (lab >= 0) {
            const Nb64 d = nb[lab];
            const double ex = bx - ax, ey = by - ay;
            // |edge| / |d| = |edge x d| / |d|^2 (the edge is perpendicular to d)
            const double ratio = fabs(ex * d.dy - ey * d.dx) / (d.dx * d.dx + d.dy * d.dy);
            const double mx = 0.5 * (ax + bx), my = 0.5 * (ay + by);
            const double ra = c0 + gx * ax + gy * ay, rb = c0 + gx * bx + gy * by, rm = c0 + gx * mx + gy * my;
            const double E0 = ratio * rm;
            const double w6 = ratio * (1.0 / 6.0);
            const double Eux = w6 * (ra * ax + 4.0 * rm * mx + rb * bx);
            const double Euy = w6 * (ra * ay + 4.0 * rm * my + rb * by);
            const double Exx = w6 * (ra * ax * ax + 4.0 * rm * mx * mx + rb * bx * bx);
            const double Eyy = w6 * (ra * ay * ay + 4.0 * rm * my * my + rb * by * by);
            const double Exy = w6 * (ra * ax * ay + 4.0 * rm * mx * my + rb * bx * by);
            double bj, ejx, ejy;
            cot(lab, bj, ejx, ejy);
            const double db = bi - bj, dex = exi - ejx, dey = eyi - ejy;
            gw += 0.5 * db * E0 + 0.5 * (dex * (xi * E0 + Eux) + dey * (yi * E0 + Euy));
            const double dx = dex * xi + dey * yi;
            gpx += (db + dx) * Eux + Exx * dex + Exy * dey;
            gpy += (db + dx) * Euy + Exy * dex + Eyy * dey;
        }
        ax = bx;
        ay = by;
    }
    M.I1 = m0 * 0.5;
    M.Iux = m1x * (1.0 / 6.0);
    M.Iuy = m1y * (1.0 / 6.0);
    M.Sxx = sxx * (1.0 / 24.0);
    M.Syy = syy * (1.0 / 24.0);
    M.Sxy = sxy * (1.0 / 24.0);
    M.Iq = q2 * (1.0 / 12.0);
    M.Icx = c3x * (1.0 / 60.0);
    M.Icy = c3y * (1.0 / 60.0);
}

// integrate_vjp in FP32 about the cell's anchor a (the mixed-precision adjoint): the
// vertices of integrate_piece32 (their radii unused), the piece's moments and each
// radical-axis edge's line integrals E0, Ev, Evv in compensated FP32 about a, then moved
// to the site-relative moments integrate_vjp gives, u = v + a, in FP64:
//   int u = Iv + a I1,  int u u^T = Svv + a Iv^T + Iv a^T + a a^T I1,
//   int |u|^2 = Iqv + 2 a.Iv + |a|^2 I1,
//   int u |u|^2 = Icv + 2 Svv a + |a|^2 Iv + a Iqv + 2 a (a.Iv) + a |a|^2 I1,
// and likewise for the edge integrals; the gradients accumulate as in integrate_vjp.
template <class Lab, class Cot>
MA_HD void integrate_vjp32(int n, const Lab& lab_of, const Slot* slots, const float* zc, double ax, double ay,
                           const Fixed& fx, double c0, double gx, double gy, double xi, double yi, double bi,
                           double exi, double eyi, const Cot& cot, PieceMoments& M, double& gw, double& gpx,
                           double& gpy)
{
    FixedA fa;
    fa.n = fx.n;
#pragma unroll
    for (int e = 0; e < 3; e++) {  // triangles
        fa.ux[e] = (float)(fx.rx[e] - ax);
        fa.uy[e] = (float)(fx.ry[e] - ay);
        fa.ur[e] = kU32 * fmaxf(fabsf(fa.ux[e]), fabsf(fa.uy[e])) + 1e-37f;
    }
    const float caf = (float)(c0 + gx * ax + gy * ay), gxf = (float)gx, gyf = (float)gy;
    float x0 = 0.0f, y0 = 0.0f, vx = 0.0f, vy = 0.0f;
    CompF m0{0, 0}, m1x{0, 0}, m1y{0, 0}, q2{0, 0}, c3x{0, 0}, c3y{0, 0}, sxx{0, 0}, syy{0, 0}, sxy{0, 0};
    for (int k = -1; k < n; k++) {
        const int lab = k < 0 ? lab_of(n - 1) : lab_of(k);
        float bx, by, br;
        if (k + 1 < n)
            vtx_anchor(lab, lab_of(k + 1), slots, zc, fa, bx, by, br);
        else {
            bx = x0;
            by = y0;
        }
        if (k < 0) {
            x0 = vx = bx;
            y0 = vy = by;
            continue;
        }
        const float cr = vx * by - vy * bx;
        const float aa = vx * vx + vy * vy, ab = vx * bx + vy * by, bb = bx * bx + by * by;
        m0.add(cr);
        m1x.add(cr * (vx + bx));
        m1y.add(cr * (vy + by));
        q2.add(cr * (aa + ab + bb));
        const float ka = 3.0f * aa + 2.0f * ab + bb, kb = aa + 2.0f * ab + 3.0f * bb;
        c3x.add(cr * (vx * ka + bx * kb));
        c3y.add(cr * (vy * ka + by * kb));
        sxx.add(cr * (2.0f * (vx * vx + bx * bx) + 2.0f * vx * bx));
        syy.add(cr * (2.0f * (vy * vy + by * by) + 2.0f * vy * by));
        sxy.add(cr * (2.0f * (vx * vy + bx * by) + vx * by + bx * vy));
        if (lab >= 0) {
            const Slot d = slots[lab];
            const float ex = bx - vx, ey = by - vy;
            const float ratio = fabsf(ex * d.dy - ey * d.dx) / (d.dx * d.dx + d.dy * d.dy);
            const float mx = 0.5f * (vx + bx), my = 0.5f * (vy + by);
            const float ra = caf + gxf * vx + gyf * vy, rb = caf + gxf * bx + gyf * by, rm = caf + gxf * mx + gyf * my;
            const float w6 = ratio * (1.0f / 6.0f);
            const double E0 = (double)(ratio * rm);
            const double Evx = (double)(w6 * (ra * vx + 4.0f * rm * mx + rb * bx));
            const double Evy = (double)(w6 * (ra * vy + 4.0f * rm * my + rb * by));
            const double Evxx = (double)(w6 * (ra * vx * vx + 4.0f * rm * mx * mx + rb * bx * bx));
            const double Evyy = (double)(w6 * (ra * vy * vy + 4.0f * rm * my * my + rb * by * by));
            const double Evxy = (double)(w6 * (ra * vx * vy + 4.0f * rm * mx * my + rb * bx * by));
            const double Eux = Evx + ax * E0, Euy = Evy + ay * E0;
            const double Exx = Evxx + 2.0 * ax * Evx + ax * ax * E0;
            const double Eyy = Evyy + 2.0 * ay * Evy + ay * ay * E0;
            const double Exy = Evxy + ax * Evy + ay * Evx + ax * ay * E0;
            double bj, ejx, ejy;
            cot(lab, bj, ejx, ejy);
            const double db = bi - bj, dex = exi - ejx, dey = eyi - ejy;
            gw += 0.5 * db * E0 + 0.5 * (dex * (xi * E0 + Eux) + dey * (yi * E0 + Euy));
            const double dxi = dex * xi + dey * yi;
            gpx += (db + dxi) * Eux + Exx * dex + Exy * dey;
            gpy += (db + dxi) * Euy + Exy * dex + Eyy * dey;
        }
        vx = bx;
        vy = by;
    }
    const double I1 = 0.5 * (double)m0.val();
    const double Ivx = (double)m1x.val() * (1.0 / 6.0), Ivy = (double)m1y.val() * (1.0 / 6.0);
    const double Sxx = (double)sxx.val() * (1.0 / 24.0), Syy = (double)syy.val() * (1.0 / 24.0),
                 Sxy = (double)sxy.val() * (1.0 / 24.0);
    const double Iqv = (double)q2.val() * (1.0 / 12.0);
    const double Icvx = (double)c3x.val() * (1.0 / 60.0), Icvy = (double)c3y.val() * (1.0 / 60.0);
    const double aIv = ax * Ivx + ay * Ivy, a2 = ax * ax + ay * ay;
    M.I1 = I1;
    M.Iux = Ivx + ax * I1;
    M.Iuy = Ivy + ay * I1;
    M.Sxx = Sxx + 2.0 * ax * Ivx + ax * ax * I1;
    M.Syy = Syy + 2.0 * ay * Ivy + ay * ay * I1;
    M.Sxy = Sxy + ax * Ivy + ay * Ivx + ax * ay * I1;
    M.Iq = Iqv + 2.0 * aIv + a2 * I1;
    M.Icx = Icvx + 2.0 * (ax * Sxx + ay * Sxy) + a2 * Ivx + ax * Iqv + 2.0 * ax * aIv + ax * a2 * I1;
    M.Icy = Icvy + 2.0 * (ax * Sxy + ay * Syy) + a2 * Ivy + ay * Iqv + 2.0 * ay * aIv + ay * a2 * I1;
}

template <int CAP, bool MOM>
MA_HD void integrate_piece(const Poly<CAP>& P, const Nb64* nb, const Fixed& fx, double c0, double gx,
                           double gy, Acc& acc, double* hv, Bits<CAP>& touched)
{
    integrate_labels<MOM>(
        P.n, [&](int k) { return P.lab[k]; }, nb, fx, c0, gx, gy, acc,
        [&](int, int lab, double v) {
            hv[lab] += v;
            touched.set(lab);
        });
}

}  // namespace ma
