/*
 * ma_oracle.c -- CPU FP64 restatement of the MongeAmpere++ hot path:
 * Laguerre (power) cells intersected with a triangulated piecewise-linear
 * density, giving the Kantorovich value, the cell masses (gradient), the sparse
 * Hessian triplets and the first / second moments.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle.  It is loaded by the
 * test-suite, by the smoke check and by the CPU-baseline leg of the benchmark,
 * never by the product library.
 *
 * Reference files followed (paths inside the MongeAmpere++ tree):
 *   include/MA/kantorovich.hpp:59-139          value, gradient, Hessian triplets
 *   include/MA/voronoi_triangulation_intersection.hpp:42-199   Tri_intersector
 *       (symbolic EDGE_T / EDGE_DT edges, inside(), Sutherland-Hodgman clip)
 *   include/MA/voronoi_triangulation_intersection.hpp:219-313  flood fill over
 *       (site, triangle) pairs
 *   include/MA/voronoi_triangulation_intersection.hpp:315-343  materialised pieces
 *   include/MA/predicates.hpp:21-135           Construct_dual, Side1, Side2, Side3
 *   include/MA/quadrature.hpp:24-42,69-85,122-143   Albrecht-Collatz, centroid,
 *       segment midpoint, polygon fans
 *   include/MA/functions.hpp:25-80             barycentric / extrapolate /
 *       Linear_function
 *   include/MA/lloyd.hpp:30-123                first and second moments
 *
 * The reference takes its regular triangulation and its filtered-exact predicates
 * from CGAL 4.11 (not part of the reference tree).  They are restated here:
 *   - the regular-triangulation neighbours of a site are recomputed by exact
 *     half-plane clipping of a box that contains the mesh (a neighbour whose edge
 *     lies outside the mesh never changes a piece, so the pieces are the same);
 *   - Side1 / Side2 / Side3 are evaluated as signs of polynomials in the input
 *     doubles, first with a certified running-error filter and, when the filter
 *     cannot decide, exactly with floating-point expansions (Shewchuk 1997,
 *     "Adaptive precision floating-point arithmetic and fast robust geometric
 *     predicates").  Ties count as "not inside", the reference's strict SMALLER.
 *
 * Parity unpinned against reference outputs: the reference cannot be compiled
 * here (CGAL, Eigen and GMP are absent) and its tests hold no golden vectors.  The
 * oracle is pinned instead to exact-rational fixtures (tests/golden) and to the
 * invariants the reference's drivers print (total area, mass conservation,
 * finite-difference consistency).
 *
 * Build: gcc -O2 -fPIC -shared -ffp-contract=off -fopenmp (oracle/build.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* exact expansion arithmetic                                                */
/* ------------------------------------------------------------------------- */

#define EXMAX 2048

static void two_sum(double a, double b, double *x, double *y)
{
    double s = a + b;
    double bv = s - a;
    double av = s - bv;
    *x = s;
    *y = (a - av) + (b - bv);
}

static void two_prod(double a, double b, double *x, double *y)
{
    double p = a * b;
    *x = p;
    *y = fma(a, b, -p);
}

/* h = e + b (e nonoverlapping, increasing magnitude); zero components dropped.
 * h may alias e. */
static int ex_grow(int elen, const double *e, double b, double *h)
{
    double q = b, qn, hh;
    int hi = 0;
    for (int i = 0; i < elen; i++) {
        two_sum(q, e[i], &qn, &hh);
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}

/* e += f, in place on e (capacity EXMAX) */
static int ex_add(int elen, double *e, int flen, const double *f)
{
    for (int j = 0; j < flen; j++) elen = ex_grow(elen, e, f[j], e);
    return elen;
}

/* h = e * b, zero components dropped */
static int ex_scale(int elen, const double *e, double b, double *h)
{
    double q, hh, p1, p0, s;
    int hi = 0;
    two_prod(e[0], b, &q, &hh);
    if (hh != 0.0) h[hi++] = hh;
    for (int i = 1; i < elen; i++) {
        two_prod(e[i], b, &p1, &p0);
        two_sum(q, p0, &s, &hh);
        if (hh != 0.0) h[hi++] = hh;
        two_sum(p1, s, &q, &hh);
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}

/* h = e * f */
static int ex_mul(int elen, const double *e, int flen, const double *f, double *h)
{
    double t[EXMAX];
    int hl = 1;
    h[0] = 0.0;
    for (int j = 0; j < flen; j++) {
        int tl = ex_scale(elen, e, f[j], t);
        hl = ex_add(hl, h, tl, t);
    }
    return hl;
}

static int ex_neg(int elen, const double *e, double *h)
{
    for (int i = 0; i < elen; i++) h[i] = -e[i];
    return elen;
}

static int ex_sign(int elen, const double *e)
{
    double top = e[elen - 1];
    return (top > 0.0) - (top < 0.0);
}

/* ------------------------------------------------------------------------- */
/* certified running-error arithmetic (value, absolute error bound)          */
/* ------------------------------------------------------------------------- */

typedef struct { double v, e; } rd;
#define RD_U 0x1p-52 /* twice the unit roundoff */

static rd rd_c(double x) { rd r = {x, 0.0}; return r; }
static rd rd_add(rd a, rd b) { rd r; r.v = a.v + b.v; r.e = a.e + b.e + RD_U * fabs(r.v); return r; }
static rd rd_sub(rd a, rd b) { rd r; r.v = a.v - b.v; r.e = a.e + b.e + RD_U * fabs(r.v); return r; }
static rd rd_mul(rd a, rd b)
{
    rd r;
    r.v = a.v * b.v;
    r.e = fabs(a.v) * b.e + fabs(b.v) * a.e + a.e * b.e + RD_U * fabs(r.v);
    return r;
}
/* +1 / -1 when the sign is certain, 0 when the filter cannot decide */
static int rd_sign(rd a)
{
    double eb = a.e * (1.0 + 0x1p-30);
    if (a.v > eb) return 1;
    if (-a.v > eb) return -1;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* double-double arithmetic (about 106 significant bits)                     */
/* ------------------------------------------------------------------------- */
/* The reference builds polygon vertices and integrals in FP64 from absolute
 * coordinates (CGAL EPICK constructions).  Their rounding is large enough that a
 * mere translation of the input moves short-edge Hessian entries by ~1e-10, so the
 * oracle can also run those constructions and integrals in double-double
 * (Dekker 1971; Hida, Li, Bailey 2001), with the same formulas and the same
 * quadrature rules.  Combinatorics (predicates) are exact either way. */

typedef struct { double hi, lo; } dd;

static dd dd_c(double a) { dd r = {a, 0.0}; return r; }
static dd dd_norm(double s, double e)
{
    dd r;
    r.hi = s + e;
    r.lo = e - (r.hi - s);
    return r;
}
static dd dd_add(dd a, dd b)
{
    double s, e, t, f;
    two_sum(a.hi, b.hi, &s, &e);
    two_sum(a.lo, b.lo, &t, &f);
    e += t;
    dd r = dd_norm(s, e);
    e = r.lo + f;
    return dd_norm(r.hi, e);
}
static dd dd_neg(dd a) { dd r = {-a.hi, -a.lo}; return r; }
static dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
static dd dd_mul(dd a, dd b)
{
    double p, e;
    two_prod(a.hi, b.hi, &p, &e);
    e += a.hi * b.lo + a.lo * b.hi;
    return dd_norm(p, e);
}
static dd dd_muld(dd a, double b) { return dd_mul(a, dd_c(b)); }
static dd dd_div(dd a, dd b)
{
    double q1 = a.hi / b.hi;
    dd r = dd_sub(a, dd_muld(b, q1));
    double q2 = r.hi / b.hi;
    r = dd_sub(r, dd_muld(b, q2));
    double q3 = r.hi / b.hi;
    dd q = dd_norm(q1, q2);
    return dd_add(q, dd_c(q3));
}
static dd dd_sqrt(dd a)
{
    if (a.hi <= 0.0) return dd_c(0.0);
    double x = sqrt(a.hi);
    dd xx = dd_mul(dd_c(x), dd_c(x));
    dd corr = dd_div(dd_sub(a, xx), dd_c(2.0 * x));
    return dd_add(dd_c(x), corr);
}
static double dd_d(dd a) { return a.hi + a.lo; }

/* ------------------------------------------------------------------------- */
/* weighted points and the three predicates of predicates.hpp                */
/* ------------------------------------------------------------------------- */

typedef struct { double x, y, w; } site_t;

typedef struct {
    long filter_calls;
    long exact_calls;
} pred_stats;

/* exact pow(E,v) - pow(E,w) with pow(E,p) = |E-p|^2 - p.w, E a double point */
static int ex_pi(const site_t *v, const site_t *w, double ex, double ey, double *h)
{
    double t[20];
    int n = 0;
    double hi, lo;
    two_prod(2.0 * ex, w->x, &hi, &lo); t[n++] = lo; t[n++] = hi;
    two_prod(-2.0 * ex, v->x, &hi, &lo); t[n++] = lo; t[n++] = hi;
    two_prod(2.0 * ey, w->y, &hi, &lo); t[n++] = lo; t[n++] = hi;
    two_prod(-2.0 * ey, v->y, &hi, &lo); t[n++] = lo; t[n++] = hi;
    two_prod(v->x, v->x, &hi, &lo); t[n++] = lo; t[n++] = hi;
    two_prod(v->y, v->y, &hi, &lo); t[n++] = lo; t[n++] = hi;
    two_prod(-w->x, w->x, &hi, &lo); t[n++] = lo; t[n++] = hi;
    two_prod(-w->y, w->y, &hi, &lo); t[n++] = lo; t[n++] = hi;
    t[n++] = -v->w;
    t[n++] = w->w;
    int hl = 1;
    h[0] = 0.0;
    for (int k = 0; k < n; k++) hl = ex_grow(hl, h, t[k], h);
    return hl;
}

static rd rd_pi(const site_t *v, const site_t *w, double ex, double ey)
{
    rd ax = rd_sub(rd_c(ex), rd_c(v->x)), ay = rd_sub(rd_c(ey), rd_c(v->y));
    rd bx = rd_sub(rd_c(ex), rd_c(w->x)), by = rd_sub(rd_c(ey), rd_c(w->y));
    rd s = rd_add(rd_mul(ax, ax), rd_mul(ay, ay));
    s = rd_sub(s, rd_add(rd_mul(bx, bx), rd_mul(by, by)));
    return rd_add(s, rd_sub(rd_c(w->w), rd_c(v->w)));
}

/* Side1 (predicates.hpp:73-99): compare_power_distance(E, v, w) == SMALLER */
static int side1(const site_t *v, const site_t *w, double ex, double ey, pred_stats *st)
{
    st->filter_calls++;
    int s = rd_sign(rd_pi(v, w, ex, ey));
    if (s == 0) {
        double h[32];
        st->exact_calls++;
        int hl = ex_pi(v, w, ex, ey, h);
        s = ex_sign(hl, h);
    }
    return s < 0;
}

/* sign of pow(E,v) - pow(E,w): -1 closer to v, 0 tie, +1 closer to w */
static int pi_sign(const site_t *v, const site_t *w, double ex, double ey)
{
    int s = rd_sign(rd_pi(v, w, ex, ey));
    if (s == 0) {
        double h[32];
        int hl = ex_pi(v, w, ex, ey, h);
        s = ex_sign(hl, h);
    }
    return s;
}

/* Side3 (predicates.hpp:117-135): E = line(p,q) ∩ radical_axis(v,u);
 * with A = pow(.,v)-pow(.,u), B = pow(.,v)-pow(.,w):
 *   B(E) = (A(p)B(q) - A(q)B(p)) / (A(p) - A(q)). */
static int side3(const site_t *v, const site_t *u, double px, double py, double qx, double qy,
                 const site_t *w, pred_stats *st)
{
    st->filter_calls++;
    rd Ap = rd_pi(v, u, px, py), Aq = rd_pi(v, u, qx, qy);
    rd Bp = rd_pi(v, w, px, py), Bq = rd_pi(v, w, qx, qy);
    int sd = rd_sign(rd_sub(rd_mul(Ap, Bq), rd_mul(Aq, Bp)));
    int sn = rd_sign(rd_sub(Ap, Aq));
    if (sd == 0 || sn == 0) {
        static __thread double eAp[32], eAq[32], eBp[32], eBq[32], t1[EXMAX], t2[EXMAX];
        st->exact_calls++;
        int lAp = ex_pi(v, u, px, py, eAp), lAq = ex_pi(v, u, qx, qy, eAq);
        int lBp = ex_pi(v, w, px, py, eBp), lBq = ex_pi(v, w, qx, qy, eBq);
        int l1 = ex_mul(lAp, eAp, lBq, eBq, t1);
        int l2 = ex_mul(lAq, eAq, lBp, eBp, t2);
        l2 = ex_neg(l2, t2, t2);
        l1 = ex_add(l1, t1, l2, t2);
        sd = ex_sign(l1, t1);
        double nq[32];
        int lq = ex_neg(lAq, eAq, nq);
        double den[64];
        memcpy(den, eAp, sizeof(double) * lAp);
        int ld = ex_add(lAp, den, lq, nq);
        sn = ex_sign(ld, den);
    }
    if (sn == 0) return 0; /* radical axis parallel to the segment: no vertex */
    return sd * sn < 0;
}

/* exact two-term difference a - b */
static int ex_diff(double a, double b, double *h)
{
    double x, y;
    two_sum(a, -b, &x, &y);
    h[0] = y;
    h[1] = x;
    if (y == 0.0) { h[0] = x; return 1; }
    return 2;
}

/* Side2 (predicates.hpp:101-115): E = weighted circumcenter of (v, a, b).
 * In coordinates relative to v, with d_k = x_k - x_v and z_k = |d_k|^2 - (w_k - w_v),
 * pow(E,v) - pow(E,w) = M / D where
 *   D = d_a x d_b,
 *   M = d_w.x (z_a d_b.y - z_b d_a.y) + d_w.y (d_a.x z_b - d_b.x z_a) - z_w D. */
static int side2(const site_t *v, const site_t *a, const site_t *b, const site_t *w,
                 pred_stats *st)
{
    st->filter_calls++;
    rd dax = rd_sub(rd_c(a->x), rd_c(v->x)), day = rd_sub(rd_c(a->y), rd_c(v->y));
    rd dbx = rd_sub(rd_c(b->x), rd_c(v->x)), dby = rd_sub(rd_c(b->y), rd_c(v->y));
    rd dwx = rd_sub(rd_c(w->x), rd_c(v->x)), dwy = rd_sub(rd_c(w->y), rd_c(v->y));
    rd za = rd_sub(rd_add(rd_mul(dax, dax), rd_mul(day, day)), rd_sub(rd_c(a->w), rd_c(v->w)));
    rd zb = rd_sub(rd_add(rd_mul(dbx, dbx), rd_mul(dby, dby)), rd_sub(rd_c(b->w), rd_c(v->w)));
    rd zw = rd_sub(rd_add(rd_mul(dwx, dwx), rd_mul(dwy, dwy)), rd_sub(rd_c(w->w), rd_c(v->w)));
    rd D = rd_sub(rd_mul(dax, dby), rd_mul(day, dbx));
    rd M = rd_mul(dwx, rd_sub(rd_mul(za, dby), rd_mul(zb, day)));
    M = rd_add(M, rd_mul(dwy, rd_sub(rd_mul(dax, zb), rd_mul(dbx, za))));
    M = rd_sub(M, rd_mul(zw, D));
    int sm = rd_sign(M), sd = rd_sign(D);
    if (sm == 0 || sd == 0) {
        static __thread double A[8][4], Z[3][64], T1[EXMAX], T2[EXMAX], T3[EXMAX], Mx[EXMAX];
        static __thread double Dx[256];
        int la[6];
        st->exact_calls++;
        la[0] = ex_diff(a->x, v->x, A[0]);
        la[1] = ex_diff(a->y, v->y, A[1]);
        la[2] = ex_diff(b->x, v->x, A[2]);
        la[3] = ex_diff(b->y, v->y, A[3]);
        la[4] = ex_diff(w->x, v->x, A[4]);
        la[5] = ex_diff(w->y, v->y, A[5]);
        const site_t *ps[3] = {a, b, w};
        int lz[3];
        for (int k = 0; k < 3; k++) {
            double sq[32], dw[4];
            int l = ex_mul(la[2 * k], A[2 * k], la[2 * k], A[2 * k], Z[k]);
            int l2 = ex_mul(la[2 * k + 1], A[2 * k + 1], la[2 * k + 1], A[2 * k + 1], sq);
            l = ex_add(l, Z[k], l2, sq);
            int l3 = ex_diff(ps[k]->w, v->w, dw);
            l3 = ex_neg(l3, dw, dw);
            lz[k] = ex_add(l, Z[k], l3, dw);
        }
        /* D = dax*dby - day*dbx */
        int l1 = ex_mul(la[0], A[0], la[3], A[3], T1);
        int l2 = ex_mul(la[1], A[1], la[2], A[2], T2);
        l2 = ex_neg(l2, T2, T2);
        int lD = ex_add(l1, T1, l2, T2);
        memcpy(Dx, T1, sizeof(double) * lD);
        sd = ex_sign(lD, Dx);
        /* t = za*dby - zb*day */
        l1 = ex_mul(lz[0], Z[0], la[3], A[3], T1);
        l2 = ex_mul(lz[1], Z[1], la[1], A[1], T2);
        l2 = ex_neg(l2, T2, T2);
        l1 = ex_add(l1, T1, l2, T2);
        int lM = ex_mul(l1, T1, la[4], A[4], Mx);
        /* t = dax*zb - dbx*za */
        l1 = ex_mul(la[0], A[0], lz[1], Z[1], T1);
        l2 = ex_mul(la[2], A[2], lz[0], Z[0], T2);
        l2 = ex_neg(l2, T2, T2);
        l1 = ex_add(l1, T1, l2, T2);
        int l3 = ex_mul(l1, T1, la[5], A[5], T3);
        lM = ex_add(lM, Mx, l3, T3);
        /* - zw * D */
        l3 = ex_mul(lz[2], Z[2], lD, Dx, T3);
        l3 = ex_neg(l3, T3, T3);
        lM = ex_add(lM, Mx, l3, T3);
        sm = ex_sign(lM, Mx);
    }
    if (sd == 0) return 0; /* collinear: no weighted circumcenter */
    return sm * sd < 0;
}

/* ------------------------------------------------------------------------- */
/* symbolic polygons (Tri_intersector, vti.hpp:42-199)                       */
/* ------------------------------------------------------------------------- */

/* t == 0: EDGE_T between points a, b of the point table
 * t == 1: EDGE_DT, bisector between owner site a and site b */
typedef struct { int t, a, b; } pedge;

typedef struct {
    const double *px, *py; /* point table: mesh vertices, then 4 box corners */
    const site_t *s;
    pred_stats st;
} geo_t;

static int common_pt(pedge f, pedge g)
{
    if (f.a == g.a) return f.a;
    if (f.a == g.b) return f.a;
    return f.b;
}

/* inside(): is the vertex between edges a and b strictly closer (power
 * distance) to v than to w (vti.hpp:129-166) */
static int inside(geo_t *G, int v, int w, pedge a, pedge b)
{
    const site_t *S = G->s;
    if (a.t == 0 && b.t == 0) {
        int p = common_pt(a, b);
        return side1(&S[v], &S[w], G->px[p], G->py[p], &G->st);
    }
    if (a.t == 1 && b.t == 1) return side2(&S[v], &S[b.b], &S[a.b], &S[w], &G->st);
    int p, q, u;
    if (a.t == 0) { p = a.a; q = a.b; u = b.b; }
    else { p = b.a; q = b.b; u = a.b; }
    return side3(&S[v], &S[u], G->px[p], G->py[p], G->px[q], G->py[q], &S[w], &G->st);
}

#define PMAX 512

/* Sutherland-Hodgman clip of P by the half-plane of v against w (vti.hpp:168-198) */
static int clip(geo_t *G, const pedge *P, int n, int v, int w, pedge *R)
{
    if (n == 0) return 0;
    pedge L = {1, v, w};
    int m = 0;
    int prev_in = inside(G, v, w, P[n - 1], P[0]);
    for (int i = 0; i < n; i++) {
        int ii = (i + 1) % n;
        int cur_in = inside(G, v, w, P[i], P[ii]);
        if (prev_in) {
            R[m++] = P[i];
            if (!cur_in) R[m++] = L;
        } else if (cur_in) {
            R[m++] = P[i];
        }
        prev_in = cur_in;
        if (m >= PMAX - 1) abort();
    }
    return m;
}

/* homogeneous line a x + b y + c = 0 of an edge (edge_to_line, vti.hpp:98-110) */
static void edge_line(const geo_t *G, pedge e, double *a, double *b, double *c)
{
    if (e.t == 0) {
        double px = G->px[e.a], py = G->py[e.a], qx = G->px[e.b], qy = G->py[e.b];
        *a = py - qy;
        *b = qx - px;
        *c = px * qy - py * qx;
    } else {
        const site_t *v = &G->s[e.a], *w = &G->s[e.b];
        /* radical axis: 2 x.(w - v) + |v|^2 - v.w - |w|^2 + w.w = 0 */
        *a = 2.0 * (w->x - v->x);
        *b = 2.0 * (w->y - v->y);
        *c = (v->x * v->x + v->y * v->y - v->w) - (w->x * w->x + w->y * w->y - w->w);
    }
}

/* vertex_to_point (vti.hpp:112-123; predicates.hpp:21-30) */
static void vertex_to_point(const geo_t *G, pedge e1, pedge e2, double *x, double *y)
{
    double a1, b1, c1, a2, b2, c2;
    edge_line(G, e1, &a1, &b1, &c1);
    edge_line(G, e2, &a2, &b2, &c2);
    double den = a1 * b2 - a2 * b1;
    *x = (b1 * c2 - b2 * c1) / den;
    *y = (a2 * c1 - a1 * c2) / den;
}

/* ------------------------------------------------------------------------- */
/* quadrature (quadrature.hpp) and the linear density (functions.hpp)        */
/* ------------------------------------------------------------------------- */

typedef struct { double a, b, c; } linfn;

/* functions.hpp:25-53 barycentric coordinates / extrapolate */
static double extrapolate(double px, double py, double ax, double ay, double fa, double bx,
                          double by, double fb, double cx, double cy, double fc)
{
    double v0x = bx - ax, v0y = by - ay, v1x = cx - ax, v1y = cy - ay, v2x = px - ax, v2y = py - ay;
    double d00 = v0x * v0x + v0y * v0y, d01 = v0x * v1x + v0y * v1y, d11 = v1x * v1x + v1y * v1y;
    double d20 = v2x * v0x + v2y * v0y, d21 = v2x * v1x + v2y * v1y;
    double den = d00 * d11 - d01 * d01;
    double v = (d11 * d20 - d01 * d21) / den;
    double w = (d00 * d21 - d01 * d20) / den;
    double u = 1.0 - v - w;
    return u * fa + v * fb + w * fc;
}

/* functions.hpp:55-80 Linear_function(p, fp, q, fq, r, fr) */
static linfn make_linfn(double px, double py, double fp, double qx, double qy, double fq, double rx,
                        double ry, double fr)
{
    linfn L;
    L.c = extrapolate(0, 0, px, py, fp, qx, qy, fq, rx, ry, fr);
    L.a = extrapolate(1, 0, px, py, fp, qx, qy, fq, rx, ry, fr) - L.c;
    L.b = extrapolate(0, 1, px, py, fp, qx, qy, fq, rx, ry, fr) - L.c;
    return L;
}

static double lf(const linfn *L, double x, double y) { return L->a * x + L->b * y + L->c; }

/* CGAL::area(a,b,c): signed area */
static double tri_area(double ax, double ay, double bx, double by, double cx, double cy)
{
    return ((bx - ax) * (cy - ay) - (cx - ax) * (by - ay)) / 2.0;
}

/* integrand of kantorovich.hpp:126-131 and lloyd.hpp:57-62, 300-313:
 * out[0] = rho |x - s|^2, out[1..6] = rho, rho x, rho y, rho x^2, rho y^2, rho x y */
#define NQ 7
static void integrand(const linfn *L, double sx, double sy, double x, double y, double *out)
{
    double r = lf(L, x, y);
    double dx = x - sx, dy = y - sy;
    out[0] = r * (dx * dx + dy * dy);
    out[1] = r;
    out[2] = r * x;
    out[3] = r * y;
    out[4] = r * x * x;
    out[5] = r * y * y;
    out[6] = r * x * y;
}

/* quadrature.hpp:24-42 integrate_albrecht_collatz (6 points, degree 3) */
static void albrecht_collatz(const linfn *L, double sx, double sy, double ax, double ay, double bx,
                             double by, double cx, double cy, double *acc)
{
    const double h = 1.0 / 2.0, s6 = 1.0 / 6.0, t3 = 2.0 / 3.0, w1 = 1.0 / 30.0, w9 = 9.0 / 30.0;
    double ux = bx - ax, uy = by - ay, vx = cx - ax, vy = cy - ay;
    double q[6][2] = {
        {ax + h * ux + h * vx, ay + h * uy + h * vy},
        {ax + h * ux, ay + h * uy},
        {ax + h * vx, ay + h * vy},
        {ax + s6 * ux + t3 * vx, ay + s6 * uy + t3 * vy},
        {ax + s6 * vx + t3 * ux, ay + s6 * vy + t3 * uy},
        {ax + s6 * ux + s6 * vx, ay + s6 * uy + s6 * vy},
    };
    const double wt[6] = {w1, w1, w1, w9, w9, w9};
    double sum[NQ] = {0};
    for (int k = 0; k < 6; k++) {
        double f[NQ];
        integrand(L, sx, sy, q[k][0], q[k][1], f);
        for (int j = 0; j < NQ; j++) sum[j] += wt[k] * f[j];
    }
    double A = tri_area(ax, ay, bx, by, cx, cy);
    for (int j = 0; j < NQ; j++) acc[j] += A * sum[j];
}

/* ------------------------------------------------------------------------- */
/* problem state                                                             */
/* ------------------------------------------------------------------------- */

typedef struct {
    int face, site;
    double mass;      /* integrate_1(polygon) with the centroid rule */
    double second;    /* integrate_3(rho |x - s|^2) */
    double mom[6];    /* integrate_3 of rho, rho x, rho y, rho x^2, rho y^2, rho xy */
    double area;
    int nv;           /* polygon size */
    long poly_off;    /* offset into the polygon store (keep_pieces) */
} piece_t;

typedef struct {
    int row, col, face, aux;
    double val;
} trip_t;

typedef struct {
    piece_t *p;
    long n, cap;
    trip_t *t;
    long nt, capt;
    double *pxy;      /* polygon vertex store (keep_pieces) */
    int *plab;        /* edge labels: >=0 site index of an EDGE_DT edge, -1 for EDGE_T */
    long npv, cappv, cappl;
    pred_stats st;
} piece_buf;

static void *grow_buf(void *p, long *cap, long need, size_t elt)
{
    if (need <= *cap) return p;
    long nc = *cap ? *cap : 1024;
    while (nc < need) nc *= 2;
    void *q = realloc(p, nc * elt);
    if (!q) abort();
    *cap = nc;
    return q;
}

typedef struct {
    int nv, nt, n;
    const double *vx, *vy, *vval;
    const int *tri;
    double *ptx, *pty;  /* point table: nv mesh vertices + 4 box corners */
    site_t *s;
    int *fnbr;          /* 3*nt: neighbour face opposite local vertex k, -1 on boundary */
    linfn *fn;
    /* site grid */
    double gx0, gy0, gcw, gch;
    int gnx, gny;
    int *gstart, *gidx;
    double wmax;
    /* box B' (contains the mesh) */
    double bx0, by0, bx1, by1;
    /* regular-triangulation neighbours restricted to B' */
    int *nstart, *nlist;
    int keep_pieces;
    /* candidate neighbour lists (a superset of the regular-triangulation neighbours) */
    const int *cstart, *clist;
    /* cell bounding boxes and a bin grid over them, for point location */
    double *cbox;
    int bnx, bny;
    double bx0b, by0b, bcwb, bchb;
    int *bstart, *blist;
} prob_t;

/* ------------------------------------------------------------------------- */
/* site grid and regular-triangulation neighbours                            */
/* ------------------------------------------------------------------------- */

static void build_grid(prob_t *P)
{
    double x0 = P->bx0, y0 = P->by0, x1 = P->bx1, y1 = P->by1;
    for (int i = 0; i < P->n; i++) {
        if (P->s[i].x < x0) x0 = P->s[i].x;
        if (P->s[i].x > x1) x1 = P->s[i].x;
        if (P->s[i].y < y0) y0 = P->s[i].y;
        if (P->s[i].y > y1) y1 = P->s[i].y;
    }
    double W = x1 - x0, H = y1 - y0;
    int g = (int)ceil(sqrt((double)P->n));
    if (g < 1) g = 1;
    P->gnx = g;
    P->gny = g;
    P->gx0 = x0;
    P->gy0 = y0;
    P->gcw = W / g;
    P->gch = H / g;
    if (P->gcw <= 0) P->gcw = 1;
    if (P->gch <= 0) P->gch = 1;
    int nc = P->gnx * P->gny;
    P->gstart = calloc(nc + 1, sizeof(int));
    P->gidx = malloc(sizeof(int) * (P->n > 0 ? P->n : 1));
    int *cell = malloc(sizeof(int) * (P->n > 0 ? P->n : 1));
    for (int i = 0; i < P->n; i++) {
        int cx = (int)floor((P->s[i].x - P->gx0) / P->gcw);
        int cy = (int)floor((P->s[i].y - P->gy0) / P->gch);
        if (cx < 0) cx = 0;
        if (cx >= P->gnx) cx = P->gnx - 1;
        if (cy < 0) cy = 0;
        if (cy >= P->gny) cy = P->gny - 1;
        cell[i] = cy * P->gnx + cx;
        P->gstart[cell[i] + 1]++;
    }
    for (int c = 0; c < nc; c++) P->gstart[c + 1] += P->gstart[c];
    int *fill = malloc(sizeof(int) * nc);
    memcpy(fill, P->gstart, sizeof(int) * nc);
    for (int i = 0; i < P->n; i++) P->gidx[fill[cell[i]]++] = i;
    free(fill);
    free(cell);
    P->wmax = -INFINITY;
    for (int i = 0; i < P->n; i++)
        if (P->s[i].w > P->wmax) P->wmax = P->s[i].w;
}

/* distance from (x, y) to the complement of the block of grid cells
 * [cx-r, cx+r] x [cy-r, cy+r]; INFINITY when the block covers the grid */
static double block_gap(const prob_t *P, double x, double y, int cx, int cy, int r)
{
    double d = INFINITY;
    int covers = 1;
    if (cx - r > 0) { covers = 0; double e = x - (P->gx0 + (cx - r) * P->gcw); if (e < d) d = e; }
    if (cx + r < P->gnx - 1) { covers = 0; double e = (P->gx0 + (cx + r + 1) * P->gcw) - x; if (e < d) d = e; }
    if (cy - r > 0) { covers = 0; double e = y - (P->gy0 + (cy - r) * P->gch); if (e < d) d = e; }
    if (cy + r < P->gny - 1) { covers = 0; double e = (P->gy0 + (cy + r + 1) * P->gch) - y; if (e < d) d = e; }
    if (covers) return INFINITY;
    if (d < 0) d = 0;
    return d * (1.0 - 1e-12);
}

static void home_cell(const prob_t *P, double x, double y, int *cx, int *cy)
{
    int a = (int)floor((x - P->gx0) / P->gcw), b = (int)floor((y - P->gy0) / P->gch);
    if (a < 0) a = 0;
    if (a >= P->gnx) a = P->gnx - 1;
    if (b < 0) b = 0;
    if (b >= P->gny) b = P->gny - 1;
    *cx = a;
    *cy = b;
}

/* power cell of site i clipped to the box B' (edges between the 4 corner points
 * nv..nv+3); returns the DT labels of the final polygon in *nb */
static int site_neighbors(prob_t *P, int i, int *nb, pred_stats *st)
{
    geo_t G = {P->ptx, P->pty, P->s, {0, 0}};
    pedge A[PMAX], B[PMAX];
    int c0 = P->nv;
    int n = 4;
    for (int k = 0; k < 4; k++) { A[k].t = 0; A[k].a = c0 + k; A[k].b = c0 + (k + 1) % 4; }
    pedge *cur = A, *nxt = B;
    const site_t *si = &P->s[i];
    int cx, cy;
    home_cell(P, si->x, si->y, &cx, &cy);
    for (int r = 0;; r++) {
        int any = 0;
        for (int yy = cy - r; yy <= cy + r; yy++) {
            if (yy < 0 || yy >= P->gny) continue;
            for (int xx = cx - r; xx <= cx + r; xx++) {
                if (xx < 0 || xx >= P->gnx) continue;
                if (yy != cy - r && yy != cy + r && xx != cx - r && xx != cx + r) continue;
                any = 1;
                int c = yy * P->gnx + xx;
                for (int k = P->gstart[c]; k < P->gstart[c + 1] && n > 0; k++) {
                    int j = P->gidx[k];
                    if (j == i) continue;
                    const site_t *sj = &P->s[j];
                    if (sj->x == si->x && sj->y == si->y) {
                        /* duplicate point: the larger weight (then the lower index) survives */
                        if (sj->w > si->w || (sj->w == si->w && j < i)) n = 0;
                        continue;
                    }
                    int m = clip(&G, cur, n, i, j, nxt);
                    pedge *t = cur; cur = nxt; nxt = t;
                    n = m;
                }
            }
        }
        if (n == 0) break;
        double R2 = 0;
        for (int k = 0; k < n; k++) {
            double x, y;
            vertex_to_point(&G, cur[(k + n - 1) % n], cur[k], &x, &y);
            double dx = x - si->x, dy = y - si->y;
            double d2 = dx * dx + dy * dy;
            if (d2 > R2) R2 = d2;
        }
        double R = sqrt(R2) * (1.0 + 1e-7) + 1e-300;
        double d = block_gap(P, si->x, si->y, cx, cy, r);
        if (d == INFINITY || !any) break;
        double slack = 1e-9 * (R2 + fabs(P->wmax) + fabs(si->w));
        if (d > R && d * d - 2.0 * d * R >= (P->wmax - si->w) + slack) break;
    }
    *st = G.st;
    int m = 0;
    for (int k = 0; k < n; k++)
        if (cur[k].t == 1) nb[m++] = cur[k].b;
    return m;
}

/* power cell of site i clipped to the box B' by its candidate list (exact); the
 * polygon's bounding box goes to cbox[4i..4i+3] */
static int site_neighbors_cand(prob_t *P, int i, int *nb, pred_stats *st)
{
    geo_t G = {P->ptx, P->pty, P->s, {0, 0}};
    pedge A[PMAX], B[PMAX];
    int c0 = P->nv;
    int n = 4;
    for (int k = 0; k < 4; k++) { A[k].t = 0; A[k].a = c0 + k; A[k].b = c0 + (k + 1) % 4; }
    pedge *cur = A, *nxt = B;
    const site_t *si = &P->s[i];
    for (int q = P->cstart[i]; q < P->cstart[i + 1] && n > 0; q++) {
        int j = P->clist[q];
        if (j == i) continue;
        const site_t *sj = &P->s[j];
        if (sj->x == si->x && sj->y == si->y) {
            if (sj->w > si->w || (sj->w == si->w && j < i)) n = 0;
            continue;
        }
        int m = clip(&G, cur, n, i, j, nxt);
        pedge *t = cur; cur = nxt; nxt = t;
        n = m;
    }
    double bx0 = INFINITY, by0 = INFINITY, bx1 = -INFINITY, by1 = -INFINITY;
    for (int k = 0; k < n; k++) {
        double x, y;
        vertex_to_point(&G, cur[(k + n - 1) % n], cur[k], &x, &y);
        if (x < bx0) bx0 = x;
        if (x > bx1) bx1 = x;
        if (y < by0) by0 = y;
        if (y > by1) by1 = y;
    }
    double mg = 1e-9 * (P->bx1 - P->bx0 + P->by1 - P->by0);
    P->cbox[4 * i] = bx0 - mg;
    P->cbox[4 * i + 1] = by0 - mg;
    P->cbox[4 * i + 2] = bx1 + mg;
    P->cbox[4 * i + 3] = by1 + mg;
    *st = G.st;
    int m = 0;
    for (int k = 0; k < n; k++)
        if (cur[k].t == 1) nb[m++] = cur[k].b;
    return m;
}

/* bin grid over the cell bounding boxes */
static void build_cell_bins(prob_t *P)
{
    int g = (int)ceil(sqrt((double)P->n));
    if (g < 1) g = 1;
    P->bnx = g;
    P->bny = g;
    P->bx0b = P->bx0;
    P->by0b = P->by0;
    P->bcwb = (P->bx1 - P->bx0) / g;
    P->bchb = (P->by1 - P->by0) / g;
    int nb = g * g;
    P->bstart = calloc(nb + 1, sizeof(int));
    for (int pass = 0; pass < 2; pass++) {
        int *fill = pass ? malloc(sizeof(int) * nb) : NULL;
        if (pass) memcpy(fill, P->bstart, sizeof(int) * nb);
        for (int i = 0; i < P->n; i++) {
            const double *b = &P->cbox[4 * i];
            if (!(b[2] >= b[0])) continue; /* empty cell */
            int x0 = (int)floor((b[0] - P->bx0b) / P->bcwb), x1 = (int)floor((b[2] - P->bx0b) / P->bcwb);
            int y0 = (int)floor((b[1] - P->by0b) / P->bchb), y1 = (int)floor((b[3] - P->by0b) / P->bchb);
            if (x0 < 0) x0 = 0;
            if (y0 < 0) y0 = 0;
            if (x1 >= g) x1 = g - 1;
            if (y1 >= g) y1 = g - 1;
            for (int yy = y0; yy <= y1; yy++)
                for (int xx = x0; xx <= x1; xx++) {
                    if (pass == 0) P->bstart[yy * g + xx + 1]++;
                    else P->blist[fill[yy * g + xx]++] = i;
                }
        }
        if (pass == 0) {
            for (int b = 0; b < nb; b++) P->bstart[b + 1] += P->bstart[b];
            P->blist = malloc(sizeof(int) * (P->bstart[nb] > 0 ? P->bstart[nb] : 1));
        }
        free(fill);
    }
}

/* the sites whose closed power cell contains (x, y), by exact point location */
static int locate(const prob_t *P, double x, double y, int *out, int cap)
{
    int bx = (int)floor((x - P->bx0b) / P->bcwb), by = (int)floor((y - P->by0b) / P->bchb);
    if (bx < 0) bx = 0;
    if (by < 0) by = 0;
    if (bx >= P->bnx) bx = P->bnx - 1;
    if (by >= P->bny) by = P->bny - 1;
    int b = by * P->bnx + bx, m = 0;
    for (int q = P->bstart[b]; q < P->bstart[b + 1]; q++) {
        int i = P->blist[q];
        const double *c = &P->cbox[4 * i];
        if (x < c[0] || x > c[2] || y < c[1] || y > c[3]) continue;
        int inside = 1;
        for (int k = P->nstart[i]; k < P->nstart[i + 1] && inside; k++)
            if (pi_sign(&P->s[i], &P->s[P->nlist[k]], x, y) > 0) inside = 0;
        if (inside && m < cap) out[m++] = i;
    }
    return m;
}

/* sites whose power distance at (x, y) is within tol of the minimum */
static int seeds_at(const prob_t *P, double x, double y, int *out, int cap)
{
    int cx, cy;
    home_cell(P, x, y, &cx, &cy);
    double best = INFINITY;
    int nb = 0;
    for (int pass = 0; pass < 2; pass++) {
        for (int r = 0;; r++) {
            int any = 0;
            for (int yy = cy - r; yy <= cy + r; yy++) {
                if (yy < 0 || yy >= P->gny) continue;
                for (int xx = cx - r; xx <= cx + r; xx++) {
                    if (xx < 0 || xx >= P->gnx) continue;
                    if (yy != cy - r && yy != cy + r && xx != cx - r && xx != cx + r) continue;
                    any = 1;
                    int c = yy * P->gnx + xx;
                    for (int k = P->gstart[c]; k < P->gstart[c + 1]; k++) {
                        int j = P->gidx[k];
                        double dx = x - P->s[j].x, dy = y - P->s[j].y;
                        double pd = dx * dx + dy * dy - P->s[j].w;
                        if (pass == 0) {
                            if (pd < best) best = pd;
                        } else {
                            double tol = 1e-9 * (fabs(best) + dx * dx + dy * dy + fabs(P->s[j].w)) + 1e-300;
                            if (pd <= best + tol && nb < cap) out[nb++] = j;
                        }
                    }
                }
            }
            double d = block_gap(P, x, y, cx, cy, r);
            if (d == INFINITY || !any) break;
            double lim = best + 1e-9 * (fabs(best) + d * d + fabs(P->wmax));
            if (d * d - P->wmax > lim) break;
        }
    }
    return nb;
}

/* ------------------------------------------------------------------------- */
/* the per-piece callback (kantorovich.hpp:87-136, lloyd.hpp:244-267)        */
/* ------------------------------------------------------------------------- */

static void emit_piece(prob_t *P, piece_buf *B, geo_t *G, int f, int v, const pedge *R, int n)
{
    if (n == 0) return; /* empty pieces contribute nothing (integrate_* return 0) */
    double px[PMAX], py[PMAX];
    int adj[PMAX];
    for (int i = 0; i < n; i++) {
        int ii = (i == 0) ? n - 1 : i - 1;
        vertex_to_point(G, R[i], R[ii], &px[i], &py[i]);
        adj[i] = (R[i].t == 1) ? R[i].b : -1;
    }
    const linfn *L = &P->fn[f];
    const site_t *sv = &P->s[v];
    /* Hessian triplets (kantorovich.hpp:110-122) */
    for (int i = 0; i < n; i++) {
        if (adj[i] < 0) continue;
        int w = adj[i];
        int i1 = (i + 1) % n;
        double ex = px[i1] - px[i], ey = py[i1] - py[i];
        double r = sqrt(ex * ex + ey * ey) * lf(L, (px[i] + px[i1]) / 2.0, (py[i] + py[i1]) / 2.0);
        double dx = sv->x - P->s[w].x, dy = sv->y - P->s[w].y;
        double d = 2.0 * sqrt(dx * dx + dy * dy);
        B->t = grow_buf(B->t, &B->capt, B->nt + 2, sizeof(trip_t));
        trip_t t1 = {v, w, f, -1, -r / d};
        trip_t t2 = {v, v, f, w, r / d};
        B->t[B->nt++] = t1;
        B->t[B->nt++] = t2;
    }
    piece_t pc;
    memset(&pc, 0, sizeof(pc));
    pc.face = f;
    pc.site = v;
    pc.nv = n;
    /* warea = integrate_1(p) with the centroid rule (quadrature.hpp:122-131, 69-77) */
    double warea = 0.0, area = 0.0;
    if (n > 2) {
        for (int i = 1; i < n - 1; i++) {
            double A = tri_area(px[0], py[0], px[i], py[i], px[i + 1], py[i + 1]);
            double gx = (px[0] + px[i] + px[i + 1]) / 3.0, gy = (py[0] + py[i] + py[i + 1]) / 3.0;
            warea += A * lf(L, gx, gy);
            area += A;
        }
    }
    pc.mass = warea;
    pc.area = area;
    /* intg = integrate_3(rho |x - s|^2) (quadrature.hpp:133-143) with the fan of
     * kantorovich.hpp (apex p[0]); moments with the fan of lloyd.hpp (vertices
     * vertex_to_point(R[i], R[i+1]) = p[i+1], apex p[1]) */
    double acc[NQ] = {0}, acm[NQ] = {0};
    if (n > 2) {
        for (int i = 1; i < n - 1; i++)
            albrecht_collatz(L, sv->x, sv->y, px[0], py[0], px[i], py[i], px[i + 1], py[i + 1], acc);
        for (int i = 1; i < n - 1; i++) {
            int a = 1 % n, b = (i + 1) % n, c = (i + 2) % n;
            albrecht_collatz(L, sv->x, sv->y, px[a], py[a], px[b], py[b], px[c], py[c], acm);
        }
    }
    pc.second = acc[0];
    for (int j = 0; j < 6; j++) pc.mom[j] = acm[1 + j];
    if (P->keep_pieces) {
        B->pxy = grow_buf(B->pxy, &B->cappv, 2 * (B->npv + n), sizeof(double));
        B->plab = grow_buf(B->plab, &B->cappl, B->npv + n, sizeof(int));
        pc.poly_off = B->npv;
        for (int i = 0; i < n; i++) {
            B->pxy[2 * (B->npv + i)] = px[i];
            B->pxy[2 * (B->npv + i) + 1] = py[i];
            B->plab[B->npv + i] = adj[i];
        }
        B->npv += n;
    }
    B->p = grow_buf(B->p, &B->cap, B->n + 1, sizeof(piece_t));
    B->p[B->n++] = pc;
}

/* ---- the same constructions and rules in double-double ---- */

typedef struct { dd a, b, c; } dd_lin;

static void edge_line_dd(const geo_t *G, pedge e, dd *a, dd *b, dd *c)
{
    if (e.t == 0) {
        double px = G->px[e.a], py = G->py[e.a], qx = G->px[e.b], qy = G->py[e.b];
        *a = dd_sub(dd_c(py), dd_c(qy));
        *b = dd_sub(dd_c(qx), dd_c(px));
        *c = dd_sub(dd_mul(dd_c(px), dd_c(qy)), dd_mul(dd_c(py), dd_c(qx)));
    } else {
        const site_t *v = &G->s[e.a], *w = &G->s[e.b];
        *a = dd_muld(dd_sub(dd_c(w->x), dd_c(v->x)), 2.0);
        *b = dd_muld(dd_sub(dd_c(w->y), dd_c(v->y)), 2.0);
        dd pv = dd_sub(dd_add(dd_mul(dd_c(v->x), dd_c(v->x)), dd_mul(dd_c(v->y), dd_c(v->y))), dd_c(v->w));
        dd pw = dd_sub(dd_add(dd_mul(dd_c(w->x), dd_c(w->x)), dd_mul(dd_c(w->y), dd_c(w->y))), dd_c(w->w));
        *c = dd_sub(pv, pw);
    }
}

static void vertex_to_point_dd(const geo_t *G, pedge e1, pedge e2, dd *x, dd *y)
{
    dd a1, b1, c1, a2, b2, c2;
    edge_line_dd(G, e1, &a1, &b1, &c1);
    edge_line_dd(G, e2, &a2, &b2, &c2);
    dd den = dd_sub(dd_mul(a1, b2), dd_mul(a2, b1));
    *x = dd_div(dd_sub(dd_mul(b1, c2), dd_mul(b2, c1)), den);
    *y = dd_div(dd_sub(dd_mul(a2, c1), dd_mul(a1, c2)), den);
}

static dd extrapolate_dd(double px, double py, double ax, double ay, double fa, double bx, double by, double fb,
                         double cx, double cy, double fc)
{
    dd v0x = dd_sub(dd_c(bx), dd_c(ax)), v0y = dd_sub(dd_c(by), dd_c(ay));
    dd v1x = dd_sub(dd_c(cx), dd_c(ax)), v1y = dd_sub(dd_c(cy), dd_c(ay));
    dd v2x = dd_sub(dd_c(px), dd_c(ax)), v2y = dd_sub(dd_c(py), dd_c(ay));
    dd d00 = dd_add(dd_mul(v0x, v0x), dd_mul(v0y, v0y)), d01 = dd_add(dd_mul(v0x, v1x), dd_mul(v0y, v1y));
    dd d11 = dd_add(dd_mul(v1x, v1x), dd_mul(v1y, v1y));
    dd d20 = dd_add(dd_mul(v2x, v0x), dd_mul(v2y, v0y)), d21 = dd_add(dd_mul(v2x, v1x), dd_mul(v2y, v1y));
    dd den = dd_sub(dd_mul(d00, d11), dd_mul(d01, d01));
    dd v = dd_div(dd_sub(dd_mul(d11, d20), dd_mul(d01, d21)), den);
    dd w = dd_div(dd_sub(dd_mul(d00, d21), dd_mul(d01, d20)), den);
    dd u = dd_sub(dd_sub(dd_c(1.0), v), w);
    return dd_add(dd_add(dd_muld(u, fa), dd_muld(v, fb)), dd_muld(w, fc));
}

static dd_lin make_linfn_dd(const prob_t *P, int f)
{
    const int *t = &P->tri[3 * f];
    double px = P->vx[t[0]], py = P->vy[t[0]], fp = P->vval[t[0]];
    double qx = P->vx[t[1]], qy = P->vy[t[1]], fq = P->vval[t[1]];
    double rx = P->vx[t[2]], ry = P->vy[t[2]], fr = P->vval[t[2]];
    dd_lin L;
    L.c = extrapolate_dd(0, 0, px, py, fp, qx, qy, fq, rx, ry, fr);
    L.a = dd_sub(extrapolate_dd(1, 0, px, py, fp, qx, qy, fq, rx, ry, fr), L.c);
    L.b = dd_sub(extrapolate_dd(0, 1, px, py, fp, qx, qy, fq, rx, ry, fr), L.c);
    return L;
}

static dd lf_dd(const dd_lin *L, dd x, dd y) { return dd_add(dd_add(dd_mul(L->a, x), dd_mul(L->b, y)), L->c); }

static dd tri_area_dd(dd ax, dd ay, dd bx, dd by, dd cx, dd cy)
{
    dd t = dd_sub(dd_mul(dd_sub(bx, ax), dd_sub(cy, ay)), dd_mul(dd_sub(cx, ax), dd_sub(by, ay)));
    return dd_muld(t, 0.5);
}

static void integrand_dd(const dd_lin *L, double sx, double sy, dd x, dd y, dd *out)
{
    dd r = lf_dd(L, x, y);
    dd dx = dd_sub(x, dd_c(sx)), dy = dd_sub(y, dd_c(sy));
    out[0] = dd_mul(r, dd_add(dd_mul(dx, dx), dd_mul(dy, dy)));
    out[1] = r;
    out[2] = dd_mul(r, x);
    out[3] = dd_mul(r, y);
    out[4] = dd_mul(dd_mul(r, x), x);
    out[5] = dd_mul(dd_mul(r, y), y);
    out[6] = dd_mul(dd_mul(r, x), y);
}

static void albrecht_collatz_dd(const dd_lin *L, double sx, double sy, dd ax, dd ay, dd bx, dd by, dd cx, dd cy,
                                dd *acc)
{
    dd ux = dd_sub(bx, ax), uy = dd_sub(by, ay), vx = dd_sub(cx, ax), vy = dd_sub(cy, ay);
    /* 1/2, 1/6, 2/3 and the weights 1/30, 9/30 as double-double constants */
    dd h = dd_c(0.5);
    dd s6 = dd_div(dd_c(1.0), dd_c(6.0)), t3 = dd_div(dd_c(2.0), dd_c(3.0));
    dd w1 = dd_div(dd_c(1.0), dd_c(30.0)), w9 = dd_div(dd_c(9.0), dd_c(30.0));
    dd cu[6][2] = {{h, h}, {h, dd_c(0)}, {dd_c(0), h}, {s6, t3}, {t3, s6}, {s6, s6}};
    dd wt[6] = {w1, w1, w1, w9, w9, w9};
    dd sum[NQ];
    for (int j = 0; j < NQ; j++) sum[j] = dd_c(0.0);
    for (int k = 0; k < 6; k++) {
        dd qx = dd_add(ax, dd_add(dd_mul(cu[k][0], ux), dd_mul(cu[k][1], vx)));
        dd qy = dd_add(ay, dd_add(dd_mul(cu[k][0], uy), dd_mul(cu[k][1], vy)));
        dd f[NQ];
        integrand_dd(L, sx, sy, qx, qy, f);
        for (int j = 0; j < NQ; j++) sum[j] = dd_add(sum[j], dd_mul(wt[k], f[j]));
    }
    dd A = tri_area_dd(ax, ay, bx, by, cx, cy);
    for (int j = 0; j < NQ; j++) acc[j] = dd_add(acc[j], dd_mul(A, sum[j]));
}

/* emit_piece with the constructions and rules evaluated in double-double */
static void emit_piece_dd(prob_t *P, piece_buf *B, geo_t *G, int f, int v, const pedge *R, int n)
{
    if (n == 0) return;
    dd px[PMAX], py[PMAX];
    int adj[PMAX];
    for (int i = 0; i < n; i++) {
        int ii = (i == 0) ? n - 1 : i - 1;
        vertex_to_point_dd(G, R[i], R[ii], &px[i], &py[i]);
        adj[i] = (R[i].t == 1) ? R[i].b : -1;
    }
    dd_lin L = make_linfn_dd(P, f);
    const site_t *sv = &P->s[v];
    for (int i = 0; i < n; i++) {
        if (adj[i] < 0) continue;
        int w = adj[i];
        int i1 = (i + 1) % n;
        dd ex = dd_sub(px[i1], px[i]), ey = dd_sub(py[i1], py[i]);
        dd len = dd_sqrt(dd_add(dd_mul(ex, ex), dd_mul(ey, ey)));
        dd mx = dd_muld(dd_add(px[i], px[i1]), 0.5), my = dd_muld(dd_add(py[i], py[i1]), 0.5);
        dd r = dd_mul(len, lf_dd(&L, mx, my));
        dd dx = dd_sub(dd_c(sv->x), dd_c(P->s[w].x)), dy = dd_sub(dd_c(sv->y), dd_c(P->s[w].y));
        dd d = dd_muld(dd_sqrt(dd_add(dd_mul(dx, dx), dd_mul(dy, dy))), 2.0);
        double q = dd_d(dd_div(r, d));
        B->t = grow_buf(B->t, &B->capt, B->nt + 2, sizeof(trip_t));
        trip_t t1 = {v, w, f, -1, -q};
        trip_t t2 = {v, v, f, w, q};
        B->t[B->nt++] = t1;
        B->t[B->nt++] = t2;
    }
    piece_t pc;
    memset(&pc, 0, sizeof(pc));
    pc.face = f;
    pc.site = v;
    pc.nv = n;
    dd warea = dd_c(0.0), area = dd_c(0.0);
    dd acc[NQ], acm[NQ];
    for (int j = 0; j < NQ; j++) {
        acc[j] = dd_c(0.0);
        acm[j] = dd_c(0.0);
    }
    if (n > 2) {
        dd third = dd_div(dd_c(1.0), dd_c(3.0));
        for (int i = 1; i < n - 1; i++) {
            dd A = tri_area_dd(px[0], py[0], px[i], py[i], px[i + 1], py[i + 1]);
            dd gx = dd_mul(dd_add(dd_add(px[0], px[i]), px[i + 1]), third);
            dd gy = dd_mul(dd_add(dd_add(py[0], py[i]), py[i + 1]), third);
            warea = dd_add(warea, dd_mul(A, lf_dd(&L, gx, gy)));
            area = dd_add(area, A);
        }
        for (int i = 1; i < n - 1; i++)
            albrecht_collatz_dd(&L, sv->x, sv->y, px[0], py[0], px[i], py[i], px[i + 1], py[i + 1], acc);
        for (int i = 1; i < n - 1; i++) {
            int a = 1 % n, b = (i + 1) % n, c = (i + 2) % n;
            albrecht_collatz_dd(&L, sv->x, sv->y, px[a], py[a], px[b], py[b], px[c], py[c], acm);
        }
    }
    pc.mass = dd_d(warea);
    pc.area = dd_d(area);
    pc.second = dd_d(acc[0]);
    for (int j = 0; j < 6; j++) pc.mom[j] = dd_d(acm[1 + j]);
    if (P->keep_pieces) {
        B->pxy = grow_buf(B->pxy, &B->cappv, 2 * (B->npv + n), sizeof(double));
        B->plab = grow_buf(B->plab, &B->cappl, B->npv + n, sizeof(int));
        pc.poly_off = B->npv;
        for (int i = 0; i < n; i++) {
            B->pxy[2 * (B->npv + i)] = dd_d(px[i]);
            B->pxy[2 * (B->npv + i) + 1] = dd_d(py[i]);
            B->plab[B->npv + i] = adj[i];
        }
        B->npv += n;
    }
    B->p = grow_buf(B->p, &B->cap, B->n + 1, sizeof(piece_t));
    B->p[B->n++] = pc;
}

static int g_dd = 0;

void ora_set_precision(int double_double) { g_dd = double_double; }

static void emit(prob_t *P, piece_buf *B, geo_t *G, int f, int v, const pedge *R, int n)
{
    if (g_dd)
        emit_piece_dd(P, B, G, f, v, R, n);
    else
        emit_piece(P, B, G, f, v, R, n);
}

/* clip triangle f by the neighbours of v (vti.hpp:255-274) */
static int clip_piece(prob_t *P, geo_t *G, int f, int v, pedge *out)
{
    pedge A[PMAX], Bv[PMAX];
    const int *t = &P->tri[3 * f];
    A[0].t = 0; A[0].a = t[0]; A[0].b = t[1];
    A[1].t = 0; A[1].a = t[1]; A[1].b = t[2];
    A[2].t = 0; A[2].a = t[2]; A[2].b = t[0];
    int n = 3;
    pedge *cur = A, *nxt = Bv;
    for (int k = P->nstart[v]; k < P->nstart[v + 1] && n > 0; k++) {
        int m = clip(G, cur, n, v, P->nlist[k], nxt);
        pedge *tmp = cur; cur = nxt; nxt = tmp;
        n = m;
    }
    memcpy(out, cur, sizeof(pedge) * n);
    return n;
}

/* ------------------------------------------------------------------------- */
/* visited set (open addressing on 64-bit keys)                              */
/* ------------------------------------------------------------------------- */

typedef struct { uint64_t *k; long cap, n; long *used; long ucap; } hset;

static uint64_t hmix(uint64_t x)
{
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

static int hs_insert(hset *h, uint64_t key) /* returns 1 if newly inserted */
{
    if (2 * (h->n + 1) > h->cap) {
        long nc = h->cap ? 2 * h->cap : 1024;
        uint64_t *nk = malloc(sizeof(uint64_t) * nc);
        for (long i = 0; i < nc; i++) nk[i] = UINT64_MAX;
        for (long i = 0; i < h->cap; i++) {
            if (h->k[i] == UINT64_MAX) continue;
            long p = hmix(h->k[i]) & (nc - 1);
            while (nk[p] != UINT64_MAX) p = (p + 1) & (nc - 1);
            nk[p] = h->k[i];
        }
        free(h->k);
        h->k = nk;
        h->cap = nc;
        h->n = 0;
        for (long i = 0; i < nc; i++)
            if (nk[i] != UINT64_MAX) {
                h->used = grow_buf(h->used, &h->ucap, h->n + 1, sizeof(long));
                h->used[h->n++] = i;
            }
    }
    long p = hmix(key) & (h->cap - 1);
    while (h->k[p] != UINT64_MAX) {
        if (h->k[p] == key) return 0;
        p = (p + 1) & (h->cap - 1);
    }
    h->k[p] = key;
    h->used = grow_buf(h->used, &h->ucap, h->n + 1, sizeof(long));
    h->used[h->n++] = p;
    return 1;
}

/* empty the set in time proportional to its size */
static void hs_clear(hset *h)
{
    for (long i = 0; i < h->n; i++) h->k[h->used[i]] = UINT64_MAX;
    h->n = 0;
}

/* ------------------------------------------------------------------------- */
/* result                                                                    */
/* ------------------------------------------------------------------------- */

typedef struct {
    int n;
    double value, total_mass, total_area;
    double *g;        /* masses */
    double *mom;      /* 6 per site: rho, rho x, rho y, rho x^2, rho y^2, rho xy */
    long nnz;
    int *hr, *hc;
    double *hv;
    long npieces;
    int *pface, *psite, *pnv;
    long *poff;
    double *pxy;
    int *plab;
    long filter_calls, exact_calls;
    int *nstart, *nlist;
} ora_result;

static int cmp_piece(const void *a, const void *b)
{
    const piece_t *x = a, *y = b;
    if (x->face != y->face) return x->face < y->face ? -1 : 1;
    if (x->site != y->site) return x->site < y->site ? -1 : 1;
    return 0;
}

static int cmp_trip(const void *a, const void *b)
{
    const trip_t *x = a, *y = b;
    if (x->row != y->row) return x->row < y->row ? -1 : 1;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    if (x->face != y->face) return x->face < y->face ? -1 : 1;
    if (x->aux != y->aux) return x->aux < y->aux ? -1 : 1;
    return 0;
}

static void build_faces(prob_t *P)
{
    /* face adjacency from shared edges (what Triangulation_incremental_builder_2
     * sets up, CGAL/Triangulation_incremental_builder_2.h:128-151) */
    int nt = P->nt;
    P->fnbr = malloc(sizeof(int) * 3 * (nt > 0 ? nt : 1));
    for (int i = 0; i < 3 * nt; i++) P->fnbr[i] = -1;
    long cap = 1;
    while (cap < 6L * nt + 16) cap <<= 1;
    uint64_t *key = malloc(sizeof(uint64_t) * cap);
    int *val = malloc(sizeof(int) * cap);
    for (long i = 0; i < cap; i++) key[i] = UINT64_MAX;
    for (int f = 0; f < nt; f++) {
        for (int k = 0; k < 3; k++) {
            int a = P->tri[3 * f + (k + 1) % 3], b = P->tri[3 * f + (k + 2) % 3];
            uint64_t lo = a < b ? a : b, hi = a < b ? b : a;
            uint64_t kk = (lo << 32) | hi;
            long p = hmix(kk) & (cap - 1);
            while (key[p] != UINT64_MAX && key[p] != kk) p = (p + 1) & (cap - 1);
            if (key[p] == UINT64_MAX) {
                key[p] = kk;
                val[p] = 3 * f + k;
            } else {
                int g = val[p] / 3, kg = val[p] % 3;
                P->fnbr[3 * f + k] = g;
                P->fnbr[3 * g + kg] = f;
            }
        }
    }
    free(key);
    free(val);
    P->fn = malloc(sizeof(linfn) * (nt > 0 ? nt : 1));
    for (int f = 0; f < nt; f++) {
        const int *t = &P->tri[3 * f];
        P->fn[f] = make_linfn(P->vx[t[0]], P->vy[t[0]], P->vval[t[0]], P->vx[t[1]], P->vy[t[1]],
                              P->vval[t[1]], P->vx[t[2]], P->vy[t[2]], P->vval[t[2]]);
    }
}

static int g_threads = 0;

void ora_set_threads(int n) { g_threads = n; }

int ora_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * ora_kantorovich: one evaluation of the reference's kantorovich() plus the
 * moments of first_moment()/second_moment().
 *   mode 0: the reference's global flood fill over (site, triangle) pairs
 *           (vti.hpp:219-313), single thread;
 *   mode 1: the same pieces found triangle by triangle (one flood fill over the
 *           sites inside each triangle), OpenMP over triangles.
 * Both modes emit the same pieces with the same symbolic polygons, and the
 * accumulation is done in (face, site) order, so both give identical bits.
 */
ora_result *ora_kantorovich(int nv, const double *vx, const double *vy, const double *vval, int nt,
                            const int *tri, int n, const double *x, const double *y, const double *w,
                            int mode, int keep_pieces, const int *cand_start, const int *cand_list)
{
    prob_t P;
    memset(&P, 0, sizeof(P));
    P.nv = nv; P.nt = nt; P.n = n;
    P.vx = vx; P.vy = vy; P.vval = vval; P.tri = tri;
    P.keep_pieces = keep_pieces;
    P.cstart = cand_start;
    P.clist = cand_list;
#ifdef _OPENMP
    if (g_threads > 0) omp_set_num_threads(g_threads);
#endif
    /* box B' around the mesh */
    double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    for (int i = 0; i < nv; i++) {
        if (vx[i] < x0) x0 = vx[i];
        if (vx[i] > x1) x1 = vx[i];
        if (vy[i] < y0) y0 = vy[i];
        if (vy[i] > y1) y1 = vy[i];
    }
    double mw = (x1 - x0) * 1e-3, mh = (y1 - y0) * 1e-3;
    P.bx0 = x0 - mw; P.by0 = y0 - mh; P.bx1 = x1 + mw; P.by1 = y1 + mh;
    P.ptx = malloc(sizeof(double) * (nv + 4));
    P.pty = malloc(sizeof(double) * (nv + 4));
    memcpy(P.ptx, vx, sizeof(double) * nv);
    memcpy(P.pty, vy, sizeof(double) * nv);
    P.ptx[nv] = P.bx0; P.pty[nv] = P.by0;
    P.ptx[nv + 1] = P.bx1; P.pty[nv + 1] = P.by0;
    P.ptx[nv + 2] = P.bx1; P.pty[nv + 2] = P.by1;
    P.ptx[nv + 3] = P.bx0; P.pty[nv + 3] = P.by1;
    P.s = malloc(sizeof(site_t) * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++) { P.s[i].x = x[i]; P.s[i].y = y[i]; P.s[i].w = w[i]; }
    build_faces(&P);
    build_grid(&P);

    ora_result *res = calloc(1, sizeof(ora_result));
    res->n = n;

    /* regular-triangulation neighbours (restricted to B') */
    int **nbl = malloc(sizeof(int *) * (n > 0 ? n : 1));
    int *nbc = calloc(n > 0 ? n : 1, sizeof(int));
    P.cbox = malloc(sizeof(double) * 4 * (n > 0 ? n : 1));
    long fc = 0, ec = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : fc, ec) if (mode == 1)
    for (int i = 0; i < n; i++) {
        int tmp[PMAX];
        pred_stats st = {0, 0};
        int m = P.cstart ? site_neighbors_cand(&P, i, tmp, &st) : site_neighbors(&P, i, tmp, &st);
        nbl[i] = malloc(sizeof(int) * (m > 0 ? m : 1));
        memcpy(nbl[i], tmp, sizeof(int) * m);
        nbc[i] = m;
        fc += st.filter_calls;
        ec += st.exact_calls;
    }
    P.nstart = malloc(sizeof(int) * (n + 1));
    P.nstart[0] = 0;
    for (int i = 0; i < n; i++) P.nstart[i + 1] = P.nstart[i] + nbc[i];
    P.nlist = malloc(sizeof(int) * (P.nstart[n] > 0 ? P.nstart[n] : 1));
    for (int i = 0; i < n; i++) {
        memcpy(P.nlist + P.nstart[i], nbl[i], sizeof(int) * nbc[i]);
        free(nbl[i]);
    }
    free(nbl);
    free(nbc);
    if (P.cstart) build_cell_bins(&P);

    int nthreads = 1;
#ifdef _OPENMP
    if (mode == 1) nthreads = omp_get_max_threads();
#endif
    piece_buf *bufs = calloc(nthreads, sizeof(piece_buf));

    if (n > 0 && nt > 0 && mode == 0) {
        /* global flood fill (vti.hpp:234-305), FIFO order; faces never reached
         * from face 0 (a disconnected mesh) are seeded in turn */
        geo_t G = {P.ptx, P.pty, P.s, {0, 0}};
        hset vis = {0, 0, 0, 0, 0};
        char *covered = calloc(nt, 1);
        long qcap = 1024, qh = 0, qt = 0;
        uint64_t *Q = malloc(sizeof(uint64_t) * qcap);
        pedge R[PMAX];
        int seeds[256];
        for (int f0 = 0; f0 < nt; f0++) {
            if (covered[f0]) continue;
            int ns = P.cstart ? locate(&P, vx[tri[3 * f0]], vy[tri[3 * f0]], seeds, 256)
                              : seeds_at(&P, vx[tri[3 * f0]], vy[tri[3 * f0]], seeds, 256);
            for (int k = 0; k < ns; k++) {
                uint64_t key = (uint64_t)seeds[k] * (uint64_t)nt + f0;
                if (hs_insert(&vis, key)) {
                    if (qt >= qcap) { qcap *= 2; Q = realloc(Q, sizeof(uint64_t) * qcap); }
                    Q[qt++] = key;
                }
            }
            while (qh < qt) {
                uint64_t key = Q[qh++];
                int v = (int)(key / (uint64_t)nt), f = (int)(key % (uint64_t)nt);
                int m = clip_piece(&P, &G, f, v, R);
                if (m > 0) covered[f] = 1;
                for (int e = 0; e < m; e++) {
                    uint64_t nk;
                    if (R[e].t == 0) {
                        const int *t = &tri[3 * f];
                        int i = (R[e].a == t[0]) ? 0 : (R[e].a == t[1]) ? 1 : 2;
                        int j = (R[e].b == t[0]) ? 0 : (R[e].b == t[1]) ? 1 : 2;
                        int fn = P.fnbr[3 * f + (3 - i - j)];
                        if (fn < 0) continue;
                        nk = (uint64_t)v * (uint64_t)nt + fn;
                    } else {
                        nk = (uint64_t)R[e].b * (uint64_t)nt + f;
                    }
                    if (!hs_insert(&vis, nk)) continue;
                    if (qt >= qcap) { qcap *= 2; Q = realloc(Q, sizeof(uint64_t) * qcap); }
                    Q[qt++] = nk;
                }
                emit(&P, &bufs[0], &G, f, v, R, m);
            }
        }
        bufs[0].st.filter_calls += G.st.filter_calls;
        bufs[0].st.exact_calls += G.st.exact_calls;
        free(Q);
        free(vis.k);
        free(vis.used);
        free(covered);
    } else if (n > 0 && nt > 0) {
#pragma omp parallel
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            piece_buf *B = &bufs[tid];
            geo_t G = {P.ptx, P.pty, P.s, {0, 0}};
            pedge R[PMAX];
            int seeds[256];
            long scap = 1024;
            int *stack = malloc(sizeof(int) * scap);
            hset seen = {0, 0, 0, 0, 0};
#pragma omp for schedule(dynamic, 16)
            for (int f = 0; f < nt; f++) {
                int ns = P.cstart ? locate(&P, vx[tri[3 * f]], vy[tri[3 * f]], seeds, 256)
                                  : seeds_at(&P, vx[tri[3 * f]], vy[tri[3 * f]], seeds, 256);
                long nsk = 0;
                hs_clear(&seen);
                for (int k = 0; k < ns; k++) {
                    stack = grow_buf(stack, &scap, nsk + 1, sizeof(int));
                    stack[nsk++] = seeds[k];
                    hs_insert(&seen, (uint64_t)seeds[k]);
                }
                while (nsk > 0) {
                    int v = stack[--nsk];
                    int m = clip_piece(&P, &G, f, v, R);
                    for (int e = 0; e < m; e++) {
                        if (R[e].t != 1) continue;
                        int u = R[e].b;
                        if (!hs_insert(&seen, (uint64_t)u)) continue;
                        stack = grow_buf(stack, &scap, nsk + 1, sizeof(int));
                        stack[nsk++] = u;
                    }
                    emit(&P, B, &G, f, v, R, m);
                }
            }
            B->st.filter_calls += G.st.filter_calls;
            B->st.exact_calls += G.st.exact_calls;
            free(stack);
            free(seen.k);
            free(seen.used);
        }
    }

    /* merge the piece records and accumulate in canonical order */
    long np = 0, ntr = 0, npv = 0;
    for (int t = 0; t < nthreads; t++) { np += bufs[t].n; ntr += bufs[t].nt; npv += bufs[t].npv; }
    piece_t *all = malloc(sizeof(piece_t) * (np > 0 ? np : 1));
    trip_t *tr = malloc(sizeof(trip_t) * (ntr > 0 ? ntr : 1));
    double *allxy = keep_pieces ? malloc(sizeof(double) * 2 * (npv > 0 ? npv : 1)) : NULL;
    int *alllab = keep_pieces ? malloc(sizeof(int) * (npv > 0 ? npv : 1)) : NULL;
    long op = 0, ot = 0, ov = 0;
    for (int t = 0; t < nthreads; t++) {
        for (long k = 0; k < bufs[t].n; k++) {
            all[op] = bufs[t].p[k];
            if (keep_pieces) all[op].poly_off += ov;
            op++;
        }
        memcpy(tr + ot, bufs[t].t, sizeof(trip_t) * bufs[t].nt);
        ot += bufs[t].nt;
        if (keep_pieces && bufs[t].npv) {
            memcpy(allxy + 2 * ov, bufs[t].pxy, sizeof(double) * 2 * bufs[t].npv);
            memcpy(alllab + ov, bufs[t].plab, sizeof(int) * bufs[t].npv);
        }
        ov += bufs[t].npv;
        fc += bufs[t].st.filter_calls;
        ec += bufs[t].st.exact_calls;
        free(bufs[t].p);
        free(bufs[t].t);
        free(bufs[t].pxy);
        free(bufs[t].plab);
    }
    free(bufs);
    qsort(all, np, sizeof(piece_t), cmp_piece);
    qsort(tr, ntr, sizeof(trip_t), cmp_trip);

    res->g = calloc(n > 0 ? n : 1, sizeof(double));
    res->mom = calloc(6 * (n > 0 ? n : 1), sizeof(double));
    double fval = 0.0, total = 0.0, tarea = 0.0;
    for (long k = 0; k < np; k++) {
        const piece_t *pc = &all[k];
        fval = fval + pc->mass * w[pc->site] - pc->second;
        res->g[pc->site] += pc->mass;
        for (int j = 0; j < 6; j++) res->mom[6 * pc->site + j] += pc->mom[j];
        total += pc->mass;
        tarea += pc->area;
    }
    res->value = fval;
    res->total_mass = total;
    res->total_area = tarea;
    /* setFromTriplets: duplicates summed (kantorovich.hpp:137-139) */
    res->hr = malloc(sizeof(int) * (ntr > 0 ? ntr : 1));
    res->hc = malloc(sizeof(int) * (ntr > 0 ? ntr : 1));
    res->hv = malloc(sizeof(double) * (ntr > 0 ? ntr : 1));
    long nnz = 0;
    for (long k = 0; k < ntr; k++) {
        if (nnz > 0 && res->hr[nnz - 1] == tr[k].row && res->hc[nnz - 1] == tr[k].col) {
            res->hv[nnz - 1] += tr[k].val;
        } else {
            res->hr[nnz] = tr[k].row;
            res->hc[nnz] = tr[k].col;
            res->hv[nnz] = tr[k].val;
            nnz++;
        }
    }
    res->nnz = nnz;
    res->npieces = np;
    res->pface = malloc(sizeof(int) * (np > 0 ? np : 1));
    res->psite = malloc(sizeof(int) * (np > 0 ? np : 1));
    res->pnv = malloc(sizeof(int) * (np > 0 ? np : 1));
    res->poff = malloc(sizeof(long) * (np > 0 ? np : 1));
    for (long k = 0; k < np; k++) {
        res->pface[k] = all[k].face;
        res->psite[k] = all[k].site;
        res->pnv[k] = all[k].nv;
        res->poff[k] = all[k].poly_off;
    }
    res->pxy = allxy;
    res->plab = alllab;
    res->filter_calls = fc;
    res->exact_calls = ec;
    res->nstart = P.nstart;
    res->nlist = P.nlist;
    free(all);
    free(tr);
    free(P.ptx); free(P.pty); free(P.s); free(P.fnbr); free(P.fn); free(P.gstart); free(P.gidx);
    free(P.cbox); free(P.bstart); free(P.blist);
    return res;
}

double ora_value(const ora_result *r) { return r->value; }
double ora_total_mass(const ora_result *r) { return r->total_mass; }
double ora_total_area(const ora_result *r) { return r->total_area; }
void ora_masses(const ora_result *r, double *g) { memcpy(g, r->g, sizeof(double) * r->n); }
void ora_moments(const ora_result *r, double *m) { memcpy(m, r->mom, sizeof(double) * 6 * r->n); }
long ora_nnz(const ora_result *r) { return r->nnz; }
void ora_hessian(const ora_result *r, int *row, int *col, double *val)
{
    memcpy(row, r->hr, sizeof(int) * r->nnz);
    memcpy(col, r->hc, sizeof(int) * r->nnz);
    memcpy(val, r->hv, sizeof(double) * r->nnz);
}
long ora_npieces(const ora_result *r) { return r->npieces; }
void ora_pieces(const ora_result *r, int *face, int *site, int *nvert)
{
    memcpy(face, r->pface, sizeof(int) * r->npieces);
    memcpy(site, r->psite, sizeof(int) * r->npieces);
    memcpy(nvert, r->pnv, sizeof(int) * r->npieces);
}
/* polygon vertices of every piece, in piece order (requires keep_pieces) */
long ora_piece_vertices(const ora_result *r, double *xy, int *lab)
{
    if (!r->pxy) return -1;
    long o = 0;
    for (long k = 0; k < r->npieces; k++) {
        memcpy(xy + 2 * o, r->pxy + 2 * r->poff[k], sizeof(double) * 2 * r->pnv[k]);
        memcpy(lab + o, r->plab + r->poff[k], sizeof(int) * r->pnv[k]);
        o += r->pnv[k];
    }
    return o;
}
long ora_neighbor_count(const ora_result *r) { return r->nstart[r->n]; }
void ora_neighbors(const ora_result *r, int *start, int *list)
{
    memcpy(start, r->nstart, sizeof(int) * (r->n + 1));
    memcpy(list, r->nlist, sizeof(int) * r->nstart[r->n]);
}
void ora_pred_stats(const ora_result *r, long *out)
{
    out[0] = r->filter_calls;
    out[1] = r->exact_calls;
}
void ora_free(ora_result *r)
{
    if (!r) return;
    free(r->g); free(r->mom); free(r->hr); free(r->hc); free(r->hv);
    free(r->pface); free(r->psite); free(r->pnv); free(r->poff); free(r->pxy); free(r->plab);
    free(r->nstart); free(r->nlist);
    free(r);
}

/* quadrature.hpp:24-42 on one triangle tri = (ax, ay, bx, by, cx, cy), for the tests
 * that check the rule (tests/test_quadrature_triangle.cpp:10-21 integrates x y^2): the
 * seven integrands of `integrand` for the linear function a x + b y + c and the site
 * (sx, sy), added to out[0..6] */
void ora_albrecht_collatz(double a, double b, double c, double sx, double sy, const double *tri, double *out)
{
    const linfn L = {a, b, c};
    albrecht_collatz(&L, sx, sy, tri[0], tri[1], tri[2], tri[3], tri[4], tri[5], out);
}

/* exact predicate entry points, for the tests that check the filters */
int ora_side1(const double *v, const double *w, double ex, double ey)
{
    site_t a = {v[0], v[1], v[2]}, b = {w[0], w[1], w[2]};
    pred_stats st = {0, 0};
    return side1(&a, &b, ex, ey, &st);
}
int ora_side2(const double *v, const double *a, const double *b, const double *w)
{
    site_t A = {v[0], v[1], v[2]}, B = {a[0], a[1], a[2]}, C = {b[0], b[1], b[2]}, D = {w[0], w[1], w[2]};
    pred_stats st = {0, 0};
    return side2(&A, &B, &C, &D, &st);
}
int ora_side3(const double *v, const double *u, const double *p, const double *q, const double *w)
{
    site_t A = {v[0], v[1], v[2]}, U = {u[0], u[1], u[2]}, W = {w[0], w[1], w[2]};
    pred_stats st = {0, 0};
    return side3(&A, &U, p[0], p[1], q[0], q[1], &W, &st);
}

/* ------------------------------------------------------------------------- */
/* one cell clipped to a polygon (voronoi_polygon_intersection.hpp:27-188)    */
/* ------------------------------------------------------------------------- */

/* MA::voronoi_polygon_intersection(P, dt, v) for site v: the polygon (qx, qy)[0..k)
 * as the symbolic edges (e, e+1) (:160-161), clipped in turn by the half-plane of v
 * against each candidate neighbour (Pgon_intersector::operator(), :116-149, the same
 * Sutherland-Hodgman step as Tri_intersector's), then each vertex -- the pair of its
 * two edges -- made a point (vertex_to_point, :64-69).  The reference clips by the
 * triangulation's neighbours of v; the candidates here are a superset (the regular
 * triangulation's neighbours and theirs), which changes nothing because every test
 * is exact.  Coordinates in double-double rounded to double (the corners of P
 * copied).  Vertex j is the start of edge lab[j]: a neighbour's index, or -1-e for
 * edge e of P.  Returns the vertex count (0: empty), or -1 beyond `cap`. */
int ora_polygon_cell(int n, const double *x, const double *y, const double *w, int v, const int *cand,
                     int ncand, int k, const double *qx, const double *qy, int cap, double *xy, int *lab)
{
    site_t *S = (site_t *)malloc(sizeof(site_t) * (size_t)n);
    pedge *A = (pedge *)malloc(sizeof(pedge) * PMAX), *B = (pedge *)malloc(sizeof(pedge) * PMAX);
    for (int i = 0; i < n; i++) { S[i].x = x[i]; S[i].y = y[i]; S[i].w = w[i]; }
    geo_t G;
    memset(&G, 0, sizeof G);
    G.px = qx;
    G.py = qy;
    G.s = S;
    int m = k;
    for (int e = 0; e < k; e++) { A[e].t = 0; A[e].a = e; A[e].b = (e + 1) % k; }
    for (int c = 0; c < ncand && m > 0; c++) {
        int u = cand[c];
        if (u == v) continue;
        if (S[u].x == S[v].x && S[u].y == S[v].y) {
            /* coincident sites: the larger weight, then the lower index, keeps the cell */
            if (S[u].w > S[v].w || (S[u].w == S[v].w && u < v)) m = 0;
            continue;
        }
        m = clip(&G, A, m, v, u, B);
        pedge *t = A; A = B; B = t;
    }
    int out = m;
    if (m > cap) {
        out = -1;
    } else {
        for (int j = 0; j < m; j++) {
            pedge e0 = A[(j + m - 1) % m], e1 = A[j];
            if (e0.t == 0 && e1.t == 0) {
                int p = common_pt(e0, e1);
                xy[2 * j] = qx[p];
                xy[2 * j + 1] = qy[p];
            } else {
                dd X, Y;
                vertex_to_point_dd(&G, e0, e1, &X, &Y);
                xy[2 * j] = dd_d(X);
                xy[2 * j + 1] = dd_d(Y);
            }
            lab[j] = e1.t == 0 ? -1 - e1.a : e1.b;
        }
    }
    free(S);
    free(A);
    free(B);
    return out;
}
