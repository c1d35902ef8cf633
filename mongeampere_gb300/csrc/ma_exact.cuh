// ma_exact.cuh -- arithmetic building blocks for certified geometric decisions.
//
//  * uncontracted FP64 operations (the device never fuses them into FMAs, so
//    error-free transformations stay error free);
//  * floating-point expansions: an exact real number held as a sum of doubles
//    with non-overlapping bits (Shewchuk, "Adaptive precision floating-point
//    arithmetic and fast robust geometric predicates", DCG 18, 1997):
//    two_sum, two_prod, grow, scale, compress;
//  * running-error arithmetic in FP32 (F) and FP64 (R): a computed value plus a
//    rigorous bound on its distance to the exact value of the same expression on
//    the exact inputs.  A sign is certain when |value| exceeds the bound.
//
// Everything here is __host__ __device__ so the same code can be checked on a
// CPU.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define MA_HD __host__ __device__ __forceinline__
#define MA_HDNI inline __host__ __device__ __noinline__
#else
#define MA_HD inline
#define MA_HDNI
#endif

namespace ma {

// ---------------------------------------------------------------------------
// uncontracted FP64
// ---------------------------------------------------------------------------
MA_HD double dadd(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    volatile double r = a + b;
    return r;
#endif
}
MA_HD double dsub(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    volatile double r = a - b;
    return r;
#endif
}
MA_HD double dmul(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;
    return r;
#endif
}
MA_HD double dfma(double a, double b, double c)
{
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

// ---------------------------------------------------------------------------
// expansions
// ---------------------------------------------------------------------------
MA_HD void two_sum(double a, double b, double& s, double& e)
{
    s = dadd(a, b);
    double bv = dsub(s, a);
    double av = dsub(s, bv);
    e = dadd(dsub(a, av), dsub(b, bv));
}

MA_HD void two_prod(double a, double b, double& p, double& e)
{
    p = dmul(a, b);
    e = dfma(a, b, -p);
}

// Fixed-capacity expansion.  `ok` turns false if a result would not fit; the
// caller then reports an error instead of trusting the sign.
template <int CAP>
struct Exp {
    int n;
    double c[CAP];
};

// h += b   (h non-overlapping, increasing magnitude; zero components dropped)
template <int CAP>
MA_HD void ex_grow(Exp<CAP>& h, double b, bool& ok)
{
    double q = b, qn, hh;
    int hi = 0;
    for (int i = 0; i < h.n; i++) {
        two_sum(q, h.c[i], qn, hh);
        q = qn;
        if (hh != 0.0) h.c[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) {
        if (hi >= CAP) { ok = false; return; }
        h.c[hi++] = q;
    }
    h.n = hi;
}

// Shewchuk's Compress: same value, fewer components.
template <int CAP>
MA_HD void ex_compress(Exp<CAP>& e)
{
    if (e.n <= 1) return;
    double g[CAP];
    int bottom = e.n - 1;
    double Q = e.c[bottom], Qn, q;
    for (int i = e.n - 2; i >= 0; i--) {
        two_sum(Q, e.c[i], Qn, q);
        if (q != 0.0) {
            g[bottom--] = Qn;
            Q = q;
        } else {
            Q = Qn;
        }
    }
    int top = 0;
    for (int i = bottom + 1; i < e.n; i++) {
        two_sum(g[i], Q, Qn, q);
        if (q != 0.0) e.c[top++] = q;
        Q = Qn;
    }
    e.c[top++] = Q;
    e.n = top;
}

template <int CAP>
MA_HD void ex_set(Exp<CAP>& h, double a)
{
    h.n = 1;
    h.c[0] = a;
}

template <int CAP>
MA_HD void ex_add(Exp<CAP>& h, const Exp<CAP>& f, bool& ok)
{
    for (int j = 0; j < f.n && ok; j++) ex_grow(h, f.c[j], ok);
    if (h.n > CAP / 2) ex_compress(h);
}

template <int CAP>
MA_HD void ex_sub(Exp<CAP>& h, const Exp<CAP>& f, bool& ok)
{
    for (int j = 0; j < f.n && ok; j++) ex_grow(h, -f.c[j], ok);
    if (h.n > CAP / 2) ex_compress(h);
}

// h = a * b
template <int CAP>
MA_HD void ex_mul(Exp<CAP>& h, const Exp<CAP>& a, const Exp<CAP>& b, bool& ok)
{
    ex_set(h, 0.0);
    for (int j = 0; j < b.n && ok; j++) {
        for (int i = 0; i < a.n && ok; i++) {
            double p, e;
            two_prod(a.c[i], b.c[j], p, e);
            ex_grow(h, e, ok);
            if (ok) ex_grow(h, p, ok);
        }
        if (h.n > CAP / 2) ex_compress(h);
    }
}

// h = a - b exactly (two components)
template <int CAP>
MA_HD void ex_diff(Exp<CAP>& h, double a, double b)
{
    double s, e;
    two_sum(a, -b, s, e);
    if (e != 0.0) {
        h.n = 2;
        h.c[0] = e;
        h.c[1] = s;
    } else {
        h.n = 1;
        h.c[0] = s;
    }
}

template <int CAP>
MA_HD int ex_sign(const Exp<CAP>& e)
{
    double t = e.c[e.n - 1];
    return (t > 0.0) - (t < 0.0);
}

// ---------------------------------------------------------------------------
// running-error FP32:  |v - exact| <= e
// ---------------------------------------------------------------------------
struct F {
    float v, e;
};

constexpr float kU32 = 1.1920929e-07f;  // 2^-23: covers one rounding plus slack

MA_HD F fv(float v, float e) { return F{v, e}; }
MA_HD F f_add(F a, F b)
{
    float s = a.v + b.v;
    return F{s, a.e + b.e + kU32 * fabsf(s)};
}
MA_HD F f_sub(F a, F b)
{
    float s = a.v - b.v;
    return F{s, a.e + b.e + kU32 * fabsf(s)};
}
MA_HD F f_mul(F a, F b)
{
    float p = a.v * b.v;
    return F{p, fabsf(a.v) * b.e + fabsf(b.v) * a.e + a.e * b.e + kU32 * fabsf(p)};
}
MA_HD F f_scale2(F a) { return F{2.0f * a.v, 2.0f * a.e}; }
// a / b; an infinite bound when b may be zero
MA_HD F f_div(F a, F b)
{
    float q = a.v / b.v;
    float den = fabsf(b.v) - b.e;
    if (!(den > 0.0f)) return F{q, INFINITY};
    float e = (a.e + fabsf(q) * b.e) / den;
    return F{q, e * 1.0000001f + kU32 * fabsf(q)};
}

// ---------------------------------------------------------------------------
// running-error FP64
// ---------------------------------------------------------------------------
struct R {
    double v, e;
};

constexpr double kU64 = 2.220446049250313e-16;  // 2^-52

MA_HD R rv(double v) { return R{v, 0.0}; }
MA_HD R r_add(R a, R b)
{
    double s = dadd(a.v, b.v);
    return R{s, a.e + b.e + kU64 * fabs(s)};
}
MA_HD R r_sub(R a, R b)
{
    double s = dsub(a.v, b.v);
    return R{s, a.e + b.e + kU64 * fabs(s)};
}
MA_HD R r_mul(R a, R b)
{
    double p = dmul(a.v, b.v);
    return R{p, fabs(a.v) * b.e + fabs(b.v) * a.e + a.e * b.e + kU64 * fabs(p)};
}
// +1 / -1 when certain, 0 otherwise
MA_HD int r_sign(R a)
{
    double b = a.e * (1.0 + 1e-9) + 1e-300;
    if (a.v > b) return 1;
    if (-a.v > b) return -1;
    return 0;
}

}  // namespace ma
