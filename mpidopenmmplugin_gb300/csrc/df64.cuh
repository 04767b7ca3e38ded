// Double-float ("df") arithmetic: a value is the unevaluated sum hi + lo of two floats
// with |lo| <= ulp(hi)/2, about 48 significant bits.  GB300 runs FP32 at many times its
// FP64 rate, so the mixed path's FP64-accurate residual field is evaluated in df on the
// FP32 pipes.  The building blocks are the error-free transformations of Knuth (TwoSum),
// Dekker (FastTwoSum) and the FMA-based TwoProd, combined as in the double-double /
// double-float literature (Dekker 1971; Hida, Li & Bailey, "Algorithms for quad-double
// precision floating point arithmetic", 2001).  Every function is __host__ __device__,
// so the host tests check the device arithmetic against long double.
#pragma once
#include <math.h>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#define __forceinline__ inline
#endif
#endif
#define DF_HD __host__ __device__ __forceinline__

namespace mpid {

// Rounded add and multiply that the compiler may not contract into an FMA (the
// error-free transformations below depend on each operation being rounded on its own).
#if defined(__CUDA_ARCH__)
DF_HD float df_radd(float a, float b) { return __fadd_rn(a, b); }
DF_HD float df_rsub(float a, float b) { return __fsub_rn(a, b); }
DF_HD float df_rmul(float a, float b) { return __fmul_rn(a, b); }
#else
DF_HD float df_radd(float a, float b) { return a + b; }
DF_HD float df_rsub(float a, float b) { return a - b; }
DF_HD float df_rmul(float a, float b) { return a * b; }
#endif

struct dfloat {
    float hi, lo;
};

DF_HD dfloat df_make(float hi, float lo) {
    dfloat r;
    r.hi = hi;
    r.lo = lo;
    return r;
}
DF_HD dfloat df_from_float(float x) { return df_make(x, 0.f); }
// Host/device conversion from double (exact split of the leading 48 bits).
DF_HD dfloat df_from_double(double x) {
    const float hi = (float) x;
    return df_make(hi, (float) (x - (double) hi));
}
DF_HD double df_to_double(dfloat a) { return (double) a.hi + (double) a.lo; }

DF_HD float df_fma(float a, float b, float c) { return fmaf(a, b, c); }

// s + e = a + b exactly
DF_HD dfloat two_sum(float a, float b) {
    const float s = df_radd(a, b);
    const float bb = df_rsub(s, a);
    const float e = df_radd(df_rsub(a, df_rsub(s, bb)), df_rsub(b, bb));
    return df_make(s, e);
}
// s + e = a + b exactly, for |a| >= |b|
DF_HD dfloat fast_two_sum(float a, float b) {
    const float s = df_radd(a, b);
    return df_make(s, df_rsub(b, df_rsub(s, a)));
}
// p + e = a * b exactly
DF_HD dfloat two_prod(float a, float b) {
    const float p = df_rmul(a, b);
    return df_make(p, df_fma(a, b, -p));
}

DF_HD dfloat df_add(dfloat a, dfloat b) {
    dfloat s = two_sum(a.hi, b.hi);
    const dfloat t = two_sum(a.lo, b.lo);
    s.lo = df_radd(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = df_radd(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
DF_HD dfloat df_add(dfloat a, float b) {
    dfloat s = two_sum(a.hi, b);
    s.lo = df_radd(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
DF_HD dfloat df_neg(dfloat a) { return df_make(-a.hi, -a.lo); }
DF_HD dfloat df_sub(dfloat a, dfloat b) { return df_add(a, df_neg(b)); }

DF_HD dfloat df_mul(dfloat a, dfloat b) {
    dfloat p = two_prod(a.hi, b.hi);
    p.lo = df_fma(a.hi, b.lo, p.lo);
    p.lo = df_fma(a.lo, b.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
DF_HD dfloat df_mul(dfloat a, float b) {
    dfloat p = two_prod(a.hi, b);
    p.lo = df_fma(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
// a * b + c
DF_HD dfloat df_fma(dfloat a, dfloat b, dfloat c) { return df_add(df_mul(a, b), c); }

// a / b: quotient estimate from the float quotient, one df correction step.
DF_HD dfloat df_div(dfloat a, dfloat b) {
    const float q1 = a.hi / b.hi;
    const dfloat r = df_sub(a, df_mul(b, q1));
    const float q2 = r.hi / b.hi;
    return fast_two_sum(q1, q2);
}
DF_HD dfloat df_recip(dfloat b) { return df_div(df_from_float(1.f), b); }

// sqrt(a), a > 0: float root, one df Newton correction (Karp & Markstein form).
DF_HD dfloat df_sqrt(dfloat a) {
    const float x = sqrtf(a.hi);
    const dfloat x2 = two_prod(x, x);
    const dfloat r = df_sub(a, x2);
    return fast_two_sum(x, r.hi / (2.f * x));
}

// exp(-s) for s >= 0 (s <= 80): s = k ln2 + t with |t| <= ln2/2 (Cody-Waite split of
// ln2), exp(-t) by its Taylor series to t^13 in Horner form, scaled by 2^-k.
DF_HD dfloat df_exp_neg(dfloat s) {
    // ln2 = L1 + L2 + L3 with L1, L2 of 16 significant bits, so k * L1 and k * L2 are
    // exact for |k| < 2^7 (s <= 80)
    const float kLn2a = 0.693145751953125f;
    const float kLn2b = 1.4286197256296873e-06f;
    const float kLn2c = -1.2905320041778356e-11f;
    const float k = rintf(s.hi * 1.44269502f);
    dfloat t = df_add(s, df_rmul(-k, kLn2a));
    t = df_add(t, df_rmul(-k, kLn2b));
    t = df_add(t, df_rmul(-k, kLn2c));
    const dfloat mt = df_neg(t);
    // coefficients 1/n! as df (n = 13 .. 0)
    const float cHi[14] = {1.605904437e-10f, 2.087675588e-09f, 2.505210794e-08f, 2.755731998e-07f, 2.755731884e-06f,
                           2.480158764e-05f, 1.984127011e-04f, 1.388888923e-03f, 8.333333768e-03f, 4.166666791e-02f,
                           1.666666716e-01f, 5.000000000e-01f, 1.000000000e+00f, 1.000000000e+00f};
    const float cLo[14] = {-5.352526512e-18f, 1.108283915e-16f, 4.417623045e-16f, -7.575112209e-15f, 3.793571224e-14f,
                           -3.406996094e-13f, -2.725596875e-12f, -3.363109444e-11f, -4.346172033e-10f, -1.241763470e-09f,
                           -4.967053879e-09f, 0.0f, 0.0f, 0.0f};
    dfloat acc = df_make(cHi[0], cLo[0]);
#pragma unroll
    for (int n = 1; n < 14; ++n) acc = df_add(df_mul(acc, mt), df_make(cHi[n], cLo[n]));
    const float sc = ldexpf(1.f, -(int) k);
    return df_make(acc.hi * sc, acc.lo * sc);
}

// Two functions tabulated as degree-D polynomials in u = r - centre[k] on K equal
// intervals from r0 (coef layout [K][D+1][f1 hi, f1 lo, f2 hi, f2 lo], lowest power
// first; see radial_tables.h).  The interval comes from r.hi.
template <int D>
DF_HD void df_table_eval(const float* __restrict__ coef, const float* __restrict__ centre, float r0, float invh, int K,
                         dfloat r, dfloat& f1, dfloat& f2) {
    int k = (int) floorf((r.hi - r0) * invh);
    k = k < 0 ? 0 : (k >= K ? K - 1 : k);
    const dfloat u = df_add(r, -centre[k]);
    const float* c = coef + (size_t) k * (D + 1) * 4;
    f1 = df_make(c[4 * D], c[4 * D + 1]);
    f2 = df_make(c[4 * D + 2], c[4 * D + 3]);
#pragma unroll
    for (int p = D - 1; p >= 0; --p) {
        f1 = df_add(df_mul(f1, u), df_make(c[4 * p], c[4 * p + 1]));
        f2 = df_add(df_mul(f2, u), df_make(c[4 * p + 2], c[4 * p + 3]));
    }
}

}  // namespace mpid
