// Radial functions of the FP32 pair kernel of the mutual solver's CG iterations, as
// polynomials fitted on the host for the context's Ewald parameter.
//
// The kernel K_u = phi_T - erf(alpha r)/r (induced-induced, MPIDReferenceForce.cpp:
// 4161-4281) needs b_1 and b_2.  Over the erfc segment of the neighbour lists
// (x = alpha r >= xq) its Ewald part is written through erfcx(x) = erfc(x) exp(x^2),
// which is smooth and slowly varying there:
//   r^3 b_1[erfc(alpha r)/r] = exp(-x^2) (erfcx(x) + 2 x / sqrt(pi))
//   r^5 b_2[erfc(alpha r)/r] = exp(-x^2) (3 erfcx(x) + 2 (3 x + 2 x^3) / sqrt(pi)),
// so a pair costs one exponential and one polynomial instead of erfc, a second
// exponential and two divisions.  Over the near segment (x < xq) the erf part is
//   b_n[erf(alpha r)/r] = 2^(n+1) alpha^(2n+1) / sqrt(pi) F_n(x^2),
// F_n(T) = int_0^1 v^(2n) exp(-T v^2) dv, with F_1 and F_2 as polynomials in T.
// Each polynomial interpolates its function at the Chebyshev nodes of the interval
// (degree kCgDeg, long double), re-expanded in powers of t in [-1, 1]; evaluated in FP32
// the result is within ~2e-7 relative of the function (the Horner rounding), checked
// against long double by tests/native/cg_radial_check.cpp.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

namespace mpid {

constexpr int kCgDeg = 8;

struct CgRadial {
    float xs, xo;                          // erfc segment: t = x xs + xo, x = alpha r in [xq, xL]
    float erfcx[kCgDeg + 1];               // erfc(x) exp(x^2) in powers of t, lowest first
    float Ts, To;                          // near segment: t = T Ts + To, T = (alpha r)^2 in [0, xq^2]
    float F1[kCgDeg + 1], F2[kCgDeg + 1];  // F_1(T), F_2(T) in powers of t
    float xq2;                             // xq^2: near-segment pairs beyond it (far covalent partners)
                                           // take the erfc-segment form
    float twoRtPi;                         // 2 / sqrt(pi)
    float h1, h2;                          // 4 alpha^3 / sqrt(pi), 8 alpha^5 / sqrt(pi)
    int usePme;                            // 0: no Ewald part (bare Thole-damped kernel)
};

namespace cg_detail {

typedef long double ld;

inline ld boys(int n, ld T) {  // sum_k (-T)^k / (k! (2n + 2k + 1)), T <= a few
    ld term = 1, sum = 0;
    for (int k = 0; k < 200; ++k) {
        const ld add = term / (2 * n + 2 * k + 1);
        sum += add;
        if (std::fabs(add) < 1e-30L * std::fabs(sum) && k > 4) break;
        term *= -T / (k + 1);
    }
    return sum;
}

// Coefficients (powers of t, lowest first) of the degree-D interpolant of f on [a, b] at
// the Chebyshev nodes, t = (2 y - (a + b)) / (b - a).
template <typename F>
inline void fit(F f, ld a, ld b, float* out) {
    const int D = kCgDeg;
    const ld pi = std::acos((ld) -1);
    std::vector<ld> fv(D + 1), c(D + 1, 0), mono(D + 1, 0), Tm2(D + 1, 0), Tm1(D + 1, 0), Tm(D + 1, 0);
    for (int j = 0; j <= D; ++j) fv[j] = f((a + b) / 2 + (b - a) / 2 * std::cos(pi * (j + 0.5L) / (D + 1)));
    for (int m = 0; m <= D; ++m) {
        ld s = 0;
        for (int j = 0; j <= D; ++j) s += fv[j] * std::cos(pi * m * (j + 0.5L) / (D + 1));
        c[m] = s * 2 / (D + 1);
    }
    c[0] *= 0.5L;
    // Chebyshev -> monomials: T_0 = 1, T_1 = t, T_m = 2 t T_(m-1) - T_(m-2)
    Tm2[0] = 1;
    Tm1[1] = 1;
    for (int p = 0; p <= D; ++p) mono[p] += c[0] * Tm2[p] + c[1] * Tm1[p];
    for (int m = 2; m <= D; ++m) {
        for (int p = 0; p <= D; ++p) Tm[p] = (p > 0 ? 2 * Tm1[p - 1] : 0) - Tm2[p];
        for (int p = 0; p <= D; ++p) mono[p] += c[m] * Tm[p];
        Tm2 = Tm1;
        Tm1 = Tm;
    }
    for (int p = 0; p <= D; ++p) out[p] = (float) mono[p];
}

}  // namespace cg_detail

#if defined(__CUDACC__)
#define CG_HD __host__ __device__ __forceinline__
#else
#define CG_HD inline
#endif

constexpr double cg_inv_factorial(int k) { return k <= 1 ? 1.0 : cg_inv_factorial(k - 1) / k; }
template <int K>
struct CgInvFactorial {
    static constexpr float v = (float) cg_inv_factorial(K);
};
// sum_{j=0}^{J} s^j / (j + OFF)! by Horner with compile-time coefficients
template <int OFF, int J, int j>
struct CgSeries {
    static CG_HD float eval(float s) { return fmaf(CgSeries<OFF, J, j + 1>::eval(s), s, CgInvFactorial<j + OFF>::v); }
};
template <int OFF, int J>
struct CgSeries<OFF, J, J> {
    static CG_HD float eval(float) { return CgInvFactorial<J + OFF>::v; }
};

CG_HD float cg_poly(const float* c, float t) {
    float p = c[kCgDeg];
#pragma unroll
    for (int k = kCgDeg - 1; k >= 0; --k) p = fmaf(p, t, c[k]);
    return p;
}

CG_HD float cg_rsqrt(float v) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(v);
#else
    return 1.f / std::sqrt(v);
#endif
}

// b_1, b_2 of K_u for one pair at squared distance r2 with Thole width a and inverse
// damping product invdd (1 / (d_i d_j)); ahi + alo = alpha.  NEAR: the pair is in the near
// segment of the lists, where 1/r comes from an IEEE square root and division (its powers
// up to 1/r^5 weigh most there); the erfc segment uses rsqrt and one Newton step.  A
// near-segment pair beyond the near range (a covalent-scale-0 partner) takes the erfc
// form.  Returns false-free: every argument gives finite values for r2 > 0.
template <bool NEAR>
CG_HD void cg_pair_radial(const CgRadial& R, float r2, float a, float invdd, float ahi, float alo, float& b1,
                          float& b2) {
    float r, ri;
    if (NEAR) {
        r = std::sqrt(r2);
        ri = 1.f / r;
    } else {
        ri = cg_rsqrt(r2);
        ri = ri * fmaf(-0.5f * r2 * ri, ri, 1.5f);  // one Newton step
        r = r2 * ri;
    }
    const float ri2 = ri * ri, ri3 = ri * ri2, ri5 = ri3 * ri2;
    const float s = fminf(a * r * invdd, 100.f);
    const float x = fmaf(ahi, r, alo * r);
    const float es = expf(-s);
    const float P1 = fmaf(s, fmaf(s, 0.5f, 1.f), 1.f);
    if (!NEAR || x * x >= R.xq2) {
        const float P2 = fmaf(s * s * s, 1.f / 6.f, P1);
        float g1 = 1.f, g2 = 3.f, ex = 1.f;  // bare kernel without PME
        if (R.usePme) {
            const float x2 = x * x, x2l = fmaf(x, x, -x2);
            ex = expf(-x2) * (1.f - x2l);
            const float ec = cg_poly(R.erfcx, fmaf(x, R.xs, R.xo));
            g1 = fmaf(R.twoRtPi, x, ec);
            g2 = fmaf(3.f, ec, R.twoRtPi * x * fmaf(2.f, x2, 3.f));
        }
        b1 = fmaf(ex, g1, -es * P1) * ri3;
        b2 = fmaf(ex, g2, -3.f * es * P2) * ri5;
    } else {
        // lambda_n bB_n - b_n[erf(alpha r)/r]; lambda from its series for s < 4 (no
        // cancellation), else 1 - e^-s P_n(s)
        const float tt = fmaf(x * x, R.Ts, R.To);
        const float H1 = R.h1 * cg_poly(R.F1, tt), H2 = R.h2 * cg_poly(R.F2, tt);
        float l1, l2;
        if (s < 4.f) {
            const float s3 = s * s * s;
            l1 = es * s3 * CgSeries<3, 17, 0>::eval(s);
            l2 = es * s3 * s * CgSeries<4, 17, 0>::eval(s);
        } else {
            l1 = fmaf(-es, P1, 1.f);
            l2 = fmaf(-es, fmaf(s * s * s, 1.f / 6.f, P1), 1.f);
        }
        b1 = fmaf(l1, ri3, -H1);
        b2 = fmaf(3.f * l2, ri5, -H2);
    }
}

// alpha: Ewald parameter (0 without PME); xq: alpha r at the near/erfc segment boundary;
// rL: the neighbour-list cutoff (the erfc segment ends at alpha rL).
inline CgRadial build_cg_radial(double alpha, double xq, double rL) {
    using cg_detail::ld;
    CgRadial R{};
    R.usePme = alpha > 0 ? 1 : 0;
    const ld sqrtpi = std::sqrt(std::acos((ld) -1));
    R.twoRtPi = (float) (2 / sqrtpi);
    const ld al = alpha;
    R.h1 = (float) (4 * al * al * al / sqrtpi);
    R.h2 = (float) (8 * al * al * al * al * al / sqrtpi);
    R.xq2 = (float) (xq * xq);
    const ld xa = xq, xb = std::max((ld) (alpha * rL), xa + 0.5L);
    R.xs = (float) (2 / (xb - xa));
    R.xo = (float) (-(xa + xb) / (xb - xa));
    cg_detail::fit([](ld x) { return std::erfc(x) * std::exp(x * x); }, xa, xb, R.erfcx);
    const ld Tb = (ld) xq * xq;
    R.Ts = (float) (2 / Tb);
    R.To = -1.f;
    cg_detail::fit([](ld T) { return cg_detail::boys(1, T); }, 0, Tb, R.F1);
    cg_detail::fit([](ld T) { return cg_detail::boys(2, T); }, 0, Tb, R.F2);
    return R;
}

}  // namespace mpid
