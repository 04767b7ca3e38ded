// Tabulated Ewald radial functions for the double-float (df) residual field.
//
// The induced-induced kernel K_u = phi_T - erf(alpha r)/r needs b_1 and b_2 of its
// Ewald part.  Over the erfc segment of the neighbour lists (alpha r >= 1.5) the table
// holds G_n(r) = r^(2n+1) b_n[erfc(alpha r)/r]; over the quadrature segment (r below
// 1.5/alpha) it holds H_n(r) = b_n[erf(alpha r)/r].  Both are smooth and bounded on their
// ranges.  Each range is cut into K equal intervals and each function is a degree-D
// polynomial in u = r - c_k about the interval centre c_k (a float), with df
// coefficients from Chebyshev interpolation at D+1 nodes.  Reference values come from
// long double (erfcl and the power series of F_n), the coefficients from long double
// arithmetic.  With K = 32 and D = 7 the df evaluation is accurate to ~1e-14 relative
// (checked against long double by df_check.cpp, run from tests/test_cpu_host.py).
#pragma once
#include <cmath>
#include <vector>

namespace mpid {

struct RadialTableHost {
    int K = 0, D = 0;
    float r0 = 0.f, h = 0.f, invh = 0.f;
    std::vector<float> centre;   // [K]
    std::vector<float> coef;     // [K][D+1][4]: (f1 hi, f1 lo, f2 hi, f2 lo), lowest power first
};

namespace radial_detail {

typedef long double ld;

inline ld sqrt_pi() { return std::sqrt(std::acos((ld) -1)); }

// b_1, b_2 of erfc(alpha r)/r times r^3, r^5 (upward recursion, all terms positive)
inline void erfc_parts(ld r, ld alpha, ld* G) {
    const ld x = alpha * r;
    const ld ex = std::exp(-x * x);
    const ld rinv2 = 1 / (r * r);
    ld b0 = std::erfc(x) / r;
    ld c = 2 * alpha / sqrt_pi() * ex;
    const ld b1 = (b0 + c) * rinv2;
    c *= 2 * alpha * alpha;
    const ld b2 = (3 * b1 + c) * rinv2;
    G[0] = b1 * r * r * r;
    G[1] = b2 * r * r * r * r * r;
}

// b_1, b_2 of erf(alpha r)/r: 2^(n+1) alpha^(2n+1)/sqrt(pi) F_n(alpha r),
// F_n(x) = sum_k (-x^2)^k / (k! (2n + 2k + 1)).
inline void erf_parts(ld r, ld alpha, ld* H) {
    const ld x2 = alpha * r * alpha * r;
    for (int n = 1; n <= 2; ++n) {
        ld term = 1, sum = 0;
        for (int k = 0; k < 200; ++k) {
            const ld add = term / (2 * n + 2 * k + 1);
            sum += add;
            if (std::fabs(add) < 1e-30L * std::fabs(sum) && k > 4) break;
            term *= -x2 / (k + 1);
        }
        H[n - 1] = std::pow((ld) 2, n + 1) * std::pow(alpha, 2 * n + 1) / sqrt_pi() * sum;
    }
}

}  // namespace radial_detail

// Build the table of f(r) = (f1, f2) on [ra, rb] (both functions from `eval`).
template <typename Eval>
RadialTableHost build_radial_table(double ra, double rb, int K, int D, Eval eval) {
    using radial_detail::ld;
    RadialTableHost t;
    t.K = K;
    t.D = D;
    t.r0 = (float) ra;
    t.h = (float) ((rb - (double) t.r0) / K);
    t.invh = 1.f / t.h;
    t.centre.resize(K);
    t.coef.assign((size_t) K * (D + 1) * 4, 0.f);
    const ld pi = std::acos((ld) -1);
    for (int k = 0; k < K; ++k) {
        const float c = t.r0 + ((float) k + 0.5f) * t.h;
        t.centre[k] = c;
        const ld half = (ld) t.h * 0.5L * 1.02L;  // fit slightly beyond the interval
        // Chebyshev interpolation in t in [-1, 1], r = c + half t
        std::vector<ld> nodes(D + 1), fv[2] = {std::vector<ld>(D + 1), std::vector<ld>(D + 1)};
        for (int j = 0; j <= D; ++j) {
            nodes[j] = std::cos(pi * (j + 0.5L) / (D + 1));
            ld f[2];
            eval((ld) c + half * nodes[j], f);
            fv[0][j] = f[0];
            fv[1][j] = f[1];
        }
        for (int fn = 0; fn < 2; ++fn) {
            // Chebyshev coefficients a_m
            std::vector<ld> a(D + 1, 0);
            for (int m = 0; m <= D; ++m) {
                ld s = 0;
                for (int j = 0; j <= D; ++j) s += fv[fn][j] * std::cos(pi * m * (j + 0.5L) / (D + 1));
                a[m] = s * 2 / (D + 1);
            }
            a[0] *= 0.5L;
            // Chebyshev -> monomials in t: T_0 = 1, T_1 = t, T_m = 2 t T_(m-1) - T_(m-2)
            std::vector<ld> mono(D + 1, 0), Tm2(D + 1, 0), Tm1(D + 1, 0), Tm(D + 1, 0);
            Tm2[0] = 1;
            if (D >= 1) Tm1[1] = 1;
            for (int p = 0; p <= D; ++p) mono[p] += a[0] * Tm2[p];
            if (D >= 1)
                for (int p = 0; p <= D; ++p) mono[p] += a[1] * Tm1[p];
            for (int m = 2; m <= D; ++m) {
                for (int p = 0; p <= D; ++p) Tm[p] = (p > 0 ? 2 * Tm1[p - 1] : 0) - Tm2[p];
                for (int p = 0; p <= D; ++p) mono[p] += a[m] * Tm[p];
                Tm2 = Tm1;
                Tm1 = Tm;
            }
            // monomials in u = r - c: coefficient of u^p is mono[p] / half^p
            ld scale = 1;
            for (int p = 0; p <= D; ++p) {
                const ld v = mono[p] * scale;
                const float hi = (float) v;
                const float lo = (float) (v - (ld) hi);
                t.coef[((size_t) k * (D + 1) + p) * 4 + 2 * fn] = hi;
                t.coef[((size_t) k * (D + 1) + p) * 4 + 2 * fn + 1] = lo;
                scale /= half;
            }
        }
    }
    return t;
}

// Tables of the erfc segment [rq, rL] (G_1, G_2) and the quadrature segment [0, rq]
// (H_1, H_2) for Ewald parameter alpha.
inline void build_ewald_tables(double alpha, double rq, double rL, int K, int D, RadialTableHost& G,
                               RadialTableHost& H) {
    using radial_detail::ld;
    G = build_radial_table(rq, rL, K, D, [alpha](ld r, ld* f) { radial_detail::erfc_parts(r, (ld) alpha, f); });
    H = build_radial_table(0.0, rq, K, D, [alpha](ld r, ld* f) { radial_detail::erf_parts(r, (ld) alpha, f); });
}

}  // namespace mpid
