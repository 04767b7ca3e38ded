// Per-atom and per-pair mathematics of the MPIDForce evaluation, templated on the
// arithmetic type (float for the mixed-precision path, double for the FP64 path).
// Everything here is __host__ __device__ and free of memory-layout decisions; the
// kernels in mpid_kernels.cu wrap these functions.
//
// Conventions (units nm, e, kJ/mol; electric constant applied by the caller):
//  * quadrupole components  XX XY XZ YY YZ ZZ   (lab frame, "Q6")
//  * octopole components    XXX XXY XXZ XYY XYZ XZZ YYY YYZ YZZ ZZZ ("O10")
//  * potential of a source multipole at field point x (s = x - source):
//        phi = q K - mu.grad K + Theta:grad grad K - Omega:grad^3 K
//    for a radial kernel K(r); derivatives are expressed through
//        b_n = (-1)^n ((1/r) d/dr)^n K,   bare 1/r:  b_n = (2n-1)!!/r^(2n+1).
//    (this is the convention of MPIDReferenceForce.cpp:839-898 and :2812-2920).
#pragma once
#include <math.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif
#define MPID_HD __host__ __device__ __forceinline__

#include "qi_tables.cuh"

namespace mpid {

// Ewald self-term constant sqrt(pi) as the reference uses it (MPIDReferenceForce.cpp:2541).
constexpr double kSqrtPiRef = 1.77245385091;
constexpr double kSqrtPi = 1.7724538509055160273;

template <typename real> struct Prec;
template <> struct Prec<float> {
    // Below this alpha*r the erf part of the kernels comes from the Boys function series
    // (the erfc recursion above it).
    static constexpr float kQuadX = 1.5f;
    static constexpr int kBoysTerms = 16;   // series truncation < 3e-11 relative at (alpha r)^2 <= 2.25
};
template <> struct Prec<double> {
    static constexpr double kQuadX = 1.5;
    static constexpr int kBoysTerms = 26;   // < 1e-16
};

MPID_HD float m_exp(float x) { return expf(x); }
MPID_HD double m_exp(double x) { return exp(x); }
MPID_HD float m_sqrt(float x) { return sqrtf(x); }
MPID_HD double m_sqrt(double x) { return sqrt(x); }
MPID_HD float m_erfc(float x) { return erfcf(x); }
MPID_HD double m_erfc(double x) { return erfc(x); }
MPID_HD float m_fabs(float x) { return fabsf(x); }
MPID_HD double m_fabs(double x) { return fabs(x); }
MPID_HD float m_copysign(float a, float b) { return copysignf(a, b); }
MPID_HD double m_copysign(double a, double b) { return copysign(a, b); }
// a * b + c with one rounding (keeps the low parts of split constants effective)
MPID_HD float m_fma(float a, float b, float c) { return fmaf(a, b, c); }
MPID_HD double m_fma(double a, double b, double c) { return fma(a, b, c); }

// ---------------------------------------------------------------------------
// Ewald parameter split so that products with alpha are formed without rounding alpha
// itself: alpha = hi + lo with hi = real(alpha).  Rounding alpha once would bias every
// erfc(alpha r) the same way (by up to ~13x its relative error near alpha r = 2.5).
template <typename real>
struct EwaldAlpha {
    real hi, lo;        // alpha
    real pre_hi, pre_lo;  // 2 alpha / sqrt(pi)
    real a2x2, a2x2_lo;   // 2 alpha^2
    MPID_HD EwaldAlpha() : hi(0), lo(0), pre_hi(0), pre_lo(0), a2x2(0), a2x2_lo(0) {}
    MPID_HD explicit EwaldAlpha(double a) {
        hi = real(a);
        lo = real(a - double(hi));
        const double p = 2.0 / kSqrtPi * a;
        pre_hi = real(p);
        pre_lo = real(p - double(pre_hi));
        a2x2 = real(2.0 * a * a);
        a2x2_lo = real(2.0 * a * a - double(a2x2));
    }
    MPID_HD real times(real r) const { return m_fma(hi, r, lo * r); }
    // v * 2 alpha^2 without the rounding of 2 alpha^2
    MPID_HD real times_a2x2(real v) const { return m_fma(a2x2, v, a2x2_lo * v); }
    // v * 2 alpha / sqrt(pi) without the rounding of the constant
    MPID_HD real times_pre(real v) const { return m_fma(pre_hi, v, pre_lo * v); }
};

// 1/m as an unevaluated sum hi + lo of the arithmetic type (so that products with it
// carry no systematic rounding of the constant).
template <typename real>
struct InvOdd {
    real hi, lo;
    MPID_HD explicit InvOdd(int m) {
        const double v = 1.0 / (double) m;
        hi = real(v);
        lo = real(v - (double) hi);
    }
    MPID_HD real times(real x) const { return m_fma(hi, x, lo * x); }
};

// b_n (n = 0..NMAX) of erf(alpha r)/r through the Boys function
//   F_n(T) = int_0^1 v^(2n) exp(-T v^2) dv,  T = (alpha r)^2:
//   b_n = 2^(n+1) alpha^(2n+1) / sqrt(pi) F_n(T).
// F_NMAX from the series exp(-T) sum_k (2T)^k / ((2N+1)(2N+3)...(2N+2k+1)), whose terms
// are all positive; lower orders by the stable downward recursion
//   F_(n-1) = (2T F_n + exp(-T)) / (2n - 1).
// No cancellation and no deterministic quadrature error (used for alpha r < 1.5, where
// the series has converged to the working precision after Prec::kBoysTerms terms).
template <typename real, int NMAX>
MPID_HD void erf_part_boys(real r, const EwaldAlpha<real>& al, real* bF) {
    constexpr int K = Prec<real>::kBoysTerms;
    const real x = al.times(r);
    const real T = x * x, twoT = T + T;
    const real ex = m_exp(-T);
    real term = InvOdd<real>(2 * NMAX + 1).times(real(1));
    real sum = term;
#pragma unroll
    for (int k = 1; k < K; ++k) {
        term = InvOdd<real>(2 * NMAX + 2 * k + 1).times(term * twoT);
        sum += term;
    }
    real F[NMAX + 1];
    F[NMAX] = ex * sum;
#pragma unroll
    for (int n = NMAX; n >= 1; --n) F[n - 1] = InvOdd<real>(2 * n - 1).times(twoT * F[n] + ex);
    // prefactor 2^(n+1) alpha^(2n+1) / sqrt(pi): (2 alpha / sqrt(pi)) (2 alpha^2)^n
    real scale = real(1);
#pragma unroll
    for (int n = 0; n <= NMAX; ++n) {
        bF[n] = al.times_pre(F[n]) * scale;
        scale = al.times_a2x2(scale);
    }
}

// b_n of erfc(alpha r)/r by upward recursion (all terms positive).
template <typename real, int NMAX>
MPID_HD void erfc_part(real r, real rinv2, const EwaldAlpha<real>& al, real* bE) {
    const real ar = al.times(r);
    const real ex = m_exp(-ar * ar);
    bE[0] = m_erfc(ar) / r;
    // c_n = (2 alpha^2)^n / (alpha sqrt(pi)) * exp(-alpha^2 r^2), starting at n = 1
    real c = al.times_pre(ex);
#pragma unroll
    for (int n = 1; n <= NMAX; ++n) {
        bE[n] = (real(2 * n - 1) * bE[n - 1] + c) * rinv2;
        c = al.times_a2x2(c);
    }
}

// b_n of the bare kernel 1/r.
template <typename real, int NMAX>
MPID_HD void bare_part(real rinv, real rinv2, real* bB) {
    bB[0] = rinv;
#pragma unroll
    for (int n = 1; n <= NMAX; ++n) bB[n] = real(2 * n - 1) * bB[n - 1] * rinv2;
}

// Thole screening of the MPID damped potential, phi_T = (1 - (1 + s/2) e^-s) / r with
// s = a r / (d_i d_j) (MPIDReferenceForce.cpp:818-833, :2678-2718, :4509-4523):
//   b_n[phi_T] = lambda_(2n+1)(s) b_n[1/r],  lambda = 1 - e^-s P_n(s).
// Returns lam[n] for n = 1..NMAX (lam[0] unused) and oneMinus[n] = e^-s P_n(s).
// For s < 4 lambda is summed as e^-s * sum_k (1/k! - p_k) s^k, which has no
// cancellation; larger s uses 1 - e^-s P_n(s).
template <typename real, int NMAX>
MPID_HD void thole_lambdas(real s, real* lam, real* oneMinus) {
    // Coefficients p_{n,k} of P_n (k = 0..7) for n = 1..6.
    const double P[7][8] = {
        {1, 0.5, 0, 0, 0, 0, 0, 0},
        {1, 1, 0.5, 0, 0, 0, 0, 0},
        {1, 1, 0.5, 1.0 / 6, 0, 0, 0, 0},
        {1, 1, 0.5, 1.0 / 6, 1.0 / 30, 0, 0, 0},
        {1, 1, 0.5, 1.0 / 6, 4.0 / 105, 1.0 / 210, 0, 0},
        {1, 1, 0.5, 1.0 / 6, 5.0 / 126, 2.0 / 315, 1.0 / 1890, 0},
        {1, 1, 0.5, 1.0 / 6, 4.0 / 99, 7.0 / 990, 17.0 / 20790, 1.0 / 20790},
    };
    const double invfact[8] = {1, 1, 0.5, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040};
    const real es = m_exp(-s);
    if (s < real(4)) {
        // tail T = sum_{k>=8} s^k/k!, by Horner on s^8/8! (1 + s/9 (1 + s/10 (...)))
        real tail = real(1);
#pragma unroll
        for (int k = 24; k >= 9; --k) tail = real(1) + s * tail / real(k);
        real s2 = s * s, s4 = s2 * s2;
        tail *= s4 * s4 * real(1.0 / 40320.0);
#pragma unroll
        for (int n = 1; n <= NMAX; ++n) {
            real acc = tail;
            real sk = real(1);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const double d = invfact[k] - P[n][k];
                if (d != 0.0) acc += real(d) * sk;
                sk *= s;
            }
            lam[n] = es * acc;
            oneMinus[n] = real(1) - lam[n];
        }
    } else {
#pragma unroll
        for (int n = 1; n <= NMAX; ++n) {
            real p = real(P[n][7]);
#pragma unroll
            for (int k = 6; k >= 0; --k) p = p * s + real(P[n][k]);
            oneMinus[n] = es * p;
            lam[n] = real(1) - oneMinus[n];
        }
    }
}

// d lambda_(2n+1) / ds = e^-s (P_n(s) - P_n'(s)) for n = 1..NMAX (dl[0] unused), the
// screening derivative of the polarisability and Thole-width gradients.  Every
// coefficient of P_n - P_n' is >= 0, so the sum has no cancellation.
template <typename real, int NMAX>
MPID_HD void thole_lambda_derivs(real s, real* dl) {
    const double P[7][8] = {
        {1, 0.5, 0, 0, 0, 0, 0, 0},
        {1, 1, 0.5, 0, 0, 0, 0, 0},
        {1, 1, 0.5, 1.0 / 6, 0, 0, 0, 0},
        {1, 1, 0.5, 1.0 / 6, 1.0 / 30, 0, 0, 0},
        {1, 1, 0.5, 1.0 / 6, 4.0 / 105, 1.0 / 210, 0, 0},
        {1, 1, 0.5, 1.0 / 6, 5.0 / 126, 2.0 / 315, 1.0 / 1890, 0},
        {1, 1, 0.5, 1.0 / 6, 4.0 / 99, 7.0 / 990, 17.0 / 20790, 1.0 / 20790},
    };
    const real es = m_exp(-s);
#pragma unroll
    for (int n = 1; n <= NMAX; ++n) {
        real p = real(P[n][7]);
#pragma unroll
        for (int k = 6; k >= 0; --k) p = p * s + real(P[n][k] - (k + 1) * P[n][k + 1]);
        dl[n] = es * p;
    }
}

// Radial functions of one pair for the three kernels of the model:
//   perm     K_p = (s - erf(alpha r)) / r                 permanent-permanent
//   ind      K_i = s phi_T - erf(alpha r)/r               permanent-induced, fields
//   uu       K_u = phi_T - erf(alpha r)/r                 induced-induced
// where s is the covalent scale of the pair (the m- and p-scales of the reference are
// always equal, MPIDReferenceForce.cpp:190-225) and the Thole width is a_i + a_j for
// s == 0, else the default width.  Each array b[n] is filled for n = 0..NMAX.
template <typename real, int NP, int NI, int NU>
struct PairRadial {
    real bP[NP + 1];
    real bI[NI + 1];
    real bU[NU + 1];
};

// Compute the requested radial arrays.  NP/NI/NU < 0 disables a kernel.  QUAD selects
// the branch at compile time (the name of the lists' near segment): true takes the erf
// part from the Boys-function series (needed where erf(alpha r)/r must not be formed as
// a difference: alpha r below the threshold, or covalent scale 0), false uses the erfc
// recursion.  pair_radial picks by alpha r.
template <typename real, int NP, int NI, int NU, bool QUAD>
MPID_HD void pair_radial_branch(real r, const EwaldAlpha<real>& alpha, real scale, real tholeA, real dampProd,
                                PairRadial<real, (NP > 0 ? NP : 0), (NI > 0 ? NI : 0), (NU > 0 ? NU : 0)>& out) {
    constexpr int NMAX = (NP > NI ? (NP > NU ? NP : NU) : (NI > NU ? NI : NU));
    const real rinv = real(1) / r;
    const real rinv2 = rinv * rinv;
    real bB[NMAX + 1];
    bare_part<real, NMAX>(rinv, rinv2, bB);
    // Thole factors (only needed for ind/uu).
    constexpr int NT = (NI > NU ? NI : NU);
    real lam[(NT > 0 ? NT : 0) + 1], oneMinus[(NT > 0 ? NT : 0) + 1];
    if (NT > 0) {
        bool undamped = !(dampProd > real(0));
        real sT = undamped ? real(0) : tholeA * r / dampProd;
        if (undamped || sT >= real(50)) {
#pragma unroll
            for (int n = 0; n <= NT; ++n) { lam[n] = real(1); oneMinus[n] = real(0); }
        } else {
            thole_lambdas<real, NT>(sT, lam, oneMinus);
        }
    }
    if (QUAD) {
        real bF[NMAX + 1];
        erf_part_boys<real, NMAX>(r, alpha, bF);
        if (NP >= 0) {
            // K_p = (s - erf)/r: for s = 1 it is erfc(alpha r)/r, whose upward recursion has
            // no cancellation, while 1/r - erf(alpha r)/r would amplify the relative error
            // of the erf part by erf/erfc (up to ~30 near the branch threshold)
            constexpr int NPP = NP > 0 ? NP : 0;
            if (scale == real(1)) {
                real bE[NMAX + 1];
                erfc_part<real, NMAX>(r, rinv2, alpha, bE);
#pragma unroll
                for (int n = 0; n <= NPP; ++n) out.bP[n] = bE[n];
            } else {
#pragma unroll
                for (int n = 0; n <= NPP; ++n) out.bP[n] = scale * bB[n] - bF[n];
            }
        }
        if (NI > 0) {
#pragma unroll
            for (int n = 1; n <= NI; ++n) out.bI[n] = scale * lam[n] * bB[n] - bF[n];
        }
        if (NU > 0) {
#pragma unroll
            for (int n = 1; n <= NU; ++n) out.bU[n] = lam[n] * bB[n] - bF[n];
        }
    } else {
        real bE[NMAX + 1];
        erfc_part<real, NMAX>(r, rinv2, alpha, bE);
        if (NP >= 0) {
            const real oneMinusS = real(1) - scale;
#pragma unroll
            for (int n = 0; n <= (NP > 0 ? NP : 0); ++n) out.bP[n] = bE[n] - oneMinusS * bB[n];
        }
        if (NI > 0) {
            const real oneMinusS = real(1) - scale;
#pragma unroll
            for (int n = 1; n <= NI; ++n) out.bI[n] = bE[n] - (oneMinusS + scale * oneMinus[n]) * bB[n];
        }
        if (NU > 0) {
#pragma unroll
            for (int n = 1; n <= NU; ++n) out.bU[n] = bE[n] - oneMinus[n] * bB[n];
        }
    }
}

// True where the quadrature branch is required: alpha r below the threshold, or a
// covalent scale of 0 (the kernel is then -erf(alpha r)/r at any distance).
template <typename real>
MPID_HD bool radial_needs_quadrature(real r, const EwaldAlpha<real>& alpha, real scale) {
    return alpha.times(r) < real(Prec<real>::kQuadX) || scale == real(0);
}

template <typename real, int NP, int NI, int NU>
MPID_HD void pair_radial(real r, const EwaldAlpha<real>& alpha, real scale, real tholeA, real dampProd,
                         PairRadial<real, (NP > 0 ? NP : 0), (NI > 0 ? NI : 0), (NU > 0 ? NU : 0)>& out) {
    if (alpha.times(r) < real(Prec<real>::kQuadX))
        pair_radial_branch<real, NP, NI, NU, true>(r, alpha, scale, tholeA, dampProd, out);
    else
        pair_radial_branch<real, NP, NI, NU, false>(r, alpha, scale, tholeA, dampProd, out);
}

// ---------------------------------------------------------------------------
// Lab-frame moments of one atom as needed by the pair kernels.
template <typename real>
struct LabMoments {
    real q;
    real d[3];      // dipole x y z
    real Q[6];      // XX XY XZ YY YZ ZZ
    real O[10];     // XXX XXY XXZ XYY XYZ XZZ YYY YYZ YZZ ZZZ
};

// Index of a symmetric Cartesian component in the Q6 / O10 layouts.
MPID_HD int q6(int i, int j) {
    if (i > j) { int t = i; i = j; j = t; }
    // (0,0)0 (0,1)1 (0,2)2 (1,1)3 (1,2)4 (2,2)5
    return i == 0 ? j : (i == 1 ? 2 + j : 5);
}
MPID_HD int o10(int i, int j, int k) {
    // sort
    if (i > j) { int t = i; i = j; j = t; }
    if (j > k) { int t = j; j = k; k = t; }
    if (i > j) { int t = i; i = j; j = t; }
    // XXX0 XXY1 XXZ2 XYY3 XYZ4 XZZ5 YYY6 YYZ7 YZZ8 ZZZ9
    if (i == 0) {
        if (j == 0) return k;        // 0,1,2
        if (j == 1) return 2 + k;    // XYY(k=1)->3, XYZ(k=2)->4
        return 5;                    // XZZ
    }
    if (i == 1) {
        if (j == 1) return 5 + k;    // YYY(k=1)->6, YYZ(k=2)->7
        return 8;                    // YZZ
    }
    return 9;
}

// Spherical components (16) of an atom's moments in the frame (ex, ey, ez):
// [q, mu_z, mu_x, mu_y, Q20, Q21c, Q21s, Q22c, Q22s, Q30, Q31c, Q31s, Q32c, Q32s, Q33c, Q33s]
// with the normalisation of MPIDReferenceForce.cpp:318-342.
template <typename real>
MPID_HD void frame_spherical(const LabMoments<real>& m, const real* ex, const real* ey, const real* ez, real* S) {
    const real sq3 = real(1.7320508075688772);
    S[0] = m.q;
    S[1] = m.d[0] * ez[0] + m.d[1] * ez[1] + m.d[2] * ez[2];
    S[2] = m.d[0] * ex[0] + m.d[1] * ex[1] + m.d[2] * ex[2];
    S[3] = m.d[0] * ey[0] + m.d[1] * ey[1] + m.d[2] * ey[2];
    // Theta e_a for a = z, x, y
    real Tz[3], Tx[3], Ty[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Tz[i] = m.Q[q6(i, 0)] * ez[0] + m.Q[q6(i, 1)] * ez[1] + m.Q[q6(i, 2)] * ez[2];
        Tx[i] = m.Q[q6(i, 0)] * ex[0] + m.Q[q6(i, 1)] * ex[1] + m.Q[q6(i, 2)] * ex[2];
        Ty[i] = m.Q[q6(i, 0)] * ey[0] + m.Q[q6(i, 1)] * ey[1] + m.Q[q6(i, 2)] * ey[2];
    }
    const real tzz = ez[0] * Tz[0] + ez[1] * Tz[1] + ez[2] * Tz[2];
    const real txz = ex[0] * Tz[0] + ex[1] * Tz[1] + ex[2] * Tz[2];
    const real tyz = ey[0] * Tz[0] + ey[1] * Tz[1] + ey[2] * Tz[2];
    const real txx = ex[0] * Tx[0] + ex[1] * Tx[1] + ex[2] * Tx[2];
    const real tyy = ey[0] * Ty[0] + ey[1] * Ty[1] + ey[2] * Ty[2];
    const real txy = ey[0] * Tx[0] + ey[1] * Tx[1] + ey[2] * Tx[2];
    S[4] = real(3) * tzz;
    S[5] = real(2) * sq3 * txz;
    S[6] = real(2) * sq3 * tyz;
    S[7] = sq3 * (txx - tyy);
    S[8] = real(2) * sq3 * txy;
    // Octopole: M_a = Omega . e_a (symmetric 3x3), then contractions.
    real Mz[6], Mx[6];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
            Mz[q6(i, j)] = m.O[o10(i, j, 0)] * ez[0] + m.O[o10(i, j, 1)] * ez[1] + m.O[o10(i, j, 2)] * ez[2];
            Mx[q6(i, j)] = m.O[o10(i, j, 0)] * ex[0] + m.O[o10(i, j, 1)] * ex[1] + m.O[o10(i, j, 2)] * ex[2];
        }
    real Mzz[3], Mzx[3], Mzy[3], Mxx[3], Mxy[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Mzz[i] = Mz[q6(i, 0)] * ez[0] + Mz[q6(i, 1)] * ez[1] + Mz[q6(i, 2)] * ez[2];
        Mzx[i] = Mz[q6(i, 0)] * ex[0] + Mz[q6(i, 1)] * ex[1] + Mz[q6(i, 2)] * ex[2];
        Mzy[i] = Mz[q6(i, 0)] * ey[0] + Mz[q6(i, 1)] * ey[1] + Mz[q6(i, 2)] * ey[2];
        Mxx[i] = Mx[q6(i, 0)] * ex[0] + Mx[q6(i, 1)] * ex[1] + Mx[q6(i, 2)] * ex[2];
        Mxy[i] = Mx[q6(i, 0)] * ey[0] + Mx[q6(i, 1)] * ey[1] + Mx[q6(i, 2)] * ey[2];
    }
    const real ozzz = ez[0] * Mzz[0] + ez[1] * Mzz[1] + ez[2] * Mzz[2];
    const real oxzz = ex[0] * Mzz[0] + ex[1] * Mzz[1] + ex[2] * Mzz[2];
    const real oyzz = ey[0] * Mzz[0] + ey[1] * Mzz[1] + ey[2] * Mzz[2];
    const real oxxz = ex[0] * Mzx[0] + ex[1] * Mzx[1] + ex[2] * Mzx[2];
    const real oyyz = ey[0] * Mzy[0] + ey[1] * Mzy[1] + ey[2] * Mzy[2];
    const real oxyz = ey[0] * Mzx[0] + ey[1] * Mzx[1] + ey[2] * Mzx[2];
    const real oxyy = ey[0] * Mxy[0] + ey[1] * Mxy[1] + ey[2] * Mxy[2];
    const real oxxy = ey[0] * Mxx[0] + ey[1] * Mxx[1] + ey[2] * Mxx[2];
    // traceless: xxx = -(xyy + xzz), yyy = -(xxy + yzz)
    const real oxxx = -(oxyy + oxzz);
    const real oyyy = -(oxxy + oyzz);
    S[9] = real(15) * ozzz;
    S[10] = real(15 * 1.2247448713915890) * oxzz;
    S[11] = real(15 * 1.2247448713915890) * oyzz;
    S[12] = real(15 * 0.77459666924148338) * (oxxz - oyyz);
    S[13] = real(30 * 0.77459666924148338) * oxyz;
    S[14] = real(15 * 0.31622776601683794) * (oxxx - real(3) * oxyy);
    S[15] = real(15 * 0.31622776601683794) * (real(3) * oxxy - oyyy);
}

// Pair frame: ez along the pair, ex the projection of the lab x axis onto the plane
// normal to ez (the lab y axis when the pair lies exactly on x), ey = ez x ex.  This is
// the convention of MPIDReferenceForce.cpp:650-684; it matters only for the
// reference-compatible anisotropic torque below, which is not invariant under
// rotations about the pair axis.  Written without cancellation:
//   ex = (rho, -ez_x ez_y / rho, -ez_x ez_z / rho),  rho = sqrt(ez_y^2 + ez_z^2).
template <typename real>
MPID_HD void complete_basis(const real* n, real* ex, real* ey) {
    const real rho2 = n[1] * n[1] + n[2] * n[2];
    if (rho2 > real(0)) {
        const real rho = m_sqrt(rho2);
        const real inv = real(1) / rho;
        ex[0] = rho;
        ex[1] = -n[0] * n[1] * inv;
        ex[2] = -n[0] * n[2] * inv;
    } else {
        ex[0] = real(0);
        ex[1] = real(1);
        ex[2] = real(0);
    }
    ey[0] = n[1] * ex[2] - n[2] * ex[1];
    ey[1] = n[2] * ex[0] - n[0] * ex[2];
    ey[2] = n[0] * ex[1] - n[1] * ex[0];
}

// Result of one real-space pair interaction (lab frame).
template <typename real>
struct PairOut {
    real energy;     // electric constant NOT applied
    real fJ[3];      // force on J (force on I is -fJ)
    real tI[3];      // torque on I
    real tJ[3];      // torque on J
};

// Real-space pair energy, force and torques in the pair-axis frame.
//   d        = R_J - R_I (minimum image), r = |d|
//   mI, mJ   lab moments; uI, uJ induced dipoles (lab); anisoI/J as in the reference
//            (induced dipoles of anisotropic atoms rotate with the frame and take torque)
//   radial   bP[0..7] (perm), bI[1..5] (perm-ind), bU[1..3] (ind-ind, MUTUAL only)
// Energy = U_pp + U_pi / 2;  force = -grad(U_pp + U_pi + [MUTUAL] U_uu)
// (MPIDReferenceForce.cpp:4335-4920 computes the same quantities).
//
// REF_ANISO_TORQUE reproduces the reference's induced-induced torque on anisotropic
// atoms, which keeps only the mu_I,x mu_J,y part of the pair-axis (z) rotation term
// (MPIDReferenceForce.cpp:4872-4873); the default evaluation follows the reference.
// With REF_ANISO_TORQUE = false the torque is the exact rotation derivative, which
// agrees with finite differences of the energy.
template <typename real, bool MUTUAL, bool REF_ANISO_TORQUE = true>
MPID_HD void qi_pair(const real* d, real r, const LabMoments<real>& mI, const LabMoments<real>& mJ, const real* uIlab,
                     const real* uJlab, bool anisoI, bool anisoJ, const real* bP, const real* bI, const real* bU,
                     PairOut<real>& out) {
    real ez[3] = {d[0] / r, d[1] / r, d[2] / r};
    real ex[3], ey[3];
    complete_basis(ez, ex, ey);
    real QI[16], QJ[16];
    frame_spherical(mI, ex, ey, ez, QI);
    frame_spherical(mJ, ex, ey, ez, QJ);
    // Induced dipoles as dipole blocks of a 16-vector (only indices 1..3 used).
    real uI[16], uJ[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) { uI[k] = real(0); uJ[k] = real(0); }
    uI[1] = uIlab[0] * ez[0] + uIlab[1] * ez[1] + uIlab[2] * ez[2];
    uI[2] = uIlab[0] * ex[0] + uIlab[1] * ex[1] + uIlab[2] * ex[2];
    uI[3] = uIlab[0] * ey[0] + uIlab[1] * ey[1] + uIlab[2] * ey[2];
    uJ[1] = uJlab[0] * ez[0] + uJlab[1] * ez[1] + uJlab[2] * ez[2];
    uJ[2] = uJlab[0] * ex[0] + uJlab[1] * ex[1] + uJlab[2] * ex[2];
    uJ[3] = uJlab[0] * ey[0] + uJlab[1] * ey[1] + uJlab[2] * ey[2];

    real rp[8];
    rp[0] = real(1);
#pragma unroll
    for (int k = 1; k < 8; ++k) rp[k] = rp[k - 1] * r;
    real Cp[QI_NCH_PP], dCp[QI_NCH_PP], Ci[QI_NCH_PP], dCi[QI_NCH_PP];
    qi_channels_pp<real>(bP, rp, Cp, dCp);
    // The permanent-induced and induced-induced couplings use the same channel
    // formulas with their own radial arrays (only channels touching a dipole are read).
    real bIx[8];
    bIx[0] = real(0);
#pragma unroll
    for (int n = 1; n < 6; ++n) bIx[n] = bI[n];
    bIx[6] = real(0);
    bIx[7] = real(0);
    qi_channels_pp<real>(bIx, rp, Ci, dCi);
    real Cu[QI_NCH_PP], dCu[QI_NCH_PP];
    if (MUTUAL) {
        real bUx[8];
        bUx[0] = real(0);
#pragma unroll
        for (int n = 1; n < 4; ++n) bUx[n] = bU[n];
#pragma unroll
        for (int n = 4; n < 8; ++n) bUx[n] = real(0);
        qi_channels_pp<real>(bUx, rp, Cu, dCu);
    }

    real VI[16], VJ[16], WI[16], WJ[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) { VI[k] = VJ[k] = WI[k] = WJ[k] = real(0); }
    real dU = real(0);
#define MPID_QI_PP(a, b, c)                         \
    VI[a] += Cp[c] * QJ[b];                         \
    VJ[b] += Cp[c] * QI[a];                         \
    dU += dCp[c] * QI[a] * QJ[b];
    QI_PAIR_LIST(MPID_QI_PP)
#undef MPID_QI_PP
    // permanent(I) - induced(J): b in 1..3 ; induced(I) - permanent(J): a in 1..3
#define MPID_QI_PI(a, b, c)                                   \
    if (b >= 1 && b <= 3) {                                   \
        VI[a] += Ci[c] * uJ[b];                               \
        WJ[b] += Ci[c] * QI[a];                               \
        dU += dCi[c] * QI[a] * uJ[b];                         \
    }                                                         \
    if (a >= 1 && a <= 3) {                                   \
        VJ[b] += Ci[c] * uI[a];                               \
        WI[a] += Ci[c] * QJ[b];                               \
        dU += dCi[c] * uI[a] * QJ[b];                         \
    }
    QI_PAIR_LIST(MPID_QI_PI)
#undef MPID_QI_PI
    if (MUTUAL) {
#define MPID_QI_UU(a, b, c)                                   \
    if (a >= 1 && a <= 3 && b >= 1 && b <= 3) {               \
        WI[a] += Cu[c] * uJ[b];                               \
        WJ[b] += Cu[c] * uI[a];                               \
        dU += dCu[c] * uI[a] * uJ[b];                         \
    }
        QI_PAIR_LIST(MPID_QI_UU)
#undef MPID_QI_UU
    }
    real e = real(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) e += QI[k] * VI[k] + QJ[k] * VJ[k];
    out.energy = real(0.5) * e;

    // Rotation derivatives: E_Iu = V_I . (G_u Q_I) etc.
    real G[16];
    real EI[3], EJ[3], iEI[3], iEJ[3];
    qi_rotgen_x<real>(QI, G);
    EI[0] = real(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) EI[0] += VI[k] * G[k];
    qi_rotgen_y<real>(QI, G);
    EI[1] = real(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) EI[1] += VI[k] * G[k];
    qi_rotgen_z<real>(QI, G);
    EI[2] = real(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) EI[2] += VI[k] * G[k];
    qi_rotgen_x<real>(QJ, G);
    EJ[0] = real(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) EJ[0] += VJ[k] * G[k];
    qi_rotgen_y<real>(QJ, G);
    EJ[1] = real(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) EJ[1] += VJ[k] * G[k];
    qi_rotgen_z<real>(QJ, G);
    EJ[2] = real(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) EJ[2] += VJ[k] * G[k];
    // induced dipoles: dipole block of the generators
    qi_rotgen_x<real>(uI, G);
    iEI[0] = WI[1] * G[1] + WI[2] * G[2] + WI[3] * G[3];
    qi_rotgen_y<real>(uI, G);
    iEI[1] = WI[1] * G[1] + WI[2] * G[2] + WI[3] * G[3];
    qi_rotgen_z<real>(uI, G);
    iEI[2] = WI[1] * G[1] + WI[2] * G[2] + WI[3] * G[3];
    qi_rotgen_x<real>(uJ, G);
    iEJ[0] = WJ[1] * G[1] + WJ[2] * G[2] + WJ[3] * G[3];
    qi_rotgen_y<real>(uJ, G);
    iEJ[1] = WJ[1] * G[1] + WJ[2] * G[2] + WJ[3] * G[3];
    qi_rotgen_z<real>(uJ, G);
    iEJ[2] = WJ[1] * G[1] + WJ[2] * G[2] + WJ[3] * G[3];

    if (MUTUAL && REF_ANISO_TORQUE) {
        // Drop -C(1,1,1) mu_I,y mu_J,x from the z rotation term of each induced dipole.
        iEI[2] += Cu[QI_CH_DIPOLE_DIPOLE_M1] * uJ[2] * uI[3];
        iEJ[2] += Cu[QI_CH_DIPOLE_DIPOLE_M1] * uI[2] * uJ[3];
    }
    const real rinv = real(1) / r;
    // Force on J in the pair frame (x, y, z).
    const real fx = rinv * (EI[1] + EJ[1] + iEI[1] + iEJ[1]);
    const real fy = -rinv * (EI[0] + EJ[0] + iEI[0] + iEJ[0]);
    const real fz = -dU;
    real tI[3] = {-EI[0], -EI[1], -EI[2]};
    real tJ[3] = {-EJ[0], -EJ[1], -EJ[2]};
    if (anisoI) { tI[0] -= iEI[0]; tI[1] -= iEI[1]; tI[2] -= iEI[2]; }
    if (anisoJ) { tJ[0] -= iEJ[0]; tJ[1] -= iEJ[1]; tJ[2] -= iEJ[2]; }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        out.fJ[i] = fx * ex[i] + fy * ey[i] + fz * ez[i];
        out.tI[i] = tI[0] * ex[i] + tI[1] * ey[i] + tI[2] * ez[i];
        out.tJ[i] = tJ[0] * ex[i] + tJ[1] * ey[i] + tJ[2] * ez[i];
    }
}

// ---------------------------------------------------------------------------
// Cartesian field of a source multipole (lab frame) at displacement s = x - R_src,
// with radial array b (b[1..4] used):
//   E(s) = s [q b1 + b2 (mu.s) + b3 (s.Theta.s) + b4 (Omega:sss)] - b1 mu - 2 b2 Theta s
//          - 3 b3 (Omega:ss)
template <typename real>
MPID_HD void multipole_field(const LabMoments<real>& m, const real* s, const real* b, real* E) {
    real Ts[3], Oss[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) Ts[i] = m.Q[q6(i, 0)] * s[0] + m.Q[q6(i, 1)] * s[1] + m.Q[q6(i, 2)] * s[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        real acc = real(0);
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) acc += m.O[o10(i, j, k)] * s[j] * s[k];
        Oss[i] = acc;
    }
    const real ms = m.d[0] * s[0] + m.d[1] * s[1] + m.d[2] * s[2];
    const real sTs = s[0] * Ts[0] + s[1] * Ts[1] + s[2] * Ts[2];
    const real osss = s[0] * Oss[0] + s[1] * Oss[1] + s[2] * Oss[2];
    const real radial = m.q * b[1] + b[2] * ms + b[3] * sTs + b[4] * osss;
#pragma unroll
    for (int i = 0; i < 3; ++i) E[i] = s[i] * radial - b[1] * m.d[i] - real(2) * b[2] * Ts[i] - real(3) * b[3] * Oss[i];
}

// Field of a point dipole mu at displacement s with radial array b (b[1..2]):
//   E = -b1 mu + b2 (mu.s) s
// and, optionally, its gradient E_ab = b2 (mu_a s_b + mu_b s_a + (mu.s) delta_ab)
//   - b3 (mu.s) s_a s_b in the order xx yy zz xy xz yz.
template <typename real, bool GRAD>
MPID_HD void dipole_field(const real* mu, const real* s, const real* b, real* E, real* dE) {
    const real ms = mu[0] * s[0] + mu[1] * s[1] + mu[2] * s[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) E[i] = -b[1] * mu[i] + b[2] * ms * s[i];
    if (GRAD) {
        dE[0] = b[2] * (real(2) * mu[0] * s[0] + ms) - b[3] * ms * s[0] * s[0];
        dE[1] = b[2] * (real(2) * mu[1] * s[1] + ms) - b[3] * ms * s[1] * s[1];
        dE[2] = b[2] * (real(2) * mu[2] * s[2] + ms) - b[3] * ms * s[2] * s[2];
        dE[3] = b[2] * (mu[0] * s[1] + mu[1] * s[0]) - b[3] * ms * s[0] * s[1];
        dE[4] = b[2] * (mu[0] * s[2] + mu[2] * s[0]) - b[3] * ms * s[0] * s[2];
        dE[5] = b[2] * (mu[1] * s[2] + mu[2] * s[1]) - b[3] * ms * s[1] * s[2];
    }
}

// ---------------------------------------------------------------------------
// Cardinal B-splines and derivatives.  For fractional grid coordinate u with
// w = u - floor(u), the atom touches grid points floor(u) - ORDER + 1 + i,
// i = 0..ORDER-1, with weights theta_i = M_ORDER(w + ORDER - 1 - i) (the layout of
// MPIDReferenceForce.cpp:3049-3075).  th[k][i] holds the k-th derivative, k = 0..4.
// M_1 is the unit box; M_n(t) = [t M_(n-1)(t) + (n - t) M_(n-1)(t - 1)] / (n - 1);
// the k-th derivative of M_n is the k-th backward difference of M_(n-k).
template <typename real, int ORDER>
MPID_HD void bspline_derivs(real w, real th[5][ORDER]) {
    // A[n][m] = M_n(w + m), m = 0..n-1, for n = 1..ORDER
    real A[ORDER + 1][ORDER];
#pragma unroll
    for (int n = 0; n <= ORDER; ++n)
#pragma unroll
        for (int m = 0; m < ORDER; ++m) A[n][m] = real(0);
    A[1][0] = real(1);
#pragma unroll
    for (int n = 2; n <= ORDER; ++n) {
        const real inv = real(1) / real(n - 1);
#pragma unroll
        for (int m = 0; m < n; ++m) {
            const real t = w + real(m);
            const real left = (m < n - 1) ? A[n - 1][m] : real(0);
            const real right = (m >= 1) ? A[n - 1][m - 1] : real(0);
            A[n][m] = (t * left + (real(n) - t) * right) * inv;
        }
    }
    const real binom[5][5] = {{1, 0, 0, 0, 0}, {1, 1, 0, 0, 0}, {1, 2, 1, 0, 0}, {1, 3, 3, 1, 0}, {1, 4, 6, 4, 1}};
#pragma unroll
    for (int k = 0; k <= 4; ++k) {
#pragma unroll
        for (int i = 0; i < ORDER; ++i) {
            const int m = ORDER - 1 - i;
            real acc = real(0);
            if (ORDER - k >= 1) {
#pragma unroll
                for (int j = 0; j <= k; ++j) {
                    const int mm = m - j;
                    if (mm >= 0 && mm < ORDER - k) {
                        const real v = A[ORDER - k][mm];
                        acc += ((j & 1) ? -binom[k][j] : binom[k][j]) * v;
                    }
                }
            }
            th[k][i] = acc;
        }
    }
}

// The 35 fractional potential derivatives phi_tuv (t+u+v <= 4) in the order of
// MPIDReferenceForce.cpp:3495-3528.
MPID_HD int hermite_index(int t, int u, int v) {
    const int n = t + u + v;
    if (n == 0) return 0;
    if (n == 1) return t ? 1 : (u ? 2 : 3);
    if (n == 2) {
        if (t == 2) return 4;
        if (u == 2) return 5;
        if (v == 2) return 6;
        if (t && u) return 7;
        if (t && v) return 8;
        return 9;
    }
    if (n == 3) {
        if (t == 3) return 10;
        if (u == 3) return 11;
        if (v == 3) return 12;
        if (t == 2 && u == 1) return 13;
        if (t == 2 && v == 1) return 14;
        if (t == 1 && u == 2) return 15;
        if (u == 2 && v == 1) return 16;
        if (t == 1 && v == 2) return 17;
        if (u == 1 && v == 2) return 18;
        return 19;  // 111
    }
    if (t == 4) return 20;
    if (u == 4) return 21;
    if (v == 4) return 22;
    if (t == 3 && u == 1) return 23;
    if (t == 3 && v == 1) return 24;
    if (t == 1 && u == 3) return 25;
    if (u == 3 && v == 1) return 26;
    if (t == 1 && v == 3) return 27;
    if (u == 1 && v == 3) return 28;
    if (t == 2 && u == 2) return 29;
    if (t == 2 && v == 2) return 30;
    if (u == 2 && v == 2) return 31;
    if (t == 2) return 32;  // 211
    if (u == 2) return 33;  // 121
    return 34;              // 112
}

// ---------------------------------------------------------------------------
// Local axis frames (MPIDReferenceForce.cpp:399-458).  Rows of R are the frame's
// x, y, z axes in lab coordinates.  NoAxisType keeps the identity.
enum AxisType { ZThenX = 0, Bisector = 1, ZBisect = 2, ThreeFold = 3, ZOnly = 4, NoAxisType = 5 };

template <typename real>
MPID_HD real normalize3(real* v) {
    const real n = m_sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (n > real(0)) {
        const real inv = real(1) / n;
        v[0] *= inv; v[1] *= inv; v[2] *= inv;
    }
    return n;
}

template <typename real>
MPID_HD void local_frame(int axis, const real* pI, const real* pZ, const real* pX, const real* pY, real R[3][3]) {
    if (axis == NoAxisType) {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) R[i][j] = real(i == j);
        return;
    }
    real vz[3] = {pZ[0] - pI[0], pZ[1] - pI[1], pZ[2] - pI[2]};
    normalize3(vz);
    real vx[3], vy[3];
    if (axis == ZOnly) {
        const bool useX = m_fabs(vz[0]) < real(0.866);
        vx[0] = useX ? real(1) : real(0);
        vx[1] = useX ? real(0) : real(1);
        vx[2] = real(0);
    } else {
        for (int k = 0; k < 3; ++k) vx[k] = pX[k] - pI[k];
        if (axis == Bisector) {
            normalize3(vx);
            for (int k = 0; k < 3; ++k) vz[k] += vx[k];
            normalize3(vz);
        } else if (axis == ZBisect) {
            normalize3(vx);
            for (int k = 0; k < 3; ++k) vy[k] = pY[k] - pI[k];
            normalize3(vy);
            for (int k = 0; k < 3; ++k) vx[k] += vy[k];
            normalize3(vx);
        } else if (axis == ThreeFold) {
            normalize3(vx);
            for (int k = 0; k < 3; ++k) vy[k] = pY[k] - pI[k];
            normalize3(vy);
            for (int k = 0; k < 3; ++k) vz[k] += vx[k] + vy[k];
            normalize3(vz);
        }
    }
    const real dot = vz[0] * vx[0] + vz[1] * vx[1] + vz[2] * vx[2];
    for (int k = 0; k < 3; ++k) vx[k] -= vz[k] * dot;
    normalize3(vx);
    vy[0] = vz[1] * vx[2] - vz[2] * vx[1];
    vy[1] = vz[2] * vx[0] - vz[0] * vx[2];
    vy[2] = vz[0] * vx[1] - vz[1] * vx[0];
    for (int k = 0; k < 3; ++k) { R[0][k] = vx[k]; R[1][k] = vy[k]; R[2][k] = vz[k]; }
}

// Molecular-frame parameters in the MPIDForce::addMultipole orders
// (dipole XYZ; quadrupole XX XY YY XZ YZ ZZ; octopole XXX XXY XYY YYY XXZ XYZ YYZ XZZ YYZ ZZZ).
template <typename real>
struct MolParams {
    real q;
    real d[3];
    real Q[6];
    real O[10];
    real pol[3];
};

// Rotate molecular moments and the polarisability diagonal to the lab frame
// (MPIDReferenceForce.cpp:459-563).  `flipY` applies the chirality inversion of
// MPIDReferenceForce.cpp:357-381, which negates dipole-y, QXY and QYZ only.
template <typename real>
MPID_HD void rotate_to_lab(const MolParams<real>& p, const real R[3][3], bool flipY, LabMoments<real>& lab,
                           real alphaLab[6]) {
    real d[3] = {p.d[0], p.d[1], p.d[2]};
    // API order -> symmetric access
    real Qm[3][3] = {{p.Q[0], p.Q[1], p.Q[3]}, {p.Q[1], p.Q[2], p.Q[4]}, {p.Q[3], p.Q[4], p.Q[5]}};
    if (flipY) {
        d[1] = -d[1];
        Qm[0][1] = Qm[1][0] = -Qm[0][1];
        Qm[1][2] = Qm[2][1] = -Qm[1][2];
    }
    // octopole API order -> O10 order of the symmetric access helper
    // API: XXX0 XXY1 XYY2 YYY3 XXZ4 XYZ5 YYZ6 XZZ7 YZZ8 ZZZ9
    real Om[10];
    Om[o10(0, 0, 0)] = p.O[0];
    Om[o10(0, 0, 1)] = p.O[1];
    Om[o10(0, 1, 1)] = p.O[2];
    Om[o10(1, 1, 1)] = p.O[3];
    Om[o10(0, 0, 2)] = p.O[4];
    Om[o10(0, 1, 2)] = p.O[5];
    Om[o10(1, 1, 2)] = p.O[6];
    Om[o10(0, 2, 2)] = p.O[7];
    Om[o10(1, 2, 2)] = p.O[8];
    Om[o10(2, 2, 2)] = p.O[9];
    lab.q = p.q;
    for (int i = 0; i < 3; ++i) lab.d[i] = d[0] * R[0][i] + d[1] * R[1][i] + d[2] * R[2][i];
    // Q_lab = R^T Q R ; alpha_lab = R^T diag(pol) R
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) {
            real acc = real(0), aacc = real(0);
            for (int k = 0; k < 3; ++k) {
                aacc += R[k][i] * R[k][j] * p.pol[k];
                for (int m = 0; m < 3; ++m) acc += R[k][i] * R[m][j] * Qm[k][m];
            }
            lab.Q[q6(i, j)] = acc;
            alphaLab[q6(i, j)] = aacc;
        }
    // O_lab[ijk] = R[l][i] R[m][j] R[o][k] O[lmo], done one index at a time.
    real T1[3][3][3];  // T1[i][m][o] = sum_l R[l][i] O[l m o]
    for (int i = 0; i < 3; ++i)
        for (int m = 0; m < 3; ++m)
            for (int o = 0; o < 3; ++o) {
                real acc = real(0);
                for (int l = 0; l < 3; ++l) acc += R[l][i] * Om[o10(l, m, o)];
                T1[i][m][o] = acc;
            }
    real T2[3][3][3];  // T2[i][j][o] = sum_m R[m][j] T1[i][m][o]
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int o = 0; o < 3; ++o) {
                real acc = real(0);
                for (int m = 0; m < 3; ++m) acc += R[m][j] * T1[i][m][o];
                T2[i][j][o] = acc;
            }
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j)
            for (int k = j; k < 3; ++k) {
                real acc = real(0);
                for (int o = 0; o < 3; ++o) acc += R[o][k] * T2[i][j][o];
                lab.O[o10(i, j, k)] = acc;
            }
}

// Chirality test of MPIDReferenceForce.cpp:357-381 for ZThenX atoms with a Y atom.
template <typename real>
MPID_HD bool chiral_flip(int axis, bool hasY, const real* pI, const real* pZ, const real* pX, const real* pY) {
    if (axis != ZThenX || !hasY) return false;
    const real ad[3] = {pI[0] - pY[0], pI[1] - pY[1], pI[2] - pY[2]};
    const real bd[3] = {pZ[0] - pY[0], pZ[1] - pY[1], pZ[2] - pY[2]};
    const real cd[3] = {pX[0] - pY[0], pX[1] - pY[1], pX[2] - pY[2]};
    const real c[3] = {bd[1] * cd[2] - bd[2] * cd[1], bd[2] * cd[0] - bd[0] * cd[2], bd[0] * cd[1] - bd[1] * cd[0]};
    return c[0] * ad[0] + c[1] * ad[1] + c[2] * ad[2] < real(0);
}

// ---------------------------------------------------------------------------
// Reciprocal space helpers.  A[j][i] converts Cartesian to fractional grid
// coordinates: frac_j = sum_i A[j][i] x_i, A[j][i] = n_j recip[i][j]
// (MPIDReferenceForce.cpp:3080-3083).
//
// Weighted fractional multipole, 20 components in the order
// q, x y z, xx yy zz xy xz yz, xxx yyy zzz xxy xxz xyy yyz xzz yzz xyz
// (the first 20 entries of the 35-term derivative order) times the multinomial
// weight n!/(t!u!v!) of each component.
template <typename real>
MPID_HD void frac_multipole(const LabMoments<real>& m, const real A[3][3], real Mf[20]) {
    Mf[0] = m.q;
    for (int j = 0; j < 3; ++j) Mf[1 + j] = A[j][0] * m.d[0] + A[j][1] * m.d[1] + A[j][2] * m.d[2];
    // Q_f = A Q A^T
    real AQ[3][3];
    for (int a = 0; a < 3; ++a)
        for (int j = 0; j < 3; ++j) AQ[a][j] = A[a][0] * m.Q[q6(0, j)] + A[a][1] * m.Q[q6(1, j)] + A[a][2] * m.Q[q6(2, j)];
    real Qf[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) Qf[a][b] = AQ[a][0] * A[b][0] + AQ[a][1] * A[b][1] + AQ[a][2] * A[b][2];
    Mf[4] = Qf[0][0];
    Mf[5] = Qf[1][1];
    Mf[6] = Qf[2][2];
    Mf[7] = real(2) * Qf[0][1];
    Mf[8] = real(2) * Qf[0][2];
    Mf[9] = real(2) * Qf[1][2];
    // O_f[abc] = A[a][i] A[b][j] A[c][k] O[ijk]
    real T1[3][6];  // T1[a][jk] = sum_i A[a][i] O[i j k]
    for (int a = 0; a < 3; ++a)
        for (int j = 0; j < 3; ++j)
            for (int k = j; k < 3; ++k)
                T1[a][q6(j, k)] = A[a][0] * m.O[o10(0, j, k)] + A[a][1] * m.O[o10(1, j, k)] + A[a][2] * m.O[o10(2, j, k)];
    real T2[3][3][3];  // T2[a][b][k] = sum_j A[b][j] T1[a][jk]
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int k = 0; k < 3; ++k)
                T2[a][b][k] = A[b][0] * T1[a][q6(0, k)] + A[b][1] * T1[a][q6(1, k)] + A[b][2] * T1[a][q6(2, k)];
    auto of = [&](int a, int b, int c) {
        return A[c][0] * T2[a][b][0] + A[c][1] * T2[a][b][1] + A[c][2] * T2[a][b][2];
    };
    // order (from index 10): xxx yyy zzz xxy xxz xyy yyz xzz yzz xyz
    Mf[10] = of(0, 0, 0);
    Mf[11] = of(1, 1, 1);
    Mf[12] = of(2, 2, 2);
    Mf[13] = real(3) * of(0, 0, 1);
    Mf[14] = real(3) * of(0, 0, 2);
    Mf[15] = real(3) * of(0, 1, 1);
    Mf[16] = real(3) * of(1, 1, 2);
    Mf[17] = real(3) * of(0, 2, 2);
    Mf[18] = real(3) * of(1, 2, 2);
    Mf[19] = real(6) * of(0, 1, 2);
}

// (t,u,v) of the first 20 derivative slots.
MPID_HD void hermite_tuv(int k, int& t, int& u, int& v) {
    const int T[20] = {0, 1, 0, 0, 2, 0, 0, 1, 1, 0, 3, 0, 0, 2, 2, 1, 0, 1, 0, 1};
    const int U[20] = {0, 0, 1, 0, 0, 2, 0, 1, 0, 1, 0, 3, 0, 1, 0, 2, 2, 0, 1, 1};
    const int V[20] = {0, 0, 0, 1, 0, 0, 2, 0, 1, 1, 0, 0, 3, 0, 1, 0, 1, 2, 2, 1};
    t = T[k]; u = U[k]; v = V[k];
}

// Cartesian potential-derivative tensors from the 35 fractional derivatives:
// Phi1[i], Phi2[i][j], Phi3[i][j][k] (full symmetric), Phi_0 = phi[0].
template <typename real>
MPID_HD void cartesian_potential(const real* phi, const real A[3][3], real& Phi0, real Phi1[3], real Phi2[3][3],
                                 real Phi3[3][3][3]) {
    Phi0 = phi[0];
    for (int i = 0; i < 3; ++i) Phi1[i] = A[0][i] * phi[1] + A[1][i] * phi[2] + A[2][i] * phi[3];
    // Phi2 = A^T H A and Phi3 = (A^T)^3 G, one index at a time (separable contraction)
    real H[3][3], T[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            int c[3] = {0, 0, 0};
            c[a]++; c[b]++;
            H[a][b] = phi[hermite_index(c[0], c[1], c[2])];
        }
    for (int i = 0; i < 3; ++i)
        for (int b = 0; b < 3; ++b) T[i][b] = A[0][i] * H[0][b] + A[1][i] * H[1][b] + A[2][i] * H[2][b];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Phi2[i][j] = A[0][j] * T[i][0] + A[1][j] * T[i][1] + A[2][j] * T[i][2];
    real G[3][3][3], U[3][3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int c = 0; c < 3; ++c) {
                int n[3] = {0, 0, 0};
                n[a]++; n[b]++; n[c]++;
                G[a][b][c] = phi[hermite_index(n[0], n[1], n[2])];
            }
    for (int i = 0; i < 3; ++i)
        for (int b = 0; b < 3; ++b)
            for (int c = 0; c < 3; ++c) U[i][b][c] = A[0][i] * G[0][b][c] + A[1][i] * G[1][b][c] + A[2][i] * G[2][b][c];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int c = 0; c < 3; ++c) G[i][j][c] = A[0][j] * U[i][0][c] + A[1][j] * U[i][1][c] + A[2][j] * U[i][2][c];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                Phi3[i][j][k] = A[0][k] * G[i][j][0] + A[1][k] * G[i][j][1] + A[2][k] * G[i][j][2];
}

// Torque on a multipole (q, dipole d, Q6, O10) in an external potential with
// Cartesian derivative tensors Phi: tau = -sum_n n (M^(n) x Phi^(n)), the cross
// product taken over the first index of both tensors.
template <typename real>
MPID_HD void multipole_torque(const real* d, const real* Q, const real* O, const real Phi1[3], const real Phi2[3][3],
                              const real Phi3[3][3][3], real* tau) {
    for (int a = 0; a < 3; ++a) {
        const int j = (a + 1) % 3, k = (a + 2) % 3;
        real t = -(d[j] * Phi1[k] - d[k] * Phi1[j]);
        real t2 = real(0), t3 = real(0);
        for (int m = 0; m < 3; ++m) {
            t2 += Q[q6(j, m)] * Phi2[k][m] - Q[q6(k, m)] * Phi2[j][m];
            for (int n = 0; n < 3; ++n) t3 += O[o10(j, m, n)] * Phi3[k][m][n] - O[o10(k, m, n)] * Phi3[j][m][n];
        }
        tau[a] = t - real(2) * t2 - real(3) * t3;
    }
}

// Map the torque on atom I onto forces on I and its frame atoms
// (MPIDReferenceForce.cpp:1895-2110).  Writes up to four force vectors:
// fI, fZ (U atom), fX (V atom), fY (W atom).
template <typename real>
MPID_HD void torque_to_force(int axis, const real* pI, const real* pZ, const real* pX, const real* pY, bool hasY,
                             const real* torque, real* fI, real* fZ, real* fX, real* fY) {
    for (int k = 0; k < 3; ++k) fI[k] = fZ[k] = fX[k] = fY[k] = real(0);
    if (axis == NoAxisType) return;
    auto cross = [](const real* a, const real* b, real* c) {
        c[0] = a[1] * b[2] - a[2] * b[1];
        c[1] = a[2] * b[0] - a[0] * b[2];
        c[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto dot = [](const real* a, const real* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    real u[3], v[3], w[3];
    for (int k = 0; k < 3; ++k) { u[k] = pZ[k] - pI[k]; v[k] = pX[k] - pI[k]; }
    const real nu = normalize3(u);
    if (axis == ZOnly) {
        // The second frame vector of a Z-only frame is the fixed lab axis chosen in
        // local_frame (as the reference CUDA platform does, multipoles.cu:527-533); the
        // reference CPU code reads an x atom that Z-only frames do not have.
        const bool useX = m_fabs(u[0]) < real(0.866);
        v[0] = useX ? real(1) : real(0);
        v[1] = useX ? real(0) : real(1);
        v[2] = real(0);
    }
    const real nv = normalize3(v);
    if (hasY && (axis == ZBisect || axis == ThreeFold)) {
        for (int k = 0; k < 3; ++k) w[k] = pY[k] - pI[k];
    } else {
        cross(u, v, w);
    }
    const real nw = normalize3(w);
    real uv[3], uw[3], vw[3];
    cross(v, u, uv);
    cross(w, u, uw);
    cross(w, v, vw);
    normalize3(uv);
    normalize3(uw);
    normalize3(vw);
    const real cUV = dot(u, v), sUV = m_sqrt(real(1) - cUV * cUV);
    const real cUW = dot(u, w), sUW = m_sqrt(real(1) - cUW * cUW);
    const real cVW = dot(v, w), sVW = m_sqrt(real(1) - cVW * cVW);
    const real dU = -dot(u, torque), dV = -dot(v, torque), dW = -dot(w, torque);
    if (axis == ZThenX || axis == Bisector) {
        const real f1 = dV / (nu * sUV);
        real f2 = dW / nu;
        const real f3 = -dU / (nv * sUV);
        real f4 = real(0);
        if (axis == Bisector) {
            f2 *= real(0.5);
            f4 = real(0.5) * dW / nv;
        }
        for (int k = 0; k < 3; ++k) {
            const real forceU = uv[k] * f1 + f2 * uw[k];
            const real forceV = uv[k] * f3 + f4 * vw[k];
            fZ[k] = -forceU;
            fX[k] = -forceV;
            fI[k] = forceU + forceV;
        }
    } else if (axis == ZBisect) {
        real rr[3] = {v[0] + w[0], v[1] + w[1], v[2] + w[2]};
        real ss[3];
        cross(u, rr, ss);
        normalize3(rr);
        normalize3(ss);
        real ur[3], us[3], vs[3], ws[3];
        cross(rr, u, ur);
        cross(ss, u, us);
        cross(ss, v, vs);
        cross(ss, w, ws);
        normalize3(ur);
        normalize3(us);
        normalize3(vs);
        normalize3(ws);
        const real cUR = dot(u, rr), sUR = m_sqrt(real(1) - cUR * cUR);
        const real cVS = dot(v, ss), sVS = m_sqrt(real(1) - cVS * cVS);
        const real cWS = dot(w, ss), sWS = m_sqrt(real(1) - cWS * cWS);
        real t1[3], t2[3];
        for (int k = 0; k < 3; ++k) { t1[k] = v[k] - ss[k] * cVS; t2[k] = w[k] - ss[k] * cWS; }
        normalize3(t1);
        normalize3(t2);
        const real ut1c = dot(u, t1), ut1s = m_sqrt(real(1) - ut1c * ut1c);
        const real ut2c = dot(u, t2), ut2s = m_sqrt(real(1) - ut2c * ut2c);
        const real dR = -dot(rr, torque), dS = -dot(ss, torque);
        const real f1 = dR / (nu * sUR);
        const real f2 = dS / nu;
        const real f3 = dU / (nv * (ut1s + ut2s));
        const real f4 = dU / (nw * (ut1s + ut2s));
        for (int k = 0; k < 3; ++k) {
            const real forceU = ur[k] * f1 + us[k] * f2;
            const real forceV = (ss[k] * sVS - t1[k] * cVS) * f3;
            const real forceW = (ss[k] * sWS - t2[k] * cWS) * f4;
            fZ[k] = -forceU;
            fX[k] = -forceV;
            fY[k] = -forceW;
            fI[k] = forceU + forceV + forceW;
        }
    } else if (axis == ThreeFold) {
        for (int k = 0; k < 3; ++k) {
            real du = uw[k] * dW / (nu * sUW) + uv[k] * dV / (nu * sUV) - uw[k] * dU / (nu * sUW) - uv[k] * dU / (nu * sUV);
            real dv = vw[k] * dW / (nv * sVW) - uv[k] * dU / (nv * sUV) - vw[k] * dV / (nv * sVW) + uv[k] * dV / (nv * sUV);
            real dw = -uw[k] * dU / (nw * sUW) - vw[k] * dV / (nw * sVW) + uw[k] * dW / (nw * sUW) + vw[k] * dW / (nw * sVW);
            du /= real(3);
            dv /= real(3);
            dw /= real(3);
            fZ[k] = -du;
            fX[k] = -dv;
            if (hasY) fY[k] = -dw;
            fI[k] = du + dv + dw;
        }
    } else if (axis == ZOnly) {
        for (int k = 0; k < 3; ++k) {
            const real du = uv[k] * dV / (nu * sUV) + uw[k] * dW / nu;
            fZ[k] = -du;
            fI[k] = du;
        }
    }
}

}  // namespace mpid
