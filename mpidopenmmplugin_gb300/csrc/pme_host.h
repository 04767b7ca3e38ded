// Host-side PME set-up computed once per grid / box in FP64: B-spline moduli and the
// reciprocal box.  Used by the context (mpid_context.cu) to build device tables.
#pragma once
#include <cmath>
#include <vector>

namespace mpid {

// Cardinal B-spline M_order evaluated at the integers 1..order (M_order(order) = 0).
inline std::vector<double> bspline_at_integers(int order) {
    // values of M_n(t) at t = 1..n by the Cox-de Boor recursion on integer points
    std::vector<double> cur = {1.0};  // M_1(1) is the right end of the unit box: treat M_1 on [0,1)
    // Build M_n(k) for k = 0..n using M_n(t) = [t M_(n-1)(t) + (n - t) M_(n-1)(t-1)]/(n-1)
    std::vector<double> prev(3, 0.0);  // M_1 at t = 0,1,2 -> 1, 0, 0 (left-closed box)
    prev[0] = 1.0;
    for (int n = 2; n <= order; ++n) {
        std::vector<double> next(n + 2, 0.0);
        for (int t = 0; t <= n; ++t) {
            double a = (t < (int) prev.size()) ? prev[t] : 0.0;
            double b = (t - 1 >= 0 && t - 1 < (int) prev.size()) ? prev[t - 1] : 0.0;
            next[t] = (t * a + (n - t) * b) / (n - 1);
        }
        prev = next;
    }
    std::vector<double> out(order, 0.0);
    for (int k = 0; k < order; ++k) out[k] = (k + 1 < (int) prev.size()) ? prev[k + 1] : 0.0;
    return out;
}

// |b(m)|^-2 style moduli of the B-spline structure factor along one grid axis, with the
// exponential-Euler-spline fix and the optimal-zeta lattice-sum correction of
// MPIDReferenceForce.cpp:2720-2810 (restated; the zeta sums run over |j| <= 50).
inline std::vector<double> bspline_moduli(int order, int n) {
    std::vector<double> Mk = bspline_at_integers(order);  // Mk[k] = M_order(k + 1)
    std::vector<double> mod(n, 0.0);
    for (int i = 0; i < n; ++i) {
        double s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < order && k + 1 <= n - 1; ++k) {
            const double arg = 2.0 * M_PI * (double) i * (double) (k + 1) / (double) n;
            s1 += Mk[k] * std::cos(arg);
            s2 += Mk[k] * std::sin(arg);
        }
        mod[i] = s1 * s1 + s2 * s2;
    }
    const double eps = 1.0e-7;
    if (mod[0] < eps) mod[0] = 0.5 * mod[1];
    for (int i = 1; i < n - 1; ++i)
        if (mod[i] < eps) mod[i] = 0.5 * (mod[i - 1] + mod[i + 1]);
    if (mod[n - 1] < eps) mod[n - 1] = 0.5 * mod[n - 2];
    for (int i = 0; i < n; ++i) {
        int k = i;
        if (i + 1 > n / 2) k = i - n;
        double zeta = 1.0;
        if (k != 0) {
            const double f = M_PI * k / n;
            double s1 = 1.0, s2 = 1.0;
            for (int j = 1; j <= 50; ++j) {
                const double a = f / (f + M_PI * j), b = f / (f - M_PI * j);
                s1 += std::pow(a, order) + std::pow(b, order);
                s2 += std::pow(a, 2 * order) + std::pow(b, 2 * order);
            }
            zeta = s2 / s1;
        }
        mod[i] *= zeta * zeta;
    }
    return mod;
}

// Reciprocal box of a box whose first vector lies on x and second in the xy plane
// (rows; MPIDReferenceForce.cpp:2615-2633 uses the same reduced form).
inline void reciprocal_box(const double box[9], double recip[9]) {
    const double ax = box[0], bx = box[3], by = box[4], cx = box[6], cy = box[7], cz = box[8];
    const double inv = 1.0 / (ax * by * cz);
    recip[0] = by * cz * inv; recip[1] = 0; recip[2] = 0;
    recip[3] = -bx * cz * inv; recip[4] = ax * cz * inv; recip[5] = 0;
    recip[6] = (bx * cy - by * cx) * inv; recip[7] = -ax * cy * inv; recip[8] = ax * by * inv;
}

}  // namespace mpid
