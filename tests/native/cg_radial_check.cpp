// CPU check of the FP32 radial functions of the CG pair kernel (cg_radial.h) against
// long double: b_1 and b_2 of K_u = phi_T - erf(alpha r)/r for pairs over the whole list
// range (near and erfc segments), for the Thole arguments of water-like atoms.
//
//   g++ -O2 -std=c++17 -I mpidopenmmplugin_gb300/csrc tests/native/cg_radial_check.cpp -o /tmp/cg_radial_check
//   /tmp/cg_radial_check 3.4 0.9
//
// Prints, for the polynomial form and for the general FP32 radial functions of the
// other pair kernels (pair_radial_branch in mpid_math.cuh, for comparison), the largest
// error of b_1 and b_2 relative to the bare 1/r^3 and 3/r^5 of the pair (the scale of
// the pair's contribution to the field) and relative to |b_n| itself over pairs where
// |b_n| is at least 1 % of that scale.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "cg_radial.h"
#include "mpid_math.cuh"

typedef long double ld;

static void reference(ld alpha, ld xq, ld r, ld s, ld* b) {
    const ld x = alpha * r, rinv = 1 / r, rinv2 = rinv * rinv;
    const ld bB1 = rinv * rinv2, bB2 = 3 * bB1 * rinv2;
    const ld es = std::exp(-s);
    const ld om1 = es * (1 + s + s * s / 2), om2 = om1 + es * s * s * s / 6;
    const ld sqrtpi = std::sqrt(std::acos((ld) -1));
    if (x >= xq) {
        const ld ex = std::exp(-x * x);
        const ld b0 = std::erfc(x) * rinv;
        ld c = 2 * alpha / sqrtpi * ex;
        const ld e1 = (b0 + c) * rinv2;
        c *= 2 * alpha * alpha;
        const ld e2 = (3 * e1 + c) * rinv2;
        b[0] = e1 - om1 * bB1;
        b[1] = e2 - om2 * bB2;
    } else {
        const ld T = x * x;
        const ld H1 = 4 * alpha * alpha * alpha / sqrtpi * mpid::cg_detail::boys(1, T);
        const ld H2 = 8 * alpha * alpha * alpha * alpha * alpha / sqrtpi * mpid::cg_detail::boys(2, T);
        b[0] = (1 - om1) * bB1 - H1;
        b[1] = (1 - om2) * bB2 - H2;
    }
}

int main(int argc, char** argv) {
    const double alpha = argc > 1 ? atof(argv[1]) : 3.4;
    const double cutoff = argc > 2 ? atof(argv[2]) : 0.9;
    const double xq = 1.5, rL = cutoff * (1.0 + 1e-6) + 1e-5;
    const mpid::CgRadial R = mpid::build_cg_radial(alpha, xq, rL);
    // Thole width a and d_i d_j of O-O, O-H, H-H pairs (polarisabilities 1e-3 and 3e-4 nm^3)
    const double widths[2] = {1.3, 0.65};
    const double dd[3] = {std::pow(1e-3, 1.0 / 3.0), std::pow(1e-3 * 3e-4, 1.0 / 6.0), std::pow(3e-4, 1.0 / 3.0)};
    double worstScale[2][2] = {{0, 0}, {0, 0}}, worstRel[2][2] = {{0, 0}, {0, 0}};
    const mpid::EwaldAlpha<float> ew(alpha);
    const int N = 200000;
    for (int w = 0; w < 2; ++w)
        for (int p = 0; p < 3; ++p)
            for (int k = 0; k < N; ++k) {
                const double r = 0.05 + (rL - 0.05) * (k + 0.5) / N;
                const float rf = (float) r;
                const float r2 = rf * rf;
                const float invd = (float) (1.0 / dd[p]);
                const float ahi = (float) alpha, alo = (float) (alpha - (double) ahi);  // the split alpha
                // the segment as the list builder assigns it (alpha r below 1.5)
                const bool nearSeg = rf * rf < (float) std::pow(xq / alpha, 2);
                float b1, b2;
                if (nearSeg)
                    mpid::cg_pair_radial<true>(R, r2, (float) widths[w], invd, ahi, alo, b1, b2);
                else
                    mpid::cg_pair_radial<false>(R, r2, (float) widths[w], invd, ahi, alo, b1, b2);
                // the kernel's r and Thole argument, for the references
                const float rr = nearSeg ? std::sqrt(r2) : r2 * (1.f / std::sqrt(r2));
                const float s = fminf((float) widths[w] * rr * invd, 100.f);
                const float x = fmaf(ahi, rr, alo * rr);
                // the general path at the same r (Thole argument from the damping product)
                const float ddf = (float) dd[p];
                mpid::PairRadial<float, 0, 0, 2> old;
                if (x * x < R.xq2)
                    mpid::pair_radial_branch<float, -1, -1, 2, true>(rr, ew, 1.f, (float) widths[w], ddf, old);
                else
                    mpid::pair_radial_branch<float, -1, -1, 2, false>(rr, ew, 1.f, (float) widths[w], ddf, old);
                ld ref[2];
                reference((ld) alpha, (ld) xq, (ld) rr, (ld) s, ref);
                ld refOld[2];
                reference((ld) alpha, (ld) xq, (ld) rr, (ld) widths[w] * (ld) rr / (ld) ddf, refOld);
                const ld bare[2] = {1 / ((ld) rr * rr * rr), 3 / ((ld) rr * rr * rr * rr * rr)};
                const float got[2][2] = {{b1, b2}, {old.bU[1], old.bU[2]}};
                for (int v = 0; v < 2; ++v)
                    for (int n = 0; n < 2; ++n) {
                        const ld rf = v == 0 ? ref[n] : refOld[n];
                        const double eScale = (double) (std::fabs((ld) got[v][n] - rf) / bare[n]);
                        if (eScale > worstScale[v][n]) worstScale[v][n] = eScale;
                        if (std::fabs(rf) > 0.01L * bare[n]) {
                            const double eRel = (double) (std::fabs((ld) got[v][n] - rf) / std::fabs(rf));
                            if (eRel > worstRel[v][n]) worstRel[v][n] = eRel;
                        }
                    }
            }
    for (int v = 0; v < 2; ++v)
        printf("%s b1 scale %.3e rel %.3e b2 scale %.3e rel %.3e\n", v == 0 ? "polynomial" : "general", worstScale[v][0],
               worstRel[v][0], worstScale[v][1], worstRel[v][1]);
    return 0;
}
