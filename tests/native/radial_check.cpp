// Host check of the Ewald radial functions of the pair kernels (mpid_math.cuh) against
// long double: b_n (n = 0..7) of erf(alpha r)/r below the branch threshold (Boys
// function series) and of erfc(alpha r)/r above it, in float and in double.
//
//   g++ -O2 -std=c++17 -I mpidopenmmplugin_gb300/csrc tests/native/radial_check.cpp -o /tmp/radial_check
//   /tmp/radial_check alpha cutoff
//
// Prints "name max_relative_error mean_signed_relative_error" per check; the mean of the
// signed error exposes systematic bias.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "mpid_math.cuh"

using namespace mpid;
typedef long double ld;

// b_n of erf(alpha r)/r (n = 0..7): 2^(n+1) alpha^(2n+1)/sqrt(pi) F_n(T), F_n by its
// power series in long double.
static void ref_erf(ld r, ld alpha, ld* b) {
    const ld T = alpha * r * alpha * r, sp = std::sqrt(std::acos((ld) -1));
    for (int n = 0; n <= 7; ++n) {
        ld term = 1, sum = 0;
        for (int k = 0; k < 300; ++k) {
            sum += term / (2 * n + 2 * k + 1);
            term *= -T / (k + 1);
            if (std::fabs(term) < 1e-40L) break;
        }
        b[n] = std::pow((ld) 2, n + 1) * std::pow(alpha, 2 * n + 1) / sp * sum;
    }
}
static void ref_erfc(ld r, ld alpha, ld* b) {
    const ld x = alpha * r, sp = std::sqrt(std::acos((ld) -1)), rinv2 = 1 / (r * r);
    b[0] = std::erfc(x) / r;
    ld c = 2 * alpha / sp * std::exp(-x * x);
    for (int n = 1; n <= 7; ++n) {
        b[n] = ((2 * n - 1) * b[n - 1] + c) * rinv2;
        c *= 2 * alpha * alpha;
    }
}

template <typename real>
static void check(const char* name, double alpha, double r0, double r1, bool erfBranch) {
    std::mt19937_64 gen(7);
    const EwaldAlpha<real> al(alpha);
    long double worst = 0, mean = 0;
    const int N = 200000;
    for (int i = 0; i < N; ++i) {
        const real r = (real) (r0 + (r1 - r0) * std::uniform_real_distribution<double>(0, 1)(gen));
        real b[8];
        ld ref[8];
        if (erfBranch) {
            erf_part_boys<real, 7>(r, al, b);
            ref_erf((ld) r, (ld) alpha, ref);
        } else {
            const real rinv = real(1) / r;
            erfc_part<real, 7>(r, rinv * rinv, al, b);
            ref_erfc((ld) r, (ld) alpha, ref);
        }
        for (int n = 0; n <= 7; ++n) {
            const ld e = (ld) b[n] / ref[n] - 1;
            worst = std::fmax(worst, std::fabs(e));
            mean += e / (8.0L * N);
        }
    }
    printf("%s %.3Le %.3Le\n", name, worst, mean);
}

int main(int argc, char** argv) {
    const double alpha = argc > 1 ? atof(argv[1]) : 3.4;
    const double cutoff = argc > 2 ? atof(argv[2]) : 0.9;
    const double rq = 1.5 / alpha;
    check<float>("erf_float", alpha, 0.05, rq, true);
    check<float>("erfc_float", alpha, rq, cutoff, false);
    check<double>("erf_double", alpha, 0.05, rq, true);
    check<double>("erfc_double", alpha, rq, cutoff, false);
    return 0;
}
