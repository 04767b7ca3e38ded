// Host check of the double-float arithmetic and the tabulated Ewald radial functions
// used by the mixed path's residual field, against long double.
//
//   g++ -O2 -std=c++17 -I mpidopenmmplugin_gb300/csrc tests/native/df_check.cpp -o /tmp/df_check
//   /tmp/df_check alpha cutoff
//
// Prints one line "name max_relative_error" per check.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "df64.cuh"
#include "radial_tables.h"

using namespace mpid;
typedef long double ld;

static ld as_ld(dfloat a) { return (ld) a.hi + (ld) a.lo; }

int main(int argc, char** argv) {
    const double alpha = argc > 1 ? atof(argv[1]) : 3.4;
    const double cutoff = argc > 2 ? atof(argv[2]) : 0.9;
    const double rq = 1.5 / alpha, rL = cutoff * (1.0 + 1e-6) + 1e-5;
    RadialTableHost G, H;
    build_ewald_tables(alpha, rq, rL, 32, 7, G, H);
    std::mt19937_64 gen(12345);
    ld eG = 0, eH = 0, eExp = 0, eDiv = 0, eSqrt = 0;
    for (int i = 0; i < 100000; ++i) {
        const double r = rq + (rL - rq) * std::uniform_real_distribution<double>(0, 1)(gen);
        dfloat rd = df_from_double(r), f1, f2;
        df_table_eval<7>(G.coef.data(), G.centre.data(), G.r0, G.invh, G.K, rd, f1, f2);
        ld ref[2];
        radial_detail::erfc_parts(as_ld(rd), (ld) alpha, ref);
        eG = std::fmax(eG, std::fabs(as_ld(f1) / ref[0] - 1));
        eG = std::fmax(eG, std::fabs(as_ld(f2) / ref[1] - 1));
        const double r2 = rq * std::uniform_real_distribution<double>(0, 1)(gen);
        rd = df_from_double(r2);
        df_table_eval<7>(H.coef.data(), H.centre.data(), H.r0, H.invh, H.K, rd, f1, f2);
        radial_detail::erf_parts(as_ld(rd), (ld) alpha, ref);
        eH = std::fmax(eH, std::fabs(as_ld(f1) / ref[0] - 1));
        eH = std::fmax(eH, std::fabs(as_ld(f2) / ref[1] - 1));
        const double s = 50.0 * std::uniform_real_distribution<double>(0, 1)(gen);
        dfloat sd = df_from_double(s);
        eExp = std::fmax(eExp, std::fabs(as_ld(df_exp_neg(sd)) / std::exp(-as_ld(sd)) - 1));
        const double a = std::uniform_real_distribution<double>(0.05, 5)(gen), b = std::uniform_real_distribution<double>(0.05, 5)(gen);
        dfloat A = df_from_double(a), B = df_from_double(b);
        eDiv = std::fmax(eDiv, std::fabs(as_ld(df_div(A, B)) / (as_ld(A) / as_ld(B)) - 1));
        eSqrt = std::fmax(eSqrt, std::fabs(as_ld(df_sqrt(A)) / std::sqrt(as_ld(A)) - 1));
    }
    printf("erfc_table %.3Le\nerf_table %.3Le\nexp_neg %.3Le\ndiv %.3Le\nsqrt %.3Le\n", eG, eH, eExp, eDiv, eSqrt);
    return 0;
}
