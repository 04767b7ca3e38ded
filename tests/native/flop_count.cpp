// Operation count per interacting pair of the real-space pair kernels, taken from the
// kernel source itself: the per-pair mathematics of mpid_math.cuh is instantiated with
// a number type that counts every arithmetic operation it performs.
//
//   g++ -O0 -std=c++17 -I mpidopenmmplugin_gb300/csrc tests/native/flop_count.cpp -o /tmp/flop_count
//   /tmp/flop_count
//
// Convention: add, sub, mul = 1; an FMA appears as its mul + add = 2; div, sqrt, exp,
// erfc, rint = 1 each (they are also reported separately, as special functions).
// Two representative pairs are counted: alpha r below the near-segment threshold (erf
// part from the Boys-function series and its downward recursion) and above it (erfc
// recursion); the per-pair average weights them by the fraction of pair volume inside a
// 0.9 nm cutoff with alpha = 3.4: r < 1.5 / 3.4 nm holds (0.441 / 0.9)^3 = 11.8 % of the
// pairs.  tests/test_cpu_host.py checks that the averages are the FLOP/pair figures that
// bench.py uses for the roofline.
#include <cmath>
#include <cstdio>

struct Counts {
    long long add = 0, mul = 0, div = 0, special = 0, cmp = 0;
    long long flops() const { return add + mul + div + special; }
};
static Counts g;

struct CF {
    float v;
    CF() : v(0) {}
    CF(double x) : v((float) x) {}
    CF(float x) : v(x) {}
    CF(int x) : v((float) x) {}
    explicit operator float() const { return v; }
    explicit operator double() const { return v; }
};
static inline CF mk(float x) { CF r; r.v = x; return r; }
static inline CF operator+(CF a, CF b) { ++g.add; return mk(a.v + b.v); }
static inline CF operator-(CF a, CF b) { ++g.add; return mk(a.v - b.v); }
static inline CF operator*(CF a, CF b) { ++g.mul; return mk(a.v * b.v); }
static inline CF operator/(CF a, CF b) { ++g.div; return mk(a.v / b.v); }
static inline CF operator-(CF a) { return mk(-a.v); }
static inline CF& operator+=(CF& a, CF b) { ++g.add; a.v += b.v; return a; }
static inline CF& operator-=(CF& a, CF b) { ++g.add; a.v -= b.v; return a; }
static inline CF& operator*=(CF& a, CF b) { ++g.mul; a.v *= b.v; return a; }
static inline CF& operator/=(CF& a, CF b) { ++g.div; a.v /= b.v; return a; }
static inline bool operator<(CF a, CF b) { ++g.cmp; return a.v < b.v; }
static inline bool operator>(CF a, CF b) { ++g.cmp; return a.v > b.v; }
static inline bool operator<=(CF a, CF b) { ++g.cmp; return a.v <= b.v; }
static inline bool operator>=(CF a, CF b) { ++g.cmp; return a.v >= b.v; }
static inline bool operator==(CF a, CF b) { ++g.cmp; return a.v == b.v; }
static inline bool operator!=(CF a, CF b) { ++g.cmp; return a.v != b.v; }
static inline bool operator!(CF a) { return !a.v; }

namespace mpid {
static inline CF m_exp(CF x) { ++g.special; return mk(std::exp(x.v)); }
static inline CF m_sqrt(CF x) { ++g.special; return mk(std::sqrt(x.v)); }
static inline CF m_erfc(CF x) { ++g.special; return mk(std::erfc(x.v)); }
static inline CF m_fabs(CF x) { return mk(std::fabs(x.v)); }
static inline CF m_copysign(CF a, CF b) { return mk(std::copysign(a.v, b.v)); }
static inline CF m_fma(CF a, CF b, CF c) { g.mul++; g.add++; return mk(std::fma(a.v, b.v, c.v)); }
}  // namespace mpid
static inline CF sqrt(CF x) { ++g.special; return mk(std::sqrt(x.v)); }

#include "mpid_math.cuh"

namespace mpid {
template <> struct Prec<CF> {
    static constexpr float kQuadX = 1.5f;
    static constexpr int kBoysTerms = 16;
};
}  // namespace mpid

using namespace mpid;

// Kernel-level work per pair that is not in mpid_math.cuh (mpid_kernels.cuh):
// pair_delta = 3 x (sub, add, mul, rint, fma-sub = 2) = 18; r2 = 5; sqrt = 1;
// the Thole width select and damping product = 2.
static const long long kPairSetup = 18 + 5 + 1 + 2;

static void fill_moments(LabMoments<CF>& m, float s) {
    m.q = CF(0.4f * s);
    for (int k = 0; k < 3; ++k) m.d[k] = CF(0.01f * s * (k + 1));
    for (int k = 0; k < 6; ++k) m.Q[k] = CF(0.002f * s * (k + 1));
    for (int k = 0; k < 10; ++k) m.O[k] = CF(0.0003f * s * (k + 1));
}

template <bool MUTUAL>
static Counts electrostatics_pair(float rr) {
    g = Counts();
    CF d[3] = {CF(rr * 0.6f), CF(rr * 0.48f), CF(rr * 0.64f)};
    CF r = CF(rr);
    LabMoments<CF> mi, mj;
    fill_moments(mi, 1.0f);
    fill_moments(mj, -0.7f);
    CF ui[3] = {CF(0.001f), CF(-0.002f), CF(0.0005f)};
    CF uj[3] = {CF(-0.001f), CF(0.0015f), CF(0.002f)};
    const EwaldAlpha<CF> ew(3.4);
    const Counts before = g;
    PairRadial<CF, 7, 5, MUTUAL ? 3 : 0> pr;
    pair_radial<CF, 7, 5, MUTUAL ? 3 : -1>(r, ew, CF(1.0f), CF(1.3f), CF(0.1f), pr);
    PairOut<CF> po;
    qi_pair<CF, MUTUAL, true>(d, r, mi, mj, ui, uj, false, false, pr.bP, pr.bI, pr.bU, po);
    // accumulation into the i registers and j shared-memory accumulators: 12 adds
    g.add += 12;
    (void) before;
    return g;
}

static Counts dipole_field_pair(float rr) {
    g = Counts();
    CF d[3] = {CF(rr * 0.6f), CF(rr * 0.48f), CF(rr * 0.64f)};
    CF r = CF(rr);
    const EwaldAlpha<CF> ew(3.4);
    PairRadial<CF, 0, 0, 2> pr;
    pair_radial<CF, -1, -1, 2>(r, ew, CF(1.0f), CF(1.3f), CF(0.1f), pr);
    CF b[4] = {CF(0.0f), pr.bU[1], pr.bU[2], CF(0.0f)};
    CF ui[3] = {CF(0.001f), CF(-0.002f), CF(0.0005f)}, uj[3] = {CF(-0.001f), CF(0.0015f), CF(0.002f)};
    CF sI[3] = {-d[0], -d[1], -d[2]};
    CF e[3], gr[6];
    dipole_field<CF, false>(uj, sI, b, e, gr);
    dipole_field<CF, false>(ui, d, b, e, gr);
    g.add += 6;  // accumulation of the two fields
    return g;
}

static Counts fixed_field_pair(float rr) {
    g = Counts();
    CF d[3] = {CF(rr * 0.6f), CF(rr * 0.48f), CF(rr * 0.64f)};
    CF r = CF(rr);
    const EwaldAlpha<CF> ew(3.4);
    PairRadial<CF, 0, 4, 0> pr;
    pair_radial<CF, -1, 4, -1>(r, ew, CF(1.0f), CF(1.3f), CF(0.1f), pr);
    LabMoments<CF> mi, mj;
    fill_moments(mi, 1.0f);
    fill_moments(mj, -0.7f);
    CF sI[3] = {-d[0], -d[1], -d[2]};
    CF E[3];
    multipole_field(mj, sI, pr.bI, E);
    multipole_field(mi, d, pr.bI, E);
    g.add += 6;
    return g;
}

static void report(const char* name, Counts lo, Counts hi) {
    const double wLo = std::pow(1.5 / 3.4 / 0.9, 3.0);
    const double avg = wLo * (lo.flops() + kPairSetup) + (1 - wLo) * (hi.flops() + kPairSetup);
    std::printf("%-22s quad branch %5lld (special %3lld)  erfc branch %5lld (special %3lld)  mean %.0f FLOP/pair\n", name,
                lo.flops() + kPairSetup, lo.special, hi.flops() + kPairSetup, hi.special, avg);
}

int main() {
    report("k_electrostatics mut", electrostatics_pair<true>(0.3f), electrostatics_pair<true>(0.7f));
    report("k_electrostatics", electrostatics_pair<false>(0.3f), electrostatics_pair<false>(0.7f));
    report("k_dipole_field", dipole_field_pair(0.3f), dipole_field_pair(0.7f));
    report("k_fixed_field", fixed_field_pair(0.3f), fixed_field_pair(0.7f));
    return 0;
}
