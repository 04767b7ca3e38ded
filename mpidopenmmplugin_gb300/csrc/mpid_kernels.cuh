// CUDA kernels of the MPIDForce evaluation (sm_103a).  Templated on the arithmetic
// type: float for the mixed-precision path, double for the FP64 path.
//
// Layout in HBM (all per-atom arrays in spatially sorted order, SoA, padded to a
// multiple of 32 so that each 32-atom tile is one warp):
//   off[3][npad]       position minus its tile centre (real)
//   mom[20][npad]      lab-frame q, dipole[3], Q6[6], O10[10] (real)
//   alab[6][npad]      lab-frame polarisability, sroot[6][npad] its square root
//   prm[npad]          (thole, damp, aniso flag, 1/damp or 0) in the arithmetic type; orig[npad]
// Forces, torques and fields accumulate as 64-bit fixed point with 2^32 units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "mpid_math.cuh"
#include "df64.cuh"
#include "cg_radial.h"

namespace mpid {

// Every kernel is written as a device body that takes its block index and block count
// from a KGrid instead of blockIdx.x / gridDim.x, so that the same body runs either as
// a launch of its own (the block index is the hardware one) or as the share of one box
// in a launch over many boxes (the block index is the block's rank within its box; see
// the launch wrappers in mpid_context.cu).  MT and MB are the body's launch bounds
// (maximum threads per block, minimum resident blocks per SM; 0 when it has none).
template <int MT = 0, int MB = 0>
struct KGrid {
    unsigned bx;  // block index within the launch (or within the box)
    unsigned nb;  // blocks of the launch (or of the box)
};
#define MPID_KERNEL __device__ __forceinline__

constexpr double kFixedScale = 4294967296.0;       // 2^32
constexpr double kFixedInv = 1.0 / 4294967296.0;
constexpr double kElectric = 138.935455846;        // MPIDReferenceForce.cpp:38

__device__ __forceinline__ void fx_add(unsigned long long* p, float v) {
    atomicAdd(p, (unsigned long long) __float2ll_rn(v * 4294967296.0f));
}
__device__ __forceinline__ void fx_add(unsigned long long* p, double v) {
    atomicAdd(p, (unsigned long long) __double2ll_rn(v * kFixedScale));
}
__device__ __forceinline__ double fx_get(const unsigned long long* p, int i) {
    return (double) (long long) p[i] * kFixedInv;
}

template <typename real> struct Vec4;
template <> struct Vec4<float> {
    typedef float4 type;
    static __host__ __device__ __forceinline__ float4 make(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
};
template <> struct Vec4<double> {
    typedef double4_16a type;
    static __host__ __device__ __forceinline__ double4_16a make(double a, double b, double c, double d) { return make_double4_16a(a, b, c, d); }
};

// Periodic box in OpenMM's reduced form: rows a = (ax, 0, 0), b = (bx, by, 0),
// c = (cx, cy, cz) with |bx|, |cx| <= ax / 2 and |cy| <= by / 2 (rectangular when the
// off-diagonal entries are 0).
struct BoxDev {
    double L[3], invL[3];    // ax, by, cz and their inverses
    double V[9];             // a, b, c as rows
    double R[3][3];          // reciprocal vectors as the reference stores them (fractional w_j = sum_i x_i R[i][j])
    double A[3][3];          // Cartesian -> fractional grid, frac_j = sum_i A[j][i] x_i = grid_j w_j
    int grid[3];
    int tri;                 // off-diagonal entries present
};

// Minimum image of a displacement in a reduced-form box (c, then b, then a; the order of
// MPIDReferenceForce.cpp:2673-2675).  V: box rows, iL: 1/ax, 1/by, 1/cz.  With a
// rectangular box the off-diagonal products are exact zeros, so the result equals the
// per-axis image.
template <typename real>
__host__ __device__ __forceinline__ void min_image(real* d, const real* V, const real* iL) {
    real s = rint(d[2] * iL[2]);
    d[0] -= s * V[6];
    d[1] -= s * V[7];
    d[2] -= s * V[8];
    s = rint(d[1] * iL[1]);
    d[0] -= s * V[3];
    d[1] -= s * V[4];
    s = rint(d[0] * iL[0]);
    d[0] -= s * V[0];
}

// ---------------------------------------------------------------------------
// Spatial sort into near-cubic 32-atom tiles: the box is cut into x-y columns about
// (32 / density)^(1/3) wide, columns are visited in a snake order, and atoms are sorted
// along z inside each column (ascending in even, descending in odd columns so that a
// tile running past the end of a column continues next to it).  Key: column index above
// zBits bits of quantised z (the radix sort then runs over the bits in use only); the
// value is the atom index.  Atoms of one column closer in z than the quantum keep their
// input order (the sort is stable).
MPID_KERNEL void k_sort_keys(KGrid<> kg, int n, const double* __restrict__ pos, BoxDev box, int ncx, int ncy, int zBits,
                            unsigned* __restrict__ keys, int* __restrict__ vals, double* __restrict__ wpos) {
    int i = kg.bx * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double w[3], x[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    // into [0, ax) x [0, by) x [0, cz): c, then b, then a (a lattice translation)
    for (int k = 2; k >= 0; --k) {
        double f = floor(x[k] * box.invL[k]);
        if (x[k] - f * box.L[k] >= box.L[k]) f += 1.0;  // rounding at the upper edge
        for (int q = 0; q <= k; ++q) x[q] -= f * box.V[3 * k + q];
    }
    for (int k = 0; k < 3; ++k) {
        wpos[3 * i + k] = x[k];
        w[k] = x[k] * box.invL[k];
    }
    int cx = min(ncx - 1, (int) (w[0] * ncx));
    int cy = min(ncy - 1, (int) (w[1] * ncy));
    if (cx & 1) cy = ncy - 1 - cy;  // snake through the columns
    const unsigned int col = (unsigned int) (cx * ncy + cy);
    double zf = (col & 1) ? 1.0 - w[2] : w[2];
    const unsigned int zq = (unsigned int) fmin(4294967295.0, zf * 4294967296.0);
    keys[i] = (col << zBits) | (zq >> (32 - zBits));
    vals[i] = i;
}

// The same order as the radix sort of (key, atom index) pairs, for one box of at most
// kBlockSortMax atoms in one block of 1024 threads: a bitonic sort of the 64-bit words
// key << 32 | index in shared memory (keys are distinct once the index is appended, so
// any correct sort gives the stable order).  Used where many boxes are set up in one
// launch, one block per box.
constexpr int kBlockSortMax = 4096;
MPID_KERNEL void k_sort_block(KGrid<1024> kg, int n, const unsigned* __restrict__ keys, const int* __restrict__ vals,
                              int* __restrict__ order) {
    __shared__ unsigned long long s[kBlockSortMax];
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x)
        s[i] = i < n ? ((unsigned long long) keys[i] << 32) | (unsigned) vals[i] : ~0ull;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned long long a = s[i], b = s[l];
                    if ((a > b) == ((i & k) == 0)) {
                        s[i] = b;
                        s[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) order[i] = (int) (unsigned) s[i];
}

// No-cutoff systems keep the caller's order.
MPID_KERNEL void k_identity_order(KGrid<> kg, int n, const double* __restrict__ pos, int* __restrict__ order,
                                 double* __restrict__ wpos) {
    const int i = kg.bx * blockDim.x + threadIdx.x;
    if (i >= n) return;
    order[i] = i;
    for (int k = 0; k < 3; ++k) wpos[3 * i + k] = pos[3 * i + k];
}

// Tile centres and half extents from the wrapped positions of the sorted atoms: one warp
// per tile, one lane per atom, minima and maxima by shuffles.
MPID_KERNEL void k_tile_bounds(KGrid<> kg, int n, int ntiles, const int* __restrict__ order,
                              const double* __restrict__ wpos, double* __restrict__ center,
                              double* __restrict__ half, float4* __restrict__ centerF, float4* __restrict__ halfF) {
    const int t = (kg.bx * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (t >= ntiles) return;  // whole warps
    const int s = t * 32 + lane;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    if (s < n) {
        const int i = order[s];
        for (int k = 0; k < 3; ++k) lo[k] = hi[k] = wpos[3 * i + k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fmin(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmax(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    if (lane < 3) {
        const double l = lane == 0 ? lo[0] : (lane == 1 ? lo[1] : lo[2]);
        const double h = lane == 0 ? hi[0] : (lane == 1 ? hi[1] : hi[2]);
        center[3 * t + lane] = 0.5 * (l + h);
        half[3 * t + lane] = 0.5 * (h - l);
    }
    if (lane == 0) {
        centerF[t] = make_float4((float) (0.5 * (lo[0] + hi[0])), (float) (0.5 * (lo[1] + hi[1])),
                                 (float) (0.5 * (lo[2] + hi[2])), 0.f);
        halfF[t] = make_float4((float) (0.5 * (hi[0] - lo[0])), (float) (0.5 * (hi[1] - lo[1])),
                               (float) (0.5 * (hi[2] - lo[2])), 0.f);
    }
}

// ---------------------------------------------------------------------------
// Neighbour lists.  Real-space work is organised per 32-atom tile I (one warp):
//  * tile list: the tiles J whose bounding boxes come within the list cutoff of I's, in
//    ascending order, with the minimum-image shift of the tile centres (float and double)
//    and a flag when a dimension is so short against the cutoff that each pair must be
//    imaged on its own;
//  * atom lists: for every atom (lane) the atoms j within the list cutoff, both
//    directions (each pair appears in the lists of both atoms), lane-interleaved
//    [tile][entry][lane] so that a warp reads 128 contiguous bytes per entry.
// An entry is (slot << 7) | (flag << 5) | jlane: slot indexes I's tile list, jlane is
// j's lane in that tile, flag is 0 for covalent scale 1, 1 for scale 0, 2 for any other
// scale (looked up again by the kernel).  Every lane's entries run over J tiles in
// ascending order and jlane ascending, so the lists and all sums over them are
// reproducible.

// Bounding-box test of tiles I and J.  A dimension whose extents plus the cutoff reach
// half the box always counts as overlapping and marks the pair for per-pair imaging
// (`wrap`); in a triclinic box the boxes are tested at every lattice image next to the
// minimum image of the centres, and every hit is imaged pair by pair.
__device__ __forceinline__ bool tile_pair_hit(int J, const float* cI, const float* hI,
                                              const float4* __restrict__ centerF, const float4* __restrict__ halfF,
                                              const BoxDev& box, double cutoff, int usePbc, bool& wrap) {
    const float4 cJ = centerF[J], hJ = halfF[J];
    const float cJv[3] = {cJ.x, cJ.y, cJ.z}, hJv[3] = {hJ.x, hJ.y, hJ.z};
    const float cut = (float) cutoff * 1.0001f + 1e-4f;  // margin far above the float rounding
    wrap = false;
    if (usePbc && box.tri) {
        float Vf[9], iLf[3];
        for (int q = 0; q < 9; ++q) Vf[q] = (float) box.V[q];
        for (int q = 0; q < 3; ++q) iLf[q] = (float) box.invL[q];
        float dc[3], ext[3];
        for (int k = 0; k < 3; ++k) {
            dc[k] = cJv[k] - cI[k];
            ext[k] = hI[k] + hJv[k];
        }
        min_image(dc, Vf, iLf);
        float best = 3.0e38f;
        for (int ia = -1; ia <= 1; ++ia)
            for (int ib = -1; ib <= 1; ++ib)
                for (int ic = -1; ic <= 1; ++ic) {
                    const float v[3] = {dc[0] + ia * Vf[0] + ib * Vf[3] + ic * Vf[6], dc[1] + ib * Vf[4] + ic * Vf[7],
                                        dc[2] + ic * Vf[8]};
                    float d2 = 0.f;
                    for (int k = 0; k < 3; ++k) {
                        const float g = fabsf(v[k]) - ext[k];
                        if (g > 0.f) d2 += g * g;
                    }
                    best = fminf(best, d2);
                }
        wrap = true;
        return best < cut * cut;
    }
    float d2 = 0.f;
    for (int k = 0; k < 3; ++k) {
        const float Lk = (float) box.L[k];
        float dc = cJv[k] - cI[k];
        const float ext = hI[k] + hJv[k];
        bool always = false;
        if (usePbc) {
            always = ext + cut >= 0.5f * Lk;
            wrap = wrap || always;
            dc -= Lk * rintf(dc * (float) box.invL[k]);
        }
        const float g = fabsf(dc) - ext;
        if (!always && g > 0.f) d2 += g * g;
    }
    return d2 < cut * cut;
}

// One block of kTileListWarps warps per tile I; warp w scans the w-th contiguous range of
// tiles J.  A first pass counts each warp's hits, a prefix sum over the warps gives their
// offsets, and a second pass writes the hits in ascending J (an ordered ballot compaction
// within each warp), so the list order is deterministic.
constexpr int kTileListWarps = 8;

MPID_KERNEL void k_tile_list(KGrid<(32 * kTileListWarps)> kg, int ntiles, const double* __restrict__ center, const float4* __restrict__ centerF,
            const float4* __restrict__ halfF, BoxDev box, double cutoff, int usePbc, int tcap, int* __restrict__ tileCount, int* __restrict__ tileJ,
            float4* __restrict__ shF, double* __restrict__ shD, float2* __restrict__ shDF,
            int* __restrict__ maxTiles) {
    __shared__ int wcount[kTileListWarps];
    const int I = kg.bx, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (I >= ntiles) return;  // whole blocks
    const float4 cI4 = centerF[I], hI4 = halfF[I];
    const float cI[3] = {cI4.x, cI4.y, cI4.z}, hI[3] = {hI4.x, hI4.y, hI4.z};
    const int span = (ntiles + kTileListWarps - 1) / kTileListWarps;
    const int j0 = min(ntiles, w * span), j1 = min(ntiles, j0 + span);
    int count = 0;
    for (int J0 = j0; J0 < j1; J0 += 32) {
        const int J = J0 + lane;
        bool wrap = false;
        const bool hit = J < j1 && tile_pair_hit(J, cI, hI, centerF, halfF, box, cutoff, usePbc, wrap);
        count += __popc(__ballot_sync(0xffffffffu, hit));
    }
    if (lane == 0) wcount[w] = count;
    __syncthreads();
    int base = 0, total = 0;
    for (int v = 0; v < kTileListWarps; ++v) {
        if (v < w) base += wcount[v];
        total += wcount[v];
    }
    for (int J0 = j0; J0 < j1; J0 += 32) {
        const int J = J0 + lane;
        bool wrap = false;
        const bool hit = J < j1 && tile_pair_hit(J, cI, hI, centerF, halfF, box, cutoff, usePbc, wrap);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int pos = base + __popc(m & ((1u << lane) - 1u));
            if (pos < tcap) {
                // minimum-image shift of the centres in FP64
                double sh[3];
                for (int k = 0; k < 3; ++k) sh[k] = center[3 * J + k] - center[3 * I + k];
                if (usePbc) {
                    if (box.tri)
                        min_image(sh, box.V, box.invL);
                    else
                        for (int k = 0; k < 3; ++k) sh[k] -= box.L[k] * rint(sh[k] * box.invL[k]);
                }
                const size_t s = (size_t) I * tcap + pos;
                const int code = J | (wrap ? (int) 0x80000000 : 0);
                tileJ[s] = code;
                shF[s] = make_float4((float) sh[0], (float) sh[1], (float) sh[2], __int_as_float(code));
                for (int k = 0; k < 3; ++k) {
                    shD[3 * s + k] = sh[k];
                    const dfloat v = df_from_double(sh[k]);
                    shDF[3 * s + k] = make_float2(v.hi, v.lo);
                }
            }
        }
        base += __popc(m);
    }
    if (threadIdx.x == 0) {
        tileCount[I] = min(total, tcap);
        atomicMax(maxTiles, total);
    }
}

// ---------------------------------------------------------------------------
// Per-atom parameters in sorted order: lab frame, polarisability and its square root.
template <typename real>
struct AtomArrays {
    int n, npad;
    real* off;       // [3][npad]
    real* mom;       // [20][npad]
    real* alab;      // [6][npad]
    real* sroot;     // [6][npad]
    typename Vec4<real>::type* prm;  // thole, damp, aniso, 0
    int* orig;       // [npad], -1 for padding
    int* rank;       // [n]  sorted slot of each original atom
};

struct MolArrays {  // original order, FP64, as given through the API
    const double* charge;
    const double* dipole;
    const double* quad;
    const double* oct;
    const double* thole;
    const double* pol;
    const int* axis;
    const int* az;
    const int* ax;
    const int* ay;
};

template <typename real>
MPID_KERNEL void k_gather_atoms(KGrid<> kg, int n, int npad, const int* __restrict__ order, MolArrays mol,
                               const double* __restrict__ pos, const double* __restrict__ wpos,
                               const double* __restrict__ center, AtomArrays<real> at, double* __restrict__ mom64,
                               double* __restrict__ prm64) {
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    if (s >= n) {
        for (int k = 0; k < 3; ++k) at.off[k * npad + s] = real(0);
        for (int k = 0; k < 20; ++k) at.mom[k * npad + s] = real(0);
        for (int k = 0; k < 6; ++k) { at.alab[k * npad + s] = real(0); at.sroot[k * npad + s] = real(0); }
        at.prm[s] = Vec4<real>::make(real(0), real(0), real(0), real(0));
        at.orig[s] = -1;
        if (mom64)
            for (int k = 0; k < 20; ++k) mom64[k * npad + s] = 0.0;
        return;
    }
    const int i = order[s];
    at.orig[s] = i;
    at.rank[i] = s;
    const int t = s >> 5;
    for (int k = 0; k < 3; ++k) at.off[k * npad + s] = real(wpos[3 * i + k] - center[3 * t + k]);
    MolParams<double> p;
    p.q = mol.charge[i];
    for (int k = 0; k < 3; ++k) p.d[k] = mol.dipole[3 * i + k];
    for (int k = 0; k < 6; ++k) p.Q[k] = mol.quad[6 * i + k];
    for (int k = 0; k < 10; ++k) p.O[k] = mol.oct[10 * i + k];
    for (int k = 0; k < 3; ++k) p.pol[k] = mol.pol[3 * i + k];
    const int ax = mol.axis[i], iz = mol.az[i], ix = mol.ax[i], iy = mol.ay[i];
    const double* pI = pos + 3 * i;
    const double* pZ = (iz >= 0 && iz < n) ? pos + 3 * iz : pI;
    const double* pX = (ix >= 0 && ix < n) ? pos + 3 * ix : pI;
    const double* pY = (iy >= 0 && iy < n) ? pos + 3 * iy : pI;
    double R[3][3];
    local_frame<double>(ax, pI, pZ, pX, pY, R);
    const bool flip = chiral_flip<double>(ax, iy >= 0, pI, pZ, pX, pY);
    LabMoments<double> L;
    double al[6];
    rotate_to_lab(p, R, flip, L, al);
    if (mom64) {
        mom64[s] = L.q;
        for (int k = 0; k < 3; ++k) mom64[(1 + k) * npad + s] = L.d[k];
        for (int k = 0; k < 6; ++k) mom64[(4 + k) * npad + s] = L.Q[k];
        for (int k = 0; k < 10; ++k) mom64[(10 + k) * npad + s] = L.O[k];
    }
    at.mom[s] = real(L.q);
    for (int k = 0; k < 3; ++k) at.mom[(1 + k) * npad + s] = real(L.d[k]);
    for (int k = 0; k < 6; ++k) at.mom[(4 + k) * npad + s] = real(L.Q[k]);
    for (int k = 0; k < 10; ++k) at.mom[(10 + k) * npad + s] = real(L.O[k]);
    for (int k = 0; k < 6; ++k) at.alab[k * npad + s] = real(al[k]);
    for (int a = 0; a < 3; ++a)
        for (int b = a; b < 3; ++b) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc += R[k][a] * R[k][b] * sqrt(fmax(p.pol[k], 0.0));
            at.sroot[q6(a, b) * npad + s] = real(acc);
        }
    const bool aniso = p.pol[0] != p.pol[1] || p.pol[0] != p.pol[2];
    const double damp = pow((p.pol[0] + p.pol[1] + p.pol[2]) / 3.0, 1.0 / 6.0);
    at.prm[s] = Vec4<real>::make(real(mol.thole[i]), real(damp), aniso ? real(1) : real(0),
                                 real(damp > 0.0 ? 1.0 / damp : 0.0));
    if (prm64) {
        prm64[2 * i] = mol.thole[i];
        prm64[2 * i + 1] = damp;
    }
}

template <typename real>
__device__ __forceinline__ void load_moments(const real* mom, int npad, int s, LabMoments<real>& m) {
    m.q = mom[s];
#pragma unroll
    for (int k = 0; k < 3; ++k) m.d[k] = mom[(1 + k) * npad + s];
#pragma unroll
    for (int k = 0; k < 6; ++k) m.Q[k] = mom[(4 + k) * npad + s];
#pragma unroll
    for (int k = 0; k < 10; ++k) m.O[k] = mom[(10 + k) * npad + s];
}

// Covalent scale of an (original-index) pair from the symmetric partner list.
__device__ __forceinline__ double pair_scale(int oi, int oj, const int* __restrict__ covOff,
                                             const int* __restrict__ covJ, const double* __restrict__ covS) {
    const int b = covOff[oi], e = covOff[oi + 1];
    for (int k = b; k < e; ++k)
        if (covJ[k] == oj) return covS[k];
    return 1.0;
}

// Flag of a covalent scale as stored in list entries.
__device__ __forceinline__ unsigned scale_flag(double sc) { return sc == 1.0 ? 0u : (sc == 0.0 ? 1u : 2u); }

// Atom lists: one block of kListWarps warps per tile I; warp w scans a contiguous range
// of I's tile list, each lane testing the 32 atoms of every J tile in the range (float
// arithmetic; cutoff2 includes a small skin so that both the FP32 and the FP64 kernels,
// which apply the exact cutoff, see every pair).  Each lane's list has two segments so
// that the pair kernels never mix the two radial branches in a warp: the erfc segment
// grows from the front (count nL), the quadrature segment (alpha r below the threshold,
// r2 < quadR2, or covalent scale 0 under PME) from the back (nS).  A first pass counts
// per warp, a second writes at the lane's running offset, so the entries of every lane
// are in ascending J order (and ascending j).
constexpr int kListWarps = 8;

// Covalent partners of an atom as bit masks over the 32 atoms of tile J: m1 the partners
// of scale 0 (entry flag 1), m2 those of any other scale but 1 (flag 2).  pS holds the
// sorted slots of the first kCache partners (-1 for none), pF their flags (2 bits each);
// the partners beyond those are read from covJ.
template <int kCache>
__device__ __forceinline__ void partner_masks(int J, const int* pS, unsigned pF, int rest0, int rest1,
                                              const int* __restrict__ covJ, const double* __restrict__ covS,
                                              const int* __restrict__ rank, unsigned& m1, unsigned& m2) {
    m1 = 0u;
    m2 = 0u;
#pragma unroll
    for (int k = 0; k < kCache; ++k)
        if ((pS[k] >> 5) == J) {
            const unsigned b = 1u << (pS[k] & 31), f = (pF >> (2 * k)) & 3u;
            if (f == 1u) m1 |= b;
            else if (f == 2u) m2 |= b;
        }
    for (int k = rest0; k < rest1; ++k) {
        const int sp = rank[covJ[k]];
        if ((sp >> 5) == J) {
            const unsigned f = scale_flag(covS[k]), b = 1u << (sp & 31);
            if (f == 1u) m1 |= b;
            else if (f == 2u) m2 |= b;
        }
    }
}

template <typename real>
MPID_KERNEL void k_atom_list(KGrid<(32 * kListWarps), 3> kg, int ntiles, int npad, const real* __restrict__ off, const int* __restrict__ orig,
            const int* __restrict__ rank, BoxDev box, float cutoff2, float quadR2, int usePme, int tcap,
            const int* __restrict__ tileCount, const int* __restrict__ tileJ, const float4* __restrict__ shF,
            const int* __restrict__ covOff, const int* __restrict__ covJ, const double* __restrict__ covS, int cap,
            int* __restrict__ countL, int* __restrict__ countS, int* __restrict__ loL, int* __restrict__ loS,
            int* __restrict__ tmaxL, int* __restrict__ tmaxS, unsigned* __restrict__ list, int* __restrict__ maxCounts) {
    constexpr int kCache = 8;
    constexpr int kMasks = 16;  // tile pairs per warp whose hits the first pass keeps for the second
    __shared__ int cnt[kListWarps][4][32];  // nL, nS, lowL, lowS per warp and lane
    __shared__ unsigned hits[kListWarps][kMasks][32], near[kListWarps][kMasks][32];
    __shared__ float4 jat[kListWarps][32];  // the current J tile: offset and original index of each atom
    const int I = kg.bx, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (I >= ntiles) return;
    const int si = I * 32 + lane;
    const float oi[3] = {(float) off[si], (float) off[npad + si], (float) off[2 * npad + si]};
    const int origI = orig[si];
    const float iL[3] = {(float) box.invL[0], (float) box.invL[1], (float) box.invL[2]};
    float Vb[9];
    for (int q = 0; q < 9; ++q) Vb[q] = (float) box.V[q];
    // covalent partners of this atom by sorted slot: the first kCache in registers
    int cb = 0, ce = 0;
    if (origI >= 0) { cb = covOff[origI]; ce = covOff[origI + 1]; }
    const int ncached = min(ce - cb, kCache);
    int pS[kCache];
    unsigned pF = 0u;
#pragma unroll
    for (int k = 0; k < kCache; ++k) {
        pS[k] = k < ncached ? rank[covJ[cb + k]] : -1;
        if (k < ncached) pF |= scale_flag(covS[cb + k]) << (2 * k);
    }
    const int rest0 = cb + ncached, rest1 = ce;
    const int nt = tileCount[I];
    const int s0 = (w * nt) / kListWarps, s1 = ((w + 1) * nt) / kListWarps;
    unsigned* out = list + (size_t) I * cap * 32 + lane;
    int baseL = 0, baseS = 0;
    bool fits = true;
    for (int pass = 0; pass < 2; ++pass) {
        int nL = 0, nS = 0, lowL = 0, lowS = 0;
        for (int s = s0; s < s1; ++s) {
            const int Jw = tileJ[(size_t) I * tcap + s];
            const int J = Jw & 0x7fffffff;
            unsigned m1, m2;
            partner_masks<kCache>(J, pS, pF, rest0, rest1, covJ, covS, rank, m1, m2);
            if (pass == 1 && s - s0 < kMasks) {
                // second pass over a kept tile pair: only its hits, in the same order
                if (!fits) continue;
                unsigned m = hits[w][s - s0][lane];
                const unsigned q = near[w][s - s0][lane];
                while (m) {
                    const int jl = __ffs(m) - 1;
                    m &= m - 1;
                    const unsigned flag = ((m1 >> jl) & 1u) ? 1u : (((m2 >> jl) & 1u) ? 2u : 0u);
                    const bool quad = usePme && (((q >> jl) & 1u) || flag == 1u);
                    const unsigned code = ((unsigned) s << 7) | (flag << 5) | (unsigned) jl;
                    out[(size_t) (quad ? cap - 1 - (baseS + nS) : baseL + nL) * 32] = code;
                    if (quad) ++nS; else ++nL;
                }
                continue;
            }
            unsigned hitMask = 0, nearMask = 0;
            const bool wrap = Jw < 0;
            const float4 sh = shF[(size_t) I * tcap + s];
            const int sj = J * 32 + lane;
            __syncwarp();
            jat[w][lane] = make_float4((float) off[sj], (float) off[npad + sj], (float) off[2 * npad + sj],
                                       __int_as_float(orig[sj]));
            __syncwarp();
            for (int jl = 0; jl < 32; ++jl) {
                const float4 aj = jat[w][jl];
                float d[3] = {sh.x + (aj.x - oi[0]), sh.y + (aj.y - oi[1]), sh.z + (aj.z - oi[2])};
                const int oj = __float_as_int(aj.w);
                if (wrap) min_image(d, Vb, iL);
                const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                if (origI < 0 || oj < 0 || r2 >= cutoff2 || (J == I && jl == lane)) continue;
                const unsigned flag = ((m1 >> jl) & 1u) ? 1u : (((m2 >> jl) & 1u) ? 2u : 0u);
                const bool quad = usePme && (r2 < quadR2 || flag == 1u);
                if (pass == 1 && fits) {
                    const unsigned code = ((unsigned) s << 7) | (flag << 5) | (unsigned) jl;
                    out[(size_t) (quad ? cap - 1 - (baseS + nS) : baseL + nL) * 32] = code;
                }
                hitMask |= 1u << jl;
                if (r2 < quadR2) nearMask |= 1u << jl;
                const int low = J * 32 + jl < si;
                if (quad) { ++nS; lowS += low; } else { ++nL; lowL += low; }
            }
            if (pass == 0 && s - s0 < kMasks) {
                hits[w][s - s0][lane] = hitMask;
                near[w][s - s0][lane] = nearMask;
            }
        }
        if (pass == 0) {
            cnt[w][0][lane] = nL;
            cnt[w][1][lane] = nS;
            cnt[w][2][lane] = lowL;
            cnt[w][3][lane] = lowS;
            __syncthreads();
            int tL = 0, tS = 0;
            for (int v = 0; v < kListWarps; ++v) {
                if (v == w) { baseL = tL; baseS = tS; }
                tL += cnt[v][0][lane];
                tS += cnt[v][1][lane];
            }
            fits = tL + tS <= cap;
        }
    }
    if (w == 0) {
        int nL = 0, nS = 0, lowL = 0, lowS = 0;
        for (int v = 0; v < kListWarps; ++v) {
            nL += cnt[v][0][lane];
            nS += cnt[v][1][lane];
            lowL += cnt[v][2][lane];
            lowS += cnt[v][3][lane];
        }
        countL[si] = nL;
        countS[si] = nS;
        loL[si] = lowL;
        loS[si] = lowS;
        int mt = nL + nS, ml = nL, ms = nS;
        for (int o = 16; o > 0; o >>= 1) {
            mt = max(mt, __shfl_xor_sync(0xffffffffu, mt, o));
            ml = max(ml, __shfl_xor_sync(0xffffffffu, ml, o));
            ms = max(ms, __shfl_xor_sync(0xffffffffu, ms, o));
        }
        if (lane == 0) {
            tmaxL[I] = ml;
            tmaxS[I] = ms;
            atomicMax(maxCounts, mt);
            atomicMax(maxCounts + 1, ml);
            atomicMax(maxCounts + 2, ms);
        }
    }
}

// Pair constants of one arithmetic type, computed on the host (no FP64 in FP32 loops).
template <typename real>
struct PairConsts {
    real L[3], iL[3];
    real V[9];      // box rows (reduced form)
    real rc2;       // exact cutoff squared
    real thole;     // default Thole width
    EwaldAlpha<real> ew;
};

// Neighbour lists and pair constants as the pair kernels see them.
struct NbrList {
    int ntiles, tcap, cap, chunk;
    int nchunksL, nchunksS;   // work items per tile over the erfc / quadrature segments
    const int* tileJ;
    const float4* shF;
    const double* shD;
    const float2* shDF;       // the same shifts as double-float
    const int* countL;
    const int* countS;
    const int* loL;           // entries with j < i at the head of each segment
    const int* loS;
    const int* tmaxL;
    const int* tmaxS;
    const unsigned* list;
    int usePbc;
    int split;                // sub-ranges per work item (PairTask::init), a power of two dividing chunk
    PairConsts<float> cf;
    PairConsts<double> cd;
    const int* covOff;
    const int* covJ;
    const double* covS;
};

template <typename real> __device__ __forceinline__ const PairConsts<real>& pair_consts(const NbrList& nl);
template <> __device__ __forceinline__ const PairConsts<float>& pair_consts<float>(const NbrList& nl) { return nl.cf; }
template <> __device__ __forceinline__ const PairConsts<double>& pair_consts<double>(const NbrList& nl) { return nl.cd; }

// Work item of a pair kernel: entries [k0, k0 + chunk) of one segment of the lists of
// tile I.  quad is uniform over the warp.
struct PairTask {
    int I, k0, k1, lane, si;
    bool quad;
    __device__ __forceinline__ int tasks(const NbrList& nl) const {
        return nl.ntiles * (nl.nchunksL + nl.nchunksS) * nl.split;
    }
    // Work items: all erfc-segment items (tile-major), then all quadrature-segment items,
    // so that resident warps mostly run the same branch of the code.
    __device__ __forceinline__ bool init(const NbrList& nl, unsigned bx) { return init_split(nl, nl.split, bx); }
    // The same items, each cut into `split` consecutive sub-ranges of chunk / split
    // entries (split divides the chunk), one warp per sub-range: more warps for kernels
    // whose per-pair work is long (the FP64 gradient passes of small systems).
    __device__ __forceinline__ bool init_split(const NbrList& nl, int split, unsigned bx) {
        const int w = (bx * blockDim.x + threadIdx.x) >> 5;
        const int item = w / split, part = w - item * split;
        const int nLong = nl.ntiles * nl.nchunksL;
        lane = threadIdx.x & 31;
        quad = item >= nLong;
        const int wq = quad ? item - nLong : item, nch = quad ? nl.nchunksS : nl.nchunksL;
        I = nch > 0 ? wq / nch : nl.ntiles;
        const int span = nl.chunk / split;
        k0 = (wq - I * nch) * nl.chunk + part * span;
        si = I * 32 + lane;
        if (I >= nl.ntiles || k0 >= (quad ? nl.tmaxS[I] : nl.tmaxL[I])) return false;
        k1 = min(k0 + span, quad ? nl.countS[si] : nl.countL[si]);
        return true;
    }
};

template <typename real>
__device__ __forceinline__ void tile_shift(const NbrList& nl, size_t s, real* sh);
template <>
__device__ __forceinline__ void tile_shift<float>(const NbrList& nl, size_t s, float* sh) {
    const float4 v = nl.shF[s];
    sh[0] = v.x; sh[1] = v.y; sh[2] = v.z;
}
template <>
__device__ __forceinline__ void tile_shift<double>(const NbrList& nl, size_t s, double* sh) {
    sh[0] = nl.shD[3 * s]; sh[1] = nl.shD[3 * s + 1]; sh[2] = nl.shD[3 * s + 2];
}

// Decode entry k of lane `lane` in segment QUAD of tile I into j's sorted index, the
// displacement d = R_j - R_i and r^2; returns false for pairs beyond the cutoff.
template <typename real, bool QUAD>
__device__ __forceinline__ bool list_pair(const NbrList& nl, const PairConsts<real>& pc, const AtomArrays<real>& at,
                                          int I, int k, int lane, const real* oi, int& sj, unsigned& flag, real* d,
                                          real& r2) {
    const int pos = QUAD ? nl.cap - 1 - k : k;
    const unsigned code = nl.list[((size_t) I * nl.cap + pos) * 32 + lane];
    const size_t s = (size_t) I * nl.tcap + (code >> 7);
    const int Jw = nl.tileJ[s];
    sj = (Jw & 0x7fffffff) * 32 + (int) (code & 31u);
    flag = (code >> 5) & 3u;
    real sh[3];
    tile_shift<real>(nl, s, sh);
    const int npad = at.npad;
#pragma unroll
    for (int q = 0; q < 3; ++q) d[q] = sh[q] + (at.off[q * npad + sj] - oi[q]);
    if (Jw < 0) min_image(d, pc.V, pc.iL);
    r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    return !(nl.usePbc && r2 > pc.rc2);
}

template <typename real>
__device__ __forceinline__ real list_scale(const NbrList& nl, unsigned flag, int origI, int origJ) {
    return flag == 0u ? real(1) : (flag == 1u ? real(0) : (real) pair_scale(origI, origJ, nl.covOff, nl.covJ, nl.covS));
}

constexpr int kWarpsPerBlock = 4;

// ---------------------------------------------------------------------------
// Real-space permanent field at every atom (kernel K_i with the pair's covalent scale):
// the PME real-space part of MPIDReferenceForce.cpp:2812-2920 / :911-934.
template <typename real, bool QUAD>
__device__ __forceinline__ void fixed_field_loop(const NbrList& nl, const AtomArrays<real>& at, const PairTask& t,
                                                 int origI, real* Ei) {
    const PairConsts<real>& pc = pair_consts<real>(nl);
    const int npad = at.npad, si = t.si;
    const real oi[3] = {at.off[si], at.off[npad + si], at.off[2 * npad + si]};
    const typename Vec4<real>::type pi = at.prm[si];
    for (int k = t.k0; k < t.k1; ++k) {
        int sj;
        unsigned flag;
        real d[3], r2;
        if (!list_pair<real, QUAD>(nl, pc, at, t.I, k, t.lane, oi, sj, flag, d, r2)) continue;
        const real r = sqrt(r2);
        const real scale = list_scale<real>(nl, flag, origI, at.orig[sj]);
        const typename Vec4<real>::type pj = at.prm[sj];
        const real a = scale == real(0) ? pi.x + pj.x : pc.thole;
        PairRadial<real, 0, 4, 0> pr;
        pair_radial_branch<real, -1, 4, -1, QUAD>(r, pc.ew, scale, a, pi.y * pj.y, pr);
        LabMoments<real> mj;
        load_moments(at.mom, npad, sj, mj);
        const real sI[3] = {-d[0], -d[1], -d[2]};
        real e[3];
        multipole_field(mj, sI, pr.bI, e);
        Ei[0] += e[0]; Ei[1] += e[1]; Ei[2] += e[2];
    }
}

template <typename real>
MPID_KERNEL void k_fixed_field(KGrid<(32 * kWarpsPerBlock)> kg, NbrList nl, AtomArrays<real> at, unsigned long long* __restrict__ field) {
    PairTask t;
    if (!t.init(nl, kg.bx)) return;
    const int origI = at.orig[t.si];
    if (origI < 0) return;
    real Ei[3] = {real(0), real(0), real(0)};
    if (t.quad)
        fixed_field_loop<real, true>(nl, at, t, origI, Ei);
    else
        fixed_field_loop<real, false>(nl, at, t, origI, Ei);
    for (int q = 0; q < 3; ++q) fx_add(field + q * at.npad + t.si, Ei[q]);
}

// Real-space field of point dipoles (kernel K_u), optionally with its gradient:
// MPIDReferenceForce.cpp:4161-4281.  mu is [3][npad] in sorted order.
// HALF: only the pairs with j > i, whose field at j is added with fixed-point atomics
// (half the pair evaluations; used by the FP64 kernels, where arithmetic dominates).
template <typename real, bool GRAD, bool QUAD, bool HALF>
__device__ __forceinline__ void dipole_field_loop(const NbrList& nl, const AtomArrays<real>& at, const real* mu,
                                                  const PairTask& t, real* acc, unsigned long long* field,
                                                  unsigned long long* grad) {
    const PairConsts<real>& pc = pair_consts<real>(nl);
    const int npad = at.npad, si = t.si;
    const real oi[3] = {at.off[si], at.off[npad + si], at.off[2 * npad + si]};
    const real ui[3] = {mu[si], mu[npad + si], mu[2 * npad + si]};
    const typename Vec4<real>::type pi = at.prm[si];
    const int kb = HALF ? max(t.k0, QUAD ? nl.loS[si] : nl.loL[si]) : t.k0;
    for (int k = kb; k < t.k1; ++k) {
        int sj;
        unsigned flag;
        real d[3], r2;
        if (!list_pair<real, QUAD>(nl, pc, at, t.I, k, t.lane, oi, sj, flag, d, r2)) continue;
        const real r = sqrt(r2);
        const typename Vec4<real>::type pj = at.prm[sj];
        const real a = flag == 1u ? pi.x + pj.x : pc.thole;  // flag 1: covalent scale 0
        PairRadial<real, 0, 0, GRAD ? 3 : 2> pr;
        pair_radial_branch<real, -1, -1, GRAD ? 3 : 2, QUAD>(r, pc.ew, real(1), a, pi.y * pj.y, pr);
        const real b[4] = {real(0), pr.bU[1], pr.bU[2], GRAD ? pr.bU[GRAD ? 3 : 2] : real(0)};
        const real uj[3] = {mu[sj], mu[npad + sj], mu[2 * npad + sj]};
        const real sI[3] = {-d[0], -d[1], -d[2]};
        real e[3], gr[6];
        dipole_field<real, GRAD>(uj, sI, b, e, gr);
#pragma unroll
        for (int q = 0; q < 3; ++q) acc[q] += e[q];
        if (GRAD)
#pragma unroll
            for (int q = 0; q < 6; ++q) acc[3 + q] += gr[q];
        if (HALF) {
            dipole_field<real, GRAD>(ui, d, b, e, gr);
            for (int q = 0; q < 3; ++q) fx_add(field + q * npad + sj, e[q]);
            if (GRAD)
                for (int q = 0; q < 6; ++q) fx_add(grad + q * npad + sj, gr[q]);
        }
    }
}

template <typename real, bool GRAD, bool HALF>
MPID_KERNEL void k_dipole_field(KGrid<(32 * kWarpsPerBlock)> kg, NbrList nl, AtomArrays<real> at, const real* __restrict__ mu, unsigned long long* __restrict__ field,
               unsigned long long* __restrict__ grad, const int* __restrict__ skip) {
    if (skip && *skip) return;
    PairTask t;
    if (!t.init(nl, kg.bx)) return;
    if (at.orig[t.si] < 0) return;
    constexpr int NACC = GRAD ? 9 : 3;
    real acc[NACC];
#pragma unroll
    for (int q = 0; q < NACC; ++q) acc[q] = real(0);
    if (t.quad)
        dipole_field_loop<real, GRAD, true, HALF>(nl, at, mu, t, acc, field, grad);
    else
        dipole_field_loop<real, GRAD, false, HALF>(nl, at, mu, t, acc, field, grad);
    const int npad = at.npad;
    for (int q = 0; q < 3; ++q) fx_add(field + q * npad + t.si, acc[q]);
    if (GRAD)
        for (int q = 0; q < 6; ++q) fx_add(grad + q * npad + t.si, acc[3 + q]);
}

// FP32 T.mu of the CG iterations: the induced-induced kernel K_u with the Thole width of
// the pair (MPIDReferenceForce.cpp:4161-4281), with the radial functions of cg_radial.h
// (one exponential and one polynomial for the Ewald part, 1/r from rsqrt and a Newton
// step, Thole factors from the inverse damping factors).  Per pair one 16-byte load of
// the tile slot (shift, J in .w) and two of atom j: A0 = (offset, Thole width) and
// A1 = (S p, 1 / damping factor).  An atom without polarisability has 1/damping 0, which
// fully damps its pairs; the operator B = I - S T S multiplies those pairs by its S = 0,
// so that choice does not change the product.

template <bool QUAD>
__device__ __forceinline__ void cg_field_loop(const NbrList& nl, const CgRadial& R, const float4* __restrict__ A0,
                                              const float4* __restrict__ A1, const PairTask& t, float* acc) {
    const PairConsts<float>& pc = nl.cf;
    const float4 ai = A0[t.si], bi = A1[t.si];
    for (int k = t.k0; k < t.k1; ++k) {
        const int pos = QUAD ? nl.cap - 1 - k : k;
        const unsigned code = nl.list[((size_t) t.I * nl.cap + pos) * 32 + t.lane];
        const float4 sh = nl.shF[(size_t) t.I * nl.tcap + (code >> 7)];
        const int Jw = __float_as_int(sh.w);
        const int sj = (Jw & 0x7fffffff) * 32 + (int) (code & 31u);
        const float4 aj = A0[sj], bj = A1[sj];
        float d[3] = {sh.x + (aj.x - ai.x), sh.y + (aj.y - ai.y), sh.z + (aj.z - ai.z)};
        if (Jw < 0) min_image(d, pc.V, pc.iL);
        const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (nl.usePbc && r2 > pc.rc2) continue;
        const unsigned flag = (code >> 5) & 3u;
        const float a = flag == 1u ? ai.w + aj.w : pc.thole;  // flag 1: covalent scale 0
        float b1, b2;
        cg_pair_radial<QUAD>(R, r2, a, bi.w * bj.w, pc.ew.hi, pc.ew.lo, b1, b2);
        const float b[4] = {0.f, b1, b2, 0.f};
        const float uj[3] = {bj.x, bj.y, bj.z};
        const float sI[3] = {-d[0], -d[1], -d[2]};
        float e[3], gr[6];
        dipole_field<float, false>(uj, sI, b, e, gr);
        acc[0] += e[0];
        acc[1] += e[1];
        acc[2] += e[2];
    }
}

MPID_KERNEL void k_dipole_field_cg(KGrid<(32 * kWarpsPerBlock)> kg, NbrList nl, CgRadial R, const float4* __restrict__ A0, const float4* __restrict__ A1, int npad,
                  const int* __restrict__ orig, unsigned long long* __restrict__ field, const int* __restrict__ skip) {
    if (*skip) return;
    __shared__ float part[kWarpsPerBlock][3][32];
    PairTask t;
    const bool active = t.init(nl, kg.bx) && orig[t.si] >= 0;
    float acc[3] = {0.f, 0.f, 0.f};
    if (active) {
        if (t.quad)
            cg_field_loop<true>(nl, R, A0, A1, t, acc);
        else
            cg_field_loop<false>(nl, R, A0, A1, t, acc);
    }
    // The sub-ranges of one work item are consecutive warps; within a block they add
    // their partial fields in shared memory, so that an item makes one set of atomics
    // per block (a fixed order: the sums stay deterministic).
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = min(nl.split, kWarpsPerBlock);
    if (g > 1) {
#pragma unroll
        for (int q = 0; q < 3; ++q) part[w][q][lane] = acc[q];
        __syncthreads();
        if (w % g != 0) return;
        for (int o = 1; o < g; ++o)
#pragma unroll
            for (int q = 0; q < 3; ++q) acc[q] += part[w + o][q][lane];
    }
    if (active)
        for (int q = 0; q < 3; ++q) fx_add(field + q * npad + t.si, acc[q]);
}

// A0 = (offset, Thole width) of the float engine's atoms.
MPID_KERNEL void k_pack_atoms(KGrid<> kg, int npad, const float* __restrict__ off, const float4* __restrict__ prm,
                             float4* __restrict__ A0) {
    const int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    A0[s] = make_float4(off[s], off[npad + s], off[2 * npad + s], prm[s].x);
}

// ---------------------------------------------------------------------------
// Residual field of the mixed path's refinement in double-float arithmetic: the
// real-space T.mu of k_dipole_field<double> (MPIDReferenceForce.cpp:4161-4281) to
// ~1e-14 relative, on the FP32 pipes.  The Ewald parts of b_1, b_2 come from the tables
// of radial_tables.h; Thole factors and geometry are computed in df.  Pairs j > i only,
// with the field at j added by fixed-point atomics.

// Per-atom df inputs: offsets [3][npad] from the FP64 engine, dipoles [3][npad], Thole
// width and damping factor [npad].
struct DfAtoms {
    int npad;
    const float2* off;
    const float2* mu;
    const float2* thole;
    const float2* damp;  // 1 / damping factor (0 for an atom without polarisability)
};

struct DfRadial {
    const float* Gcoef;
    const float* Gcentre;
    const float* Hcoef;
    const float* Hcentre;
    float Gr0, Ginvh, Hr0, Hinvh;
    int GK, HK;
    int usePme;
    float rc2;
    float L[3], iL[3];
    float2 Vdf[9];  // box rows as double-float
    float2 tholeDefault;
};

__device__ __forceinline__ dfloat df_load(const float2* p, int i) {
    const float2 v = p[i];
    return df_make(v.x, v.y);
}

__device__ __forceinline__ void fx_add_df(unsigned long long* p, dfloat v) {
    const long long a = __float2ll_rn(v.hi * 4294967296.0f) + __float2ll_rn(v.lo * 4294967296.0f);
    atomicAdd(p, (unsigned long long) a);
}

// float2 copies of FP64 arrays
MPID_KERNEL void k_to_df(KGrid<> kg, int count, const double* __restrict__ src, float2* __restrict__ dst) {
    const int i = kg.bx * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const dfloat v = df_from_double(src[i]);
    dst[i] = make_float2(v.hi, v.lo);
}

// df offsets, Thole widths and damping factors of the FP64 engine's atoms
MPID_KERNEL void k_df_atoms(KGrid<> kg, int npad, const double* __restrict__ off, const double4_16a* __restrict__ prm,
                           float2* __restrict__ offDF, float2* __restrict__ tholeDF, float2* __restrict__ dampDF) {
    const int i = kg.bx * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    for (int k = 0; k < 3; ++k) {
        const dfloat v = df_from_double(off[k * npad + i]);
        offDF[k * npad + i] = make_float2(v.hi, v.lo);
    }
    const double4_16a p = prm[i];
    const dfloat t = df_from_double(p.x), d = df_from_double(p.w);  // Thole width, 1 / damping (0: none)
    tholeDF[i] = make_float2(t.hi, t.lo);
    dampDF[i] = make_float2(d.hi, d.lo);
}

template <bool QUAD>
__device__ __forceinline__ void df_field_loop(const NbrList& nl, const DfRadial& R, const DfAtoms& A, const PairTask& t,
                                              dfloat* acc, unsigned long long* field) {
    const int npad = A.npad, si = t.si;
    const dfloat oi[3] = {df_load(A.off, si), df_load(A.off, npad + si), df_load(A.off, 2 * npad + si)};
    const dfloat ui[3] = {df_load(A.mu, si), df_load(A.mu, npad + si), df_load(A.mu, 2 * npad + si)};
    const dfloat thi = df_load(A.thole, si), dpi = df_load(A.damp, si);
    const dfloat one = df_from_float(1.f);
    const dfloat third = df_make(0.333333343f, -9.93410776e-09f);  // 1/3
    const int kb = max(t.k0, QUAD ? nl.loS[si] : nl.loL[si]);
    for (int k = kb; k < t.k1; ++k) {
        const int pos = QUAD ? nl.cap - 1 - k : k;
        const unsigned code = nl.list[((size_t) t.I * nl.cap + pos) * 32 + t.lane];
        const size_t s = (size_t) t.I * nl.tcap + (code >> 7);
        const int Jw = nl.tileJ[s];
        const int sj = (Jw & 0x7fffffff) * 32 + (int) (code & 31u);
        const unsigned flag = (code >> 5) & 3u;
        dfloat d[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) d[q] = df_add(df_sub(df_load(A.off, q * npad + sj), oi[q]), df_load(nl.shDF, 3 * s + q));
        if (Jw < 0)  // minimum image in double-float: c, then b, then a
#pragma unroll
            for (int k = 2; k >= 0; --k) {
                const float m = rintf(d[k].hi * R.iL[k]);
#pragma unroll
                for (int q = 0; q <= k; ++q) d[q] = df_sub(d[q], df_mul(df_make(R.Vdf[3 * k + q].x, R.Vdf[3 * k + q].y), m));
            }
        const dfloat r2 = df_add(df_add(df_mul(d[0], d[0]), df_mul(d[1], d[1])), df_mul(d[2], d[2]));
        if (R.usePme && r2.hi > R.rc2) continue;
        const dfloat r = df_sqrt(r2);
        const dfloat rinv = df_recip(r);
        const dfloat rinv2 = df_mul(rinv, rinv);
        const dfloat bB1 = df_mul(rinv, rinv2);        // 1/r^3
        const dfloat r5inv = df_mul(bB1, rinv2);       // 1/r^5
        // Thole: oneMinus_n = e^-s P_n(s), P_1 = 1 + s + s^2/2, P_2 = P_1 + s^3/6
        dfloat om1 = df_from_float(0.f), om2 = df_from_float(0.f);
        const dfloat dd = df_mul(dpi, df_load(A.damp, sj));  // 1 / (d_i d_j), 0 without damping
        if (dd.hi > 0.f) {
            const dfloat a = flag == 1u ? df_add(thi, df_load(A.thole, sj)) : df_make(R.tholeDefault.x, R.tholeDefault.y);
            const dfloat sT = df_mul(df_mul(a, r), dd);
            if (sT.hi < 50.f) {
                const dfloat e = df_exp_neg(sT);
                const dfloat s2h = df_mul(df_mul(sT, sT), 0.5f);
                const dfloat P1 = df_add(df_add(sT, 1.f), s2h);
                const dfloat P2 = df_add(P1, df_mul(df_mul(s2h, sT), third));
                om1 = df_mul(e, P1);
                om2 = df_mul(e, P2);
            }
        }
        dfloat b1, b2;
        if (QUAD) {
            dfloat H1, H2;
            df_table_eval<7>(R.Hcoef, R.Hcentre, R.Hr0, R.Hinvh, R.HK, r, H1, H2);
            b1 = df_sub(df_mul(df_sub(one, om1), bB1), H1);
            b2 = df_sub(df_mul(df_mul(df_sub(one, om2), r5inv), 3.f), H2);
        } else {
            dfloat G1 = df_from_float(1.f), G2 = df_from_float(3.f);  // no Ewald part without PME
            if (R.usePme) df_table_eval<7>(R.Gcoef, R.Gcentre, R.Gr0, R.Ginvh, R.GK, r, G1, G2);
            b1 = df_mul(df_sub(G1, om1), bB1);
            b2 = df_mul(df_sub(G2, df_mul(om2, 3.f)), r5inv);
        }
        // field at i from mu_j and at j from mu_i: E = -b1 mu + b2 (mu.d) d
        const dfloat uj[3] = {df_load(A.mu, sj), df_load(A.mu, npad + sj), df_load(A.mu, 2 * npad + sj)};
        const dfloat mjd = df_add(df_add(df_mul(uj[0], d[0]), df_mul(uj[1], d[1])), df_mul(uj[2], d[2]));
        const dfloat mid = df_add(df_add(df_mul(ui[0], d[0]), df_mul(ui[1], d[1])), df_mul(ui[2], d[2]));
        const dfloat b2mj = df_mul(b2, mjd), b2mi = df_mul(b2, mid);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            acc[q] = df_add(acc[q], df_sub(df_mul(b2mj, d[q]), df_mul(b1, uj[q])));
            fx_add_df(field + q * npad + sj, df_sub(df_mul(b2mi, d[q]), df_mul(b1, ui[q])));
        }
    }
}

MPID_KERNEL void k_dipole_field_df(KGrid<(32 * kWarpsPerBlock)> kg, NbrList nl, DfRadial R, DfAtoms A, const int* __restrict__ orig, unsigned long long* __restrict__ field) {
    PairTask t;
    if (!t.init(nl, kg.bx)) return;
    if (orig[t.si] < 0) return;
    dfloat acc[3] = {df_from_float(0.f), df_from_float(0.f), df_from_float(0.f)};
    if (t.quad)
        df_field_loop<true>(nl, R, A, t, acc, field);
    else
        df_field_loop<false>(nl, R, A, t, acc, field);
    for (int q = 0; q < 3; ++q) fx_add_df(field + q * A.npad + t.si, acc[q]);
}

// Compensated running sum (TwoSum) for the FP32 pair energies.
template <typename real>
struct KahanSum {
    real s = real(0), c = real(0);
    __device__ __forceinline__ void add(real x) {
        const real y = x - c;
        const real t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double) s - (double) c; }
};

// Real-space energy, forces and torques (MPIDReferenceForce.cpp:4335-4920).  Each lane
// evaluates its atom's pairs and adds force and torque on its own atom; with HALF only
// the pairs with j > i (sorted order), adding the pair's force and torque on j with
// fixed-point atomics (measured on the 24,000-atom box: FP32 0.52 -> 0.50 ms, FP64 path
// 8 % faster overall; the same for the CG field kernel, whose pairs are cheap, was
// slower: 87 -> 103 us).  The energy of pairs with i < j is counted; pairs of covalent
// scale other than 1 leave their energy to k_scaled_pair_energy.
template <typename real, bool MUTUAL, bool REF_ANISO_TORQUE, bool QUAD, bool HALF>
__device__ __forceinline__ void electrostatics_loop(const NbrList& nl, const AtomArrays<real>& at, const real* mu,
                                                    const PairTask& t, int origI, real* accF, real* accT,
                                                    KahanSum<real>& eSum, unsigned long long* __restrict__ force,
                                                    unsigned long long* __restrict__ torque) {
    const PairConsts<real>& pc = pair_consts<real>(nl);
    const int npad = at.npad, si = t.si;
    const real oi[3] = {at.off[si], at.off[npad + si], at.off[2 * npad + si]};
    const real ui[3] = {mu[si], mu[npad + si], mu[2 * npad + si]};
    LabMoments<real> mi;
    load_moments(at.mom, npad, si, mi);
    const typename Vec4<real>::type pi = at.prm[si];
    const int kb = HALF ? max(t.k0, QUAD ? nl.loS[si] : nl.loL[si]) : t.k0;
    for (int k = kb; k < t.k1; ++k) {
        int sj;
        unsigned flag;
        real d[3], r2;
        if (!list_pair<real, QUAD>(nl, pc, at, t.I, k, t.lane, oi, sj, flag, d, r2)) continue;
        const real r = sqrt(r2);
        const real scale = list_scale<real>(nl, flag, origI, at.orig[sj]);
        const typename Vec4<real>::type pj = at.prm[sj];
        const real a = scale == real(0) ? pi.x + pj.x : pc.thole;
        PairRadial<real, 7, 5, MUTUAL ? 3 : 0> pr;
        pair_radial_branch<real, 7, 5, MUTUAL ? 3 : -1, QUAD>(r, pc.ew, scale, a, pi.y * pj.y, pr);
        LabMoments<real> mj;
        load_moments(at.mom, npad, sj, mj);
        const real uj[3] = {mu[sj], mu[npad + sj], mu[2 * npad + sj]};
        PairOut<real> po;
        qi_pair<real, MUTUAL, REF_ANISO_TORQUE>(d, r, mi, mj, ui, uj, pi.z != real(0), pj.z != real(0), pr.bP, pr.bI,
                                                 pr.bU, po);
        if (flag == 0u && si < sj) eSum.add(po.energy);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            accF[q] -= po.fJ[q];
            accT[q] += po.tI[q];
        }
        if (HALF) {  // j > i only: the pair's force and torque on j as well
            const real E = real(kElectric);
            for (int q = 0; q < 3; ++q) {
                fx_add(force + q * npad + sj, E * po.fJ[q]);
                fx_add(torque + q * npad + sj, E * po.tJ[q]);
            }
        }
    }
}

// out: force[3][npad], torque[3][npad] fixed point; energy[warp task] (already x kElectric).
template <typename real, bool MUTUAL, bool REF_ANISO_TORQUE, bool HALF>
MPID_KERNEL void k_electrostatics(KGrid<(32 * kWarpsPerBlock), (sizeof(real) == 4 ? 4 : 1)> kg, NbrList nl, AtomArrays<real> at, const real* __restrict__ mu, unsigned long long* __restrict__ force,
                 unsigned long long* __restrict__ torque, double* __restrict__ energy) {
    PairTask t;
    const bool active = t.init(nl, kg.bx);
    const int npad = at.npad, si = t.si;
    const int origI = active ? at.orig[si] : -1;
    KahanSum<real> eSum;
    if (origI >= 0) {
        real accF[3] = {real(0), real(0), real(0)}, accT[3] = {real(0), real(0), real(0)};
        if (t.quad)
            electrostatics_loop<real, MUTUAL, REF_ANISO_TORQUE, true, HALF>(nl, at, mu, t, origI, accF, accT, eSum,
                                                                             force, torque);
        else
            electrostatics_loop<real, MUTUAL, REF_ANISO_TORQUE, false, HALF>(nl, at, mu, t, origI, accF, accT, eSum,
                                                                              force, torque);
        const real E = real(kElectric);
        for (int q = 0; q < 3; ++q) {
            fx_add(force + q * npad + si, E * accF[q]);
            fx_add(torque + q * npad + si, E * accT[q]);
        }
    }
    // FP64 energy of the work item: warp sum, written per item (fixed-order reduction later)
    double e = eSum.value();
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    const int w = (kg.bx * blockDim.x + threadIdx.x) >> 5;
    if (t.lane == 0 && w < t.tasks(nl)) energy[w] = e * kElectric;
}

// Energy of covalently scaled pairs (scale != 1) in FP64.  Their real-space terms remove
// most of the reciprocal interaction of bonded atoms and are far larger than the total,
// so they are summed at full precision; forces and torques stay in the tile kernel.
template <bool MUTUAL>
MPID_KERNEL void k_scaled_pair_energy(KGrid<> kg, int npairs, const int2* __restrict__ pr, const double* __restrict__ prs,
                                     const int* __restrict__ rank, int npad, const double* __restrict__ mom64,
                                     const double* __restrict__ prm64, const void* __restrict__ muv, int muIsFloat,
                                     const double* __restrict__ pos, BoxDev box, int usePbc, double cutoff,
                                     double ewald, double defaultThole, double* __restrict__ partial) {
    __shared__ double red[128];
    const int p = kg.bx * blockDim.x + threadIdx.x;
    const EwaldAlpha<double> ew(ewald);
    double e = 0.0;
    if (p < npairs) {
        const int i = pr[p].x, j = pr[p].y;
        const int si = rank[i], sj = rank[j];
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = pos[3 * j + k] - pos[3 * i + k];
        if (usePbc) min_image(d, box.V, box.invL);
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (!usePbc || r2 <= cutoff * cutoff) {
            const double r = sqrt(r2), s = prs[p];
            const double a = s == 0.0 ? prm64[2 * i] + prm64[2 * j] : defaultThole;
            PairRadial<double, 7, 5, MUTUAL ? 3 : 0> rad;
            pair_radial<double, 7, 5, MUTUAL ? 3 : -1>(r, ew, s, a, prm64[2 * i + 1] * prm64[2 * j + 1], rad);
            LabMoments<double> mi, mj;
            load_moments(mom64, npad, si, mi);
            load_moments(mom64, npad, sj, mj);
            double ui[3], uj[3];
            for (int c = 0; c < 3; ++c) {
                ui[c] = muIsFloat ? (double) ((const float*) muv)[c * npad + si] : ((const double*) muv)[c * npad + si];
                uj[c] = muIsFloat ? (double) ((const float*) muv)[c * npad + sj] : ((const double*) muv)[c * npad + sj];
            }
            PairOut<double> po;
            qi_pair<double, MUTUAL>(d, r, mi, mj, ui, uj, false, false, rad.bP, rad.bI, rad.bU, po);
            e = po.energy * kElectric;
        }
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[kg.bx] = red[0];
}

// ---------------------------------------------------------------------------
// getElectrostaticPotential (MPIDReferenceForce.cpp:2464-2528): at each grid point the
// bare Coulomb potential of every atom's charge, permanent + induced dipole and
// quadrupole (octopoles are not included there), minimum-imaged under PME, times the
// electric constant.  FP64; one thread per grid point, all threads reading the same atom
// at the same time.
template <typename real>
MPID_KERNEL void k_potential_grid(KGrid<> kg, int n, int npad, int ngrid, const double* __restrict__ grid,
                                 const double* __restrict__ wpos, const int* __restrict__ rank,
                                 const double* __restrict__ mom64, const real* __restrict__ mu, BoxDev box, int usePbc,
                                 double* __restrict__ out) {
    const int g = kg.bx * blockDim.x + threadIdx.x;
    if (g >= ngrid) return;
    const double gx = grid[3 * g], gy = grid[3 * g + 1], gz = grid[3 * g + 2];
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
        const int s = rank[i];
        double d[3] = {wpos[3 * i] - gx, wpos[3 * i + 1] - gy, wpos[3 * i + 2] - gz};
        if (usePbc) min_image(d, box.V, box.invL);
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const double rr1 = 1.0 / sqrt(r2), rr2 = rr1 * rr1, rr3 = rr1 * rr2;
        const double q = mom64[s];
        double sd = 0.0;
        for (int k = 0; k < 3; ++k) sd += (mom64[(1 + k) * npad + s] + (double) mu[k * npad + s]) * d[k];
        // Q6 order XX XY XZ YY YZ ZZ
        const double* Q = mom64 + 4 * (size_t) npad + s;
        const double qxx = Q[0], qxy = Q[npad], qxz = Q[2 * npad], qyy = Q[3 * npad], qyz = Q[4 * npad],
                     qzz = Q[5 * npad];
        const double sq = d[0] * (qxx * d[0] + qxy * d[1] + qxz * d[2]) + d[1] * (qxy * d[0] + qyy * d[1] + qyz * d[2]) +
                          d[2] * (qxz * d[0] + qyz * d[1] + qzz * d[2]);
        acc += q * rr1 - sd * rr3 + sq * 3.0 * rr3 * rr2;
    }
    out[g] = acc * kElectric;
}

// getSystemMultipoleMoments (MPIDReferenceForce.cpp:2349-2462), per-block partials:
// pass 0 sums (m, m x, m y, m z); pass 1 (after the centre of mass is known from
// com = red[1..3] / red[0]) sums charge, dipole (3), traced second moment (6: xx xy xz yy
// yz zz) and the atoms' lab quadrupoles (6).
template <typename real>
MPID_KERNEL void k_moment_partials(KGrid<256> kg, int n, int npad, int pass, const double* __restrict__ pos, const double* __restrict__ masses,
                  const int* __restrict__ rank, const double* __restrict__ mom64, const real* __restrict__ mu,
                  const double* __restrict__ red, double* __restrict__ partial) {
    constexpr int NV = 16;
    __shared__ double sh[NV][256];
    const int i = kg.bx * blockDim.x + threadIdx.x;
    double v[NV];
    for (int k = 0; k < NV; ++k) v[k] = 0.0;
    if (i < n) {
        if (pass == 0) {
            const double m = masses[i];
            v[0] = m;
            for (int k = 0; k < 3; ++k) v[1 + k] = m * pos[3 * i + k];
        } else {
            const double tm = red[0];
            double x[3];
            for (int k = 0; k < 3; ++k) x[k] = pos[3 * i + k] - (tm > 0.0 ? red[1 + k] / tm : 0.0);
            const int s = rank[i];
            const double q = mom64[s];
            double dn[3];
            for (int k = 0; k < 3; ++k) dn[k] = mom64[(1 + k) * npad + s] + (double) mu[k * npad + s];
            v[0] = q;
            for (int k = 0; k < 3; ++k) v[1 + k] = x[k] * q + dn[k];
            v[4] = x[0] * x[0] * q + 2.0 * x[0] * dn[0];
            v[5] = x[0] * x[1] * q + x[0] * dn[1] + x[1] * dn[0];
            v[6] = x[0] * x[2] * q + x[0] * dn[2] + x[2] * dn[0];
            v[7] = x[1] * x[1] * q + 2.0 * x[1] * dn[1];
            v[8] = x[1] * x[2] * q + x[1] * dn[2] + x[2] * dn[1];
            v[9] = x[2] * x[2] * q + 2.0 * x[2] * dn[2];
            for (int k = 0; k < 6; ++k) v[10 + k] = mom64[(4 + k) * npad + s];
        }
    }
    for (int k = 0; k < NV; ++k) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int k = 0; k < NV; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < NV) partial[threadIdx.x * kg.nb + kg.bx] = sh[threadIdx.x][0];
}

// ---------------------------------------------------------------------------
// Parameter gradients.  At stationary induced dipoles (Mutual; and, because their
// response matrices are symmetric, Direct and OPT) the derivative of the energy with
// respect to atom I's lab multipole M_I is d(U_pp + U_pi)/dM_I at fixed dipoles: the
// potential derivatives at I of every other atom's permanent multipoles (kernel K_p)
// and induced dipoles (kernel K_i), plus reciprocal and self terms.  Components are the
// 20 unique lab components (charge, dipole, quadrupole XX XY XZ YY YZ ZZ, octopole XXX
// XXY XXZ XYY XYZ XZZ YYY YYZ YZZ ZZZ) weighted by their multiplicities.

// Unique components: (t, u, v) x/y/z counts, and the multinomial weight.
__device__ __forceinline__ void comp_tuv(int c, int& t, int& u, int& v, int& w) {
    const int T[20] = {0, 1, 0, 0, 2, 1, 1, 0, 0, 0, 3, 2, 2, 1, 1, 1, 0, 0, 0, 0};
    const int U[20] = {0, 0, 1, 0, 0, 1, 0, 2, 1, 0, 0, 1, 0, 2, 1, 0, 3, 2, 1, 0};
    const int V[20] = {0, 0, 0, 1, 0, 0, 1, 0, 1, 2, 0, 0, 1, 0, 1, 2, 0, 1, 2, 3};
    const int W[20] = {1, 1, 1, 1, 1, 2, 2, 1, 2, 1, 1, 3, 3, 3, 6, 3, 1, 3, 3, 1};
    t = T[c]; u = U[c]; v = V[c]; w = W[c];
}

// Index of (t, u, v) among all tuples of rank <= some L, rank-major.
__host__ __device__ __forceinline__ constexpr int tuv_index(int t, int u, int v) {
    return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 + (u + v) * (u + v + 1) / 2 + v;
}

// Cartesian derivatives D(t,u,v) = d^t/dx^t d^u/dy^u d^v/dz^v f(|R|), t+u+v <= L, from
// g_n = ((1/r) d/dr)^n f by the recursion R^(n)_(t+1,u,v) = t R^(n+1)_(t-1,u,v) +
// X R^(n+1)_(t,u,v) (and y, z), level n from n + 1, down to n = 0.
template <typename real, int L>
__device__ __forceinline__ void cart_derivatives(const real* R, const real* g, real* D) {
    constexpr int NT = (L + 1) * (L + 2) * (L + 3) / 6;
    real nxt[NT];
    nxt[0] = g[L];
#pragma unroll
    for (int n = L - 1; n >= 0; --n) {
        const int K = L - n;
        real cur[NT];
#pragma unroll
        for (int k = 0; k <= K; ++k)
#pragma unroll
            for (int m = 0; m <= k; ++m)
#pragma unroll
                for (int v = 0; v <= m; ++v) {
                    const int u = m - v, t = k - m;
                    real val;
                    if (k == 0) {
                        val = g[n];
                    } else if (t > 0) {
                        val = R[0] * nxt[tuv_index(t - 1, u, v)];
                        if (t > 1) val += real(t - 1) * nxt[tuv_index(t - 2, u, v)];
                    } else if (u > 0) {
                        val = R[1] * nxt[tuv_index(t, u - 1, v)];
                        if (u > 1) val += real(u - 1) * nxt[tuv_index(t, u - 2, v)];
                    } else {
                        val = R[2] * nxt[tuv_index(t, u, v - 1)];
                        if (v > 1) val += real(v - 1) * nxt[tuv_index(t, u, v - 2)];
                    }
                    cur[tuv_index(t, u, v)] = val;
                }
#pragma unroll
        for (int q = 0; q < NT; ++q) nxt[q] = cur[q];
    }
#pragma unroll
    for (int q = 0; q < NT; ++q) D[q] = nxt[q];
}

// Lab multipole of a sorted atom as 20 unique components.
template <typename real>
__device__ __forceinline__ void unique_moments(const real* mom, int npad, int s, real* M) {
#pragma unroll
    for (int c = 0; c < 20; ++c) M[c] = mom[c * npad + s];
}

// Real-space part of the gradient: per lane G_I[a] = w_a sum_j [ sum_b (-1)^rank(a) w_b
// M_J[b] D_P(a+b) + sum_(b dipole) (-1)^rank(a) mu_J[b] D_I(a+b) ], kE applied.
template <typename real, bool QUAD>
__device__ __forceinline__ void gradient_loop(const NbrList& nl, const AtomArrays<real>& at, const real* mu,
                                              const PairTask& t, int origI, real* G) {
    const PairConsts<real>& pc = pair_consts<real>(nl);
    const int npad = at.npad, si = t.si;
    const real oi[3] = {at.off[si], at.off[npad + si], at.off[2 * npad + si]};
    const typename Vec4<real>::type pi = at.prm[si];
    for (int k = t.k0; k < t.k1; ++k) {
        int sj;
        unsigned flag;
        real d[3], r2;
        if (!list_pair<real, QUAD>(nl, pc, at, t.I, k, t.lane, oi, sj, flag, d, r2)) continue;
        const real r = sqrt(r2);
        const real scale = list_scale<real>(nl, flag, origI, at.orig[sj]);
        const typename Vec4<real>::type pj = at.prm[sj];
        const real a = scale == real(0) ? pi.x + pj.x : pc.thole;
        PairRadial<real, 6, 4, 0> pr;
        pair_radial_branch<real, 6, 4, -1, QUAD>(r, pc.ew, scale, a, pi.y * pj.y, pr);
        real gP[7], gI[5];
#pragma unroll
        for (int n = 0; n <= 6; ++n) gP[n] = (n & 1) ? -pr.bP[n] : pr.bP[n];
        gI[0] = real(0);
#pragma unroll
        for (int n = 1; n <= 4; ++n) gI[n] = (n & 1) ? -pr.bI[n] : pr.bI[n];
        real DP[84], DI[35];
        cart_derivatives<real, 6>(d, gP, DP);
        cart_derivatives<real, 4>(d, gI, DI);
        real MJ[20];
        unique_moments(at.mom, npad, sj, MJ);
        const real uj[3] = {mu[sj], mu[npad + sj], mu[2 * npad + sj]};
#pragma unroll
        for (int ca = 0; ca < 20; ++ca) {
            int ta, ua, va, wa;
            comp_tuv(ca, ta, ua, va, wa);
            const int ra = ta + ua + va;
            real x = real(0);
#pragma unroll
            for (int cb = 0; cb < 20; ++cb) {
                int tb, ub, vb, wb;
                comp_tuv(cb, tb, ub, vb, wb);
                x += real(wb) * MJ[cb] * DP[tuv_index(ta + tb, ua + ub, va + vb)];
            }
            if (ra <= 3)
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    x += uj[q] * DI[tuv_index(ta + (q == 0), ua + (q == 1), va + (q == 2))];
            G[ca] += real(wa) * ((ra & 1) ? -x : x);
        }
    }
}

// Segments of the neighbour lists a gradient launch covers (bit 0: erfc segment, bit 1:
// quadrature segment).  The mixed path runs the erfc segment in FP32 and the quadrature
// segment, which holds the excluded and short pairs whose terms cancel against the
// reciprocal potentials, in FP64.
constexpr int kSegErfc = 1, kSegQuad = 2, kSegAll = 3;

template <typename real>
MPID_KERNEL void k_multipole_gradient(KGrid<(32 * kWarpsPerBlock)> kg, NbrList nl, AtomArrays<real> at, const real* __restrict__ mu, unsigned long long* __restrict__ gfx,
                     int segments, int split) {
    PairTask t;
    if (!t.init_split(nl, split, kg.bx)) return;
    if (!(segments & (t.quad ? kSegQuad : kSegErfc))) return;
    const int origI = at.orig[t.si];
    if (origI < 0) return;
    real G[20];
#pragma unroll
    for (int c = 0; c < 20; ++c) G[c] = real(0);
    if (t.quad)
        gradient_loop<real, true>(nl, at, mu, t, origI, G);
    else
        gradient_loop<real, false>(nl, at, mu, t, origI, G);
    const real E = real(kElectric);
    for (int c = 0; c < 20; ++c) fx_add(gfx + (size_t) c * at.npad + t.si, E * G[c]);
}

// Local frame R of original atom i (FP64 positions; lab = R^T local R) and whether its
// chirality flips the parameters.
__device__ __forceinline__ bool api_frame(const MolArrays& mol, const double* __restrict__ pos, int n, int i,
                                          double R[3][3]) {
    const int ax = mol.axis[i], iz = mol.az[i], ix = mol.ax[i], iy = mol.ay[i];
    const double* pI = pos + 3 * i;
    const double* pZ = (iz >= 0 && iz < n) ? pos + 3 * iz : pI;
    const double* pX = (ix >= 0 && ix < n) ? pos + 3 * ix : pI;
    const double* pY = (iy >= 0 && iy < n) ? pos + 3 * iy : pI;
    local_frame<double>(ax, pI, pZ, pX, pY, R);
    return chiral_flip<double>(ax, iy >= 0, pI, pZ, pX, pY);
}

// Per atom: real-space part + reciprocal (Cartesian derivatives of both reciprocal
// potentials) + Ewald self terms, then the molecular-frame parameters of the API
// (charge, dipole X Y Z, quadrupole XX XY YY XZ YZ ZZ, octopole XXX XXY XYY YYY XXZ XYZ
// YYZ XZZ YZZ ZZZ) through the frame rotation and the chirality flip.  out[20 n] by
// original index, FP64.
template <typename real>
MPID_KERNEL void k_gradient_finish(KGrid<> kg, int n, int npad, BoxDev box, double alpha, int usePme, const int* __restrict__ order,
                                  MolArrays mol, const double* __restrict__ pos, const unsigned long long* __restrict__ gfx,
                                  const real* __restrict__ phiP, const real* __restrict__ phiD,
                                  const double* __restrict__ mom64, const real* __restrict__ mu, double* __restrict__ out) {
    const int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = order[s];
    double g[20];
    for (int c = 0; c < 20; ++c) g[c] = fx_get(gfx, c * npad + s);
    if (usePme) {
        real A[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) A[a][b] = real(box.A[a][b]);
        for (int which = 0; which < 2; ++which) {
            const real* phi = which == 0 ? phiP : phiD;
            real ph[35], P0, P1[3], P2[3][3], P3[3][3][3];
            for (int k = 0; k < 35; ++k) ph[k] = phi[k * npad + s];
            cartesian_potential(ph, A, P0, P1, P2, P3);
            for (int c = 0; c < 20; ++c) {
                int t, u, v, w;
                comp_tuv(c, t, u, v, w);
                int idx[3], m = 0;
                for (int k = 0; k < t; ++k) idx[m++] = 0;
                for (int k = 0; k < u; ++k) idx[m++] = 1;
                for (int k = 0; k < v; ++k) idx[m++] = 2;
                const real x = m == 0 ? P0 : m == 1 ? P1[idx[0]] : m == 2 ? P2[idx[0]][idx[1]] : P3[idx[0]][idx[1]][idx[2]];
                g[c] += kElectric * w * (double) x;
            }
        }
        // Ewald self energy (MPIDReferenceForce.cpp:4283-4318); the d.mu term is half the
        // permanent-induced self interaction, all of which enters at stationary dipoles
        LabMoments<double> m;
        load_moments(mom64, npad, s, m);
        const double pre = -alpha * kElectric / kSqrtPiRef, a2 = alpha * alpha;
        const double u3[3] = {(double) mu[s], (double) mu[npad + s], (double) mu[2 * npad + s]};
        g[0] += pre * 2 * m.q;
        for (int k = 0; k < 3; ++k) g[1 + k] += pre * 2.0 / 3.0 * a2 * (2 * m.d[k] + 2 * u3[k]);
        const double s3 = sqrt(3.0), r15 = sqrt(1.5), r06 = sqrt(0.6), r01 = sqrt(0.1);
        // quadrupole (XX XY XZ YY YZ ZZ) and octopole spherical components as the
        // reference forms them (MPIDReferenceForce.cpp:318-342), then d(sum S^2)
        const double* Q = m.Q;
        const double* O = m.O;
        const double S4 = 3 * Q[5], S5 = 2 * s3 * Q[2], S6 = 2 * s3 * Q[4], S7 = s3 * (Q[0] - Q[3]), S8 = 2 * s3 * Q[1];
        const double cq = pre * 4.0 / 15.0 * a2 * a2, co = pre * 8.0 / 105.0 * a2 * a2 * a2;
        g[4] += cq * 2 * S7 * s3;
        g[7] -= cq * 2 * S7 * s3;
        g[9] += cq * 2 * S4 * 3;
        g[6] += cq * 2 * S5 * 2 * s3;
        g[8] += cq * 2 * S6 * 2 * s3;
        g[5] += cq * 2 * S8 * 2 * s3;
        // O10: 0 XXX 1 XXY 2 XXZ 3 XYY 4 XYZ 5 XZZ 6 YYY 7 YYZ 8 YZZ 9 ZZZ
        const double S9 = 15 * O[9], S10 = 15 * r15 * O[5], S11 = 15 * r15 * O[8], S12 = 15 * r06 * (O[2] - O[7]),
                     S13 = 30 * r06 * O[4], S14 = 15 * r01 * (O[0] - 3 * O[3]), S15 = 15 * r01 * (3 * O[1] - O[6]);
        g[19] += co * 2 * S9 * 15;
        g[15] += co * 2 * S10 * 15 * r15;
        g[18] += co * 2 * S11 * 15 * r15;
        g[12] += co * 2 * S12 * 15 * r06;
        g[17] -= co * 2 * S12 * 15 * r06;
        g[14] += co * 2 * S13 * 30 * r06;
        g[10] += co * 2 * S14 * 15 * r01;
        g[13] -= co * 2 * S14 * 45 * r01;
        g[11] += co * 2 * S15 * 45 * r01;
        g[16] -= co * 2 * S15 * 15 * r01;
    }
    double R[3][3];
    const bool flip = api_frame(mol, pos, n, i, R);
    // full-entry lab derivatives, rotated into the molecular frame (lab = R^T local R)
    double* o = out + 20 * (size_t) i;
    o[0] = g[0];
    for (int k = 0; k < 3; ++k) o[1 + k] = R[k][0] * g[1] + R[k][1] * g[2] + R[k][2] * g[3];
    double GQ[3][3];
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) {
            const int c = q6(x, y);
            GQ[x][y] = g[4 + c] / (x == y ? 1.0 : 2.0);
        }
    const int QAPI[6][2] = {{0, 0}, {0, 1}, {1, 1}, {0, 2}, {1, 2}, {2, 2}};
    for (int c = 0; c < 6; ++c) {
        const int k = QAPI[c][0], mm = QAPI[c][1];
        double LQkm = 0.0, LQmk = 0.0;
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) {
                LQkm += R[k][x] * R[mm][y] * GQ[x][y];
                LQmk += R[mm][x] * R[k][y] * GQ[x][y];
            }
        o[4 + c] = k == mm ? LQkm : LQkm + LQmk;
    }
    // full-entry lab octopole derivative (symmetric), rotated one index at a time; the
    // molecular-frame tensor is symmetric too, so an API component is its entry times
    // the number of distinct orderings of its index triple
    double GO[3][3][3], W1[3][3][3];
    for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y)
            for (int z = 0; z < 3; ++z) {
                const int w = (x == y && y == z) ? 1 : ((x == y || y == z || x == z) ? 3 : 6);
                GO[x][y][z] = g[10 + o10(x, y, z)] / w;
            }
    for (int k = 0; k < 3; ++k)
        for (int y = 0; y < 3; ++y)
            for (int z = 0; z < 3; ++z) W1[k][y][z] = R[k][0] * GO[0][y][z] + R[k][1] * GO[1][y][z] + R[k][2] * GO[2][y][z];
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l)
            for (int z = 0; z < 3; ++z) GO[k][l][z] = R[l][0] * W1[k][0][z] + R[l][1] * W1[k][1][z] + R[l][2] * W1[k][2][z];
    const int OAPI[10][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {0, 0, 2},
                             {0, 1, 2}, {1, 1, 2}, {0, 2, 2}, {1, 2, 2}, {2, 2, 2}};
    for (int c = 0; c < 10; ++c) {
        const int a0 = OAPI[c][0], a1 = OAPI[c][1], a2i = OAPI[c][2];
        const int nperm = (a0 == a1 && a1 == a2i) ? 1 : ((a0 == a1 || a1 == a2i || a0 == a2i) ? 3 : 6);
        const double LO = R[a2i][0] * GO[a0][a1][0] + R[a2i][1] * GO[a0][a1][1] + R[a2i][2] * GO[a0][a1][2];
        o[10 + c] = nperm * LO;
    }
    if (flip) {  // the flipped parameters enter with the opposite sign
        o[2] = -o[2];
        o[4 + 1] = -o[4 + 1];
        o[4 + 4] = -o[4 + 4];
    }
}

// ---------------------------------------------------------------------------
// Polarisability and Thole-width gradients (Mutual, Direct).  At stationary dipoles the
// energy equals F(mu) = U_pp + U_pi + U_uu + kE/2 mu.alpha^-1.mu with U_pi = -mu.E_perm
// and U_uu = -1/2 mu.T.mu (absent for Direct), so the derivatives are taken at fixed
// dipoles.  The parameters enter through alpha^-1 and through the screening argument
// st = a r / (d_i d_j) of the ind and uu kernels, d_i = mean(p_i)^(1/6):
//   dst/dp_ik = -st / (18 mean(p_i)),   dst/da_i = st / a  (pairs of covalent scale 0,
//   whose width is a_i + a_j; other pairs use the default width).
// The pair loop sums, per atom, W_I = sum_j st dF_ij/dst and Z_I over the scale-0 pairs
// of st/a dF_ij/dst, where dF_ij/dst is the pair's U_pi + U_uu with the kernels' st
// derivatives, kE applied.
// Perturbation orders of the Extrapolated (OPT) solver for the polarisation gradient:
// nPT dipole sets [3][npad] each, and cbar_k = sum_(j >= k) c_j.
template <typename real>
struct OptOrders {
    int nPT;  // 0: not Extrapolated
    double cbar[8];
    const real* mu;
};

template <typename real, bool QUAD>
__device__ __forceinline__ void polarization_loop(const NbrList& nl, const AtomArrays<real>& at, const real* mu,
                                                  bool mutual, const OptOrders<real>& opt, const PairTask& t, int origI,
                                                  real& W, real& Z) {
    const PairConsts<real>& pc = pair_consts<real>(nl);
    const int npad = at.npad, si = t.si;
    const real oi[3] = {at.off[si], at.off[npad + si], at.off[2 * npad + si]};
    const typename Vec4<real>::type pi = at.prm[si];
    real MI[20];
    unique_moments(at.mom, npad, si, MI);
    const real ui[3] = {mu[si], mu[npad + si], mu[2 * npad + si]};
    // OPT: A_m = sum_(j <= nPT-2-m) cbar_(j+m+1) mu_(j,i), so that the pair's sums are
    // S1 = sum_m A_m.mu_(m,l) and S2 = sum_m (A_m.d)(mu_(m,l).d)
    real A[7][3];
    const int nm = opt.nPT > 1 ? opt.nPT - 1 : 0;
    for (int m = 0; m < 7; ++m)
        for (int q = 0; q < 3; ++q) A[m][q] = real(0);
    for (int m = 0; m < nm; ++m)
        for (int j = 0; j + m + 1 < opt.nPT; ++j)
            for (int q = 0; q < 3; ++q)
                A[m][q] += real(opt.cbar[j + m + 1]) * opt.mu[((size_t) j * 3 + q) * npad + si];
    for (int k = t.k0; k < t.k1; ++k) {
        int sj;
        unsigned flag;
        real d[3], r2;
        if (!list_pair<real, QUAD>(nl, pc, at, t.I, k, t.lane, oi, sj, flag, d, r2)) continue;
        const typename Vec4<real>::type pj = at.prm[sj];
        const real dmp = pi.y * pj.y;
        if (!(dmp > real(0))) continue;
        const real r = sqrt(r2);
        const real scale = list_scale<real>(nl, flag, origI, at.orig[sj]);
        const real a = scale == real(0) ? pi.x + pj.x : pc.thole;
        const real st = a * r / dmp;
        if (st >= real(50)) continue;
        real dl[5];
        thole_lambda_derivs<real, 4>(st, dl);
        const real rinv2 = real(1) / r2;
        real bB[5];
        bare_part<real, 4>(real(1) / r, rinv2, bB);
        // st derivatives of the ind kernel (scale lambda' b_n[1/r]) as signed g_n
        real g[5];
        g[0] = real(0);
#pragma unroll
        for (int n = 1; n <= 4; ++n) g[n] = ((n & 1) ? -scale : scale) * dl[n] * bB[n];
        real D[35];
        cart_derivatives<real, 4>(d, g, D);
        real MJ[20];
        unique_moments(at.mom, npad, sj, MJ);
        const real uj[3] = {mu[sj], mu[npad + sj], mu[2 * npad + sj]};
        real x = real(0);
#pragma unroll
        for (int ca = 0; ca < 20; ++ca) {
            int ta, ua, va, wa;
            comp_tuv(ca, ta, ua, va, wa);
            real s1 = real(0), s2 = real(0);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const real dq = D[tuv_index(ta + (q == 0), ua + (q == 1), va + (q == 2))];
                s1 += uj[q] * dq;
                s2 += ui[q] * dq;
            }
            const int ra = ta + ua + va;
            x += real(wa) * (((ra & 1) ? -MI[ca] : MI[ca]) * s1 - MJ[ca] * s2);
        }
        if (mutual) {  // -(g1' mu_i.mu_j + g2' (mu_i.d)(mu_j.d)), g1' = -lambda_1' b_1, g2' = lambda_2' b_2
            const real mm = ui[0] * uj[0] + ui[1] * uj[1] + ui[2] * uj[2];
            const real mi = ui[0] * d[0] + ui[1] * d[1] + ui[2] * d[2];
            const real mj = uj[0] * d[0] + uj[1] * d[1] + uj[2] * d[2];
            x += dl[1] * bB[1] * mm - dl[2] * bB[2] * mi * mj;
        } else if (nm > 0) {  // OPT: -(g1' S1 + g2' S2)
            real S1 = real(0), S2 = real(0);
            for (int m = 0; m < nm; ++m) {
                const real* um = opt.mu + (size_t) m * 3 * npad;
                const real ul[3] = {um[sj], um[npad + sj], um[2 * npad + sj]};
                S1 += A[m][0] * ul[0] + A[m][1] * ul[1] + A[m][2] * ul[2];
                S2 += (A[m][0] * d[0] + A[m][1] * d[1] + A[m][2] * d[2]) * (ul[0] * d[0] + ul[1] * d[1] + ul[2] * d[2]);
            }
            x += dl[1] * bB[1] * S1 - dl[2] * bB[2] * S2;
        }
        W += st * x;
        if (scale == real(0)) Z += st / a * x;
    }
}

template <typename real>
MPID_KERNEL void k_polarization_gradient(KGrid<(32 * kWarpsPerBlock)> kg, NbrList nl, AtomArrays<real> at, const real* __restrict__ mu, int mutual,
                        OptOrders<real> opt, unsigned long long* __restrict__ gfx, int segments, int split) {
    PairTask t;
    if (!t.init_split(nl, split, kg.bx)) return;
    if (!(segments & (t.quad ? kSegQuad : kSegErfc))) return;
    const int origI = at.orig[t.si];
    if (origI < 0) return;
    real W = real(0), Z = real(0);
    if (t.quad)
        polarization_loop<real, true>(nl, at, mu, mutual != 0, opt, t, origI, W, Z);
    else
        polarization_loop<real, false>(nl, at, mu, mutual != 0, opt, t, origI, W, Z);
    const real E = real(kElectric);
    fx_add(gfx + t.si, E * W);
    fx_add(gfx + at.npad + t.si, E * Z);
}

// out[4 n] by original index: dE/d(molecular-frame polarisability X Y Z, Thole width).
// Extrapolated: the alpha^-1 term is replaced by -1/2 sum_k cbar_k sum_(j <= k) F_j F_(k-j)
// (molecular frame, per axis) with F_0 = the permanent field (Efix) and F_j = the field
// of order j - 1 (ptE).
template <typename real>
MPID_KERNEL void k_polarization_gradient_finish(KGrid<> kg, int n, int npad, const int* __restrict__ order, MolArrays mol,
                                               const double* __restrict__ pos, const unsigned long long* __restrict__ gfx,
                                               const real* __restrict__ mu, OptOrders<real> opt,
                                               const real* __restrict__ Efix, const real* __restrict__ ptE,
                                               double* __restrict__ out) {
    const int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = order[s];
    const double W = fx_get(gfx, s), Z = fx_get(gfx, npad + s);
    double R[3][3];
    api_frame(mol, pos, n, i, R);
    const double* p = mol.pol + 3 * i;
    const double pbar = (p[0] + p[1] + p[2]) / 3.0;
    const double u[3] = {(double) mu[s], (double) mu[npad + s], (double) mu[2 * npad + s]};
    double* o = out + 4 * (size_t) i;
    double F[8][3];
    for (int j = 0; j < opt.nPT; ++j) {
        const real* v = j == 0 ? Efix : ptE + (size_t) (j - 1) * 3 * npad;
        const double lab[3] = {(double) v[s], (double) v[npad + s], (double) v[2 * npad + s]};
        for (int k = 0; k < 3; ++k) F[j][k] = R[k][0] * lab[0] + R[k][1] * lab[1] + R[k][2] * lab[2];
    }
    for (int k = 0; k < 3; ++k) {
        double g = 0.0;
        if (opt.nPT > 0) {
            for (int ko = 0; ko < opt.nPT; ++ko)
                for (int j = 0; j <= ko; ++j) g -= 0.5 * kElectric * opt.cbar[ko] * F[j][k] * F[ko - j][k];
        } else {
            const double nu = R[k][0] * u[0] + R[k][1] * u[1] + R[k][2] * u[2];
            g = p[k] > 0.0 ? -0.5 * kElectric * nu * nu / (p[k] * p[k]) : 0.0;
        }
        if (pbar > 0.0) g -= W / (18.0 * pbar);
        o[k] = g;
    }
    o[3] = Z;
}

// ---------------------------------------------------------------------------
// PME.  B-spline coefficients and weighted fractional multipoles per sorted atom.
// theta layout: [3 dims][5 derivs][ORDER][npad]; igrid [3][npad].
template <typename real, int ORDER>
MPID_KERNEL void k_bsplines(KGrid<> kg, int npad, int n, const int* __restrict__ order, const double* __restrict__ wpos,
                           BoxDev box, real* __restrict__ theta, int* __restrict__ igrid) {
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    if (s >= n) {
        for (int d = 0; d < 3; ++d) {
            igrid[d * npad + s] = 0;
            for (int k = 0; k < 5 * ORDER; ++k) theta[(d * 5 * ORDER + k) * npad + s] = real(0);
        }
        return;
    }
    const int i = order[s];
    for (int d = 0; d < 3; ++d) {
        // Fractional coordinate with the grid origin of MPIDReferenceForce.cpp:3058-3060:
        // the minimum-image coordinate w in [-1/2, 1/2) maps to n (w + 1/2).
        // fractional coordinate w_d = sum_k x_k R[k][d] (MPIDReferenceForce.cpp:3058)
        double w = wpos[3 * i] * box.R[0][d] + wpos[3 * i + 1] * box.R[1][d] + wpos[3 * i + 2] * box.R[2][d] + 0.5;
        w -= floor(w);
        double fr = box.grid[d] * w;
        int ifr = (int) floor(fr);
        if (ifr >= box.grid[d]) ifr -= box.grid[d];
        const real ww = real(fr - floor(fr));
        int ig = ifr - ORDER + 1;
        if (ig < 0) ig += box.grid[d];
        igrid[d * npad + s] = ig;
        real th[5][ORDER];
        bspline_derivs<real, ORDER>(ww, th);
        for (int k = 0; k < 5; ++k)
            for (int m = 0; m < ORDER; ++m) theta[((d * 5 + k) * ORDER + m) * npad + s] = th[k][m];
    }
}

template <typename real>
MPID_KERNEL void k_frac_multipoles(KGrid<> kg, int npad, BoxDev box, const real* __restrict__ mom, real* __restrict__ mf) {
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    LabMoments<real> m;
    load_moments(mom, npad, s, m);
    real A[3][3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) A[a][b] = real(box.A[a][b]);
    real f[20];
    frac_multipole(m, A, f);
    for (int k = 0; k < 20; ++k) mf[k * npad + s] = f[k];
}

template <typename real> struct GridAcc;
template <> struct GridAcc<float> {
    typedef unsigned long long type;
    static __device__ __forceinline__ void add(type* g, size_t idx, float v) { fx_add(g + idx, v); }
};
template <> struct GridAcc<double> {
    typedef double type;
    static __device__ __forceinline__ void add(type* g, size_t idx, double v) { atomicAdd(g + idx, v); }
};

// Spread NCOMP weighted fractional components (20 = full multipole, 4 = charge +
// dipole) on the grid: one thread per (atom, x, y) stencil column.
template <typename real, int ORDER, int NCOMP>
MPID_KERNEL void k_spread(KGrid<> kg, int n, int npad, BoxDev box, const real* __restrict__ mf, const real* __restrict__ theta,
                         const int* __restrict__ igrid, typename GridAcc<real>::type* __restrict__ grid,
                         const int* __restrict__ skip) {
    if (skip && *skip) return;
    const long long tid = (long long) kg.bx * blockDim.x + threadIdx.x;
    if (tid >= (long long) n * ORDER * ORDER) return;
    const int s = (int) (tid / (ORDER * ORDER));
    const int ix = (int) (tid % (ORDER * ORDER)) / ORDER, iy = (int) (tid % ORDER);
    const int nx = box.grid[0], ny = box.grid[1], nz = box.grid[2];
    auto TH = [&](int d, int k, int m) { return theta[((d * 5 + k) * ORDER + m) * npad + s]; };
    // z polynomial coefficients c_v = sum over components with z-order v
    real cv[4] = {real(0), real(0), real(0), real(0)};
#pragma unroll
    for (int c = 0; c < NCOMP; ++c) {
        int t, u, v;
        hermite_tuv(c, t, u, v);
        cv[v] += mf[c * npad + s] * TH(0, t, ix) * TH(1, u, iy);
    }
    int gx = igrid[s] + ix;
    if (gx >= nx) gx -= nx;
    int gy = igrid[npad + s] + iy;
    if (gy >= ny) gy -= ny;
    const int gz0 = igrid[2 * npad + s];
    const size_t base = ((size_t) gx * ny + gy) * nz;
#pragma unroll
    for (int iz = 0; iz < ORDER; ++iz) {
        int gz = gz0 + iz;
        if (gz >= nz) gz -= nz;
        real v = cv[0] * TH(2, 0, iz);
        if (NCOMP > 1) v += cv[1] * TH(2, 1, iz);
        if (NCOMP > 4) v += cv[2] * TH(2, 2, iz) + cv[3] * TH(2, 3, iz);
        GridAcc<real>::add(grid, base + gz, v);
    }
}

// Fixed-point (or FP64) accumulation grid -> FFT input, clearing the accumulator.
template <typename real>
MPID_KERNEL void k_grid_finish(KGrid<> kg, size_t total, typename GridAcc<real>::type* __restrict__ acc, real* __restrict__ out,
                              const int* __restrict__ skip) {
    if (skip && *skip) return;
    for (size_t i = (size_t) kg.bx * blockDim.x + threadIdx.x; i < total; i += (size_t) kg.nb * blockDim.x) {
        if constexpr (sizeof(real) == 4) {
            out[i] = (real) ((double) (long long) acc[i] * kFixedInv);
        } else {
            out[i] = (real) acc[i];
        }
        acc[i] = 0;
    }
}

// Reciprocal influence function on the half-complex grid (kx, ky, kz <= nz/2),
// MPIDReferenceForce.cpp:3329-3366: exp(-pi^2 m^2/alpha^2)/(pi V m^2 B(m)), 0 at m = 0.
MPID_KERNEL void k_influence(KGrid<> kg, BoxDev box, double alpha, const double* __restrict__ modx, const double* __restrict__ mody,
                            const double* __restrict__ modz, double volume, double* __restrict__ out) {
    const int nx = box.grid[0], ny = box.grid[1], nz = box.grid[2], nzh = nz / 2 + 1;
    const size_t total = (size_t) nx * ny * nzh;
    for (size_t idx = (size_t) kg.bx * blockDim.x + threadIdx.x; idx < total; idx += (size_t) kg.nb * blockDim.x) {
        const int kz = (int) (idx % nzh);
        const int ky = (int) ((idx / nzh) % ny);
        const int kx = (int) (idx / ((size_t) nzh * ny));
        if (kx == 0 && ky == 0 && kz == 0) { out[idx] = 0.0; continue; }
        const int mx = kx < (nx + 1) / 2 ? kx : kx - nx;
        const int my = ky < (ny + 1) / 2 ? ky : ky - ny;
        const int mz = kz < (nz + 1) / 2 ? kz : kz - nz;
        // reciprocal lattice vector m_x a* + m_y b* + m_z c* (MPIDReferenceForce.cpp:3351-3353)
        const double hx = mx * box.R[0][0];
        const double hy = mx * box.R[1][0] + my * box.R[1][1];
        const double hz = mx * box.R[2][0] + my * box.R[2][1] + mz * box.R[2][2];
        const double m2 = hx * hx + hy * hy + hz * hz;
        const double expF = M_PI * M_PI / (alpha * alpha);
        out[idx] = exp(-expF * m2) / (M_PI * volume * m2 * modx[kx] * mody[ky] * modz[kz]);
    }
}

template <typename real> struct Cplx;
template <> struct Cplx<float> { typedef float2 type; };
template <> struct Cplx<double> { typedef double2 type; };

template <typename real>
MPID_KERNEL void k_convolve(KGrid<> kg, size_t total, const double* __restrict__ influence, typename Cplx<real>::type* __restrict__ g,
                           const int* __restrict__ skip) {
    if (skip && *skip) return;
    for (size_t i = (size_t) kg.bx * blockDim.x + threadIdx.x; i < total; i += (size_t) kg.nb * blockDim.x) {
        const real f = (real) influence[i];
        typename Cplx<real>::type v = g[i];
        v.x *= f;
        v.y *= f;
        g[i] = v;
    }
}

// Gather NTERM fractional potential derivatives (4, 10 or 35) at each atom;
// MPIDReferenceForce.cpp:3368-3530.  phi layout [NTERM][npad].
//
// A block covers kGatherAtoms<...> sorted atoms with one thread per (atom, z plane of
// the stencil): each thread sums its ORDER x ORDER plane, the partial sums meet in shared
// memory, and the block adds the ORDER planes of each atom in plane order (deterministic).
// One thread per atom left a 24,000-atom box at 188 blocks of long serial loops.
template <typename real, int ORDER, int NTERM>
struct GatherShape {
    // atoms per block: the largest power of two up to 64 whose partial sums fit 48 KB
    static constexpr int bytesPerAtom = ORDER * NTERM * (int) sizeof(real);
    static constexpr int atoms = bytesPerAtom * 64 <= 49152 ? 64 : (bytesPerAtom * 32 <= 49152 ? 32 : 16);
    static constexpr int threads = ORDER * atoms;
};

template <typename real, int ORDER, int NTERM>
MPID_KERNEL void k_gather(KGrid<(GatherShape<real, ORDER, NTERM>::threads)> kg, int n, int npad, BoxDev box, const real* __restrict__ theta, const int* __restrict__ igrid,
         const real* __restrict__ grid, real* __restrict__ phi, const int* __restrict__ skip) {
    if (skip && *skip) return;
    constexpr int APB = GatherShape<real, ORDER, NTERM>::atoms;
    constexpr int MAXD = NTERM == 4 ? 1 : (NTERM == 10 ? 2 : 4);
    __shared__ real part[ORDER][NTERM][APB];
    const int a = threadIdx.x % APB, iz = threadIdx.x / APB;
    const int s0 = kg.bx * APB, s = s0 + a;
    real acc[NTERM];
#pragma unroll
    for (int k = 0; k < NTERM; ++k) acc[k] = real(0);
    if (s < n) {
        const int nx = box.grid[0], ny = box.grid[1], nz = box.grid[2];
        auto TH = [&](int d, int k, int m) { return theta[((d * 5 + k) * ORDER + m) * npad + s]; };
        const int gx0 = igrid[s], gy0 = igrid[npad + s];
        int gz = igrid[2 * npad + s] + iz;
        if (gz >= nz) gz -= nz;
        real v[MAXD + 1];
#pragma unroll
        for (int k = 0; k <= MAXD; ++k) v[k] = TH(2, k, iz);
        real tu[MAXD + 1][MAXD + 1];
#pragma unroll
        for (int p = 0; p <= MAXD; ++p)
#pragma unroll
            for (int q = 0; q <= MAXD; ++q) tu[p][q] = real(0);
        for (int iy = 0; iy < ORDER; ++iy) {
            int gy = gy0 + iy;
            if (gy >= ny) gy -= ny;
            real u[MAXD + 1];
#pragma unroll
            for (int k = 0; k <= MAXD; ++k) u[k] = TH(1, k, iy);
            real t[MAXD + 1];
#pragma unroll
            for (int k = 0; k <= MAXD; ++k) t[k] = real(0);
#pragma unroll
            for (int ix = 0; ix < ORDER; ++ix) {
                int gx = gx0 + ix;
                if (gx >= nx) gx -= nx;
                const real q = grid[((size_t) gx * ny + gy) * nz + gz];
#pragma unroll
                for (int k = 0; k <= MAXD; ++k) t[k] += q * TH(0, k, ix);
            }
#pragma unroll
            for (int p = 0; p <= MAXD; ++p)
#pragma unroll
                for (int q = 0; p + q <= MAXD; ++q) tu[p][q] += t[p] * u[q];
        }
#pragma unroll
        for (int p = 0; p <= MAXD; ++p)
#pragma unroll
            for (int q = 0; p + q <= MAXD; ++q)
#pragma unroll
                for (int c = 0; p + q + c <= MAXD; ++c) acc[hermite_index(p, q, c)] += tu[p][q] * v[c];
    }
#pragma unroll
    for (int k = 0; k < NTERM; ++k) part[iz][k][a] = acc[k];
    __syncthreads();
    for (int idx = threadIdx.x; idx < NTERM * APB; idx += blockDim.x) {
        const int k = idx / APB, b = idx % APB;
        if (s0 + b >= npad) continue;
        real sum = part[0][k][b];
#pragma unroll
        for (int z = 1; z < ORDER; ++z) sum += part[z][k][b];
        phi[k * npad + s0 + b] = sum;  // 0 for the padding atoms
    }
}

}  // namespace mpid

namespace mpid {

// ---------------------------------------------------------------------------
// Per-atom kernels.

template <typename real>
__device__ __forceinline__ void sym_mul(const real* S, int npad, int s, const real* v, real* o) {
    const real a0 = S[s], a1 = S[npad + s], a2 = S[2 * npad + s], a3 = S[3 * npad + s], a4 = S[4 * npad + s],
               a5 = S[5 * npad + s];
    o[0] = a0 * v[0] + a1 * v[1] + a2 * v[2];
    o[1] = a1 * v[0] + a3 * v[1] + a4 * v[2];
    o[2] = a2 * v[0] + a4 * v[1] + a5 * v[2];
}

// Total permanent field E = real space (fixed point) - A^T grad phi_recip + self term
// (MPIDReferenceForce.cpp:2922-2949), then mu_direct = alpha E and S E.
template <typename real>
MPID_KERNEL void k_record_fixed(KGrid<> kg, int n, int npad, BoxDev box, double selfCoef, const unsigned long long* __restrict__ fx,
                               const real* __restrict__ phi, AtomArrays<real> at, real* __restrict__ Efix,
                               real* __restrict__ muD, real* __restrict__ SE) {
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    real E[3] = {real(0), real(0), real(0)};
    if (s < n) {
        for (int c = 0; c < 3; ++c) {
            double e = fx_get(fx, c * npad + s);
            if (phi) e -= box.A[0][c] * (double) phi[npad + s] + box.A[1][c] * (double) phi[2 * npad + s] +
                          box.A[2][c] * (double) phi[3 * npad + s];
            e += selfCoef * (double) at.mom[(1 + c) * npad + s];
            E[c] = real(e);
        }
    }
    real m[3], se[3];
    sym_mul(at.alab, npad, s, E, m);
    sym_mul(at.sroot, npad, s, E, se);
    for (int c = 0; c < 3; ++c) {
        Efix[c * npad + s] = E[c];
        muD[c * npad + s] = m[c];
        SE[c * npad + s] = se[c];
    }
}

// sp = S p, and its fractional dipole for the spread (charge slot zero).
template <typename real>
MPID_KERNEL void k_apply_sroot(KGrid<> kg, int npad, BoxDev box, const real* __restrict__ S, const real* __restrict__ p,
                              real* __restrict__ sp, real* __restrict__ mfd, const int* __restrict__ skip) {
    if (skip && *skip) return;
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    real v[3] = {p[s], p[npad + s], p[2 * npad + s]}, o[3];
    sym_mul(S, npad, s, v, o);
    for (int c = 0; c < 3; ++c) sp[c * npad + s] = o[c];
    if (mfd) {
        mfd[s] = real(0);
        for (int j = 0; j < 3; ++j)
            mfd[(1 + j) * npad + s] = real(box.A[j][0]) * o[0] + real(box.A[j][1]) * o[1] + real(box.A[j][2]) * o[2];
    }
}

// Fractional dipoles of a dipole field (for spreading mu directly).
template <typename real>
MPID_KERNEL void k_frac_dipoles(KGrid<> kg, int npad, BoxDev box, const real* __restrict__ mu, real* __restrict__ mfd,
                               const int* __restrict__ skip) {
    if (skip && *skip) return;
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    const real o[3] = {mu[s], mu[npad + s], mu[2 * npad + s]};
    mfd[s] = real(0);
    for (int j = 0; j < 3; ++j)
        mfd[(1 + j) * npad + s] = real(box.A[j][0]) * o[0] + real(box.A[j][1]) * o[1] + real(box.A[j][2]) * o[2];
}

// Induced-dipole field at every atom: real space (fixed point) + reciprocal + self
// (MPIDReferenceForce.cpp:4073-4141).  Writes E (and optionally the gradient with the
// reciprocal part added, MPIDReferenceForce.cpp:4094-4130).
template <typename real>
MPID_KERNEL void k_dipole_field_total(KGrid<> kg, int n, int npad, BoxDev box, double selfCoef, const unsigned long long* __restrict__ fx,
                                     const unsigned long long* __restrict__ gfx, const real* __restrict__ phi, int nterm,
                                     const real* __restrict__ mu, real* __restrict__ E, real* __restrict__ G,
                                     const int* __restrict__ skip) {
    if (skip && *skip) return;
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    for (int c = 0; c < 3; ++c) {
        double e = 0.0;
        if (s < n) {
            e = fx_get(fx, c * npad + s) + selfCoef * (double) mu[c * npad + s];
            if (phi) e -= box.A[0][c] * (double) phi[npad + s] + box.A[1][c] * (double) phi[2 * npad + s] +
                          box.A[2][c] * (double) phi[3 * npad + s];
        }
        E[c * npad + s] = real(e);
    }
    if (G) {
        const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
        double H[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        if (phi && nterm >= 10) {
            H[0][0] = phi[4 * npad + s]; H[1][1] = phi[5 * npad + s]; H[2][2] = phi[6 * npad + s];
            H[0][1] = H[1][0] = phi[7 * npad + s];
            H[0][2] = H[2][0] = phi[8 * npad + s];
            H[1][2] = H[2][1] = phi[9 * npad + s];
        }
        for (int g = 0; g < 6; ++g) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) acc += box.A[k][ia[g]] * H[k][l] * box.A[l][ib[g]];
            G[g * npad + s] = s < n ? real(fx_get(gfx, g * npad + s) - acc) : real(0);
        }
    }
}

// q = p - S E (the CG operator B = I - S T S applied to p) and per-block partial p.q.
template <typename real>
MPID_KERNEL void k_cg_finish_matvec(KGrid<> kg, int npad, const real* __restrict__ S, const real* __restrict__ p,
                                   const real* __restrict__ E, real* __restrict__ q, double* __restrict__ partial,
                                   const int* __restrict__ skip) {
    __shared__ double red[256];
    if (skip && *skip) return;
    int s = kg.bx * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (s < npad) {
        real e[3] = {E[s], E[npad + s], E[2 * npad + s]}, se[3];
        sym_mul(S, npad, s, e, se);
        for (int c = 0; c < 3; ++c) {
            const real pv = p[c * npad + s];
            const real qv = pv - se[c];
            q[c * npad + s] = qv;
            acc += (double) pv * (double) qv;
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[kg.bx] = red[0];
}

// Deterministic final reduction of per-block partials (one block).
MPID_KERNEL void k_reduce_partials(KGrid<> kg, int nblocks, int nvals, const double* __restrict__ partial, double* __restrict__ out,
                                  const int* __restrict__ skip) {
    __shared__ double red[1024];
    if (skip && *skip) return;
    for (int v = 0; v < nvals; ++v) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partial[v * nblocks + b];
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[v] = red[0];
        __syncthreads();
    }
}

// CG scalars: slot 0 rr, 1 pq, 2 rr_new, 3 |S r|^2, 4 alpha, 5 beta, 6 metric.
// x += a p, r -= a q; partials of r.r and |S r|^2.
template <typename real, typename xreal>
MPID_KERNEL void k_cg_update(KGrid<> kg, int npad, const real* __restrict__ S, double* __restrict__ sc, const real* __restrict__ p,
                            const real* __restrict__ q, xreal* __restrict__ x, real* __restrict__ r,
                            double* __restrict__ partial, int nblocks, const int* __restrict__ skip) {
    __shared__ double red[2][256];
    if (skip && *skip) return;
    const double a = sc[0] / sc[1];
    int s = kg.bx * blockDim.x + threadIdx.x;
    double rr = 0.0, sr = 0.0;
    if (s < npad) {
        real rv[3];
        for (int c = 0; c < 3; ++c) {
            x[c * npad + s] += xreal(a * (double) p[c * npad + s]);
            rv[c] = real((double) r[c * npad + s] - a * (double) q[c * npad + s]);
            r[c * npad + s] = rv[c];
            rr += (double) rv[c] * (double) rv[c];
        }
        real z[3];
        sym_mul(S, npad, s, rv, z);
        sr = (double) z[0] * z[0] + (double) z[1] * z[1] + (double) z[2] * z[2];
    }
    red[0][threadIdx.x] = rr;
    red[1][threadIdx.x] = sr;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red[0][threadIdx.x] += red[0][threadIdx.x + o];
            red[1][threadIdx.x] += red[1][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[kg.bx] = red[0][0];
        partial[nblocks + kg.bx] = red[1][0];
    }
}

// After the reductions: beta, convergence test 48.033324 sqrt(|S r|^2 / n) < target
// (MPIDReferenceForce.cpp:1219), iteration limit.  done[0] = 1 stops the loop.
MPID_KERNEL void k_cg_scalars(KGrid<> kg, double* __restrict__ sc, const double* __restrict__ red, int n, double target,
                             int* __restrict__ iter, int maxIter, int* __restrict__ done) {
    if (*done) return;
    sc[2] = red[0];
    sc[3] = red[1];
    sc[5] = sc[2] / sc[0];
    sc[0] = sc[2];
    sc[6] = 48.033324 * sqrt(sc[3] / n);
    *iter += 1;
    if (sc[6] < target || *iter >= maxIter || !(sc[6] == sc[6])) *done = 1;
}

template <typename real>
MPID_KERNEL void k_cg_direction(KGrid<> kg, int npad, const double* __restrict__ sc, const real* __restrict__ r, real* __restrict__ p,
                               const int* __restrict__ skip) {
    if (skip && *skip) return;
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    const double b = sc[5];
    for (int c = 0; c < 3; ++c) p[c * npad + s] = real((double) r[c * npad + s] + b * (double) p[c * npad + s]);
}

// Initial CG state from the right-hand side: r = p = b, x = 0, partials of r.r and |S r|^2.
template <typename real, typename xreal>
MPID_KERNEL void k_cg_start(KGrid<> kg, int npad, const real* __restrict__ S, const real* __restrict__ b, xreal* __restrict__ x,
                           real* __restrict__ r, real* __restrict__ p, double* __restrict__ partial, int nblocks) {
    __shared__ double red[2][256];
    int s = kg.bx * blockDim.x + threadIdx.x;
    double rr = 0.0, sr = 0.0;
    if (s < npad) {
        real v[3];
        for (int c = 0; c < 3; ++c) {
            v[c] = b[c * npad + s];
            x[c * npad + s] = xreal(0);
            r[c * npad + s] = v[c];
            p[c * npad + s] = v[c];
            rr += (double) v[c] * v[c];
        }
        real z[3];
        sym_mul(S, npad, s, v, z);
        sr = (double) z[0] * z[0] + (double) z[1] * z[1] + (double) z[2] * z[2];
    }
    red[0][threadIdx.x] = rr;
    red[1][threadIdx.x] = sr;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red[0][threadIdx.x] += red[0][threadIdx.x + o];
            red[1][threadIdx.x] += red[1][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[kg.bx] = red[0][0];
        partial[nblocks + kg.bx] = red[1][0];
    }
}

MPID_KERNEL void k_cg_init_scalars(KGrid<> kg, double* __restrict__ sc, const double* __restrict__ red, int n, double target,
                                  int* __restrict__ iter, int* __restrict__ done) {
    sc[0] = red[0];
    sc[3] = red[1];
    sc[6] = 48.033324 * sqrt(red[1] / n);
    *iter = 0;
    *done = (sc[6] < target) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Fused CG iteration kernels.  Each reduction writes per-block partials and the last
// block to finish sums them in block order (deterministic) and updates the scalars, so
// an iteration needs no separate reduction launches.  `counter` returns to 0 after use.

// Block sum of v over 256 threads (fixed order: warp shuffles, then the 8 warp sums);
// the result is valid in thread 0.
__device__ __forceinline__ double block_sum_256(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();  // red may still be read from the previous sum
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
        for (int o = 4; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    }
    return t;
}

// True in exactly one block: the last of the `nblocks` blocks sharing `counter` to pass
// this point (after each block has published its partials).
__device__ __forceinline__ bool last_block(unsigned* counter, unsigned nblocks) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == nblocks - 1;
    __syncthreads();
    return last;
}

// Fixed-order sum of partial[0..nblocks) by one block of 256 threads.
__device__ __forceinline__ double sum_partials_256(const double* partial, int nblocks, double* red) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += 256) acc += ((volatile const double*) partial)[b];
    return block_sum_256(acc, red);
}

// Start of an iteration: p = r + beta p (not on the first), sp = S p and the fractional
// dipoles of sp for the reciprocal-space spread.
template <typename real>
MPID_KERNEL void k_cg_direction_sroot(KGrid<> kg, int npad, BoxDev box, const real* __restrict__ S, const double* __restrict__ sc,
                                     int first, const real* __restrict__ r, real* __restrict__ p, real* __restrict__ sp,
                                     real* __restrict__ mfd, const typename Vec4<real>::type* __restrict__ prm,
                                     typename Vec4<real>::type* __restrict__ A1, const int* __restrict__ skip) {
    if (*skip) return;
    const int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    real v[3];
    if (first) {
        for (int c = 0; c < 3; ++c) v[c] = p[c * npad + s];
    } else {
        const double b = sc[5];
        for (int c = 0; c < 3; ++c) {
            v[c] = real((double) r[c * npad + s] + b * (double) p[c * npad + s]);
            p[c * npad + s] = v[c];
        }
    }
    real o[3];
    sym_mul(S, npad, s, v, o);
    for (int c = 0; c < 3; ++c) sp[c * npad + s] = o[c];
    if (A1) A1[s] = Vec4<real>::make(o[0], o[1], o[2], prm[s].w);  // (S p, 1 / damping)
    if (mfd) {
        mfd[s] = real(0);
        for (int j = 0; j < 3; ++j)
            mfd[(1 + j) * npad + s] = real(box.A[j][0]) * o[0] + real(box.A[j][1]) * o[1] + real(box.A[j][2]) * o[2];
    }
}

// E = T sp (real space from the fixed-point accumulator, which is cleared here, plus
// reciprocal and self terms), q = p - S E, and sc[1] = p.q.
template <typename real>
MPID_KERNEL void k_cg_matvec_finish(KGrid<256> kg, int n, int npad, BoxDev box, double selfCoef, unsigned long long* __restrict__ fx,
                   const real* __restrict__ phi, const real* __restrict__ S, const real* __restrict__ p,
                   const real* __restrict__ sp, real* __restrict__ q, double* __restrict__ partial,
                   unsigned* __restrict__ counter, double* __restrict__ sc, const int* __restrict__ skip) {
    __shared__ double red[256];
    if (*skip) return;
    const int s = kg.bx * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (s < npad) {
        real e[3];
        for (int c = 0; c < 3; ++c) {
            double v = 0.0;
            if (s < n) {
                v = fx_get(fx, c * npad + s) + selfCoef * (double) sp[c * npad + s];
                if (phi) v -= box.A[0][c] * (double) phi[npad + s] + box.A[1][c] * (double) phi[2 * npad + s] +
                              box.A[2][c] * (double) phi[3 * npad + s];
            }
            fx[c * npad + s] = 0ull;
            e[c] = real(v);
        }
        real se[3];
        sym_mul(S, npad, s, e, se);
        for (int c = 0; c < 3; ++c) {
            const real pv = p[c * npad + s];
            const real qv = pv - se[c];
            q[c * npad + s] = qv;
            acc += (double) pv * (double) qv;
        }
    }
    const double b = block_sum_256(acc, red);
    if (threadIdx.x == 0) partial[kg.bx] = b;
    if (last_block(counter, kg.nb)) {
        const double pq = sum_partials_256(partial, kg.nb, red);
        if (threadIdx.x == 0) {
            sc[1] = pq;
            *counter = 0u;
        }
    }
}

// x += a p, r -= a q (a = rr / pq); then beta, the convergence test
// 48.033324 sqrt(|S r|^2 / n) < target (MPIDReferenceForce.cpp:1219) and the iteration
// limit; done = 1 stops the loop.  sc: 0 rr, 1 pq, 2 rr_new, 3 |S r|^2, 5 beta, 6 metric.
template <typename real, typename xreal>
MPID_KERNEL void k_cg_update_scalars(KGrid<256> kg, int n, int npad, const real* __restrict__ S, double* __restrict__ sc, const real* __restrict__ p,
                    const real* __restrict__ q, xreal* __restrict__ x, real* __restrict__ r, double* __restrict__ partial,
                    unsigned* __restrict__ counter, double target, int* __restrict__ iter, int maxIter,
                    int* __restrict__ done, int pcg) {
    __shared__ double red[256];
    if (*done) return;
    const double a = sc[0] / sc[1];
    const int s = kg.bx * blockDim.x + threadIdx.x;
    double rr = 0.0, sr = 0.0;
    if (s < npad) {
        real rv[3];
        for (int c = 0; c < 3; ++c) {
            x[c * npad + s] += xreal(a * (double) p[c * npad + s]);
            rv[c] = real((double) r[c * npad + s] - a * (double) q[c * npad + s]);
            r[c * npad + s] = rv[c];
            rr += (double) rv[c] * (double) rv[c];
        }
        real z[3];
        sym_mul(S, npad, s, rv, z);
        sr = (double) z[0] * z[0] + (double) z[1] * z[1] + (double) z[2] * z[2];
    }
    const double b0 = block_sum_256(rr, red);
    const double b1 = block_sum_256(sr, red);
    if (threadIdx.x == 0) {
        partial[kg.bx] = b0;
        partial[kg.nb + kg.bx] = b1;
    }
    if (last_block(counter, kg.nb)) {
        const double rrNew = sum_partials_256(partial, kg.nb, red);
        const double srNew = sum_partials_256(partial + kg.nb, kg.nb, red);
        if (threadIdx.x == 0) {
            sc[2] = rrNew;
            sc[3] = srNew;
            if (!pcg) {  // plain CG: beta from r.r; PCG takes it from k_precond_finish
                sc[5] = rrNew / sc[0];
                sc[0] = rrNew;
            }
            sc[6] = 48.033324 * sqrt(srNew / n);
            *iter += 1;
            if (sc[6] < target || *iter >= maxIter || !(sc[6] == sc[6])) *done = 1;
            *counter = 0u;
        }
    }
}

// ---------------------------------------------------------------------------
// Single-reduction CG (Chronopoulos and Gear) on B y = b, B = I - S T S: each iteration
// makes one operator application w = B r and one global reduction per kernel,
//   p = r + beta p, s = w + beta s, x += alpha p, r -= alpha s          (update)
//   gamma' = r.r, beta' = gamma' / gamma                               (update)
//   w' = B r', delta' = w'.r', alpha' = gamma' / (delta' - beta' gamma' / alpha)   (finish)
// which is CG in exact arithmetic: the same iterates with two small kernels per
// iteration instead of three.  sc: 0 gamma, 1 delta, 3 |S r|^2, 4 alpha, 5 beta,
// 6 metric 48.033324 sqrt(|S r|^2 / n) (MPIDReferenceForce.cpp:1219).

// The operator input of an iteration from r: sp = S r, its fractional dipoles for the
// reciprocal-space spread and (FP32) the packed operand A1 = (S r, 1 / damping).
template <typename real>
__device__ __forceinline__ void cgcg_operator_input(int npad, int s, const BoxDev& box, const real* S, const real* v,
                                                    real* sp, real* mfd, const typename Vec4<real>::type* prm,
                                                    typename Vec4<real>::type* A1) {
    real o[3];
    sym_mul(S, npad, s, v, o);
    for (int c = 0; c < 3; ++c) sp[c * npad + s] = o[c];
    if (A1) A1[s] = Vec4<real>::make(o[0], o[1], o[2], prm[s].w);
    if (mfd) {
        mfd[s] = real(0);
        for (int j = 0; j < 3; ++j)
            mfd[(1 + j) * npad + s] = real(box.A[j][0]) * o[0] + real(box.A[j][1]) * o[1] + real(box.A[j][2]) * o[2];
    }
}

// r = b, x = p = s = 0; gamma, the metric of r and the operator input of r.
template <typename real, typename xreal>
MPID_KERNEL void k_cgcg_start(KGrid<256> kg, int n, int npad, BoxDev box, const real* __restrict__ S, const real* __restrict__ b, xreal* __restrict__ x,
             real* __restrict__ r, real* __restrict__ p, real* __restrict__ sv, real* __restrict__ sp,
             real* __restrict__ mfd, const typename Vec4<real>::type* __restrict__ prm,
             typename Vec4<real>::type* __restrict__ A1, double* __restrict__ partial, unsigned* __restrict__ counter,
             double* __restrict__ sc, double target, int* __restrict__ iter, int* __restrict__ done) {
    __shared__ double red[256];
    const int s = kg.bx * blockDim.x + threadIdx.x;
    double rr = 0.0, sr = 0.0;
    if (s < npad) {
        real v[3];
        for (int c = 0; c < 3; ++c) {
            v[c] = b[c * npad + s];
            x[c * npad + s] = xreal(0);
            r[c * npad + s] = v[c];
            p[c * npad + s] = real(0);
            sv[c * npad + s] = real(0);
            rr += (double) v[c] * v[c];
        }
        real z[3];
        sym_mul(S, npad, s, v, z);
        sr = (double) z[0] * z[0] + (double) z[1] * z[1] + (double) z[2] * z[2];
        cgcg_operator_input(npad, s, box, S, v, sp, mfd, prm, A1);
    }
    const double b0 = block_sum_256(rr, red);
    const double b1 = block_sum_256(sr, red);
    if (threadIdx.x == 0) {
        partial[kg.bx] = b0;
        partial[kg.nb + kg.bx] = b1;
    }
    if (last_block(counter, kg.nb)) {
        const double g = sum_partials_256(partial, kg.nb, red);
        const double m = sum_partials_256(partial + kg.nb, kg.nb, red);
        if (threadIdx.x == 0) {
            sc[0] = g;
            sc[3] = m;
            sc[4] = 0.0;
            sc[5] = 0.0;
            sc[6] = 48.033324 * sqrt(m / n);
            *iter = 0;
            *done = (sc[6] < target) ? 1 : 0;
            *counter = 0u;
        }
    }
}

// w = B r (real space from the fixed-point accumulator, which is cleared here, plus the
// reciprocal and self terms), delta = w.r, then alpha (first iteration: gamma / delta).
template <typename real>
MPID_KERNEL void k_cgcg_finish(KGrid<256> kg, int n, int npad, BoxDev box, double selfCoef, unsigned long long* __restrict__ fx,
              const real* __restrict__ phi, const real* __restrict__ S, const real* __restrict__ r,
              const real* __restrict__ sp, real* __restrict__ w, double* __restrict__ partial,
              unsigned* __restrict__ counter, double* __restrict__ sc, const int* __restrict__ iter,
              const int* __restrict__ skip) {
    __shared__ double red[256];
    if (*skip) return;
    const int s = kg.bx * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (s < npad) {
        real e[3];
        for (int c = 0; c < 3; ++c) {
            double v = 0.0;
            if (s < n) {
                v = fx_get(fx, c * npad + s) + selfCoef * (double) sp[c * npad + s];
                if (phi) v -= box.A[0][c] * (double) phi[npad + s] + box.A[1][c] * (double) phi[2 * npad + s] +
                              box.A[2][c] * (double) phi[3 * npad + s];
            }
            fx[c * npad + s] = 0ull;
            e[c] = real(v);
        }
        real se[3];
        sym_mul(S, npad, s, e, se);
        for (int c = 0; c < 3; ++c) {
            const real rv = r[c * npad + s];
            const real wv = rv - se[c];
            w[c * npad + s] = wv;
            acc += (double) wv * (double) rv;
        }
    }
    const double b = block_sum_256(acc, red);
    if (threadIdx.x == 0) partial[kg.bx] = b;
    if (last_block(counter, kg.nb)) {
        const double delta = sum_partials_256(partial, kg.nb, red);
        if (threadIdx.x == 0) {
            const double g = sc[0], beta = sc[5];
            sc[1] = delta;
            sc[4] = *iter == 0 ? g / delta : g / (delta - beta * g / sc[4]);
            *counter = 0u;
        }
    }
}

// p = r + beta p, s = w + beta s, x += alpha p, r -= alpha s; gamma' and beta', the
// convergence test and the iteration limit (done = 1 stops the loop: the kernels of the
// remaining iterations return at once), and the operator input of the new r.
template <typename real, typename xreal>
MPID_KERNEL void k_cgcg_update(KGrid<256> kg, int n, int npad, BoxDev box, const real* __restrict__ S, double* __restrict__ sc,
              const real* __restrict__ w, real* __restrict__ p, real* __restrict__ sv, xreal* __restrict__ x,
              real* __restrict__ r, real* __restrict__ sp, real* __restrict__ mfd,
              const typename Vec4<real>::type* __restrict__ prm, typename Vec4<real>::type* __restrict__ A1,
              double* __restrict__ partial, unsigned* __restrict__ counter, double target, int* __restrict__ iter,
              int maxIter, int* __restrict__ done) {
    __shared__ double red[256];
    if (*done) return;
    const double a = sc[4], beta = sc[5];
    const int s = kg.bx * blockDim.x + threadIdx.x;
    double rr = 0.0, sr = 0.0;
    if (s < npad) {
        real rv[3];
        for (int c = 0; c < 3; ++c) {
            const int k = c * npad + s;
            const real pv = real((double) r[k] + beta * (double) p[k]);
            const real svv = real((double) w[k] + beta * (double) sv[k]);
            p[k] = pv;
            sv[k] = svv;
            x[k] += xreal(a * (double) pv);
            rv[c] = real((double) r[k] - a * (double) svv);
            r[k] = rv[c];
            rr += (double) rv[c] * (double) rv[c];
        }
        real z[3];
        sym_mul(S, npad, s, rv, z);
        sr = (double) z[0] * z[0] + (double) z[1] * z[1] + (double) z[2] * z[2];
        cgcg_operator_input(npad, s, box, S, rv, sp, mfd, prm, A1);
    }
    const double b0 = block_sum_256(rr, red);
    const double b1 = block_sum_256(sr, red);
    if (threadIdx.x == 0) {
        partial[kg.bx] = b0;
        partial[kg.nb + kg.bx] = b1;
    }
    if (last_block(counter, kg.nb)) {
        const double g = sum_partials_256(partial, kg.nb, red);
        const double m = sum_partials_256(partial + kg.nb, kg.nb, red);
        if (threadIdx.x == 0) {
            sc[5] = g / sc[0];
            sc[0] = g;
            sc[3] = m;
            sc[6] = 48.033324 * sqrt(m / n);
            *iter += 1;
            if (sc[6] < target || *iter >= maxIter || !(sc[6] == sc[6])) *done = 1;
            *counter = 0u;
        }
    }
}

// ---------------------------------------------------------------------------
// Near-field preconditioner of the mutual CG: P = I + S T_n S, T_n the bare
// Thole-damped dipole field (b_1 = lambda_3 / r^3, b_2 = 3 lambda_5 / r^5) over the
// quadrature segment of the lists (alpha r < 1.5 and covalent pairs), where the
// coupling of induced dipoles is strongest.  P is a first-order approximation of
// B^-1 = (I - S T S)^-1 and costs one pass over about an eighth of the pairs.

// w_i = T_n v over atom i's near pairs, v_j = S_j r_j (fixed-point accumulation).
template <typename real>
MPID_KERNEL void k_precond_field(KGrid<(32 * kWarpsPerBlock)> kg, NbrList nl, AtomArrays<real> at, const real* __restrict__ r, unsigned long long* __restrict__ w,
                const int* __restrict__ skip) {
    if (*skip) return;
    const int wi = (kg.bx * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (nl.nchunksS == 0) return;
    const int I = wi / nl.nchunksS;
    const int k0 = (wi - I * nl.nchunksS) * nl.chunk;
    if (I >= nl.ntiles || k0 >= nl.tmaxS[I]) return;
    const int si = I * 32 + lane, npad = at.npad;
    if (at.orig[si] < 0) return;
    const int k1 = min(k0 + nl.chunk, nl.countS[si]);
    const PairConsts<real>& pc = pair_consts<real>(nl);
    const real oi[3] = {at.off[si], at.off[npad + si], at.off[2 * npad + si]};
    const typename Vec4<real>::type pi = at.prm[si];
    real acc[3] = {real(0), real(0), real(0)};
    for (int k = k0; k < k1; ++k) {
        int sj;
        unsigned flag;
        real d[3], r2;
        if (!list_pair<real, true>(nl, pc, at, I, k, lane, oi, sj, flag, d, r2)) continue;
        const typename Vec4<real>::type pj = at.prm[sj];
        const real dd = pi.y * pj.y;
        real lam[3] = {real(1), real(1), real(1)}, om[3];
        const real rr = sqrt(r2);
        if (dd > real(0)) {
            const real sT = (flag == 1u ? pi.x + pj.x : pc.thole) * rr / dd;
            if (sT < real(50)) thole_lambdas<real, 2>(sT, lam, om);
        }
        const real rinv2 = real(1) / r2;
        const real r3inv = rinv2 / rr;
        const real b1 = lam[1] * r3inv;
        const real b2 = real(3) * lam[2] * r3inv * rinv2;
        const real rj[3] = {r[sj], r[npad + sj], r[2 * npad + sj]};
        real v[3];
        sym_mul(at.sroot, npad, sj, rj, v);
        const real vd = v[0] * d[0] + v[1] * d[1] + v[2] * d[2];
#pragma unroll
        for (int q = 0; q < 3; ++q) acc[q] += b2 * vd * d[q] - b1 * v[q];
    }
    for (int q = 0; q < 3; ++q) fx_add(w + q * npad + si, acc[q]);
}

// z = r + S w (w read and cleared), r.z; on the first application also p = z and
// sc[0] = r.z, afterwards sc[5] = beta = (r.z)_new / (r.z)_old and sc[0] = (r.z)_new.
template <typename real>
MPID_KERNEL void k_precond_finish(KGrid<256> kg, int n, int npad, const real* __restrict__ S, unsigned long long* __restrict__ wfx,
                 const real* __restrict__ r, real* __restrict__ z, real* __restrict__ p, int first,
                 double* __restrict__ partial, unsigned* __restrict__ counter, double* __restrict__ sc,
                 const int* __restrict__ skip) {
    __shared__ double red[256];
    if (*skip) return;
    const int s = kg.bx * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (s < npad) {
        real wv[3];
        for (int c = 0; c < 3; ++c) {
            wv[c] = s < n ? real(fx_get(wfx, c * npad + s)) : real(0);
            wfx[c * npad + s] = 0ull;
        }
        real sw[3];
        sym_mul(S, npad, s, wv, sw);
        for (int c = 0; c < 3; ++c) {
            const real rv = r[c * npad + s];
            const real zv = rv + sw[c];
            z[c * npad + s] = zv;
            if (first) p[c * npad + s] = zv;
            acc += (double) rv * (double) zv;
        }
    }
    const double b = block_sum_256(acc, red);
    if (threadIdx.x == 0) partial[kg.bx] = b;
    if (last_block(counter, kg.nb)) {
        const double rz = sum_partials_256(partial, kg.nb, red);
        if (threadIdx.x == 0) {
            if (!first) sc[5] = rz / sc[0];
            sc[0] = rz;
            *counter = 0u;
        }
    }
}

// mu = S y (sorted), in the precision of the pair kernels.
template <typename xreal, typename real>
MPID_KERNEL void k_mu_from_y(KGrid<> kg, int npad, const xreal* __restrict__ S, const xreal* __restrict__ y, real* __restrict__ mu) {
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    xreal v[3] = {y[s], y[npad + s], y[2 * npad + s]}, o[3];
    sym_mul(S, npad, s, v, o);
    for (int c = 0; c < 3; ++c) mu[c * npad + s] = real(o[c]);
}

// FP64 residual of the refinement loop: res = S (E + T S y) - y with T S y already in E2
// (E2 = field of mu = S y, including reciprocal and self terms).  Partial |S res|^2.
MPID_KERNEL void k_refine_residual(KGrid<> kg, int npad, const double* __restrict__ S, const double* __restrict__ Efix,
                                  const double* __restrict__ E2, const double* __restrict__ y, double* __restrict__ res,
                                  float* __restrict__ res32, double* __restrict__ partial) {
    __shared__ double red[256];
    int s = kg.bx * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (s < npad) {
        double e[3] = {Efix[s] + E2[s], Efix[npad + s] + E2[npad + s], Efix[2 * npad + s] + E2[2 * npad + s]}, se[3];
        sym_mul(S, npad, s, e, se);
        double rv[3];
        for (int c = 0; c < 3; ++c) {
            rv[c] = se[c] - y[c * npad + s];
            res[c * npad + s] = rv[c];
            res32[c * npad + s] = (float) rv[c];
        }
        double z[3];
        sym_mul(S, npad, s, rv, z);
        acc = z[0] * z[0] + z[1] * z[1] + z[2] * z[2];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[kg.bx] = red[0];
}

template <typename real>
MPID_KERNEL void k_axpy_to_double(KGrid<> kg, int npad3, const real* __restrict__ d, double* __restrict__ y) {
    int i = kg.bx * blockDim.x + threadIdx.x;
    if (i < npad3) y[i] += (double) d[i];
}

// mu_(m+1) = alpha E_m for the extrapolated solver; mu_out accumulates cbar-weighted sum.
template <typename real>
MPID_KERNEL void k_alpha_times(KGrid<> kg, int npad, const real* __restrict__ alab, const real* __restrict__ E, real* __restrict__ out) {
    int s = kg.bx * blockDim.x + threadIdx.x;
    if (s >= npad) return;
    real v[3] = {E[s], E[npad + s], E[2 * npad + s]}, o[3];
    sym_mul(alab, npad, s, v, o);
    for (int c = 0; c < 3; ++c) out[c * npad + s] = o[c];
}

template <typename real>
MPID_KERNEL void k_axpy(KGrid<> kg, int n3, real a, const real* __restrict__ x, real* __restrict__ y) {
    int i = kg.bx * blockDim.x + threadIdx.x;
    if (i < n3) y[i] += a * x[i];
}

// Reciprocal-space and self terms per atom (MPIDReferenceForce.cpp:3739-4024,
// 4283-4333) and the extrapolated-solver response (MPIDReferenceForce.cpp:4956-4984).
struct OptArgs {
    int nPT;                 // number of perturbation orders (0 when not extrapolated)
    double cbar[8];
    const void* mu;          // nPT x [3][npad]
    const void* E;           // (nPT-1) x [3][npad]
    const void* G;           // (nPT-1) x [6][npad]
};

template <typename real>
MPID_KERNEL void k_recip_self(KGrid<> kg, int n, int npad, BoxDev box, double alpha, int polType, const real* __restrict__ phiP,
                             const real* __restrict__ phiD, const real* __restrict__ mu, AtomArrays<real> at,
                             const double* __restrict__ mom64, OptArgs opt, unsigned long long* __restrict__ force,
                             unsigned long long* __restrict__ torque, double* __restrict__ energyPartial) {
    __shared__ double red[256];
    const int s = kg.bx * blockDim.x + threadIdx.x;
    double eAcc = 0.0;
    if (s < n) {
        const bool aniso = at.prm[s].z != real(0);
        LabMoments<real> m;
        load_moments(at.mom, npad, s, m);
        const real ui[3] = {mu[s], mu[npad + s], mu[2 * npad + s]};
        real A[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) A[a][b] = real(box.A[a][b]);
        double F[3] = {0, 0, 0}, T[3] = {0, 0, 0};
        if (phiP) {
            real Mf[20];
            frac_multipole(m, A, Mf);
            real muf[3];
            for (int j = 0; j < 3; ++j) muf[j] = A[j][0] * ui[0] + A[j][1] * ui[1] + A[j][2] * ui[2];
            // energy contractions in FP64, force contractions in the kernel precision
            auto PP = [&](int t, int u, int v) { return phiP[hermite_index(t, u, v) * npad + s]; };
            auto PD = [&](int t, int u, int v) { return phiD[hermite_index(t, u, v) * npad + s]; };
            double ef = 0.0, ei = 0.0;
            real f[3] = {real(0), real(0), real(0)};
            for (int k = 0; k < 20; ++k) {
                int t, u, v;
                hermite_tuv(k, t, u, v);
                ef += (double) Mf[k] * (double) PP(t, u, v);
                f[0] += Mf[k] * (PP(t + 1, u, v) + PD(t + 1, u, v));
                f[1] += Mf[k] * (PP(t, u + 1, v) + PD(t, u + 1, v));
                f[2] += Mf[k] * (PP(t, u, v + 1) + PD(t, u, v + 1));
            }
            for (int k = 0; k < 3; ++k) {
                const int t = k == 0, u = k == 1, v = k == 2;
                ei += (double) muf[k] * (double) PP(t, u, v);
                real g0 = PP(t + 1, u, v), g1 = PP(t, u + 1, v), g2 = PP(t, u, v + 1);
                if (polType == 0) { g0 += PD(t + 1, u, v); g1 += PD(t, u + 1, v); g2 += PD(t, u, v + 1); }
                f[0] += muf[k] * g0;
                f[1] += muf[k] * g1;
                f[2] += muf[k] * g2;
            }
            eAcc += 0.5 * kElectric * (ef + ei);
            for (int c = 0; c < 3; ++c)
                F[c] -= kElectric * (double) (A[0][c] * f[0] + A[1][c] * f[1] + A[2][c] * f[2]);
            // torques from the permanent and induced reciprocal potentials
            real P0, P1[3], P2[3][3], P3[3][3][3], tau[3], dtot[3];
            for (int c = 0; c < 3; ++c) dtot[c] = m.d[c] + (aniso ? ui[c] : real(0));
            real ph[35];
            for (int k = 0; k < 35; ++k) ph[k] = phiP[k * npad + s];
            cartesian_potential(ph, A, P0, P1, P2, P3);
            multipole_torque(dtot, m.Q, m.O, P1, P2, P3, tau);
            for (int c = 0; c < 3; ++c) T[c] += kElectric * (double) tau[c];
            for (int c = 0; c < 3; ++c) dtot[c] = m.d[c] + ((aniso && polType == 0) ? ui[c] : real(0));
            for (int k = 0; k < 35; ++k) ph[k] = phiD[k * npad + s];
            cartesian_potential(ph, A, P0, P1, P2, P3);
            multipole_torque(dtot, m.Q, m.O, P1, P2, P3, tau);
            for (int c = 0; c < 3; ++c) T[c] += kElectric * (double) tau[c];
            // self torque (isotropic atoms) and self energy
            const double a3 = alpha * alpha * alpha;
            if (!aniso) {
                const double term = 2.0 / 3.0 * kElectric * a3 / kSqrtPiRef;
                const double u2[3] = {2.0 * ui[0], 2.0 * ui[1], 2.0 * ui[2]};
                T[0] += term * ((double) m.d[1] * u2[2] - (double) m.d[2] * u2[1]);
                T[1] += term * ((double) m.d[2] * u2[0] - (double) m.d[0] * u2[2]);
                T[2] += term * ((double) m.d[0] * u2[1] - (double) m.d[1] * u2[0]);
            }
            // Ewald self energy in FP64 from the FP64 lab moments
            LabMoments<double> m64;
            if (mom64) {
                load_moments(mom64, npad, s, m64);
            } else {
                m64.q = m.q;
                for (int k = 0; k < 3; ++k) m64.d[k] = m.d[k];
                for (int k = 0; k < 6; ++k) m64.Q[k] = m.Q[k];
                for (int k = 0; k < 10; ++k) m64.O[k] = m.O[k];
            }
            double ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0}, ez[3] = {0, 0, 1};
            double S[16];
            frame_spherical(m64, ex, ey, ez, S);
            double qii = 0, oii = 0, dii = 0;
            for (int k = 4; k < 9; ++k) qii += S[k] * S[k];
            for (int k = 9; k < 16; ++k) oii += S[k] * S[k];
            for (int c = 0; c < 3; ++c) dii += m64.d[c] * (m64.d[c] + (double) ui[c]);
            const double a2 = alpha * alpha;
            eAcc += -alpha * kElectric / kSqrtPiRef *
                    (m64.q * m64.q + 2.0 / 3.0 * a2 * dii + 4.0 / 15.0 * a2 * a2 * qii + 8.0 / 105.0 * a2 * a2 * a2 * oii);
        }
        if (opt.nPT > 0) {
            const real* MU = (const real*) opt.mu;
            const real* EE = (const real*) opt.E;
            const real* GG = (const real*) opt.G;
            const size_t st3 = (size_t) 3 * npad, st6 = (size_t) 6 * npad;
            for (int l = 0; l < opt.nPT - 1; ++l)
                for (int mm = 0; mm < opt.nPT - 1 - l; ++mm) {
                    const double pw = opt.cbar[l + mm + 1];
                    if (fabs(pw) < 1e-6) continue;
                    const double u[3] = {MU[l * st3 + s], MU[l * st3 + npad + s], MU[l * st3 + 2 * npad + s]};
                    double g[6];
                    for (int q = 0; q < 6; ++q) g[q] = GG[mm * st6 + q * npad + s];
                    F[0] += pw * kElectric * (u[0] * g[0] + u[1] * g[3] + u[2] * g[4]);
                    F[1] += pw * kElectric * (u[0] * g[3] + u[1] * g[1] + u[2] * g[5]);
                    F[2] += pw * kElectric * (u[0] * g[4] + u[1] * g[5] + u[2] * g[2]);
                    if (aniso) {
                        const double e[3] = {EE[mm * st3 + s], EE[mm * st3 + npad + s], EE[mm * st3 + 2 * npad + s]};
                        T[0] += pw * kElectric * (u[1] * e[2] - u[2] * e[1]);
                        T[1] += pw * kElectric * (u[2] * e[0] - u[0] * e[2]);
                        T[2] += pw * kElectric * (u[0] * e[1] - u[1] * e[0]);
                    }
                }
        }
        for (int c = 0; c < 3; ++c) {
            fx_add(force + c * npad + s, F[c]);
            fx_add(torque + c * npad + s, T[c]);
        }
    }
    red[threadIdx.x] = eAcc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) energyPartial[kg.bx] = red[0];
}

// Torque on each atom -> forces on it and its frame atoms (original order loop).
MPID_KERNEL void k_torque_map(KGrid<> kg, int n, int npad, const double* __restrict__ pos, MolArrays mol, const int* __restrict__ rank,
                             const unsigned long long* __restrict__ torque, unsigned long long* __restrict__ force) {
    int i = kg.bx * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int ax = mol.axis[i];
    if (ax == NoAxisType) return;
    const int s = rank[i];
    const double T[3] = {fx_get(torque, s), fx_get(torque, npad + s), fx_get(torque, 2 * npad + s)};
    const int iz = mol.az[i], ix = mol.ax[i], iy = mol.ay[i];
    const double* pI = pos + 3 * i;
    const double* pZ = pos + 3 * iz;
    const double* pX = ix >= 0 ? pos + 3 * ix : pI;
    const double* pY = iy >= 0 ? pos + 3 * iy : pI;
    double fI[3], fZ[3], fX[3], fY[3];
    torque_to_force<double>(ax, pI, pZ, pX, pY, iy >= 0, T, fI, fZ, fX, fY);
    for (int c = 0; c < 3; ++c) {
        fx_add(force + c * npad + s, fI[c]);
        fx_add(force + c * npad + rank[iz], fZ[c]);
        if (ix >= 0) fx_add(force + c * npad + rank[ix], fX[c]);
        if (iy >= 0) fx_add(force + c * npad + rank[iy], fY[c]);
    }
}

// out[i] += F (accumulate, as OpenMM kernels add into the context force buffer).
MPID_KERNEL void k_forces_out(KGrid<> kg, int n, int npad, const int* __restrict__ rank, const unsigned long long* __restrict__ force,
                             double* __restrict__ out) {
    int i = kg.bx * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = rank[i];
    for (int c = 0; c < 3; ++c) out[3 * i + c] += fx_get(force, c * npad + s);
}

// Dipoles in original order: which 0 induced, 1 lab permanent, 2 total.
template <typename real>
MPID_KERNEL void k_dipoles_out(KGrid<> kg, int n, int npad, int which, const int* __restrict__ rank, const real* __restrict__ mom,
                              const real* __restrict__ mu, double* __restrict__ out) {
    int i = kg.bx * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = rank[i];
    for (int c = 0; c < 3; ++c) {
        double v = 0.0;
        if (which != 1) v += (double) mu[c * npad + s];
        if (which != 0) v += (double) mom[(1 + c) * npad + s];
        out[3 * i + c] = v;
    }
}


// Byte fill and copy of one buffer, grid-stride (the memsets and device copies of an
// evaluation when many boxes run as one launch per operation).  16- or 4-byte words when
// the pointers and the size allow, else bytes.  The copy's destination may be pinned host
// memory (mapped into the device's address space).
MPID_KERNEL void k_fill_bytes(KGrid<> kg, unsigned char* __restrict__ p, int value, size_t bytes) {
    const size_t stride = (size_t) kg.nb * blockDim.x;
    const size_t t0 = (size_t) kg.bx * blockDim.x + threadIdx.x;
    if ((((uintptr_t) p | bytes) & 15) == 0) {
        const unsigned b = (unsigned) value & 0xffu, w = b * 0x01010101u;
        const uint4 v = make_uint4(w, w, w, w);
        uint4* q = (uint4*) p;
        for (size_t i = t0; i < bytes / 16; i += stride) q[i] = v;
    } else {
        for (size_t i = t0; i < bytes; i += stride) p[i] = (unsigned char) value;
    }
}
MPID_KERNEL void k_copy_bytes(KGrid<> kg, unsigned char* __restrict__ dst, const unsigned char* __restrict__ src,
                              size_t bytes) {
    const size_t stride = (size_t) kg.nb * blockDim.x;
    const size_t t0 = (size_t) kg.bx * blockDim.x + threadIdx.x;
    if ((((uintptr_t) dst | (uintptr_t) src | bytes) & 15) == 0) {
        const uint4* a = (const uint4*) src;
        uint4* q = (uint4*) dst;
        for (size_t i = t0; i < bytes / 16; i += stride) q[i] = a[i];
    } else if ((((uintptr_t) dst | (uintptr_t) src | bytes) & 3) == 0) {
        const unsigned* a = (const unsigned*) src;
        unsigned* q = (unsigned*) dst;
        for (size_t i = t0; i < bytes / 4; i += stride) q[i] = a[i];
    } else {
        for (size_t i = t0; i < bytes; i += stride) dst[i] = src[i];
    }
}


// Per-type sums of one box's parameter gradients (the 20 multipole and 4 polarisation
// components of every atom, original order) for the fitting batch: warp c sums component
// c, each lane over a stride of the atoms and per type, then a shuffle tree per type; out
// holds [ntypes][24].  Fixed summation order.  One block of 24 warps per box.
constexpr int kMaxTypeSums = 16;
MPID_KERNEL void k_type_sums(KGrid<(24 * 32)> kg, int n, const int* __restrict__ types, int ntypes,
                             const double* __restrict__ mgrad, const double* __restrict__ pgrad,
                             double* __restrict__ out) {
    const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (c >= 24) return;
    double acc[kMaxTypeSums];
#pragma unroll
    for (int t = 0; t < kMaxTypeSums; ++t) acc[t] = 0.0;
    for (int i = lane; i < n; i += 32) {
        const int t = types[i];
        const double v = c < 20 ? mgrad[20 * (size_t) i + c] : pgrad[4 * (size_t) i + (c - 20)];
#pragma unroll
        for (int q = 0; q < kMaxTypeSums; ++q)
            if (q == t) acc[q] += v;
    }
#pragma unroll
    for (int q = 0; q < kMaxTypeSums; ++q) {
        double v = acc[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && q < ntypes) out[24 * q + c] = v;
    }
}

}  // namespace mpid
