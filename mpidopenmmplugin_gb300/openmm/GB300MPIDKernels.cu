/* GB300CalcMPIDForceKernel: OpenMM CUDA-platform kernel over libmpid_gb300 (see the
 * header).  Method-for-method replacement of CudaCalcMPIDForceKernel
 * (platforms/cuda/src/MPIDCudaKernels.cpp:118-1335). */
#include "GB300MPIDKernels.h"

#include "openmm/OpenMMException.h"
#include "openmm/internal/ContextImpl.h"
#include "openmm/internal/NonbondedForceImpl.h"
#include "openmm/NonbondedForce.h"

#include <cmath>
#include <cuda_runtime.h>

using namespace OpenMM;

namespace {

// OpenMM's double-precision posq element (x, y, z, charge), 32-byte aligned.
struct alignas(32) PosqDouble {
    double x, y, z, w;
};

// OpenMM's posq (sorted order; float4 or double4, plus a float4 correction in mixed
// precision) -> positions in System order.
template <typename P>
__global__ void gb300_gather_positions(int n, const P* __restrict__ posq, const float4* __restrict__ correction,
                                       const int* __restrict__ atomIndex, double* __restrict__ pos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const P p = posq[i];
    double x = p.x, y = p.y, z = p.z;
    if (correction) {
        const float4 c = correction[i];
        x += c.x;
        y += c.y;
        z += c.z;
    }
    const int a = atomIndex[i];
    pos[3 * a] = x;
    pos[3 * a + 1] = y;
    pos[3 * a + 2] = z;
}

// System-order forces -> OpenMM's fixed-point force buffer ([3][paddedNumAtoms], sorted
// order, 2^32 units), added to.
__global__ void gb300_add_forces(int n, int padded, const double* __restrict__ force, const int* __restrict__ atomIndex,
                                 unsigned long long* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int a = atomIndex[i];
    for (int k = 0; k < 3; ++k)
        out[i + k * padded] += (unsigned long long) (long long) llrint(force[3 * a + k] * 4294967296.0);
}

// Round a grid size up to a product of 2, 3, 5 and 7 (sizes cuFFT transforms fastest).
int legalDimension(int n) {
    for (;; ++n) {
        int m = n;
        for (int f : {2, 3, 5, 7})
            while (m % f == 0) m /= f;
        if (m == 1) return n;
    }
}

} // namespace

void GB300CalcMPIDForceKernel::check(int rc) {
    if (rc != MPID_OK) throw OpenMMException(mpid_last_error());
}

GB300CalcMPIDForceKernel::GB300CalcMPIDForceKernel(std::string name, const Platform& platform, CudaContext& cu,
                                                   const System& system)
    : CalcMPIDForceKernel(name, platform), cu(cu), system(system), handle(nullptr), numAtoms(0), evaluated(false),
      devPos(nullptr), devForce(nullptr), devEnergy(nullptr) {}

GB300CalcMPIDForceKernel::~GB300CalcMPIDForceKernel() {
    cu.setAsCurrent();
    if (handle) mpid_destroy(handle);
    if (devPos) cudaFree(devPos);
    if (devForce) cudaFree(devForce);
    if (devEnergy) cudaFree(devEnergy);
}

void GB300CalcMPIDForceKernel::initialize(const System& system, const MPIDForce& force) {
    cu.setAsCurrent();
    numAtoms = force.getNumMultipoles();
    mpid_default_settings(&settings, numAtoms);
    settings.nonbonded_method = force.getNonbondedMethod() == MPIDForce::PME ? MPID_PME : MPID_NO_CUTOFF;
    settings.polarization_type = (int) force.getPolarizationType();
    settings.cutoff = force.getCutoffDistance();
    if (settings.nonbonded_method == MPID_PME) {
        double alpha;
        int nx, ny, nz;
        force.getPMEParameters(alpha, nx, ny, nz);
        if (nx == 0 || alpha == 0.0) {
            // the automatic choice of the reference kernel (MPIDCudaKernels.cpp:440-449)
            NonbondedForce nb;
            nb.setEwaldErrorTolerance(force.getEwaldErrorTolerance());
            nb.setCutoffDistance(force.getCutoffDistance());
            NonbondedForceImpl::calcPMEParameters(system, nb, alpha, nx, ny, nz, false);
        }
        settings.ewald_alpha = alpha;
        settings.grid[0] = legalDimension(nx);
        settings.grid[1] = legalDimension(ny);
        settings.grid[2] = legalDimension(nz);
        settings.pme_order = force.getPmeBSplineOrder();
    }
    settings.mutual_eps = force.getMutualInducedTargetEpsilon();
    settings.max_iter = force.getMutualInducedMaxIterations();
    const std::vector<double>& c = force.getExtrapolationCoefficients();
    if (c.size() > 8) throw OpenMMException("MPIDForce: at most 8 extrapolation coefficients are supported");
    settings.n_extrap = (int) c.size();
    for (size_t i = 0; i < c.size(); ++i) settings.extrap_coeffs[i] = c[i];
    settings.default_thole = force.getDefaultTholeWidth();
    settings.scale14 = force.get14ScaleFactor();
    settings.precision = cu.getUseDoublePrecision() ? MPID_PRECISION_DOUBLE : MPID_PRECISION_MIXED;
    // replay evaluation segments from CUDA graphs on OpenMM's stream (launches run directly
    // while OpenMM itself captures that stream)
    settings.flags |= MPID_FLAG_GRAPH_SOLVER;
    int device = 0;
    cudaGetDevice(&device);
    check(mpid_create(&settings, device, &handle));
    uploadParameters(force);
    if (cudaMalloc(&devPos, 3 * sizeof(double) * numAtoms) != cudaSuccess ||
        cudaMalloc(&devForce, 3 * sizeof(double) * numAtoms) != cudaSuccess ||
        cudaMalloc(&devEnergy, sizeof(double)) != cudaSuccess)
        throw OpenMMException("GB300CalcMPIDForceKernel: device allocation failed");
}

void GB300CalcMPIDForceKernel::uploadParameters(const MPIDForce& force) {
    if (force.getNumMultipoles() != numAtoms)
        throw OpenMMException("updateParametersInContext: The number of multipoles has changed");
    const int n = numAtoms;
    std::vector<double> q(n), d(3 * n), Q(6 * n), O(10 * n), thole(n), pol(3 * n);
    std::vector<int> ax(n), az(n), axx(n), ay(n);
    std::vector<int> offsets(8 * n + 1, 0), index;
    for (int i = 0; i < n; ++i) {
        std::vector<double> di, Qi, Oi, pi;
        force.getMultipoleParameters(i, q[i], di, Qi, Oi, ax[i], az[i], axx[i], ay[i], thole[i], pi);
        for (int k = 0; k < 3; ++k) d[3 * i + k] = di[k];
        for (int k = 0; k < 6; ++k) Q[6 * i + k] = Qi[k];
        for (int k = 0; k < 10; ++k) O[10 * i + k] = Oi[k];
        for (int k = 0; k < 3; ++k) pol[3 * i + k] = pi[k];
        std::vector<std::vector<int> > lists;
        force.getCovalentMaps(i, lists);
        for (int t = 0; t < 8; ++t) {
            if (t < (int) lists.size()) index.insert(index.end(), lists[t].begin(), lists[t].end());
            offsets[8 * i + t + 1] = (int) index.size();
        }
    }
    check(mpid_set_multipoles(handle, q.data(), d.data(), Q.data(), O.data(), ax.data(), az.data(), axx.data(),
                              ay.data(), thole.data(), pol.data()));
    check(mpid_set_covalent(handle, offsets.data(), index.empty() ? nullptr : index.data()));
    evaluated = false;
}

double GB300CalcMPIDForceKernel::execute(ContextImpl& context, bool includeForces, bool includeEnergy) {
    cu.setAsCurrent();
    cudaStream_t stream = (cudaStream_t) cu.getCurrentStream();
    const int block = 128, grid = (numAtoms + block - 1) / block;
    const int* atomIndex = (const int*) cu.getAtomIndexArray().getDevicePointer();
    if (cu.getUseDoublePrecision())
        gb300_gather_positions<PosqDouble><<<grid, block, 0, stream>>>(
            numAtoms, (const PosqDouble*) cu.getPosq().getDevicePointer(), nullptr, atomIndex, devPos);
    else
        gb300_gather_positions<float4><<<grid, block, 0, stream>>>(
            numAtoms, (const float4*) cu.getPosq().getDevicePointer(),
            cu.getUseMixedPrecision() ? (const float4*) cu.getPosqCorrection().getDevicePointer() : nullptr,
            atomIndex, devPos);
    if (cudaMemsetAsync(devForce, 0, 3 * sizeof(double) * numAtoms, stream) != cudaSuccess)
        throw OpenMMException("GB300CalcMPIDForceKernel: cudaMemsetAsync failed");
    Vec3 a, b, c;
    cu.getPeriodicBoxVectors(a, b, c);
    const double box[9] = {a[0], a[1], a[2], b[0], b[1], b[2], c[0], c[1], c[2]};
    check(mpid_evaluate_device(handle, devPos, box, devForce, devEnergy, stream));
    evaluated = true;
    if (includeForces)
        gb300_add_forces<<<grid, block, 0, stream>>>(numAtoms, cu.getPaddedNumAtoms(), devForce, atomIndex,
                                                     (unsigned long long*) cu.getForce().getDevicePointer());
    if (cudaGetLastError() != cudaSuccess) throw OpenMMException("GB300CalcMPIDForceKernel: kernel launch failed");
    if (!includeEnergy) return 0.0;
    // returned to OpenMM, which adds it to the potential energy (the reference kernel adds
    // it to the energy buffer instead); the evaluation has waited for the solver anyway
    double energy = 0.0;
    if (cudaMemcpyAsync(&energy, devEnergy, sizeof(double), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
        throw OpenMMException("GB300CalcMPIDForceKernel: energy read-back failed");
    return energy;
}

void GB300CalcMPIDForceKernel::dipoles(ContextImpl& context, int which, std::vector<Vec3>& out) {
    if (!evaluated) context.calcForcesAndEnergy(false, false, -1);
    cu.setAsCurrent();
    std::vector<double> v(3 * numAtoms);
    check(mpid_get_dipoles(handle, which, v.data()));
    out.resize(numAtoms);
    for (int i = 0; i < numAtoms; ++i) out[i] = Vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
}

void GB300CalcMPIDForceKernel::getLabFramePermanentDipoles(ContextImpl& context, std::vector<Vec3>& out) {
    dipoles(context, 1, out);
}

void GB300CalcMPIDForceKernel::getInducedDipoles(ContextImpl& context, std::vector<Vec3>& out) { dipoles(context, 0, out); }

void GB300CalcMPIDForceKernel::getTotalDipoles(ContextImpl& context, std::vector<Vec3>& out) { dipoles(context, 2, out); }

void GB300CalcMPIDForceKernel::hostState(ContextImpl& context, std::vector<double>& pos, double box[9]) {
    std::vector<Vec3> p;
    context.getPositions(p);
    pos.resize(3 * numAtoms);
    for (int i = 0; i < numAtoms; ++i)
        for (int k = 0; k < 3; ++k) pos[3 * i + k] = p[i][k];
    Vec3 a, b, c;
    context.getPeriodicBoxVectors(a, b, c);
    for (int k = 0; k < 3; ++k) {
        box[k] = a[k];
        box[3 + k] = b[k];
        box[6 + k] = c[k];
    }
}

void GB300CalcMPIDForceKernel::getElectrostaticPotential(ContextImpl& context, const std::vector<Vec3>& inputGrid,
                                                         std::vector<double>& outputElectrostaticPotential) {
    cu.setAsCurrent();
    std::vector<double> pos, grid(3 * inputGrid.size());
    double box[9];
    hostState(context, pos, box);
    for (size_t g = 0; g < inputGrid.size(); ++g)
        for (int k = 0; k < 3; ++k) grid[3 * g + k] = inputGrid[g][k];
    outputElectrostaticPotential.resize(inputGrid.size());
    check(mpid_get_electrostatic_potential(handle, pos.data(), box, grid.data(), (int) inputGrid.size(),
                                           outputElectrostaticPotential.data()));
    evaluated = true;
}

void GB300CalcMPIDForceKernel::getSystemMultipoleMoments(ContextImpl& context, std::vector<double>& outputMultipoleMoments) {
    cu.setAsCurrent();
    std::vector<double> pos, masses(numAtoms);
    double box[9];
    hostState(context, pos, box);
    for (int i = 0; i < numAtoms; ++i) masses[i] = system.getParticleMass(i);
    outputMultipoleMoments.resize(13);
    check(mpid_get_system_multipole_moments(handle, pos.data(), box, masses.data(), outputMultipoleMoments.data()));
    evaluated = true;
}

void GB300CalcMPIDForceKernel::copyParametersToContext(ContextImpl& context, const MPIDForce& force) {
    cu.setAsCurrent();
    uploadParameters(force);
}

void GB300CalcMPIDForceKernel::getPMEParameters(double& alpha, int& nx, int& ny, int& nz) const {
    if (settings.nonbonded_method != MPID_PME) throw OpenMMException("getPMEParametersInContext: MPIDForce is not using PME");
    alpha = settings.ewald_alpha;
    nx = settings.grid[0];
    ny = settings.grid[1];
    nz = settings.grid[2];
}
