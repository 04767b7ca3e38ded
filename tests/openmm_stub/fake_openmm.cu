// Test harness: definitions behind the OpenMM interface stand-ins (tests/openmm_stub),
// enough to drive GB300CalcMPIDForceKernel outside OpenMM.  A fake CUDA context holds
// posq in a permuted ("sorted") atom order, OpenMM's fixed-point force buffer and the
// atom index; harness_run() initialises the adapter from flat parameter arrays, executes
// it and returns energy, System-order forces and induced dipoles.  Built and called by
// tests/test_openmm_adapter.py on a GPU.
#include "GB300MPIDKernels.h"
#include "openmm/internal/ContextImpl.h"
#include "openmm/internal/NonbondedForceImpl.h"
#include "openmm/NonbondedForce.h"
#include "openmm/OpenMMException.h"
#include "openmm/Platform.h"
#include "openmm/System.h"

#include <cstring>
#include <cuda_runtime.h>
#include <vector>

using namespace OpenMM;

namespace {
struct FakeState {
    int n = 0, padded = 0;
    bool dbl = false;
    CUdeviceptr posq = 0, force = 0, atomIndex = 0, correction = 0;
    CudaArray aPosq, aForce, aIndex, aCorrection;
    Vec3 box[3];
    std::vector<Vec3> positions;
    std::vector<double> masses;
    // MPIDForce parameters
    int method = 1, pol = 0, order = 5, maxIter = 60;
    double cutoff = 1.0, alpha = 0.0, eps = 1e-5, defaultThole = 5.0, scale14 = 1.0, ewaldTol = 5e-4;
    int grid[3] = {0, 0, 0};
    std::vector<double> extrap, charge, dipole, quad, oct, thole, polarity;
    std::vector<int> axis, az, ax, ay;
    std::vector<std::vector<std::vector<int> > > cov;
    GB300CalcMPIDForceKernel* kernel = nullptr;
};
FakeState g;
}  // namespace

namespace OpenMM {
KernelImpl::KernelImpl(std::string, const Platform&) {}
KernelImpl::~KernelImpl() {}
CUdeviceptr& CudaArray::getDevicePointer() {
    if (this == &g.aPosq) return g.posq;
    if (this == &g.aForce) return g.force;
    if (this == &g.aIndex) return g.atomIndex;
    return g.correction;
}
void CudaContext::setAsCurrent() {}
CudaArray& CudaContext::getPosq() { return g.aPosq; }
CudaArray& CudaContext::getPosqCorrection() { return g.aCorrection; }
CudaArray& CudaContext::getForce() { return g.aForce; }
CudaArray& CudaContext::getAtomIndexArray() { return g.aIndex; }
int CudaContext::getPaddedNumAtoms() const { return g.padded; }
bool CudaContext::getUseDoublePrecision() const { return g.dbl; }
bool CudaContext::getUseMixedPrecision() const { return false; }
CUstream CudaContext::getCurrentStream() { return 0; }
void CudaContext::getPeriodicBoxVectors(Vec3& a, Vec3& b, Vec3& c) const { a = g.box[0]; b = g.box[1]; c = g.box[2]; }
void* ContextImpl::getPlatformData() { return nullptr; }
void ContextImpl::getPositions(std::vector<Vec3>& p) { p = g.positions; }
void ContextImpl::getPeriodicBoxVectors(Vec3& a, Vec3& b, Vec3& c) { a = g.box[0]; b = g.box[1]; c = g.box[2]; }
double ContextImpl::calcForcesAndEnergy(bool f, bool e, int) { return g.kernel->execute(*this, f, e); }
int System::getNumParticles() const { return g.n; }
double System::getParticleMass(int i) const { return g.masses[i]; }
void NonbondedForce::setEwaldErrorTolerance(double) {}
void NonbondedForce::setCutoffDistance(double) {}
void NonbondedForceImpl::calcPMEParameters(const System&, const NonbondedForce&, double&, int&, int&, int&, bool) {
    throw OpenMMException("the harness passes explicit PME parameters");
}
int MPIDForce::getNumMultipoles() const { return g.n; }
MPIDForce::NonbondedMethod MPIDForce::getNonbondedMethod() const { return (NonbondedMethod) g.method; }
MPIDForce::PolarizationType MPIDForce::getPolarizationType() const { return (PolarizationType) g.pol; }
double MPIDForce::getCutoffDistance() const { return g.cutoff; }
void MPIDForce::getPMEParameters(double& a, int& x, int& y, int& z) const { a = g.alpha; x = g.grid[0]; y = g.grid[1]; z = g.grid[2]; }
int MPIDForce::getPmeBSplineOrder() const { return g.order; }
double MPIDForce::getEwaldErrorTolerance() const { return g.ewaldTol; }
int MPIDForce::getMutualInducedMaxIterations() const { return g.maxIter; }
double MPIDForce::getMutualInducedTargetEpsilon() const { return g.eps; }
const std::vector<double>& MPIDForce::getExtrapolationCoefficients() const { return g.extrap; }
double MPIDForce::getDefaultTholeWidth() const { return g.defaultThole; }
double MPIDForce::get14ScaleFactor() const { return g.scale14; }
void MPIDForce::getMultipoleParameters(int i, double& q, std::vector<double>& d, std::vector<double>& Q,
                                       std::vector<double>& O, int& axisType, int& z, int& x, int& y, double& thole,
                                       std::vector<double>& polarity) const {
    q = g.charge[i];
    d.assign(&g.dipole[3 * i], &g.dipole[3 * i] + 3);
    Q.assign(&g.quad[6 * i], &g.quad[6 * i] + 6);
    O.assign(&g.oct[10 * i], &g.oct[10 * i] + 10);
    axisType = g.axis[i]; z = g.az[i]; x = g.ax[i]; y = g.ay[i];
    thole = g.thole[i];
    polarity.assign(&g.polarity[3 * i], &g.polarity[3 * i] + 3);
}
void MPIDForce::getCovalentMaps(int i, std::vector<std::vector<int> >& lists) const { lists = g.cov[i]; }
}  // namespace OpenMM

extern "C" int harness_run(int n, int dbl, const int* perm, const double* pos, const double* box, const int* settings_i,
                           const double* settings_d, const double* charge, const double* dipole, const double* quad,
                           const double* oct, const int* axis, const int* az, const int* ax, const int* ay,
                           const double* thole, const double* polarity, const int* covOffsets, const int* covIndex,
                           double* energyOut, double* forcesOut, double* inducedOut, char* message) {
    try {
        g = FakeState();
        g.n = n;
        g.padded = (n + 31) / 32 * 32;
        g.dbl = dbl != 0;
        for (int k = 0; k < 3; ++k) g.box[k] = Vec3(box[3 * k], box[3 * k + 1], box[3 * k + 2]);
        g.positions.resize(n);
        for (int i = 0; i < n; ++i) g.positions[i] = Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        g.masses.assign(n, 1.0);
        g.method = settings_i[0]; g.pol = settings_i[1]; g.order = settings_i[2]; g.maxIter = settings_i[3];
        g.grid[0] = settings_i[4]; g.grid[1] = settings_i[5]; g.grid[2] = settings_i[6];
        g.cutoff = settings_d[0]; g.alpha = settings_d[1]; g.eps = settings_d[2]; g.defaultThole = settings_d[3];
        g.scale14 = settings_d[4];
        g.extrap.assign(settings_d + 5, settings_d + 5 + settings_i[7]);
        g.charge.assign(charge, charge + n); g.dipole.assign(dipole, dipole + 3 * n);
        g.quad.assign(quad, quad + 6 * n); g.oct.assign(oct, oct + 10 * n);
        g.axis.assign(axis, axis + n); g.az.assign(az, az + n); g.ax.assign(ax, ax + n); g.ay.assign(ay, ay + n);
        g.thole.assign(thole, thole + n); g.polarity.assign(polarity, polarity + 3 * n);
        g.cov.assign(n, std::vector<std::vector<int> >(8));
        for (int i = 0; i < n; ++i)
            for (int t = 0; t < 8; ++t)
                g.cov[i][t].assign(covIndex + covOffsets[8 * i + t], covIndex + covOffsets[8 * i + t + 1]);
        // posq in the permuted order: slot s holds atom perm[s] (charge in w, unused)
        std::vector<int> index(perm, perm + n);
        size_t posqBytes = (size_t) g.padded * (g.dbl ? 32 : 16);
        std::vector<char> hostPosq(posqBytes, 0);
        for (int s = 0; s < n; ++s) {
            const double* p = pos + 3 * perm[s];
            if (g.dbl) {
                double* d = (double*) hostPosq.data() + 4 * s;
                d[0] = p[0]; d[1] = p[1]; d[2] = p[2]; d[3] = charge[perm[s]];
            } else {
                float* f = (float*) hostPosq.data() + 4 * s;
                f[0] = (float) p[0]; f[1] = (float) p[1]; f[2] = (float) p[2]; f[3] = (float) charge[perm[s]];
            }
        }
        void *dPosq, *dForce, *dIndex;
        cudaMalloc(&dPosq, posqBytes);
        cudaMalloc(&dForce, (size_t) 3 * g.padded * 8);
        cudaMalloc(&dIndex, (size_t) n * 4);
        cudaMemcpy(dPosq, hostPosq.data(), posqBytes, cudaMemcpyHostToDevice);
        cudaMemset(dForce, 0, (size_t) 3 * g.padded * 8);
        cudaMemcpy(dIndex, index.data(), (size_t) n * 4, cudaMemcpyHostToDevice);
        g.posq = (CUdeviceptr) dPosq; g.force = (CUdeviceptr) dForce; g.atomIndex = (CUdeviceptr) dIndex;
        System system;
        MPIDForce force;
        ContextImpl context;
        CudaContext cu;
        Platform platform;
        GB300CalcMPIDForceKernel kernel("CalcMPIDForce", platform, cu, system);
        g.kernel = &kernel;
        kernel.initialize(system, force);
        *energyOut = kernel.execute(context, true, true);
        std::vector<unsigned long long> buf((size_t) 3 * g.padded);
        cudaMemcpy(buf.data(), dForce, buf.size() * 8, cudaMemcpyDeviceToHost);
        for (int s = 0; s < n; ++s)
            for (int k = 0; k < 3; ++k)
                forcesOut[3 * perm[s] + k] = (double) (long long) buf[s + (size_t) k * g.padded] / 4294967296.0;
        std::vector<Vec3> mu;
        kernel.getInducedDipoles(context, mu);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) inducedOut[3 * i + k] = mu[i][k];
        g.kernel = nullptr;
        cudaFree(dPosq); cudaFree(dForce); cudaFree(dIndex);
        return 0;
    } catch (const std::exception& e) {
        std::strncpy(message, e.what(), 511);
        message[511] = 0;
        return 1;
    }
}
