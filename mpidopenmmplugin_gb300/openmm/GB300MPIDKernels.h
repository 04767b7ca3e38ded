/* OpenMM platform kernel for MPIDForce on the CUDA platform, backed by libmpid_gb300.
 *
 * Implements the reference's kernel interface CalcMPIDForceKernel
 * (openmmapi/include/openmm/mpidKernels.h:50-104) in place of CudaCalcMPIDForceKernel
 * (platforms/cuda/src/MPIDCudaKernels.h): initialize reads the MPIDForce into a
 * libmpid_gb300 context; execute gathers OpenMM's reordered posq into caller-order
 * positions, evaluates through the C ABI on OpenMM's stream and adds the forces into
 * OpenMM's 64-bit fixed-point force buffer; the getters un-permute nothing because the
 * library's outputs are in caller (System) order already.
 */
#ifndef GB300_MPID_KERNELS_H
#define GB300_MPID_KERNELS_H

#include "openmm/mpidKernels.h"
#include "openmm/MPIDForce.h"
#include "openmm/System.h"
#include "openmm/cuda/CudaContext.h"
#include "mpid_gb300.h"

#include <vector>

namespace OpenMM {

class GB300CalcMPIDForceKernel : public CalcMPIDForceKernel {
public:
    GB300CalcMPIDForceKernel(std::string name, const Platform& platform, CudaContext& cu, const System& system);
    ~GB300CalcMPIDForceKernel();
    void initialize(const System& system, const MPIDForce& force);
    double execute(ContextImpl& context, bool includeForces, bool includeEnergy);
    void getLabFramePermanentDipoles(ContextImpl& context, std::vector<Vec3>& dipoles);
    void getInducedDipoles(ContextImpl& context, std::vector<Vec3>& dipoles);
    void getTotalDipoles(ContextImpl& context, std::vector<Vec3>& dipoles);
    void getElectrostaticPotential(ContextImpl& context, const std::vector<Vec3>& inputGrid,
                                   std::vector<double>& outputElectrostaticPotential);
    void getSystemMultipoleMoments(ContextImpl& context, std::vector<double>& outputMultipoleMoments);
    void copyParametersToContext(ContextImpl& context, const MPIDForce& force);
    void getPMEParameters(double& alpha, int& nx, int& ny, int& nz) const;

private:
    void uploadParameters(const MPIDForce& force);
    void dipoles(ContextImpl& context, int which, std::vector<Vec3>& out);
    void hostState(ContextImpl& context, std::vector<double>& pos, double box[9]);
    static void check(int rc);
    CudaContext& cu;
    const System& system;
    mpid_context* handle;
    mpid_settings settings;
    int numAtoms;
    bool evaluated;
    double* devPos;     // caller-order positions, 3 x numAtoms
    double* devForce;   // caller-order forces, 3 x numAtoms
    double* devEnergy;  // 1
};

} // namespace OpenMM

#endif
