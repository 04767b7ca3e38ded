/* Registers GB300CalcMPIDForceKernel as the CUDA platform's "CalcMPIDForce" kernel, as
 * the reference's MPIDCudaKernelFactory does for its own kernel
 * (platforms/cuda/src/MPIDCudaKernelFactory.cpp:45-76).  Load this plugin instead of the
 * reference's CUDA plugin; the reference's API library (MPIDForce) stays as it is. */
#include "GB300MPIDKernels.h"

#include "openmm/OpenMMException.h"
#include "openmm/internal/ContextImpl.h"
#include "openmm/KernelFactory.h"
#include "openmm/Platform.h"
#include "openmm/cuda/CudaPlatform.h"

using namespace OpenMM;

namespace {
class GB300MPIDKernelFactory : public KernelFactory {
public:
    KernelImpl* createKernelImpl(std::string name, const Platform& platform, ContextImpl& context) const {
        CudaPlatform::PlatformData& data = *static_cast<CudaPlatform::PlatformData*>(context.getPlatformData());
        CudaContext& cu = *data.contexts[0];
        if (name == CalcMPIDForceKernel::Name())
            return new GB300CalcMPIDForceKernel(name, platform, cu, context.getSystem());
        throw OpenMMException((std::string("Tried to create kernel with illegal kernel name '") + name + "'").c_str());
    }
};
} // namespace

extern "C" OPENMM_EXPORT void registerKernelFactories() {
    try {
        Platform& platform = Platform::getPlatformByName("CUDA");
        platform.registerKernelFactory(CalcMPIDForceKernel::Name(), new GB300MPIDKernelFactory());
    } catch (...) {
        // no CUDA platform: nothing to register
    }
}

extern "C" OPENMM_EXPORT void registerMPIDGB300KernelFactories() { registerKernelFactories(); }
