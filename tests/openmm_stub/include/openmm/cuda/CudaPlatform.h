// Compile-check stand-in for OpenMM's CudaPlatform::PlatformData.
#pragma once
#include <vector>
#include "openmm/cuda/CudaContext.h"
namespace OpenMM {
class CudaPlatform {
public:
    class PlatformData {
    public:
        std::vector<CudaContext*> contexts;
    };
};
}
