// Compile-check stand-in for OpenMM's CudaArray.
#pragma once
#include <cuda.h>
namespace OpenMM {
class CudaArray {
public:
    CUdeviceptr& getDevicePointer();
};
}
