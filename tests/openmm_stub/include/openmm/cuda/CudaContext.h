// Compile-check stand-in for OpenMM's CudaContext (the members the adapter uses).
#pragma once
#include <cuda.h>
#include "openmm/Vec3.h"
#include "openmm/cuda/CudaArray.h"
namespace OpenMM {
class CudaContext {
public:
    void setAsCurrent();
    CudaArray& getPosq();
    CudaArray& getPosqCorrection();
    CudaArray& getForce();
    CudaArray& getAtomIndexArray();
    int getPaddedNumAtoms() const;
    bool getUseDoublePrecision() const;
    bool getUseMixedPrecision() const;
    CUstream getCurrentStream();
    void getPeriodicBoxVectors(Vec3& a, Vec3& b, Vec3& c) const;
};
}
