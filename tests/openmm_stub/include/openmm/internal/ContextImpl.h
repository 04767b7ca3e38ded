// Compile-check stand-in for OpenMM's ContextImpl.
#pragma once
#include <vector>
#include "openmm/Vec3.h"
namespace OpenMM {
class System;
class ContextImpl {
public:
    void* getPlatformData();
    const System& getSystem() const;
    void getPositions(std::vector<Vec3>& positions);
    void getPeriodicBoxVectors(Vec3& a, Vec3& b, Vec3& c);
    double calcForcesAndEnergy(bool includeForces, bool includeEnergy, int groups = 0xFFFFFFFF);
};
}
