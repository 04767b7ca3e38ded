// Compile-check stand-in for OpenMM's NonbondedForceImpl.
#pragma once
namespace OpenMM {
class System;
class NonbondedForce;
class NonbondedForceImpl {
public:
    static void calcPMEParameters(const System& system, const NonbondedForce& force, double& alpha, int& xsize,
                                  int& ysize, int& zsize, bool lj);
};
}
