// Compile-check stand-in for the reference's kernel interface
// (openmmapi/include/openmm/mpidKernels.h:50-104).
#pragma once
#include <string>
#include <vector>
#include "openmm/KernelImpl.h"
#include "openmm/Vec3.h"
namespace OpenMM {
class System;
class MPIDForce;
class ContextImpl;
class CalcMPIDForceKernel : public KernelImpl {
public:
    static std::string Name() { return "CalcMPIDForce"; }
    CalcMPIDForceKernel(std::string name, const Platform& platform) : KernelImpl(name, platform) {}
    virtual void initialize(const System& system, const MPIDForce& force) = 0;
    virtual double execute(ContextImpl& context, bool includeForces, bool includeEnergy) = 0;
    virtual void getLabFramePermanentDipoles(ContextImpl& context, std::vector<Vec3>& dipoles) = 0;
    virtual void getInducedDipoles(ContextImpl& context, std::vector<Vec3>& dipoles) = 0;
    virtual void getTotalDipoles(ContextImpl& context, std::vector<Vec3>& dipoles) = 0;
    virtual void getElectrostaticPotential(ContextImpl& context, const std::vector<Vec3>& inputGrid,
                                           std::vector<double>& outputElectrostaticPotential) = 0;
    virtual void getSystemMultipoleMoments(ContextImpl& context, std::vector<double>& outputMultipoleMoments) = 0;
    virtual void copyParametersToContext(ContextImpl& context, const MPIDForce& force) = 0;
    virtual void getPMEParameters(double& alpha, int& nx, int& ny, int& nz) const = 0;
};
}
