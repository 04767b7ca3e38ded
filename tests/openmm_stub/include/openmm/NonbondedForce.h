// Compile-check stand-in for OpenMM's NonbondedForce.
#pragma once
namespace OpenMM {
class NonbondedForce {
public:
    void setEwaldErrorTolerance(double tol);
    void setCutoffDistance(double distance);
};
}
