// Compile-check stand-in for the reference's MPIDForce (the methods the adapter calls,
// with the signatures of openmmapi/include/openmm/MPIDForce.h).
#pragma once
#include <vector>
namespace OpenMM {
class MPIDForce {
public:
    enum NonbondedMethod { NoCutoff = 0, PME = 1 };
    enum PolarizationType { Mutual = 0, Direct = 1, Extrapolated = 2 };
    int getNumMultipoles() const;
    NonbondedMethod getNonbondedMethod() const;
    PolarizationType getPolarizationType() const;
    double getCutoffDistance() const;
    void getPMEParameters(double& alpha, int& nx, int& ny, int& nz) const;
    int getPmeBSplineOrder() const;
    double getEwaldErrorTolerance() const;
    int getMutualInducedMaxIterations() const;
    double getMutualInducedTargetEpsilon() const;
    const std::vector<double>& getExtrapolationCoefficients() const;
    double getDefaultTholeWidth() const;
    double get14ScaleFactor() const;
    void getMultipoleParameters(int index, double& charge, std::vector<double>& molecularDipole,
                                std::vector<double>& molecularQuadrupole, std::vector<double>& molecularOctopole,
                                int& axisType, int& multipoleAtomZ, int& multipoleAtomX, int& multipoleAtomY,
                                double& thole, std::vector<double>& polarity) const;
    void getCovalentMaps(int index, std::vector<std::vector<int> >& covalentLists) const;
};
}
