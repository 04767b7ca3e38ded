// Compile-check stand-in for OpenMM's System.
#pragma once
namespace OpenMM {
class System {
public:
    int getNumParticles() const;
    double getParticleMass(int index) const;
};
}
