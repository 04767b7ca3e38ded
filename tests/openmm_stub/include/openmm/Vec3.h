// Compile-check stand-in for OpenMM's Vec3 (declarations the adapter uses only).
#pragma once
namespace OpenMM {
class Vec3 {
public:
    Vec3() : d{0, 0, 0} {}
    Vec3(double x, double y, double z) : d{x, y, z} {}
    double operator[](int i) const { return d[i]; }
    double& operator[](int i) { return d[i]; }
private:
    double d[3];
};
}
