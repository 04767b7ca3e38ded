/* Oracle build shim (test infrastructure only).
 * Minimal 3-vector with the member functions that the reference's FP64 CPU force
 * (platforms/reference/src/SimTKReference/MPIDReferenceForce.cpp) uses from OpenMM's
 * Vec3: construction, indexing, +, -, unary -, scalar * and /, compound assignment,
 * dot and cross.  OpenMM itself is not installed, so the force is built against this. */
#ifndef MPID_ORACLE_SHIM_VEC3_H
#define MPID_ORACLE_SHIM_VEC3_H
#include <cassert>
#include <ostream>
namespace OpenMM {
class Vec3 {
public:
    Vec3() { v[0] = v[1] = v[2] = 0.0; }
    Vec3(double x, double y, double z) { v[0] = x; v[1] = y; v[2] = z; }
    double operator[](int i) const { return v[i]; }
    double& operator[](int i) { return v[i]; }
    bool operator==(const Vec3& o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
    bool operator!=(const Vec3& o) const { return !(*this == o); }
    Vec3 operator+() const { return *this; }
    Vec3 operator-() const { return Vec3(-v[0], -v[1], -v[2]); }
    Vec3 operator+(const Vec3& o) const { return Vec3(v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]); }
    Vec3 operator-(const Vec3& o) const { return Vec3(v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]); }
    Vec3 operator*(double s) const { return Vec3(v[0] * s, v[1] * s, v[2] * s); }
    Vec3 operator/(double s) const { double r = 1.0 / s; return Vec3(v[0] * r, v[1] * r, v[2] * r); }
    Vec3& operator+=(const Vec3& o) { v[0] += o.v[0]; v[1] += o.v[1]; v[2] += o.v[2]; return *this; }
    Vec3& operator-=(const Vec3& o) { v[0] -= o.v[0]; v[1] -= o.v[1]; v[2] -= o.v[2]; return *this; }
    Vec3& operator*=(double s) { v[0] *= s; v[1] *= s; v[2] *= s; return *this; }
    Vec3& operator/=(double s) { double r = 1.0 / s; v[0] *= r; v[1] *= r; v[2] *= r; return *this; }
    double dot(const Vec3& o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
    Vec3 cross(const Vec3& o) const {
        return Vec3(v[1] * o.v[2] - v[2] * o.v[1], v[2] * o.v[0] - v[0] * o.v[2], v[0] * o.v[1] - v[1] * o.v[0]);
    }
private:
    double v[3];
};
inline Vec3 operator*(double s, const Vec3& a) { return a * s; }
inline std::ostream& operator<<(std::ostream& o, const Vec3& a) { return o << "[" << a[0] << ", " << a[1] << ", " << a[2] << "]"; }
}
#endif
