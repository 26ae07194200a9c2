// Minimal stand-in for OpenMM's Vec3 (three doubles with vector algebra), written for this
// project so that the reference plugin's CPU sources compile without an OpenMM install.
// Test infrastructure only: used to build the oracle's copy of the reference, never the product.
#ifndef RBX_STANDIN_VEC3_H
#define RBX_STANDIN_VEC3_H
#include <cassert>
#include <ostream>

namespace OpenMM {

class Vec3 {
public:
    Vec3() : v{0.0, 0.0, 0.0} {}
    Vec3(double x, double y, double z) : v{x, y, z} {}
    double operator[](int i) const { assert(i >= 0 && i < 3); return v[i]; }
    double& operator[](int i) { assert(i >= 0 && i < 3); return v[i]; }
    bool operator==(const Vec3& o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
    bool operator!=(const Vec3& o) const { return !(*this == o); }
    Vec3 operator+() const { return *this; }
    Vec3 operator-() const { return Vec3(-v[0], -v[1], -v[2]); }
    Vec3 operator+(const Vec3& o) const { return Vec3(v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]); }
    Vec3 operator-(const Vec3& o) const { return Vec3(v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]); }
    Vec3& operator+=(const Vec3& o) { v[0] += o.v[0]; v[1] += o.v[1]; v[2] += o.v[2]; return *this; }
    Vec3& operator-=(const Vec3& o) { v[0] -= o.v[0]; v[1] -= o.v[1]; v[2] -= o.v[2]; return *this; }
    Vec3 operator*(double s) const { return Vec3(v[0] * s, v[1] * s, v[2] * s); }
    Vec3& operator*=(double s) { v[0] *= s; v[1] *= s; v[2] *= s; return *this; }
    Vec3 operator/(double s) const { double r = 1.0 / s; return Vec3(v[0] * r, v[1] * r, v[2] * r); }
    Vec3& operator/=(double s) { double r = 1.0 / s; v[0] *= r; v[1] *= r; v[2] *= r; return *this; }
    double dot(const Vec3& o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
    Vec3 cross(const Vec3& o) const {
        return Vec3(v[1] * o.v[2] - v[2] * o.v[1], v[2] * o.v[0] - v[0] * o.v[2], v[0] * o.v[1] - v[1] * o.v[0]);
    }
private:
    double v[3];
};

inline std::ostream& operator<<(std::ostream& os, const Vec3& a) {
    return os << '[' << a[0] << ", " << a[1] << ", " << a[2] << ']';
}

}  // namespace OpenMM
#endif
