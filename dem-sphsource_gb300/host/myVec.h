// double3 algebra of the host API.
//
// Case drivers written against the reference (e.g. driver/cases/damBreak.cpp)
// use double3 arithmetic, pi() and the helpers below by these names
// (core/myVec.h:10-109 in the reference), so the same names and semantics are
// provided here for source compatibility.  Host code only: the GPU kernels
// have their own FP32 / double-float math in csrc/.
#pragma once
#include <cmath>
#include <vector_types.h>
#include <vector_functions.h>

inline constexpr double pi() { return 3.14159265358979311600; }

inline double3 operator+(const double3& a, const double3& b) { return make_double3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline double3 operator-(const double3& a, const double3& b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline double3 operator-(const double3& a) { return make_double3(-a.x, -a.y, -a.z); }
inline double3 operator*(const double3& a, double s) { return make_double3(a.x * s, a.y * s, a.z * s); }
inline double3 operator*(double s, const double3& a) { return a * s; }
inline double3 operator/(const double3& a, double s) { return make_double3(a.x / s, a.y / s, a.z / s); }
inline double3& operator+=(double3& a, const double3& b) { a = a + b; return a; }
inline double3& operator-=(double3& a, const double3& b) { a = a - b; return a; }
inline double3& operator*=(double3& a, double s) { a = a * s; return a; }
inline double3& operator/=(double3& a, double s) { a = a / s; return a; }

inline double dot(const double3& a, const double3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double3 cross(const double3& a, const double3& b)
{
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline double lengthSquared(const double3& v) { return dot(v, v); }
inline double length(const double3& v) { return std::sqrt(dot(v, v)); }

// Unit vector; a zero vector is returned unchanged.
inline double3 normalize(const double3& v)
{
    const double l = length(v);
    return l > 0 ? v / l : v;
}

// Rotation of v by the rotation vector w (axis w/|w|, angle |w|), Rodrigues'
// formula; rotations below 1e-10 rad are treated as none.
inline double3 rotateVector(double3 v, double3 w)
{
    const double angle = length(w);
    if (angle < 1.e-10) return v;
    const double3 k = w / angle;
    const double c = std::cos(angle), s = std::sin(angle);
    return v * c + cross(k, v) * s + k * (dot(k, v) * (1 - c));
}
