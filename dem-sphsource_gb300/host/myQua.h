// Quaternion type of the host API (names as in the reference's core/myQua.h,
// which drivers and HostClump use).  Host code only.
#pragma once
#include "myVec.h"

struct quaternion {
    double q0, q1, q2, q3;  // scalar part first
};

inline quaternion make_quaternion(double q0, double q1, double q2, double q3)
{
    quaternion q;
    q.q0 = q0; q.q1 = q1; q.q2 = q2; q.q3 = q3;
    return q;
}
inline quaternion operator+(const quaternion& a, const quaternion& b)
{
    return make_quaternion(a.q0 + b.q0, a.q1 + b.q1, a.q2 + b.q2, a.q3 + b.q3);
}
inline quaternion operator*(const quaternion& q, double c) { return make_quaternion(q.q0 * c, q.q1 * c, q.q2 * c, q.q3 * c); }
inline quaternion operator*(double c, const quaternion& q) { return q * c; }
inline quaternion operator/(const quaternion& q, double c) { return make_quaternion(q.q0 / c, q.q1 / c, q.q2 / c, q.q3 / c); }

inline quaternion normalize(const quaternion& q)
{
    const double l = std::sqrt(q.q0 * q.q0 + q.q1 * q.q1 + q.q2 * q.q2 + q.q3 * q.q3);
    return l > 0 ? q / l : q;
}

// First-order update q + 0.5 * (0, w dt) * q, renormalised.
inline quaternion quaternionRotate(const quaternion& q, const double3& w, double dt)
{
    const double3 a = w * dt;
    const quaternion dq = make_quaternion(-q.q1 * a.x - q.q2 * a.y - q.q3 * a.z,
                                          q.q0 * a.x + q.q3 * a.y - q.q2 * a.z,
                                          -q.q3 * a.x + q.q0 * a.y + q.q1 * a.z,
                                          q.q2 * a.x - q.q1 * a.y + q.q0 * a.z) * 0.5;
    return normalize(q + dq);
}

// Rotation matrix R(q) applied to v (body -> world) and its transpose (world -> body).
inline double3 rotateVectorByQuaternion(const quaternion& q, const double3& v)
{
    const double w = q.q0, x = q.q1, y = q.q2, z = q.q3;
    const double3 r0 = make_double3(w * w + x * x - y * y - z * z, 2 * (x * y - w * z), 2 * (x * z + w * y));
    const double3 r1 = make_double3(2 * (x * y + w * z), w * w - x * x + y * y - z * z, 2 * (y * z - w * x));
    const double3 r2 = make_double3(2 * (x * z - w * y), 2 * (y * z + w * x), w * w - x * x - y * y + z * z);
    return make_double3(dot(r0, v), dot(r1, v), dot(r2, v));
}
inline double3 reverseRotateVectorByQuaternion(const double3& v, const quaternion& q)
{
    return rotateVectorByQuaternion(make_quaternion(q.q0, -q.q1, -q.q2, -q.q3), v);
}
