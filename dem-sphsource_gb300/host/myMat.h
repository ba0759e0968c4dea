// Symmetric 3x3 matrix type of the host API (names as in the reference's
// core/myMat.h; drivers build clump inertia tensors with make_symMatrix).
// Host code only.
#pragma once
#include "myQua.h"

struct symMatrix {
    double xx{0.}, yy{0.}, zz{0.}, xy{0.}, xz{0.}, yz{0.};
};

inline symMatrix make_symMatrix(double xx, double yy, double zz, double xy, double xz, double yz)
{
    symMatrix m;
    m.xx = xx; m.yy = yy; m.zz = zz; m.xy = xy; m.xz = xz; m.yz = yz;
    return m;
}

inline symMatrix operator+(const symMatrix& a, const symMatrix& b)
{
    return make_symMatrix(a.xx + b.xx, a.yy + b.yy, a.zz + b.zz, a.xy + b.xy, a.xz + b.xz, a.yz + b.yz);
}
inline symMatrix operator-(const symMatrix& a, const symMatrix& b)
{
    return make_symMatrix(a.xx - b.xx, a.yy - b.yy, a.zz - b.zz, a.xy - b.xy, a.xz - b.xz, a.yz - b.yz);
}
inline symMatrix operator*(const symMatrix& m, double s)
{
    return make_symMatrix(m.xx * s, m.yy * s, m.zz * s, m.xy * s, m.xz * s, m.yz * s);
}
inline symMatrix operator*(double s, const symMatrix& m) { return m * s; }
inline double3 operator*(const symMatrix& m, const double3& v)
{
    return make_double3(m.xx * v.x + m.xy * v.y + m.xz * v.z, m.xy * v.x + m.yy * v.y + m.yz * v.z,
                        m.xz * v.x + m.yz * v.y + m.zz * v.z);
}
inline double3 operator*(const double3& v, const symMatrix& m) { return m * v; }

// Frobenius-type norm sqrt(2 m:m) used by the reference for deviatoric stress.
inline double norm(const symMatrix& m)
{
    return std::sqrt(2 * (m.xx * m.xx + m.yy * m.yy + m.zz * m.zz + 2 * (m.xy * m.xy + m.xz * m.xz + m.yz * m.yz)));
}
inline symMatrix deviatoric(const symMatrix& m)
{
    const double t = (m.xx + m.yy + m.zz) / 3.;
    return make_symMatrix(m.xx - t, m.yy - t, m.zz - t, m.xy, m.xz, m.yz);
}

// R(q) A R(q)^T for a symmetric A.
inline symMatrix rotateInverseInertiaTensor(const quaternion& q, const symMatrix& A)
{
    const double3 c0 = rotateVectorByQuaternion(q, make_double3(1, 0, 0));
    const double3 c1 = rotateVectorByQuaternion(q, make_double3(0, 1, 0));
    const double3 c2 = rotateVectorByQuaternion(q, make_double3(0, 0, 1));
    // rows of R are (c0.x, c1.x, c2.x), ...
    const double3 r0 = make_double3(c0.x, c1.x, c2.x), r1 = make_double3(c0.y, c1.y, c2.y),
                  r2 = make_double3(c0.z, c1.z, c2.z);
    const double3 a0 = A * r0, a1 = A * r1, a2 = A * r2;
    return make_symMatrix(dot(r0, a0), dot(r1, a1), dot(r2, a2), dot(r0, a1), dot(r0, a2), dot(r1, a2));
}

// Inverse by cofactors.
inline symMatrix inverse(const symMatrix& A)
{
    const double c_xx = A.yy * A.zz - A.yz * A.yz;
    const double c_xy = A.xz * A.yz - A.xy * A.zz;
    const double c_xz = A.xy * A.yz - A.xz * A.yy;
    const double inv_det = 1. / (A.xx * c_xx + A.xy * c_xy + A.xz * c_xz);
    symMatrix B;
    // xy and yz are formed as the negated differences, as the reference does
    // (core/myMat.h:129-142): a diagonal tensor then gives -0.0 there, the
    // reference's bits
    B.xx = c_xx * inv_det;
    B.xy = -(A.xy * A.zz - A.xz * A.yz) * inv_det;
    B.xz = c_xz * inv_det;
    B.yy = (A.xx * A.zz - A.xz * A.xz) * inv_det;
    B.yz = -(A.xx * A.yz - A.xz * A.xy) * inv_det;
    B.zz = (A.xx * A.yy - A.xy * A.xy) * inv_det;
    return B;
}
