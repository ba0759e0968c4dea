// Host-side particle data of the drop-in API.
//
// Drivers read these structs back through dataBase::getHostFluidData() /
// getHostSolidData(), so their type and member names are those of the
// reference's core/hostStructs.h (HostFluid :48-75, HostSolid :77-117,
// HostClump :119-152, ...), with the same default values.  The layout is
// array-of-vectors in FP64, the form the C ABI (include/demsph_gb300.h)
// passes to the engine.
#pragma once
#include <algorithm>
#include <vector>
#include "myMat.h"

template <class T>
inline void appendVector(std::vector<T>& to, const std::vector<T>& from)
{
    to.insert(to.end(), from.begin(), from.end());
}

struct HostDynamicStateBase {
    std::vector<double3> velocities;
    std::vector<double3> accelerations;

    HostDynamicStateBase() = default;
    explicit HostDynamicStateBase(int n)
        : velocities(n, make_double3(0, 0, 0)), accelerations(n, make_double3(0, 0, 0)) {}
    void insertData(const HostDynamicStateBase& s)
    {
        appendVector(velocities, s.velocities);
        appendVector(accelerations, s.accelerations);
    }
};

struct HostPointCloud {
    int num{0};
    std::vector<double3> position;
    std::vector<double> effectiveRadii;  // search radius: smoothing length for fluid

    HostPointCloud() = default;
    explicit HostPointCloud(int n) : num(n), position(n, make_double3(0, 0, 0)), effectiveRadii(n, 0) {}
    void insertData(const HostPointCloud& p)
    {
        appendVector(position, p.position);
        appendVector(effectiveRadii, p.effectiveRadii);
        num += p.num;
    }
};

struct HostFluid {
    HostPointCloud points;
    HostDynamicStateBase dyn;
    std::vector<double> rho0;  // rest density
    std::vector<double> dRho;  // density minus rest density
    std::vector<double> c;     // speed of sound
    std::vector<double> nu;    // kinematic viscosity
    std::vector<double> chi;   // background pressure (unused by the step)

    HostFluid() = default;
    explicit HostFluid(int n) : points(n), dyn(n), rho0(n, 0.), dRho(n, 0.), c(n, 0.), nu(n, 0.), chi(n, 0.) {}
    void insertData(const HostFluid& f)
    {
        points.insertData(f.points);
        dyn.insertData(f.dyn);
        appendVector(rho0, f.rho0);
        appendVector(dRho, f.dRho);
        appendVector(c, f.c);
        appendVector(nu, f.nu);
        appendVector(chi, f.chi);
    }
};

struct HostSolid {
    HostPointCloud points;
    HostDynamicStateBase dyn;
    std::vector<double3> normal;
    std::vector<double3> torques;
    std::vector<double3> angularVelocities;
    std::vector<double> radius;
    std::vector<double> inverseMass;
    std::vector<int> materialID;
    std::vector<int> clusterID;
    std::vector<int> clumpID;
    std::vector<int> isDummyParticle;
    std::vector<double> pressure;

    HostSolid() = default;
    explicit HostSolid(int n)
        : points(n), dyn(n), normal(n, make_double3(0, 0, 0)), torques(n, make_double3(0, 0, 0)),
          angularVelocities(n, make_double3(0, 0, 0)), radius(n, 0), inverseMass(n, 0), materialID(n, 0),
          clusterID(n, -1), clumpID(n, -1), isDummyParticle(n, 0), pressure(n, 0) {}
    void insertData(const HostSolid& s)
    {
        points.insertData(s.points);
        dyn.insertData(s.dyn);
        appendVector(normal, s.normal);
        appendVector(torques, s.torques);
        appendVector(angularVelocities, s.angularVelocities);
        appendVector(radius, s.radius);
        appendVector(inverseMass, s.inverseMass);
        appendVector(materialID, s.materialID);
        appendVector(clusterID, s.clusterID);
        appendVector(clumpID, s.clumpID);
        appendVector(isDummyParticle, s.isDummyParticle);
        appendVector(pressure, s.pressure);
    }
};

struct HostClump {
    int num{0};
    HostDynamicStateBase dyn;
    std::vector<double3> centroidPosition;
    std::vector<double3> torques;
    std::vector<double3> angularVelocities;
    std::vector<quaternion> orientations;
    std::vector<symMatrix> inverseInertiaTensor;
    std::vector<double> inverseMass;
    std::vector<int> pebbleStartIndex;  // pebbles are solids [start, end)
    std::vector<int> pebbleEndIndex;

    HostClump() = default;
    explicit HostClump(int n)
        : num(n), dyn(n), centroidPosition(n, make_double3(0, 0, 0)), torques(n, make_double3(0, 0, 0)),
          angularVelocities(n, make_double3(0, 0, 0)), orientations(n, make_quaternion(1, 0, 0, 0)),
          inverseInertiaTensor(n, make_symMatrix(0, 0, 0, 0, 0, 0)), inverseMass(n, 0), pebbleStartIndex(n, -1),
          pebbleEndIndex(n, -1) {}
    void insertData(const HostClump& c)
    {
        dyn.insertData(c.dyn);
        appendVector(centroidPosition, c.centroidPosition);
        appendVector(torques, c.torques);
        appendVector(angularVelocities, c.angularVelocities);
        appendVector(orientations, c.orientations);
        appendVector(inverseInertiaTensor, c.inverseInertiaTensor);
        appendVector(inverseMass, c.inverseMass);
        appendVector(pebbleStartIndex, c.pebbleStartIndex);
        appendVector(pebbleEndIndex, c.pebbleEndIndex);
        num += c.num;
    }
};

struct HostInfiniteWall {
    int num{0};
    std::vector<double3> pointInPlane;
    std::vector<double3> normal;
    std::vector<int> materialID;

    HostInfiniteWall() = default;
    explicit HostInfiniteWall(int n)
        : num(n), pointInPlane(n, make_double3(0, 0, 0)), normal(n, make_double3(0, 0, 0)), materialID(n, 0) {}
    void insertData(const HostInfiniteWall& w)
    {
        appendVector(pointInPlane, w.pointInPlane);
        appendVector(normal, w.normal);
        appendVector(materialID, w.materialID);
        num += w.num;
    }
};

struct HostCylinderWall {
    int num{0};
    std::vector<double3> pointInAxis;
    std::vector<double3> axis;
    std::vector<double3> angularVelocity;
    std::vector<double> radius;
    std::vector<int> materialID;

    HostCylinderWall() = default;
    explicit HostCylinderWall(int n)
        : num(n), pointInAxis(n, make_double3(0, 0, 0)), axis(n, make_double3(0, 0, 0)),
          angularVelocity(n, make_double3(0, 0, 0)), radius(n, 0.), materialID(n, 0) {}
    void insertData(const HostCylinderWall& c)
    {
        appendVector(pointInAxis, c.pointInAxis);
        appendVector(axis, c.axis);
        appendVector(angularVelocity, c.angularVelocity);
        appendVector(radius, c.radius);
        appendVector(materialID, c.materialID);
        num += c.num;
    }
};

struct HostInteractionBase {
    int capacity{0}, num{0};
    std::vector<double3> force;
    std::vector<int> objectPointed;
    std::vector<int> objectPointing;

    HostInteractionBase() = default;
    explicit HostInteractionBase(int n)
        : capacity(n), num(0), force(n, make_double3(0, 0, 0)), objectPointed(n, -1), objectPointing(n, -1) {}
    void insertData(const HostInteractionBase& i)
    {
        appendVector(force, i.force);
        appendVector(objectPointed, i.objectPointed);
        appendVector(objectPointing, i.objectPointing);
        capacity += i.capacity;
    }
};

struct HostInteractionSolid2Solid {
    int capacity{0}, num{0};
    std::vector<double3> force;
    std::vector<double3> torque;
    std::vector<double3> slidingSpring;
    std::vector<double3> rollingSpring;
    std::vector<double3> torsionSpring;
    std::vector<int> objectPointed;
    std::vector<int> objectPointing;

    HostInteractionSolid2Solid() = default;
    explicit HostInteractionSolid2Solid(int n)
        : capacity(n), num(0), force(n, make_double3(0, 0, 0)), torque(n, make_double3(0, 0, 0)),
          slidingSpring(n, make_double3(0, 0, 0)), rollingSpring(n, make_double3(0, 0, 0)),
          torsionSpring(n, make_double3(0, 0, 0)), objectPointed(n, -1), objectPointing(n, -1) {}
    void insertData(const HostInteractionSolid2Solid& i)
    {
        appendVector(force, i.force);
        appendVector(torque, i.torque);
        appendVector(slidingSpring, i.slidingSpring);
        appendVector(rollingSpring, i.rollingSpring);
        appendVector(torsionSpring, i.torsionSpring);
        appendVector(objectPointed, i.objectPointed);
        appendVector(objectPointing, i.objectPointing);
        capacity += i.capacity;
    }
};

struct HostInteractionBonded {
    int num{0};
    std::vector<double3> contactNormal;
    std::vector<double3> contactPoint;
    std::vector<double3> shearForce;
    std::vector<double3> bendingTorque;
    std::vector<double> normalForce;
    std::vector<double> torsionTorque;
    std::vector<int> objectPointed;
    std::vector<int> objectPointing;
    std::vector<int> isBonded;

    HostInteractionBonded() = default;
    explicit HostInteractionBonded(int n)
        : num(n), contactNormal(n, make_double3(0, 0, 0)), contactPoint(n, make_double3(0, 0, 0)),
          shearForce(n, make_double3(0, 0, 0)), bendingTorque(n, make_double3(0, 0, 0)), normalForce(n, 0.),
          torsionTorque(n, 0.), objectPointed(n, -1), objectPointing(n, -1), isBonded(n, 0) {}
    void insertData(const HostInteractionBonded& i)
    {
        appendVector(contactNormal, i.contactNormal);
        appendVector(contactPoint, i.contactPoint);
        appendVector(shearForce, i.shearForce);
        appendVector(bendingTorque, i.bendingTorque);
        appendVector(normalForce, i.normalForce);
        appendVector(torsionTorque, i.torsionTorque);
        appendVector(objectPointed, i.objectPointed);
        appendVector(objectPointing, i.objectPointing);
        appendVector(isBonded, i.isBonded);
        num += i.num;
    }
};

// Per material-pair tables (k: stiffness, d: dissipation, mu: friction;
// n normal, s sliding, r rolling, t torsion).
struct HostHertzianContactModel {
    std::vector<double> E, G, res, k_r_k_s, k_t_k_s, mu_s, mu_r, mu_t;
    HostHertzianContactModel() = default;
    explicit HostHertzianContactModel(int n)
        : E(n, 0), G(n, 0), res(n, 1.), k_r_k_s(n, 0), k_t_k_s(n, 0), mu_s(n, 0), mu_r(n, 0), mu_t(n, 0) {}
};

struct HostLinearContactModel {
    std::vector<double> k_n, k_s, k_r, k_t, d_n, d_s, d_r, d_t, mu_s, mu_r, mu_t;
    HostLinearContactModel() = default;
    explicit HostLinearContactModel(int n)
        : k_n(n, 0), k_s(n, 0), k_r(n, 0), k_t(n, 0), d_n(n, 0), d_s(n, 0), d_r(n, 0), d_t(n, 0), mu_s(n, 0),
          mu_r(n, 0), mu_t(n, 0) {}
};

struct HostBondedContactModel {
    std::vector<double> gamma;    // bond radius multiplier
    std::vector<double> E;        // bond elastic modulus
    std::vector<double> k_n_k_s;  // normal / shear stiffness ratio
    std::vector<double> sigma_s;  // tensile strength
    std::vector<double> C;        // cohesion
    std::vector<double> mu;       // friction coefficient
    HostBondedContactModel() = default;
    explicit HostBondedContactModel(int n) : gamma(n, 1), E(n, 0), k_n_k_s(n, 2), sigma_s(n, 0), C(n, 0), mu(n, 0) {}
};

struct HostSolidContactModel {
    int nMaterial{0};
    HostHertzianContactModel hertzian;
    HostLinearContactModel linear;
    HostBondedContactModel bonded;

    HostSolidContactModel() = default;
    explicit HostSolidContactModel(int nMat)
        : nMaterial(nMat), hertzian(nMat * (nMat + 1) / 2), linear(nMat * (nMat + 1) / 2),
          bonded(nMat * (nMat + 1) / 2) {}

    // Slot of the unordered pair (mA, mB) in the upper-triangular table, or -1.
    int getCombinedIndex(int mA, int mB) const
    {
        if (mA >= nMaterial || mB >= nMaterial) return -1;
        const int i = std::min(mA, mB), j = std::max(mA, mB);
        return i * nMaterial - i * (i - 1) / 2 + (j - i);
    }
};

struct HostData {
    HostFluid fluids;
    HostSolid solids;
    HostClump clumps;
    HostInfiniteWall infiniteWalls;
    HostCylinderWall cylinderWalls;
    HostInteractionBase fluid2Fluid;
    HostInteractionBase fluid2Solid;
    HostInteractionSolid2Solid solid2Solid;
    HostInteractionBonded solidBond2Solid;
    HostSolidContactModel contactModels;
};
