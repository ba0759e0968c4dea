// SceneBuilder: see sceneBuilder.h.  Each function cites the reference setup
// call whose semantics it follows.
#include "sceneBuilder.h"

#include <cmath>

namespace demsph {

// dataBase::setDomain (core/dataBase.h:93-103): the values are stored before
// they are checked, as in the reference.
int SceneBuilder::setDomain(double3 origin, double3 size)
{
    sim.domainOrigin = origin;
    sim.domainSize = size;
    if (size.x <= 0. || size.y <= 0. || size.z <= 0.)
        return fail("Error: domain size must be positive in all directions.");
    return DEMSPH_OK;
}

int SceneBuilder::setGravity(double3 g)  // dataBase.h:105-109
{
    sim.gravity = g;
    return DEMSPH_OK;
}

int SceneBuilder::setTimeStep(double dt)  // dataBase.h:68-81
{
    if (dt <= 0.) return fail("Error: time step must be non-negative.");
    if (started) return fail("Warning: cannot change the time step during simulation.");
    sim.timeStep = dt;
    return DEMSPH_OK;
}

int SceneBuilder::setMaximumTime(double t)  // dataBase.h:38-51
{
    if (t <= 0.) return fail("Error: maximum time must be positive.");
    if (started) return fail("Warning: cannot change the number of frames during simulation.");
    sim.maximumTime = t;
    return DEMSPH_OK;
}

int SceneBuilder::setNumFrames(int n)  // dataBase.h:53-66
{
    if (n < 1) return fail("Error: number of frames must be at least 1.");
    if (started) return fail("Warning: cannot change the number of frames during simulation.");
    sim.numFrames = n;
    return DEMSPH_OK;
}

int SceneBuilder::setFluidIntegrateGap(int gap)  // dataBase.h:83-91
{
    if (gap < 1) return fail("Error: fluid integrate gap must be at least 1.");
    sim.fluidIntegrateGap = gap;
    return DEMSPH_OK;
}

int SceneBuilder::setHertzian(int mi, int mj, double E, double G, double res, double krks, double ktks,
                              double mus, double mur, double mut)  // dataBase.h:111-128
{
    const int c = hos.contactModels.getCombinedIndex(mi, mj);
    if (c < 0) return fail("Error: material index exceeds the number of materials.");
    HostHertzianContactModel& h = hos.contactModels.hertzian;
    h.E[c] = E; h.G[c] = G; h.res[c] = res; h.k_r_k_s[c] = krks; h.k_t_k_s[c] = ktks;
    h.mu_s[c] = mus; h.mu_r[c] = mur; h.mu_t[c] = mut;
    return DEMSPH_OK;
}

int SceneBuilder::setLinear(int mi, int mj, double kn, double ks, double kr, double kt, double dn, double ds,
                            double dr, double dt, double mus, double mur, double mut)  // dataBase.h:130-150
{
    const int c = hos.contactModels.getCombinedIndex(mi, mj);
    if (c < 0) return fail("Error: material index exceeds the number of materials.");
    HostLinearContactModel& l = hos.contactModels.linear;
    l.k_n[c] = kn; l.k_s[c] = ks; l.k_r[c] = kr; l.k_t[c] = kt;
    l.d_n[c] = dn; l.d_s[c] = ds; l.d_r[c] = dr; l.d_t[c] = dt;
    l.mu_s[c] = mus; l.mu_r[c] = mur; l.mu_t[c] = mut;
    return DEMSPH_OK;
}

int SceneBuilder::setBonded(int mi, int mj, double E, double knks, double gamma, double sigma, double C,
                            double mu)  // dataBase.h:152-167
{
    const int c = hos.contactModels.getCombinedIndex(mi, mj);
    if (c < 0) return fail("Error: material index exceeds the number of materials.");
    HostBondedContactModel& b = hos.contactModels.bonded;
    b.E[c] = E; b.k_n_k_s[c] = knks; b.gamma[c] = gamma; b.sigma_s[c] = sigma; b.C[c] = C; b.mu[c] = mu;
    return DEMSPH_OK;
}

// dataBase::addFluid + addFluidData (core/dataBase.cpp:3-17, 226-247): one
// smoothing length, rest density, sound speed and viscosity per call; the
// pair capacities the reference reserves (40 and 20 per particle) are not
// needed here because the engine sizes its own lists.
int SceneBuilder::addFluid(const std::vector<double3>& p, double3 v, double smoothLength, double density,
                           double soundSpeed, double kinematicViscosity)
{
    const int n = (int)p.size();
    HostFluid f(n);
    for (int i = 0; i < n; ++i) {
        f.points.position[i] = p[i];
        f.points.effectiveRadii[i] = smoothLength;
        f.dyn.velocities[i] = v;
        f.rho0[i] = density;
        f.c[i] = soundSpeed;
        f.nu[i] = kinematicViscosity;
    }
    hos.fluids.insertData(f);
    hos.fluid2Fluid.insertData(HostInteractionBase(0));
    hos.fluid2Solid.insertData(HostInteractionBase(0));
    return DEMSPH_OK;
}

// dataBase::addDummyParticleWall (core/dataBase.cpp:19-31): fixed particles
// whose "spacing" argument is used as their radius; search radius 2.6 r.
int SceneBuilder::addDummyParticleWall(const std::vector<double3>& p, double spacing)
{
    const int n = (int)p.size();
    HostSolid s(n);
    for (int i = 0; i < n; ++i) {
        s.points.position[i] = p[i];
        s.points.effectiveRadii[i] = 2.6 * spacing;
        s.radius[i] = spacing;
        s.isDummyParticle[i] = 1;
    }
    appendSolids(s);
    return DEMSPH_OK;
}

// Sphere mass 4/3 pi r^3 rho, evaluated in the reference's operand order
// (core/dataBase.cpp:49,109) so inverse masses agree to the last bit.
static double sphereInverseMass(double r, double rho) { return 1. / (4. / 3. * std::pow(r, 3) * pi() * rho); }

// dataBase::addSolid (core/dataBase.cpp:33-53).
int SceneBuilder::addSolid(const std::vector<double3>& p, double3 v, double radius, double density, int materialID)
{
    if (materialID >= hos.contactModels.nMaterial)
        return fail("Error: material index exceeds the number of materials when adding a cluster.");
    const int n = (int)p.size();
    HostSolid s(n);
    for (int i = 0; i < n; ++i) {
        s.points.position[i] = p[i];
        s.dyn.velocities[i] = v;
        s.points.effectiveRadii[i] = 1.1 * radius;
        s.radius[i] = radius;
        s.materialID[i] = materialID;
        if (density > 0) s.inverseMass[i] = sphereInverseMass(radius, density);
    }
    appendSolids(s);
    return DEMSPH_OK;
}

// dataBase::addInfiniteWall (core/dataBase.cpp:55-67): only before the start.
int SceneBuilder::addInfiniteWall(double3 p, double3 normal, int materialID)
{
    if (started) return fail("Error: infinite wall can only be added before the simulation starts.");
    HostInfiniteWall w(1);
    w.pointInPlane[0] = p;
    w.normal[0] = normal;
    w.materialID[0] = materialID;
    hos.infiniteWalls.insertData(w);
    return DEMSPH_OK;
}

// dataBase::addCylinderWall (core/dataBase.cpp:69-82).  The reference's solver
// never copies cylinder walls to the device, so they take no part in a step;
// they are recorded for completeness (with the radius, which the reference
// drops).
int SceneBuilder::addCylinderWall(double3 p, double3 axis, double3 angularVelocity, double radius, int materialID)
{
    if (started) return fail("Error: cylinder wall can only be added before the simulation starts.");
    HostCylinderWall c(1);
    c.pointInAxis[0] = p;
    c.axis[0] = axis;
    c.angularVelocity[0] = angularVelocity;
    c.radius[0] = radius;
    c.materialID[0] = materialID;
    hos.cylinderWalls.insertData(c);
    return DEMSPH_OK;
}

// dataBase::addCluster (core/dataBase.cpp:84-118): one new cluster id (one
// more than the largest so far) for all spheres of the call; touching spheres
// of one cluster are bonded at initialisation when the bond modulus is set.
int SceneBuilder::addCluster(const std::vector<double3>& p, const std::vector<double>& radius,
                             const std::vector<double>& density, double3 v, int materialID)
{
    if (p.size() != radius.size() || p.size() != density.size())
        return fail("Error: the size of position, velocity, and radius vectors must be the same when adding a "
                    "cluster.");
    if (materialID >= hos.contactModels.nMaterial)
        return fail("Error: material index exceeds the number of materials when adding a cluster.");
    int clusterID = 0;
    if (hos.solids.points.num > 0)
        clusterID = *std::max_element(hos.solids.clusterID.begin(), hos.solids.clusterID.end()) + 1;
    const int n = (int)p.size();
    HostSolid s(n);
    for (int i = 0; i < n; ++i) {
        s.points.position[i] = p[i];
        s.points.effectiveRadii[i] = 1.1 * radius[i];
        s.dyn.velocities[i] = v;
        s.radius[i] = radius[i];
        s.materialID[i] = materialID;
        s.clusterID[i] = clusterID;
        if (density[i] > 0) s.inverseMass[i] = sphereInverseMass(radius[i], density[i]);
    }
    appendSolids(s);
    return DEMSPH_OK;
}

// dataBase::addClump (core/dataBase.cpp:120-177).  The clump's mass is spread
// over its pebbles by the volume of each pebble's bounding cube (2r)^3, as in
// the reference; pebble velocities are the rigid-body field v + w x (p - c).
int SceneBuilder::addClump(const std::vector<double3>& p, const std::vector<double>& radius, double3 centroid,
                           double3 v, double3 angularVelocity, double mass, symMatrix inertia, int materialID)
{
    if (p.size() != radius.size())
        return fail("Error: the size of position and radius vectors must be the same when adding a clump.");
    if (materialID >= hos.contactModels.nMaterial)
        return fail("Error: material index exceeds the number of materials when adding a clump.");
    const int clumpID = hos.clumps.num;
    HostClump c(1);
    c.centroidPosition[0] = centroid;
    c.dyn.velocities[0] = v;
    c.angularVelocities[0] = angularVelocity;
    if (mass > 0.) c.inverseMass[0] = 1. / mass;
    c.inverseInertiaTensor[0] = inverse(inertia);
    c.pebbleStartIndex[0] = hos.solids.points.num;
    double volume = 0;
    for (double r : radius) volume += std::pow(2. * r, 3);
    const double density = volume > 0. ? mass / volume : 0.;
    const int n = (int)p.size();
    HostSolid s(n);
    for (int i = 0; i < n; ++i) {
        s.points.position[i] = p[i];
        s.points.effectiveRadii[i] = 1.1 * radius[i];
        s.dyn.velocities[i] = v + cross(angularVelocity, p[i] - centroid);
        s.angularVelocities[i] = angularVelocity;
        s.radius[i] = radius[i];
        s.materialID[i] = materialID;
        s.clumpID[i] = clumpID;
        if (density > 0. && radius[i] > 0) s.inverseMass[i] = 1. / (std::pow(2. * radius[i], 3) * density);
    }
    appendSolids(s);
    c.pebbleEndIndex[0] = hos.solids.points.num;
    hos.clumps.insertData(c);
    return DEMSPH_OK;
}

void SceneBuilder::appendSolids(const HostSolid& s)  // addSolidData, core/dataBase.cpp:249-268
{
    hos.solids.insertData(s);
    hos.solid2Solid.insertData(HostInteractionSolid2Solid(0));
}

void SceneBuilder::view(demsph_scene* s)
{
    *s = demsph_scene{};
    s->domain_origin[0] = sim.domainOrigin.x; s->domain_origin[1] = sim.domainOrigin.y;
    s->domain_origin[2] = sim.domainOrigin.z;
    s->domain_size[0] = sim.domainSize.x; s->domain_size[1] = sim.domainSize.y; s->domain_size[2] = sim.domainSize.z;
    s->gravity[0] = sim.gravity.x; s->gravity[1] = sim.gravity.y; s->gravity[2] = sim.gravity.z;
    s->time_step = sim.timeStep;
    s->fluid_integrate_gap = sim.fluidIntegrateGap;
    s->maximum_time = sim.maximumTime;
    s->num_frames = sim.numFrames;

    auto d3 = [](const std::vector<double3>& v) { return v.empty() ? nullptr : &v[0].x; };
    auto d1 = [](const std::vector<double>& v) { return v.empty() ? nullptr : v.data(); };
    auto i1 = [](const std::vector<int>& v) { return v.empty() ? nullptr : v.data(); };

    const HostFluid& f = hos.fluids;
    s->n_fluid = f.points.num;
    s->fluid_position = d3(f.points.position);
    s->fluid_velocity = d3(f.dyn.velocities);
    s->fluid_acceleration = d3(f.dyn.accelerations);
    s->fluid_smoothing_length = d1(f.points.effectiveRadii);
    s->fluid_rho0 = d1(f.rho0);
    s->fluid_drho = d1(f.dRho);
    s->fluid_sound_speed = d1(f.c);
    s->fluid_nu = d1(f.nu);

    const HostSolid& so = hos.solids;
    s->n_solid = so.points.num;
    s->solid_position = d3(so.points.position);
    s->solid_velocity = d3(so.dyn.velocities);
    s->solid_acceleration = d3(so.dyn.accelerations);
    s->solid_normal = d3(so.normal);
    s->solid_torque = d3(so.torques);
    s->solid_angular_velocity = d3(so.angularVelocities);
    s->solid_effective_radius = d1(so.points.effectiveRadii);
    s->solid_radius = d1(so.radius);
    s->solid_inverse_mass = d1(so.inverseMass);
    s->solid_material = i1(so.materialID);
    s->solid_cluster = i1(so.clusterID);
    s->solid_clump = i1(so.clumpID);
    s->solid_is_dummy = i1(so.isDummyParticle);

    const HostClump& c = hos.clumps;
    s->n_clump = c.num;
    s->clump_centroid = d3(c.centroidPosition);
    s->clump_velocity = d3(c.dyn.velocities);
    s->clump_acceleration = d3(c.dyn.accelerations);
    s->clump_angular_velocity = d3(c.angularVelocities);
    s->clump_torque = d3(c.torques);
    s->clump_orientation = c.orientations.empty() ? nullptr : &c.orientations[0].q0;
    s->clump_inverse_inertia = c.inverseInertiaTensor.empty() ? nullptr : &c.inverseInertiaTensor[0].xx;
    s->clump_inverse_mass = d1(c.inverseMass);
    s->clump_pebble_start = i1(c.pebbleStartIndex);
    s->clump_pebble_end = i1(c.pebbleEndIndex);

    const HostInfiniteWall& w = hos.infiniteWalls;
    s->n_wall = w.num;
    s->wall_point = d3(w.pointInPlane);
    s->wall_normal = d3(w.normal);
    s->wall_material = i1(w.materialID);

    const HostSolidContactModel& m = hos.contactModels;
    const int nc = m.nMaterial * (m.nMaterial + 1) / 2;
    hertzFlat_.assign(8 * nc, 0.);
    linearFlat_.assign(11 * nc, 0.);
    bondedFlat_.assign(6 * nc, 0.);
    for (int k = 0; k < nc; ++k) {
        const double h[8] = {m.hertzian.E[k], m.hertzian.G[k], m.hertzian.res[k], m.hertzian.k_r_k_s[k],
                             m.hertzian.k_t_k_s[k], m.hertzian.mu_s[k], m.hertzian.mu_r[k], m.hertzian.mu_t[k]};
        const double l[11] = {m.linear.k_n[k], m.linear.k_s[k], m.linear.k_r[k], m.linear.k_t[k],
                              m.linear.d_n[k], m.linear.d_s[k], m.linear.d_r[k], m.linear.d_t[k],
                              m.linear.mu_s[k], m.linear.mu_r[k], m.linear.mu_t[k]};
        const double b[6] = {m.bonded.gamma[k], m.bonded.E[k], m.bonded.k_n_k_s[k],
                             m.bonded.sigma_s[k], m.bonded.C[k], m.bonded.mu[k]};
        std::copy(h, h + 8, &hertzFlat_[8 * k]);
        std::copy(l, l + 11, &linearFlat_[11 * k]);
        std::copy(b, b + 6, &bondedFlat_[6 * k]);
    }
    s->n_material = m.nMaterial;
    s->hertzian = hertzFlat_.data();
    s->linear = linearFlat_.data();
    s->bonded = bondedFlat_.data();
}

}  // namespace demsph

// ---------------------------------------------------------------------------
// C ABI wrappers (include/demsph_gb300.h)
// ---------------------------------------------------------------------------
struct demsph_builder {
    demsph::SceneBuilder b;
    explicit demsph_builder(int n) : b(n) {}
};

namespace {
std::vector<double3> points(int n, const double* xyz)
{
    std::vector<double3> v(n > 0 ? n : 0);
    for (int i = 0; i < n; ++i) v[i] = make_double3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    return v;
}
double3 vec(const double* a) { return make_double3(a[0], a[1], a[2]); }
}  // namespace

extern "C" {

demsph_builder* demsph_builder_new(int n_material)
{
    if (n_material < 1) return nullptr;
    return new demsph_builder(n_material);
}
void demsph_builder_free(demsph_builder* b) { delete b; }
const char* demsph_builder_last_error(const demsph_builder* b) { return b ? b->b.lastError.c_str() : ""; }

#define DEMSPH_B(b) if (!(b)) return DEMSPH_ERR_ARGUMENT
int demsph_builder_set_domain(demsph_builder* b, const double o[3], const double s[3])
{
    DEMSPH_B(b);
    return b->b.setDomain(vec(o), vec(s));
}
int demsph_builder_set_gravity(demsph_builder* b, const double g[3])
{
    DEMSPH_B(b);
    return b->b.setGravity(vec(g));
}
int demsph_builder_set_time_step(demsph_builder* b, double dt) { DEMSPH_B(b); return b->b.setTimeStep(dt); }
int demsph_builder_set_maximum_time(demsph_builder* b, double t) { DEMSPH_B(b); return b->b.setMaximumTime(t); }
int demsph_builder_set_num_frames(demsph_builder* b, int n) { DEMSPH_B(b); return b->b.setNumFrames(n); }
int demsph_builder_set_fluid_integrate_gap(demsph_builder* b, int g)
{
    DEMSPH_B(b);
    return b->b.setFluidIntegrateGap(g);
}
int demsph_builder_set_hertzian(demsph_builder* b, int mi, int mj, double E, double G, double res, double krks,
                                double ktks, double mus, double mur, double mut)
{
    DEMSPH_B(b);
    return b->b.setHertzian(mi, mj, E, G, res, krks, ktks, mus, mur, mut);
}
int demsph_builder_set_linear(demsph_builder* b, int mi, int mj, double kn, double ks, double kr, double kt,
                              double dn, double ds, double dr, double dt, double mus, double mur, double mut)
{
    DEMSPH_B(b);
    return b->b.setLinear(mi, mj, kn, ks, kr, kt, dn, ds, dr, dt, mus, mur, mut);
}
int demsph_builder_set_bonded(demsph_builder* b, int mi, int mj, double E, double knks, double gamma, double sigma,
                              double C, double mu)
{
    DEMSPH_B(b);
    return b->b.setBonded(mi, mj, E, knks, gamma, sigma, C, mu);
}
int demsph_builder_add_fluid(demsph_builder* b, int n, const double* xyz, const double v[3], double sl,
                             double rho, double c, double nu)
{
    DEMSPH_B(b);
    if (n < 0 || (n > 0 && !xyz)) return DEMSPH_ERR_ARGUMENT;
    return b->b.addFluid(points(n, xyz), vec(v), sl, rho, c, nu);
}
int demsph_builder_add_dummy_wall(demsph_builder* b, int n, const double* xyz, double spacing)
{
    DEMSPH_B(b);
    if (n < 0 || (n > 0 && !xyz)) return DEMSPH_ERR_ARGUMENT;
    return b->b.addDummyParticleWall(points(n, xyz), spacing);
}
int demsph_builder_add_solid(demsph_builder* b, int n, const double* xyz, const double v[3], double r, double rho,
                             int mat)
{
    DEMSPH_B(b);
    if (n < 0 || (n > 0 && !xyz)) return DEMSPH_ERR_ARGUMENT;
    return b->b.addSolid(points(n, xyz), vec(v), r, rho, mat);
}
int demsph_builder_add_infinite_wall(demsph_builder* b, const double p[3], const double nrm[3], int mat)
{
    DEMSPH_B(b);
    return b->b.addInfiniteWall(vec(p), vec(nrm), mat);
}
int demsph_builder_add_cylinder_wall(demsph_builder* b, const double p[3], const double axis[3], const double w[3],
                                     double r, int mat)
{
    DEMSPH_B(b);
    return b->b.addCylinderWall(vec(p), vec(axis), vec(w), r, mat);
}
int demsph_builder_add_cluster(demsph_builder* b, int n, const double* xyz, const double* r, const double* rho,
                               const double v[3], int mat)
{
    DEMSPH_B(b);
    if (n < 0 || (n > 0 && (!xyz || !r || !rho))) return DEMSPH_ERR_ARGUMENT;
    return b->b.addCluster(points(n, xyz), std::vector<double>(r, r + n), std::vector<double>(rho, rho + n),
                           vec(v), mat);
}
int demsph_builder_add_clump(demsph_builder* b, int n, const double* xyz, const double* r, const double c[3],
                             const double v[3], const double w[3], double mass, const double I6[6], int mat)
{
    DEMSPH_B(b);
    if (n < 0 || (n > 0 && (!xyz || !r)) || !I6) return DEMSPH_ERR_ARGUMENT;
    return b->b.addClump(points(n, xyz), std::vector<double>(r, r + n), vec(c), vec(v), vec(w), mass,
                         make_symMatrix(I6[0], I6[1], I6[2], I6[3], I6[4], I6[5]), mat);
}
int demsph_builder_scene(const demsph_builder* b, demsph_scene* out)
{
    if (!b || !out) return DEMSPH_ERR_ARGUMENT;
    const_cast<demsph_builder*>(b)->b.view(out);
    return DEMSPH_OK;
}
#undef DEMSPH_B

}  // extern "C"
