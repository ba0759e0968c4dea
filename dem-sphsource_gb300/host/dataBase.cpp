// class dataBase: see dataBase.h.  Each function cites the reference call whose
// behaviour it keeps.
#include "dataBase.h"

#include <stdexcept>

dataBase::dataBase()
{
    // core/dataBase.h:8-23
    simPara.maximumTime = 1.;
    simPara.timeStep = 1.;
    simPara.numSteps = 1;
    simPara.iStep = 0;
    simPara.numFrames = 1;
    simPara.iFrame = 0;
    simPara.frameInterval = 1;
}

dataBase::~dataBase() { releaseEngine(); }

void dataBase::report(int status)
{
    if (status != DEMSPH_OK) std::cout << scene.lastError << std::endl;
}

void dataBase::check(int status, const char* what)
{
    if (status == DEMSPH_OK) return;
    std::string msg = std::string(what) + ": " + demsph_status_string(status);
    if (engine) msg += std::string(" (") + demsph_last_error(engine) + ")";
    throw std::runtime_error(msg);
}

// ---- simulation parameters (core/dataBase.h:33-91) ----
void dataBase::setGPUParameterDeviceIndex(int index) { deviceIndex = index; }

void dataBase::setSimulationParameterMaximumTime(double t)
{
    report(scene.setMaximumTime(t));
    simPara.maximumTime = scene.sim.maximumTime;
}

void dataBase::setSimulationParameterNumFrames(int n)
{
    report(scene.setNumFrames(n));
    simPara.numFrames = scene.sim.numFrames;
}

void dataBase::setSimulationParameterTimeStep(double dt)
{
    report(scene.setTimeStep(dt));
    simPara.timeStep = scene.sim.timeStep;
}

void dataBase::setFluidIntegrateGap(int gap) { report(scene.setFluidIntegrateGap(gap)); }

// core/dataBase.h:93-103.  Re-gridding a running engine is not supported.
void dataBase::setDomain(double3 origin, double3 size)
{
    if (running()) {
        std::cout << "Error: the domain cannot be changed after the simulation starts." << std::endl;
        return;
    }
    report(scene.setDomain(origin, size));
}

// core/dataBase.h:105-109
void dataBase::setGravity(double3 g)
{
    scene.setGravity(g);
    if (running()) {
        const double v[3] = {g.x, g.y, g.z};
        check(demsph_set_gravity(engine, v), "setGravity");
    }
}

// ---- contact models (core/dataBase.h:111-167): copied to the running engine ----
void dataBase::setHertzianContactModel(int mat_i, int mat_j, double E, double G, double res, double k_r_k_s,
                                       double k_t_k_s, double mu_s, double mu_r, double mu_t)
{
    const int st = scene.setHertzian(mat_i, mat_j, E, G, res, k_r_k_s, k_t_k_s, mu_s, mu_r, mu_t);
    report(st);
    if (st == DEMSPH_OK && running()) {
        demsph_scene v;
        scene.view(&v);
        check(demsph_set_contact_models(engine, &v), "setHertzianContactModel");
    }
}

void dataBase::setLinearContactModel(int mat_i, int mat_j, double k_n, double k_s, double k_r, double k_t,
                                     double d_n, double d_s, double d_r, double d_t, double mu_s, double mu_r,
                                     double mu_t)
{
    const int st = scene.setLinear(mat_i, mat_j, k_n, k_s, k_r, k_t, d_n, d_s, d_r, d_t, mu_s, mu_r, mu_t);
    report(st);
    if (st == DEMSPH_OK && running()) {
        demsph_scene v;
        scene.view(&v);
        check(demsph_set_contact_models(engine, &v), "setLinearContactModel");
    }
}

void dataBase::setBondedContactModel(int mat_i, int mat_j, double E, double k_n_k_s, double gamma, double sigma_s,
                                     double C, double mu)
{
    const int st = scene.setBonded(mat_i, mat_j, E, k_n_k_s, gamma, sigma_s, C, mu);
    report(st);
    if (st == DEMSPH_OK && running()) {
        demsph_scene v;
        scene.view(&v);
        check(demsph_set_contact_models(engine, &v), "setBondedContactModel");
    }
}

// core/dataBase.h:169-182
void dataBase::setClumpVelocity(int index, double3 velocity)
{
    if (index < 0 || index >= scene.hos.clumps.num) return;
    scene.hos.clumps.dyn.velocities[index] = velocity;
    if (running()) {
        const double v[3] = {velocity.x, velocity.y, velocity.z};
        check(demsph_set_clump_velocity(engine, index, v), "setClumpVelocity");
    }
}

// ---- particles and walls (core/dataBase.cpp:3-177) ----
// Fluids and solids added after the start go to the running engine
// (demsph_append: addFluidData / addSolidData with iStep > 0,
// core/dataBase.cpp:226-268); walls and clumps only before the start.
#define REFUSE_WHILE_RUNNING(what)                                                                   \
    if (running()) {                                                                                 \
        std::cout << "Error: " what " cannot be added after the simulation starts." << std::endl;   \
        return;                                                                                      \
    }
#define APPEND_WHILE_RUNNING(call)                                          \
    const int nf0_ = scene.hos.fluids.points.num, ns0_ = scene.hos.solids.points.num; \
    const int st_ = (call);                                                 \
    report(st_);                                                            \
    if (st_ == DEMSPH_OK && running()) appendRunning(nf0_, ns0_);

void dataBase::appendRunning(int nf0, int ns0)
{
    demsph_scene v;
    scene.view(&v);
    demsph_scene cur = v, add = v;
    cur.n_fluid = nf0;
    cur.n_solid = ns0;
    add.n_fluid = v.n_fluid - nf0;
    add.n_solid = v.n_solid - ns0;
    add.n_clump = 0;
    add.n_wall = 0;
    if (add.n_fluid == 0 && add.n_solid == 0) return;
    auto v3 = [](const double* p, int k) { return p ? p + 3 * (size_t)k : p; };
    auto d1 = [](const double* p, int k) { return p ? p + k : p; };
    auto i1 = [](const int* p, int k) { return p ? p + k : p; };
    add.fluid_position = v3(v.fluid_position, nf0);
    add.fluid_velocity = v3(v.fluid_velocity, nf0);
    add.fluid_acceleration = v3(v.fluid_acceleration, nf0);
    add.fluid_smoothing_length = d1(v.fluid_smoothing_length, nf0);
    add.fluid_rho0 = d1(v.fluid_rho0, nf0);
    add.fluid_drho = d1(v.fluid_drho, nf0);
    add.fluid_sound_speed = d1(v.fluid_sound_speed, nf0);
    add.fluid_nu = d1(v.fluid_nu, nf0);
    add.solid_position = v3(v.solid_position, ns0);
    add.solid_velocity = v3(v.solid_velocity, ns0);
    add.solid_acceleration = v3(v.solid_acceleration, ns0);
    add.solid_normal = v3(v.solid_normal, ns0);
    add.solid_torque = v3(v.solid_torque, ns0);
    add.solid_angular_velocity = v3(v.solid_angular_velocity, ns0);
    add.solid_effective_radius = d1(v.solid_effective_radius, ns0);
    add.solid_radius = d1(v.solid_radius, ns0);
    add.solid_inverse_mass = d1(v.solid_inverse_mass, ns0);
    add.solid_material = i1(v.solid_material, ns0);
    add.solid_cluster = i1(v.solid_cluster, ns0);
    add.solid_clump = i1(v.solid_clump, ns0);
    add.solid_is_dummy = i1(v.solid_is_dummy, ns0);
    check(demsph_append(engine, &cur, &add), "add");
    ++engineEpoch;
}

void dataBase::addFluid(std::vector<double3> p, double3 velocity, double smoothLength, double density,
                        double soundSpeed, double kinematicViscosity)
{
    APPEND_WHILE_RUNNING(scene.addFluid(p, velocity, smoothLength, density, soundSpeed, kinematicViscosity))
}

void dataBase::addDummyParticleWall(std::vector<double3> p, double spacing)
{
    APPEND_WHILE_RUNNING(scene.addDummyParticleWall(p, spacing))
}

void dataBase::addSolid(std::vector<double3> p, double3 velocity, double radius, double density, int materialID)
{
    APPEND_WHILE_RUNNING(scene.addSolid(p, velocity, radius, density, materialID))
}

void dataBase::addInfiniteWall(double3 p, double3 normal, int materialID)
{
    scene.started = running();
    report(scene.addInfiniteWall(p, normal, materialID));
}

void dataBase::addCylinderWall(double3 p, double3 axis, double3 angularVelocity, double radius, int materialID)
{
    scene.started = running();
    report(scene.addCylinderWall(p, axis, angularVelocity, radius, materialID));
}

void dataBase::addCluster(std::vector<double3> p, std::vector<double> radius, std::vector<double> density,
                          double3 velocity, int materialID)
{
    APPEND_WHILE_RUNNING(scene.addCluster(p, radius, density, velocity, materialID))
}

void dataBase::addClump(std::vector<double3> p, std::vector<double> radius, double3 centroidPosition,
                        double3 velocity, double3 angularVelocity, double mass, symMatrix inertiaTensor,
                        int materialID)
{
    REFUSE_WHILE_RUNNING("clumps")
    report(scene.addClump(p, radius, centroidPosition, velocity, angularVelocity, mass, inertiaTensor, materialID));
}
#undef REFUSE_WHILE_RUNNING
#undef APPEND_WHILE_RUNNING

// core/dataBase.cpp:179-195
void dataBase::addExternalForce(int index, double3 force)
{
    if (index < 0 || index >= scene.hos.solids.points.num) {
        std::cout << "Error: the index of the solid particle is out of range when adding external force." << std::endl;
        return;
    }
    if (!running()) {
        std::cout << "Error: external forces can only be added after the simulation starts." << std::endl;
        return;
    }
    const double f[3] = {force.x, force.y, force.z};
    check(demsph_add_external_force(engine, index, f), "addExternalForce");
}

// core/dataBase.cpp:197-224
void dataBase::addGlobalDamping(int index, double C_d)
{
    if (index < 0 || index >= scene.hos.solids.points.num) {
        std::cout << "Error: the index of the solid particle is out of range when adding global damping." << std::endl;
        return;
    }
    if (!running()) {
        std::cout << "Error: global damping can only be added after the simulation starts." << std::endl;
        return;
    }
    check(demsph_add_global_damping(engine, index, C_d), "addGlobalDamping");
}

// ---- host copies (core/dataBase.h:190-204) ----
const HostSolid& dataBase::getHostSolidData()
{
    if (engine && simPara.iStep >= 1) downloadSolids();
    return scene.hos.solids;
}

const HostFluid& dataBase::getHostFluidData()
{
    if (engine && simPara.iStep >= 1) downloadFluids();
    return scene.hos.fluids;
}

namespace {
void unpack3(const std::vector<double>& flat, std::vector<double3>& out)
{
    out.resize(flat.size() / 3);
    for (size_t i = 0; i < out.size(); ++i) out[i] = make_double3(flat[3 * i], flat[3 * i + 1], flat[3 * i + 2]);
}
}  // namespace

// solid::uploadState (core/deviceStructs.h:287-297)
void dataBase::downloadSolids()
{
    HostSolid& s = scene.hos.solids;
    const size_t n = (size_t)s.points.num;
    if (n == 0) return;
    std::vector<double> p(3 * n), v(3 * n), a(3 * n), nn(3 * n), t(3 * n), w(3 * n);
    check(demsph_download_solids(engine, p.data(), v.data(), a.data(), nn.data(), t.data(), w.data()),
          "getHostSolidData");
    unpack3(p, s.points.position);
    unpack3(v, s.dyn.velocities);
    unpack3(a, s.dyn.accelerations);
    unpack3(nn, s.normal);
    unpack3(t, s.torques);
    unpack3(w, s.angularVelocities);
}

// fluid::uploadState (core/deviceStructs.h:199-205)
void dataBase::downloadFluids()
{
    HostFluid& f = scene.hos.fluids;
    const size_t n = (size_t)f.points.num;
    if (n == 0) return;
    std::vector<double> p(3 * n), v(3 * n), a(3 * n);
    f.dRho.resize(n);
    check(demsph_download_fluids(engine, p.data(), v.data(), a.data(), f.dRho.data()), "getHostFluidData");
    unpack3(p, f.points.position);
    unpack3(v, f.dyn.velocities);
    unpack3(a, f.dyn.accelerations);
}

// interactionBase::upload of fluid2Solid (core/deviceStructs.h:483-520)
void dataBase::downloadFluidSolidPairs()
{
    HostInteractionBase& fs = scene.hos.fluid2Solid;
    const int nf = scene.hos.fluids.points.num;
    if (nf == 0) {
        fs.num = 0;
        return;
    }
    std::vector<int> prefix(nf);
    check(demsph_export_fluid_solid_pairs(engine, prefix.data(), nullptr, nullptr, nullptr, 0), "fluid2Solid");
    const long long m = prefix[nf - 1];
    fs.objectPointed.resize(m);
    fs.objectPointing.resize(m);
    std::vector<double> f(3 * m);
    check(demsph_export_fluid_solid_pairs(engine, prefix.data(), fs.objectPointed.data(), fs.objectPointing.data(),
                                          f.data(), m),
          "fluid2Solid");
    unpack3(f, fs.force);
    fs.num = (int)m;
}

// ---- engine life cycle: buildDeviceData + initialize (core/dataBase.cpp:434-449,
// core/solverBase.cpp:13-44) ----
void dataBase::buildEngine()
{
    ++engineEpoch;
    releaseEngine();
    demsph_scene v;
    scene.view(&v);
    demsph_options o{};
    o.device = deviceIndex;
    o.debug = keepPairForces ? 1 : 0;
    int st = demsph_create(&v, &o, &engine);
    if (st != DEMSPH_OK) {
        engine = nullptr;
        throw std::runtime_error(std::string("buildDeviceData: ") + demsph_status_string(st));
    }
    check(demsph_initialize(engine), "initialize");
}

void dataBase::releaseEngine()
{
    if (engine) demsph_destroy(engine);
    engine = nullptr;
}
