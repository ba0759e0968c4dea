// A small dam break written against the host API exactly as a case driver of
// the reference is (driver/cases/damBreak.cpp): a water column, three layers
// of dummy wall particles, a floor wall and a clump of spheres in the flow.
//
//   tinyDamBreak <output-name> [staged] [binary] [append]
//
// With "staged" the driver overrides handleDataAfterCalculateContact(), which
// makes solverBase call the five step functions one by one; without it the
// steps between two frames run as one batched call.  Both must write the
// same frames.  "binary" writes the frames as binary VTU from the background
// writer; "append" adds a block of fluid and a bonded cluster at frame 2
// (dataBase::addFluid / addCluster while the simulation runs).
#include <cstring>

#include "solverBase.h"

class tinyDamBreak : public solverBase {
public:
    tinyDamBreak(const char* name, bool staged, bool binary, bool append)
        : name_(name), staged_(staged), binary_(binary), append_(append)
    {
    }

    double particle_spacing = 0.02;
    double particle_radius = 0.5 * particle_spacing;
    double E = 0.3e9;

    void conditionInitialize() override
    {
        setProblemName(name_);
        setBinaryOutput(binary_);
        const double s = particle_spacing;
        setDomain(make_double3(-3. * s, -3. * s, -3. * s), make_double3(0.4 + 6. * s, 0.12 + 6. * s, 0.2 + 6. * s));
        std::vector<double3> fp = getRegularPackedPoints(make_double3(0, 0, 0), make_double3(0.12, 0.12, 0.1), s);
        addFluid(fp, make_double3(0, 0, 0), 1.3 * s, 1000., 20., 1.e-6);
        std::vector<double3> w0 = getRegularPackedPoints(make_double3(-3 * s, -3 * s, -3 * s),
                                                         make_double3(0.4 + 6 * s, 0.12 + 6 * s, 0.2 + 6 * s), s);
        std::vector<double3> w1;
        for (const auto& p : w0)
            if (p.x < 0 || p.y < 0 || p.z < 0 || p.x > 0.4 || p.y > 0.12) w1.push_back(p);
        addDummyParticleWall(w1, 0.5 * s);
        addInfiniteWall(make_double3(0.2, 0.06, 0), make_double3(0, 0, 1), 0);
        setHertzianContactModel(0, 1, E, 0.3 * E, 0.9, 0, 0, 0.35, 0, 0);
        setHertzianContactModel(1, 1, 0.5 * E, 0.15 * E, 0.9, 0, 0, 0.45, 0, 0);
        const double3 cube = make_double3(0.04, 0.04, 0.04);
        std::vector<double3> sp = getRegularPackedPoints(make_double3(0.25, 0.04, 0.0), cube, 2 * particle_radius);
        std::vector<double> rad(sp.size(), particle_radius);
        const double density = 800, mass = density * cube.x * cube.y * cube.z;
        symMatrix inertia = make_symMatrix(mass / 12. * (cube.y * cube.y + cube.z * cube.z),
                                           mass / 12. * (cube.x * cube.x + cube.z * cube.z),
                                           mass / 12. * (cube.x * cube.x + cube.y * cube.y), 0., 0., 0.);
        addClump(sp, rad, make_double3(0.27, 0.06, 0.02), make_double3(0, 0, 0), make_double3(0, 0, 0), mass,
                 inertia, 1);
        const double k = 0.5 * E * pi() * particle_radius;
        const double mij = 8 * particle_radius * particle_radius * particle_radius * density;
        const double dt = 0.2 * sqrt(mij / k);
        const double dt_f = 0.6 * 1.3 * s / (22. * sqrt(0.4 * 9.8));
        int gap = int(dt_f / dt);
        if (gap < 1) gap = 1;
        setSimulationParameterTimeStep(dt);
        setFluidIntegrateGap(gap);
        setSimulationParameterMaximumTime(200.5 * dt);
        setSimulationParameterNumFrames(4);
    }

    void handleDataAfterCalculateContact() override
    {
        if (!staged_) solverBase::handleDataAfterCalculateContact();
    }

    void outputData() override
    {
        outputFluidVTU();
        outputSolidVTU();
        if (append_ && ++frames_ == 3) {  // at frame 2: particles added while the simulation runs
            const double s = particle_spacing;
            addFluid(getRegularPackedPoints(make_double3(0.3, 0.02, 0.1), make_double3(0.06, 0.06, 0.06), s),
                     make_double3(0, 0, 0), 1.3 * s, 1000., 20., 1.e-6);
            std::vector<double3> cp = getRegularPackedPoints(make_double3(0.15, 0.04, 0.0),
                                                             make_double3(0.04, 0.04, 0.04), 2 * particle_radius);
            addCluster(cp, std::vector<double>(cp.size(), particle_radius), std::vector<double>(cp.size(), 800.),
                       make_double3(0, 0, 0), 1);
        }
    }

private:
    const char* name_;
    bool staged_, binary_, append_;
    int frames_ = 0;
};

int main(int argc, char** argv)
{
    bool staged = false, binary = false, append = false;
    for (int k = 2; k < argc; ++k) {
        staged |= std::strcmp(argv[k], "staged") == 0;
        binary |= std::strcmp(argv[k], "binary") == 0;
        append |= std::strcmp(argv[k], "append") == 0;
    }
    tinyDamBreak problem(argc > 1 ? argv[1] : "tinyDamBreak", staged, binary, append);
    problem.solve();
    return 0;
}
