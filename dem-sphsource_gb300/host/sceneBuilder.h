// SceneBuilder: the setup half of the reference's class dataBase
// (core/dataBase.h:33-219, core/dataBase.cpp:3-177), with the same argument
// meanings, derived quantities and validation, writing into HostData.
//
// dataBase (dataBase.h) and the C ABI builder (demsph_builder_*) both sit on
// this class, so a scene built by a C++ case driver and one built through the
// C ABI (tests, benchmarks, other languages) are the same arrays.  Validation
// failures return a status and record the reference's message instead of
// printing; dataBase prints it, as the reference does.
#pragma once
#include <string>
#include <vector>
#include "hostStructs.h"
#include "../../include/demsph_gb300.h"

namespace demsph {

struct SimulationSettings {
    double maximumTime{1.};
    double timeStep{1.};
    int numFrames{1};
    int fluidIntegrateGap{1};
    double3 domainOrigin{make_double3(0, 0, 0)};
    double3 domainSize{make_double3(1, 1, 1)};
    double3 gravity{make_double3(0, 0, -9.81)};
};

class SceneBuilder {
public:
    explicit SceneBuilder(int nMaterial = 10) { hos.contactModels = HostSolidContactModel(nMaterial); }

    HostData hos;
    SimulationSettings sim;
    bool started{false};       // simulation running: some setters refuse (dataBase.h:45-79)
    std::string lastError;

    int setDomain(double3 origin, double3 size);
    int setGravity(double3 g);
    int setTimeStep(double dt);
    int setMaximumTime(double t);
    int setNumFrames(int n);
    int setFluidIntegrateGap(int gap);
    int setHertzian(int mi, int mj, double E, double G, double res, double krks, double ktks, double mus,
                    double mur, double mut);
    int setLinear(int mi, int mj, double kn, double ks, double kr, double kt, double dn, double ds, double dr,
                  double dt, double mus, double mur, double mut);
    int setBonded(int mi, int mj, double E, double knks, double gamma, double sigma, double C, double mu);

    int addFluid(const std::vector<double3>& p, double3 v, double smoothLength, double density, double soundSpeed,
                 double kinematicViscosity);
    int addDummyParticleWall(const std::vector<double3>& p, double spacing);
    int addSolid(const std::vector<double3>& p, double3 v, double radius, double density, int materialID);
    int addInfiniteWall(double3 p, double3 normal, int materialID);
    int addCylinderWall(double3 p, double3 axis, double3 angularVelocity, double radius, int materialID);
    int addCluster(const std::vector<double3>& p, const std::vector<double>& radius,
                   const std::vector<double>& density, double3 v, int materialID);
    int addClump(const std::vector<double3>& p, const std::vector<double>& radius, double3 centroid, double3 v,
                 double3 angularVelocity, double mass, symMatrix inertia, int materialID);

    // Points the C view at this builder's arrays (valid until the next change).
    void view(demsph_scene* s);

private:
    int fail(const char* msg)
    {
        lastError = msg;
        return DEMSPH_ERR_ARGUMENT;
    }
    void appendSolids(const HostSolid& s);
    std::vector<double> hertzFlat_, linearFlat_, bondedFlat_;
};

}  // namespace demsph
