// class dataBase of the host API: the set-up and run-time calls a case driver
// makes, with the reference's names, arguments and messages
// (core/dataBase.h:33-219, core/dataBase.cpp:3-449).
//
// A driver written against the reference derives from solverBase (which
// derives from this class) and compiles unchanged against these headers,
// linking libdemsph_gb300.so.  Underneath, the set-up calls fill a
// demsph::SceneBuilder (the same arrays the C ABI builder fills) and, once the
// simulation has started, the run-time calls go to the GB300 engine through
// the C ABI of include/demsph_gb300.h.  The engine holds all device memory;
// this class holds only host arrays and the engine handle.
//
// Differences from the reference, all at run time (after initialisation):
// adding particles or changing the domain while the simulation runs is
// refused with a message (the engine's grid and lists are sized at start),
// and a CUDA or capacity failure throws std::runtime_error with the engine's
// message instead of exiting the process.
#pragma once
#include <iostream>
#include <string>
#include <vector>

#include "fileEditingTool.h"
#include "generatePoints.h"
#include "hostStructs.h"
#include "sceneBuilder.h"
#include "../../include/demsph_gb300.h"

class DEMSPH_API dataBase {
public:
    dataBase();
    virtual ~dataBase();
    dataBase(const dataBase&) = delete;
    dataBase& operator=(const dataBase&) = delete;

protected:
    void setGPUParameterDeviceIndex(int index);
    void setSimulationParameterMaximumTime(double t);
    void setSimulationParameterNumFrames(int n);
    void setSimulationParameterTimeStep(double dt);
    void setFluidIntegrateGap(int gap);
    void setDomain(double3 origin, double3 size);
    void setGravity(double3 g);
    void setHertzianContactModel(int mat_i, int mat_j, double E, double G, double res, double k_r_k_s,
                                 double k_t_k_s, double mu_s, double mu_r, double mu_t);
    void setLinearContactModel(int mat_i, int mat_j, double k_n, double k_s, double k_r, double k_t, double d_n,
                               double d_s, double d_r, double d_t, double mu_s, double mu_r, double mu_t);
    void setBondedContactModel(int mat_i, int mat_j, double E, double k_n_k_s, double gamma, double sigma_s,
                               double C, double mu);
    void setClumpVelocity(int index, double3 velocity);

    void addFluid(std::vector<double3> p, double3 velocity, double smoothLength, double density, double soundSpeed,
                  double kinematicViscosity);
    void addDummyParticleWall(std::vector<double3> p, double spacing);
    void addSolid(std::vector<double3> p, double3 velocity, double radius, double density, int materialID);
    void addInfiniteWall(double3 p, double3 normal, int materialID);
    void addCylinderWall(double3 p, double3 axis, double3 angularVelocity, double radius, int materialID);
    void addCluster(std::vector<double3> p, std::vector<double> radius, std::vector<double> density,
                    double3 velocity, int materialID);
    void addClump(std::vector<double3> p, std::vector<double> radius, double3 centroidPosition, double3 velocity,
                  double3 angularVelocity, double mass, symMatrix inertiaTensor, int materialID);
    void addExternalForce(int index, double3 force);
    void addGlobalDamping(int index, double C_d);

    double getTime() const { return simPara.iStep * simPara.timeStep; }
    // The host copy of the particle data; once the simulation has started it is
    // refreshed from the GPU first (uploadState in the reference).
    const HostSolid& getHostSolidData();
    const HostFluid& getHostFluidData();

private:
    struct simulationParameter {
        double maximumTime;
        double timeStep;
        int numSteps;
        int iStep;
        int numFrames;
        int iFrame;
        int frameInterval;
    };

    demsph::SceneBuilder scene;   // host arrays (scene.hos) and settings
    demsph_engine* engine{nullptr};
    simulationParameter simPara;
    int deviceIndex{0};
    bool keepPairForces{false};   // per-pair coupling forces kept for fluid2Solid output
    int engineEpoch{0};           // counts engine changes (builds and run-time additions)

    // Prints the builder's message when a set-up call was refused.
    void report(int status);
    // Throws std::runtime_error with the engine's message on failure.
    void check(int status, const char* what);
    bool running() const { return engine != nullptr && simPara.iStep > 0; }
    // Engine life cycle (buildDeviceData + the device part of initialize).
    void buildEngine();
    void releaseEngine();
    void downloadSolids();
    void downloadFluids();
    void downloadFluidSolidPairs();
    // The particles the host arrays gained beyond (nf0, ns0) go to the running
    // engine (addFluidData / addSolidData after the start).
    void appendRunning(int nf0, int ns0);

    friend class solverBase;
};
