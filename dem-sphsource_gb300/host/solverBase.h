// class solverBase of the host API (core/solverBase.h:1-47,
// core/solverBase.cpp:3-333 in the reference): the time loop a case driver
// runs with solve(), its three hooks and the VTU frame writers.
//
// The loop keeps the reference's schedule: initialise (frame 0), then for
// iStep = 1 .. numSteps one update() - neighbour search, the solid half-step
// before contact, the fluid step every `gap` steps, the contact phase, the
// driver's handleDataAfterCalculateContact(), the solid half-step after
// contact - and a frame (outputData()) every frameInterval steps.
//
// On the GPU the steps between two frames run as one demsph_update() call
// (replayed CUDA graphs, no host round trip per step) whenever the driver
// overrides neither update() nor handleDataAfterCalculateContact(); a driver
// that overrides either gets the five step functions called one by one, with
// its hook in between, exactly as in the reference.
#pragma once
#include <string>

#include "dataBase.h"

class DEMSPH_API solverBase : public dataBase {
public:
    solverBase() : dataBase() {}
    ~solverBase() override {}

    void solve();

protected:
    void setProblemName(const std::string& name) { dir = name + "Output"; }

    // Frame files <problem>Output/{fluid,solid,fluid2Solid}_NNNN.vtu (ASCII VTK
    // unstructured grids of vertices, the reference's names and fields).
    void outputFluidVTU();
    void outputSolidVTU();
    void outputFluid2SolidVTU();

    virtual void conditionInitialize() {}
    virtual void outputData() {}
    virtual void handleDataAfterCalculateContact() { hookIsDefault = true; }

private:
    std::string dir = "problem";
    bool hookIsDefault{false};     // set by the default hook when it runs
    bool updateIsDefault{false};   // set by the default update() when it runs
    bool batched{false};           // steps between frames go to demsph_update
    bool wantsPairForces{false};   // outputFluid2SolidVTU was called at frame 0

    void initialize();
    virtual void update();
    void frame();
};
