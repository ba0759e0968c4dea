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
    ~solverBase() override { closeFrames(); }

    void solve();

protected:
    void setProblemName(const std::string& name) { dir = name + "Output"; }

    // Frame files <problem>Output/{fluid,solid,fluid2Solid}_NNNN.vtu (VTK
    // unstructured grids of vertices, the reference's names and fields):
    // ASCII written on this thread as in the reference, or - after
    // setBinaryOutput(true) - binary VTU packed on the GPU and written by a
    // background thread while the steps go on (demsph_frame_writer).
    void outputFluidVTU();
    void outputSolidVTU();
    void outputFluid2SolidVTU();
    void setBinaryOutput(bool on) { binaryOutput = on; }

    virtual void conditionInitialize() {}
    virtual void outputData() {}
    virtual void handleDataAfterCalculateContact() { hookIsDefault = true; }

private:
    std::string dir = "problem";
    bool hookIsDefault{false};     // set by the default hook when it runs
    bool updateIsDefault{false};   // set by the default update() when it runs
    bool batched{false};           // steps between frames go to demsph_update
    bool wantsPairForces{false};   // outputFluid2SolidVTU was called at frame 0
    bool binaryOutput{false};      // frames through the binary writer
    demsph_frame_writer* frames{nullptr};
    int framesEpoch{-1};           // the engine the writer was opened for

    bool binaryFrame(int kind);    // true: the frame went to the binary writer
    void closeFrames();

    void initialize();
    virtual void update();
    void frame();
};
