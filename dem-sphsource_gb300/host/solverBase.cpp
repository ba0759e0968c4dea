// class solverBase: see solverBase.h.
#include "solverBase.h"

#include <filesystem>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>

namespace {

// ASCII VTK unstructured grid of N vertices with point data.
class VertexFile {
public:
    VertexFile(const std::string& dir, const char* stem, int frame, double time, int step, int n,
               const char* scalars)
        : n_(n)
    {
        std::filesystem::create_directories(dir);
        std::ostringstream name;
        name << dir << "/" << stem << "_" << std::setw(4) << std::setfill('0') << frame << ".vtu";
        out_.open(name.str());
        if (!out_) throw std::runtime_error("Cannot open " + name.str());
        out_ << std::fixed << std::setprecision(10);
        out_ << "<?xml version=\"1.0\"?>\n"
             << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n"
             << "  <UnstructuredGrid>\n"
             << "    <FieldData>\n"
             << "      <DataArray type=\"Float32\" Name=\"TIME\"  NumberOfTuples=\"1\" format=\"ascii\"> " << time
             << " </DataArray>\n"
             << "      <DataArray type=\"Int32\"   Name=\"STEP\"  NumberOfTuples=\"1\" format=\"ascii\"> " << step
             << " </DataArray>\n"
             << "    </FieldData>\n"
             << "    <Piece NumberOfPoints=\"" << n << "\" NumberOfCells=\"" << n << "\">\n";
        scalars_ = scalars;
    }

    template <class F>
    void points(F at)
    {
        out_ << "      <Points>\n        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"ascii\">\n";
        for (int i = 0; i < n_; ++i) {
            const double3 p = at(i);
            out_ << ' ' << p.x << ' ' << p.y << ' ' << p.z;
        }
        out_ << "\n        </DataArray>\n      </Points>\n      <Cells>\n"
             << "        <DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">\n";
        for (int i = 0; i < n_; ++i) out_ << ' ' << i;
        out_ << "\n        </DataArray>\n        <DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">\n";
        for (int i = 1; i <= n_; ++i) out_ << ' ' << i;
        out_ << "\n        </DataArray>\n        <DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n";
        for (int i = 0; i < n_; ++i) out_ << " 1";  // VTK_VERTEX
        out_ << "\n        </DataArray>\n      </Cells>\n      <PointData Scalars=\"" << scalars_ << "\">\n";
    }

    template <class F>
    void scalar(const char* type, const char* name, F at)
    {
        out_ << "        <DataArray type=\"" << type << "\" Name=\"" << name << "\" format=\"ascii\">\n";
        for (int i = 0; i < n_; ++i) out_ << ' ' << at(i);
        out_ << "\n        </DataArray>\n";
    }

    template <class F>
    void vector(const char* name, F at)
    {
        out_ << "        <DataArray type=\"Float32\" Name=\"" << name << "\" NumberOfComponents=\"3\" format=\"ascii\">\n";
        for (int i = 0; i < n_; ++i) {
            const double3 v = at(i);
            out_ << ' ' << v.x << ' ' << v.y << ' ' << v.z;
        }
        out_ << "\n        </DataArray>\n";
    }

    ~VertexFile() { out_ << "      </PointData>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n"; }

private:
    std::ofstream out_;
    int n_;
    std::string scalars_;
};

}  // namespace

// core/solverBase.cpp:3-11
void solverBase::solve()
{
    initialize();
    while (simPara.iStep <= simPara.numSteps) {
        if (batched) {
            // all steps up to the next frame (or the end) in one call
            const int fi = simPara.frameInterval;
            const int nextFrame = ((simPara.iStep + fi - 1) / fi) * fi;
            const int last = std::min(nextFrame, simPara.numSteps);
            const int n = last - simPara.iStep + 1;
            check(demsph_update(engine, simPara.timeStep, simPara.iStep, n, scene.sim.fluidIntegrateGap, 1),
                  "update");
            simPara.iStep = last;
            if (simPara.iStep % fi == 0) frame();
        } else {
            updateIsDefault = false;
            hookIsDefault = false;
            update();
            // after the first step, batch if neither update() nor the hook is the driver's
            batched = updateIsDefault && hookIsDefault;
        }
        simPara.iStep++;
    }
    check(demsph_synchronize(engine), "solve");
    if (frames) check(demsph_frame_writer_flush(frames), "frame files");
}

// core/solverBase.cpp:13-44
void solverBase::initialize()
{
    std::cout << "Initializing..." << std::endl;
    scene.hos.contactModels = HostSolidContactModel(10);
    conditionInitialize();

    std::cout << "Using GPU Device " << deviceIndex << std::endl;
    simPara.numSteps = int(simPara.maximumTime / simPara.timeStep) + 1;
    simPara.frameInterval = simPara.numSteps / simPara.numFrames;
    if (simPara.frameInterval < 1) simPara.frameInterval = 1;
    simPara.iStep = 0;
    simPara.iFrame = 0;

    // buildDeviceData, neighborSearch(0, 1), addBondData, setSolidNormal
    buildEngine();
    downloadSolids();  // the host copy now holds the wall normals, as after setSolidNormal
    removeVtuFiles(dir);
    removeDatFiles(dir);
    outputData();
    if (wantsPairForces && !keepPairForces) {
        // the driver writes fluid2Solid frames: rebuild once, keeping per-pair coupling forces
        keepPairForces = true;
        closeFrames();  // the writer belongs to the engine being replaced
        buildEngine();
    }
    std::cout << "Initialization completed." << std::endl;
    simPara.iStep++;
}

// core/solverBase.cpp:47-67
void solverBase::update()
{
    updateIsDefault = true;
    const double dt = simPara.timeStep;
    const int gap = scene.sim.fluidIntegrateGap;
    check(demsph_neighbor_search(engine, simPara.iStep, gap), "neighborSearch");
    check(demsph_solid_integrate_before_contact(engine, dt), "solidIntegrateBeforeContact");
    check(demsph_fluid_integrate(engine, dt, simPara.iStep, gap), "fluidIntegrate");
    check(demsph_solid_contact_after_fluid_integrate(engine, dt), "calSolidContactAfterFluidIntegrate");
    handleDataAfterCalculateContact();
    check(demsph_solid_integrate_after_contact(engine, dt), "solidIntegrateAfterContact");
    if (simPara.iStep % simPara.frameInterval == 0) frame();
}

void solverBase::frame()
{
    simPara.iFrame++;
    std::cout << "Frame " << simPara.iFrame << " at time " << simPara.iStep * simPara.timeStep << std::endl;
    outputData();
}

// Frames of a kind through the binary writer, opened on first use for the
// current engine.
bool solverBase::binaryFrame(int kind)
{
    if (!binaryOutput || !engine) return false;
    if (frames && framesEpoch != engineEpoch) closeFrames();  // particles were added: new counts
    if (!frames) {
        framesEpoch = engineEpoch;
        demsph_scene v;
        scene.view(&v);
        check(demsph_frame_writer_open(engine, &v, dir.c_str(), &frames), "frame files");
    }
    check(demsph_frame_writer_write(frames, kind, simPara.iFrame, simPara.iStep, getTime()), "frame files");
    return true;
}

void solverBase::closeFrames()
{
    if (!frames) return;
    const int st = demsph_frame_writer_close(frames);
    frames = nullptr;
    if (st != DEMSPH_OK) std::cerr << "frame files: " << demsph_last_error(engine) << std::endl;
}

// core/solverBase.cpp:69-171
void solverBase::outputFluidVTU()
{
    if (binaryFrame(DEMSPH_FRAME_FLUID)) return;
    if (simPara.iFrame > 0) downloadFluids();
    const HostFluid& f = scene.hos.fluids;
    VertexFile v(dir, "fluid", simPara.iFrame, getTime(), simPara.iStep, f.points.num, "smooth length");
    v.points([&](int i) { return f.points.position[i]; });
    v.scalar("Float32", "smooth length", [&](int i) { return f.points.effectiveRadii[i]; });
    v.vector("velocity", [&](int i) { return f.dyn.velocities[i]; });
    v.scalar("Float32", "density", [&](int i) { return f.rho0[i] + f.dRho[i]; });
    v.scalar("Float32", "pressure", [&](int i) { return f.dRho[i] * f.c[i] * f.c[i]; });
}

// core/solverBase.cpp:172-257
void solverBase::outputSolidVTU()
{
    if (binaryFrame(DEMSPH_FRAME_SOLID)) return;
    if (simPara.iFrame > 0) downloadSolids();
    const HostSolid& s = scene.hos.solids;
    VertexFile v(dir, "solid", simPara.iFrame, getTime(), simPara.iStep, s.points.num, "radius");
    v.points([&](int i) { return s.points.position[i]; });
    v.scalar("Float32", "radius", [&](int i) { return s.radius[i]; });
    v.scalar("Int32", "clusterID", [&](int i) { return s.clusterID[i]; });
    v.scalar("Int32", "clumpID", [&](int i) { return s.clumpID[i]; });
    v.vector("velocity", [&](int i) { return s.dyn.velocities[i]; });
    v.vector("angularVelocity", [&](int i) { return s.angularVelocities[i]; });
    v.vector("normal", [&](int i) { return s.normal[i]; });
}

// core/solverBase.cpp:259-333: one vertex per fluid-solid pair at the
// midpoint of the two particles, with the pair's coupling force.
void solverBase::outputFluid2SolidVTU()
{
    if (simPara.iFrame == 0) wantsPairForces = true;
    // frame 0 holds no pairs (the reference's host list is empty before the
    // first step): that file is the ASCII one
    if (simPara.iFrame > 0 && binaryFrame(DEMSPH_FRAME_FLUID2SOLID)) return;
    if (simPara.iFrame > 0) {
        downloadSolids();
        downloadFluids();
        downloadFluidSolidPairs();
    }
    const HostInteractionBase& fs = scene.hos.fluid2Solid;
    const HostFluid& f = scene.hos.fluids;
    const HostSolid& s = scene.hos.solids;
    const int n = simPara.iFrame > 0 ? fs.num : 0;
    VertexFile v(dir, "fluid2Solid", simPara.iFrame, getTime(), simPara.iStep, n, "force");
    v.points([&](int i) {
        return 0.5 * (f.points.position[fs.objectPointed[i]] + s.points.position[fs.objectPointing[i]]);
    });
    v.vector("force", [&](int i) { return fs.force[i]; });
}
