// Engine life cycle, step schedule, CUDA-graph batching and overflow
// recovery - the step half of the C ABI in include/demsph_gb300.h.
//
// Step schedule (solverBase::update, core/solverBase.cpp:47-67):
//   neighborSearch -> solidIntegrateBeforeContact -> fluidIntegrate ->
//   calSolidContactAfterFluidIntegrate -> [driver hook] -> solidIntegrateAfterContact
// with the reference's cadences: fluid lists and the fluid step every `gap`
// DEM steps, Shepard re-initialisation at i % (5 gap) == 0 and at i == 1, the
// coupling force every DEM step.
//
// Buffers keep fixed roles inside a step (fluid state in set [0] between
// steps; set [1] holds the mid-step copy), except the solid contact list,
// whose two parities alternate every build (the previous list is the spring
// history).  A CUDA graph therefore captures one period of steps - a multiple
// of 2 and of 5 gap - and is replayed; steps that do not fill a whole period
// run uncaptured.
//
// Overflow: list kernels record an overflow in a status word and every later
// kernel returns at once, so a failed step leaves the state as it was after
// the previous step (re-hashing and re-ordering are idempotent).  The host
// grows the list and re-runs from the first incomplete step.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include <mutex>

#include "engine_impl.cuh"

namespace demsph {

bool overlapLaunches()
{
    static const bool on = [] {
        const char* v = std::getenv("DEMSPH_OVERLAP_LAUNCHES");
        return !(v && v[0] == '0');
    }();
    return on;
}

void freeOne(demsph_engine* e, void*& p)
{
    if (!p) return;
    auto it = std::find_if(e->owned.begin(), e->owned.end(), [&](const Allocation& a) { return a.p == p; });
    if (it != e->owned.end()) e->owned.erase(it);
    cudaFreeAsync(p, e->stream);
    p = nullptr;
}

void dropGraph(demsph_engine* e)
{
    for (const auto& g : e->graphs) cudaGraphExecDestroy(g.exec);
    e->graphs.clear();
    for (const auto& r : e->rounds) cudaGraphDestroy(r.graph);
    e->rounds.clear();
}

double* scratchDoubles(demsph_engine* e, size_t n, int slot)
{
    if (n > e->dscratchN[slot]) {
        void* p = e->dscratch[slot];
        freeOne(e, p);
        e->dscratch[slot] = dalloc<double>(n, e->owned, e->stream, false);
        e->dscratchN[slot] = n;
    }
    return e->dscratch[slot];
}

// Cell and double-float offset of an absolute FP64 position.  The cell is the
// reference's hashing cell int((p - min) / cs) (core/neighborSearch.h:44-49),
// which is the floor inside the domain; outside it the floor is kept (the
// stencil centre applies the truncation).
void splitPosition(const DeviceState& d, double3 p, int4& c, float4& h, float4& l)
{
    const double q[3] = {p.x, p.y, p.z};
    int ci[3];
    float hi[3], lo[3];
    for (int a = 0; a < 3; ++a) {
        const double u = (q[a] - d.minB[a]) / d.cs[a];
        const int k = u >= 0 ? (int)u : (int)std::floor(u);
        double o = q[a] - (d.minB[a] + (double)k * d.cs[a]);
        // A point on a cell boundary (a lattice of wall particles can put
        // some exactly there) gets the reference's cell from the rounded
        // quotient above, while the offset, rounded too, may fall just outside
        // [0, cs) and would move the point to the neighbouring cell at the next
        // hash: keep it inside (a shift of at most ~1e-14 of the cell size).
        if (u >= 0.0) o = std::min(std::max(o, 0.0), d.cs[a] * (1.0 - 0x1p-44));
        ci[a] = k;
        const dfl s = df_from_double(o);
        hi[a] = s.hi;
        lo[a] = s.lo;
    }
    c = make_int4(ci[0], ci[1], ci[2], 0);
    h.x = hi[0]; h.y = hi[1]; h.z = hi[2];
    l.x = lo[0]; l.y = lo[1]; l.z = lo[2];
}

int readStatus(demsph_engine* e, int* stepsDone)
{
    int st[2] = {0, 0};
    CK(cudaMemcpyAsync(&st[0], e->d.status, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemcpyAsync(&st[1], e->d.stepsDone, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    if (stepsDone) *stepsDone = st[1];
    return st[0];
}

}  // namespace demsph

using namespace demsph;

namespace {

inline double3 v3(const double* p, int i)
{
    return p ? make_double3(p[3 * i], p[3 * i + 1], p[3 * i + 2]) : make_double3(0, 0, 0);
}

// Freed engine memory stays in the device's stream-ordered pool for the next
// engine instead of going back to the driver at every synchronisation (a
// setting of this process's pool only).
void keepPoolMemory(int dev)
{
    static std::mutex m;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lock(m);
    if (std::find(done.begin(), done.end(), dev) != done.end()) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done.push_back(dev);
}

int checkDevice(demsph_engine* e, int dev)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return fail(e, DEMSPH_ERR_NO_DEVICE, "no CUDA device");
    if (dev < 0 || dev >= n) return fail(e, DEMSPH_ERR_ARGUMENT, "device index out of range");
    // two attributes, not cudaGetDeviceProperties (which queries them all: a
    // cost every engine creation of a server would pay)
    int major = 0, minor = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
        return fail(e, DEMSPH_ERR_NO_DEVICE, "cannot query device");
    if (major * 10 + minor != 103)
        return fail(e, DEMSPH_ERR_NO_DEVICE, "this library is built for sm_103a (GB300); the device is sm_" +
                                                 std::to_string(major * 10 + minor));
    return DEMSPH_OK;
}

void allocFluidLists(demsph_engine* e)
{
    DeviceState& d = e->d;
    // in tile mode the fluid list exists only for exports (made on demand)
    if (!d.fluidTiles) d.ff = dalloc<unsigned>((size_t)d.kff * d.nf, e->owned, e->stream, false);
    d.fs = dalloc<int>((size_t)d.kfs * d.nf, e->owned, e->stream, false);
    if (e->debug & 1) d.fsPairForce = dalloc<float4>((size_t)d.kfs * d.nf, e->owned, e->stream);
}

void allocFluidCandidates(demsph_engine* e)
{
    DeviceState& d = e->d;
    d.fvc = dalloc<unsigned>((size_t)d.kvf * d.nf, e->owned, e->stream, false);
    d.fvsc = dalloc<int>((size_t)d.kvs * d.nf, e->owned, e->stream, false);
}

// Per-slot arrays of the contact rows (scap slots per row).
void allocContactLists(demsph_engine* e)
{
    DeviceState& d = e->d;
    const size_t c = (size_t)d.scap * std::max(1, d.nrow);
    d.rev = dalloc<int>(c, e->owned, e->stream);
    d.pF = dalloc<float4>(c, e->owned, e->stream);
    d.pT = dalloc<float4>(c, e->owned, e->stream);
    d.pTA = dalloc<float4>(c, e->owned, e->stream);
    d.revF = dalloc<float4>(c, e->owned, e->stream);
    d.revT = dalloc<float4>(c, e->owned, e->stream);
    for (int p = 0; p < 2; ++p) d.fwd[p] = dalloc<int>(c, e->owned, e->stream);
    for (int k = 0; k < 3; ++k) {
        d.springIn[k] = dalloc<float4>(c, e->owned, e->stream);
        for (int p = 0; p < 2; ++p) d.springOut[p][k] = dalloc<float4>(c, e->owned, e->stream);
    }
}

// Tile mode of the fluid lists and pair loops (sph_tiles.cu) is used when
// every fluid particle has the same parameters, the grid has at least three
// cells along every axis (the walk's cells are then distinct), every particle
// starts inside the domain (a particle outside it sends the lists to the
// reference's walk), the walk is not asked for (fluid_verlet_skin < 0), and
// DEMSPH_FLUID_TILES=1 is set in the environment (the list kernels measured
// faster, so they stay the default).
bool tileModeWanted(const demsph_scene* sc, const DeviceState& d, const demsph_options& o)
{
    const char* v = std::getenv("DEMSPH_FLUID_TILES");
    if (!(v && v[0] == '1') || o.fluid_verlet_skin < 0 || sc->n_fluid <= 0) return false;
    if (d.grid.gx < 3 || d.grid.gy < 3 || d.grid.gz < 3) return false;
    for (int i = 1; i < sc->n_fluid; ++i)
        if (sc->fluid_smoothing_length[i] != sc->fluid_smoothing_length[0] || sc->fluid_rho0[i] != sc->fluid_rho0[0] ||
            sc->fluid_sound_speed[i] != sc->fluid_sound_speed[0] || sc->fluid_nu[i] != sc->fluid_nu[0])
            return false;
    const int g[3] = {d.grid.gx, d.grid.gy, d.grid.gz};
    auto inside = [&](const double* p, int n) {
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) {
                const double u = (p[3 * i + a] - d.minB[a]) / d.cs[a];
                if (!(u >= 0.0) || (int)u >= g[a]) return false;
            }
        return true;
    };
    return inside(sc->fluid_position, sc->n_fluid) && inside(sc->solid_position, sc->n_solid);
}

// Bit words per particle from the initial fluid cells: room for the largest
// walk (with a margin for compression; more is added on overflow).
void sizeTiles(demsph_engine* e, const std::vector<int4>& cell)
{
    DeviceState& d = e->d;
    const GridDev& g = d.grid;
    std::vector<int> count((size_t)g.num, 0);
    for (const int4& c : cell) count[((size_t)c.z * g.gy + c.y) * g.gx + c.x]++;
    int most = 0;
    for (int z = 0; z < g.gz; ++z)
        for (int y = 0; y < g.gy; ++y)
            for (int x = 0; x < g.gx; ++x) {
                if (!count[((size_t)z * g.gy + y) * g.gx + x]) continue;
                int walk = 0;
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const int X = x + dx, Y = y + dy, Z = z + dz;
                            if (X < 0 || X >= g.gx || Y < 0 || Y >= g.gy || Z < 0 || Z >= g.gz) continue;
                            walk += count[((size_t)Z * g.gy + Y) * g.gx + X];
                        }
                most = std::max(most, walk);
            }
    d.kbits = (most + most / 4 + 31) / 32 + 1;
}

// ---- stage timing ----
struct StageTimer {
    demsph_engine* e;
    const char* tag;
    cudaEvent_t a = nullptr, b = nullptr;
    StageTimer(demsph_engine* eng, const char* t) : e(eng), tag(t)
    {
        if (!e->profiling) return;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        CK(cudaEventRecord(a, e->stream));
    }
    ~StageTimer()
    {
        if (!a) return;
        cudaEventRecord(b, e->stream);
        e->timed.push_back({tag, a, b});
    }
};
#define TIMED(tag) StageTimer _stage_timer(e, tag)

// ---- the five stages ----
// endView: the solids' integration has already opened this step (a fused
// pass): the search reads their end-of-step offsets from sphE/splE.
// detect false: the contact list is left to the contact stage's one launch
// (launchContactForces).
// beforeDetect: enqueued after the sorts and lists, before the contact
// detection (a fork to the side stream).
void stageNeighborSearch(demsph_engine* e, int iStep, int gap, bool endView = false, bool detect = true,
                         const std::function<void()>* beforeDetect = nullptr)
{
    e->keysAdvanced = false;  // this search's keys are the current ones until an integration rehashes
    const int npar = e->par ^ 1;  // the parity of the list this step builds
    DeviceState d = e->d;
    if (endView) {
        d.sph = d.sphE;
        d.spl = d.splE;
    }
    const cudaStream_t s = e->stream;
    const bool fluidStep = d.nf > 0 && (iStep % gap == 0);
    // solids that never move (walls of dummy particles, fixed spheres) are
    // hashed and sorted once, and again only after their positions are uploaded
    const bool solidsMove = e->nMassive > 0 || e->movingDummies > 0 || e->solidSortStale;
    const bool forceSort = e->forceWalk || e->solidSortStale;
    // Work needed only on some steps (sorting by cell, rebuilding candidates,
    // the walk) is launched every step and decided on the device from the
    // flags the previous step left (RunIf): the kernels return at once when
    // their work is not needed.  (Conditional graph nodes in place of these
    // launches measured slower on GB300, alone and with many scenes.)
    if (fluidStep) {
        // tile mode sorts the fluids by cell every fluid step (its tiles are
        // the reference's walk cells); frebuild, never cleared in tile mode,
        // also has the solids sorted on every fluid step
        TIMED("fluid_hash_reorder");
        launchFluidHash(d, e->forceWalk || d.fluidTiles, s);
        launchFluidReorder(d, e->forceWalk || d.fluidTiles, s);
    }
    if (solidsMove || e->forceWalk) {
        TIMED("solid_hash_sort");
        launchSolidHash(d, forceSort, fluidStep, npar, s);
        launchSolidSort(d, forceSort, fluidStep, npar, s);
        e->solidSortStale = false;
    }
    if (fluidStep) {
        if (d.fluidTiles) {
            // membership bits and solid partner lists of this step, on the tiles
            TIMED("fluid_lists");
            launchFluidTileLists(d, s);
        } else if (e->forceWalk) {
            TIMED("fluid_lists");
            launchFluidWalk(d, true, s);
        } else {
            {
                // the walk (once a fluid left the domain) or the candidate
                // rebuild: returns at once when neither is needed
                TIMED("fluid_candidates");
                launchFluidWalk(d, false, s);
            }
            TIMED("fluid_lists");
            launchFluidFilter(d, s);
        }
        if (e->nMassive > 0) {  // the coupling force moves only solids with mass
            TIMED("coupling_lists");
            launchCouplingLists(d, s);
        }
    }
    e->par = npar;
    e->walkOrder[e->par] = e->forceWalk;
    if (beforeDetect) (*beforeDetect)();
    if (!detect) return;
    TIMED("solid_contact_list");  // with the candidate rebuild when they are stale
    launchContactDetect(d, e->par, e->forceWalk, s);
}

void stageBefore(demsph_engine* e, double dt)
{
    TIMED("integrate_before");
    launchSolidIntegrate(e->d, dt, INTEGRATE_BEFORE, e->par, false, false, e->stream);
}

// countStep: the fluid stage ends the step (see fullStep) and its last pass
// counts it.
void stageFluid(demsph_engine* e, double dt, int iStep, int gap, bool countStep = false)
{
    DeviceState& d = e->d;
    if (d.nf <= 0) return;
    const cudaStream_t s = e->stream;
    const double dtf = dt * (double)gap;
    const bool fluidStep = iStep % gap == 0;
    if (iStep % (5 * gap) == 0 || iStep == 1) {
        TIMED("density_reinit");
        launchDensityReinit(d, iStep, s);
    }
    if (fluidStep) {
        TIMED("continuity");
        launchContinuityPass(d, 0, dtf, s);
    }
    if (e->nMassive > 0) {
        TIMED("coupling_force");
        launchCoupling(d, fluidStep ? 1 : 0, s);
    }
    if (d.fsPairForce) launchCouplingPairForces(d, fluidStep ? 1 : 0, d.fsPairForce, s);
    if (fluidStep) {
        {
            TIMED("momentum");
            launchMomentumPass(d, dtf, s);
        }
        TIMED("continuity");
        launchContinuityPass(d, 1, dtf, s, countStep);
    }
}

// withClumpForce: the clumps' pebble forces are summed here (the staged
// calls: the driver's hook runs between contact and integration); a whole
// step (fullStep) sums them inside the integration that follows instead.
// beforeForces: enqueued between the pair forces (with the bonds) and the
// per-solid sums (the join of a side-stream branch whose result only the
// sums read).
// integrate, countStep: the per-solid sums also run the solids' integration
// pass of that kind (see sumsIntegrate).
void stageContact(demsph_engine* e, double dt, bool withClumpForce = true,
                  const std::function<void()>* beforeForces = nullptr, int integrate = -1, bool countStep = false)
{
    DeviceState& d = e->d;
    {
        TIMED("pair_forces");  // with the bonds
        launchPairForces(d, e->par, (float)dt, e->stream);
    }
    if (beforeForces) (*beforeForces)();
    {
        TIMED("solid_forces");
        launchSolidForces(d, e->par, dt, e->stream, integrate, countStep);
    }
    if (d.nc > 0 && withClumpForce) {
        TIMED("clump_force");
        launchClumpForce(d, e->stream);
    }
}

// The solids the integration moves are exactly the contact rows (no clumps,
// no moving dummy particles): the per-solid sums can integrate them.
bool sumsIntegrate(const demsph_engine* e)
{
    const DeviceState& d = e->d;
    return e->foldIntegration && d.nc == 0 && d.nrow > 0 && d.nmove == d.nrow;
}

void stageAfter(demsph_engine* e, double dt, bool clumpForce = false, bool countStep = false)
{
    e->keysAdvanced = true;  // the rehash keeps the search's keys in skeySearch
    TIMED("integrate_after");
    launchSolidIntegrate(e->d, dt, INTEGRATE_AFTER, e->par, clumpForce, countStep, e->stream);
}

// One solverBase::update() without the driver's hook.  The clump force sum
// and the step count ride on the last integration (bit for bit what the
// staged calls compute).  opened: the solids' before-contact half of this
// step has run already (a step resumed after an overflow in its search).
void fullStep(demsph_engine* e, double dt, int iStep, int gap, bool opened = false)
{
    // a fluid step after whose fluid stage nothing runs (no solid is
    // integrated, touches another or is bonded, no clump) is counted by the
    // last continuity pass instead of a launch of its own
    const DeviceState& d = e->d;
    const bool countInFluid =
        d.nf > 0 && iStep % gap == 0 && d.nmove == 0 && d.nc == 0 && d.nb == 0 && d.nrow <= 0;
    stageNeighborSearch(e, iStep, gap, opened);
    if (!opened) stageBefore(e, dt);
    stageFluid(e, dt, iStep, gap, countInFluid);
    if (sumsIntegrate(e)) {
        stageContact(e, dt, false, nullptr, INTEGRATE_AFTER, !countInFluid);
        e->keysAdvanced = true;  // as stageAfter
        return;
    }
    stageContact(e, dt, false);
    stageAfter(e, dt, e->d.nc > 0, !countInFluid);
}

// `length` >= 2 whole steps of plain DEM (no fluid step among them) where
// each step but the last closes with the integration pass that also opens the
// next step.  The neighbour search that sits between the two halves in
// solverBase::update moves nothing and reads only the solids' end-of-step
// positions (which the pass leaves in sphE/splE); the before-contact half
// depends on nothing the search writes.  So the state after every step is
// bit for bit that of fullStep.  The solids no integration moves (dummy
// particles at rest) get their sphE/splE copy once, after the first search.
// Without bonds (a bond reads the contact list) the opened steps build their
// contact list in the contact stage, in the launch of the contact forces: the
// fluid stage of a plain DEM step (the coupling force) does not read it.
void fusedSteps(demsph_engine* e, double dt, int iStep, int length, int gap)
{
    DeviceState& d = e->d;
    const bool merge = e->mergeContacts && d.nb == 0 && d.nrow > 0;
    stageNeighborSearch(e, iStep, gap);
    const long long pebbles = std::count(e->moveKind.begin(), e->moveKind.end(), (unsigned char)0);
    if (d.ns - d.nmove - pebbles > 0) {
        CK(cudaMemcpyAsync(d.sphE, d.sph, sizeof(float4) * d.ns, cudaMemcpyDeviceToDevice, e->stream));
        CK(cudaMemcpyAsync(d.splE, d.spl, sizeof(float4) * d.ns, cudaMemcpyDeviceToDevice, e->stream));
    }
    stageBefore(e, dt);
    // the coupling force of an opened step reads the fluids and the solids as
    // the fused pass leaves them, and nothing the search writes: it runs on
    // the side stream beside the contact detection (and the coupling force
    // of a plain DEM step is all its fluid stage does)
    const bool branch = !merge && !e->profiling && e->nMassive > 0 && d.nf > 0 && d.ns > 0 && d.nrow > 0;
    const std::function<void()> fork = [&] {
        CK(cudaEventRecord(e->forkEv, e->stream));
        CK(cudaStreamWaitEvent(e->side, e->forkEv, 0));
        launchCoupling(d, 0, e->side);
        if (d.fsPairForce) launchCouplingPairForces(d, 0, d.fsPairForce, e->side);
        CK(cudaEventRecord(e->joinEv, e->side));
    };
    // the join: the per-solid sums (which read the coupling force) wait for
    // the branch; the pair forces and bonds before them do not
    const std::function<void()> join = [&] { CK(cudaStreamWaitEvent(e->stream, e->joinEv, 0)); };
    const bool fold = sumsIntegrate(e);
    bool forked = false;
    for (int k = 0; k < length; ++k) {
        if (!forked) stageFluid(e, dt, iStep + k, gap);
        const bool last = k == length - 1;
        bool integrated = false;
        if (k > 0 && merge) {
            TIMED("contact_forces");  // with the contact list of the step
            launchContactForces(d, e->par, (float)dt, e->stream);
        } else {
            // the sums close the step (the last) or close it and open the next
            integrated = fold;
            stageContact(e, dt, false, forked ? &join : nullptr,
                         fold ? (last ? INTEGRATE_AFTER : INTEGRATE_FUSED) : -1, true);
        }
        forked = false;
        if (last) {
            if (integrated) e->keysAdvanced = true;  // as stageAfter
            else stageAfter(e, dt, d.nc > 0, true);
            break;
        }
        if (!integrated) {
            TIMED("integrate_after");  // the closing half of this step and the opening half of the next
            launchSolidIntegrate(d, dt, INTEGRATE_FUSED, e->par, d.nc > 0, true, e->stream);
        }
        stageNeighborSearch(e, iStep + k + 1, gap, true, !merge, branch ? &fork : nullptr);
        forked = branch;
    }
}

// Grows whatever overflowed and clears the status.  e->par must be the parity
// of the last successful solid list build (the history the retry reads).
void grow(demsph_engine* e, int status)
{
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    if (status & (ST_FF_OVERFLOW | ST_FS_OVERFLOW)) {
        void* p = d.ff;
        freeOne(e, p);
        p = d.fs;
        freeOne(e, p);
        if (d.fsPairForce) {
            p = d.fsPairForce;
            freeOne(e, p);
            d.fsPairForce = nullptr;
        }
        if (status & ST_FF_OVERFLOW) d.kff *= 2;
        if (status & ST_FS_OVERFLOW) d.kfs *= 2;
        allocFluidLists(e);
    }
    if (status & (ST_SS_OVERFLOW | ST_VERLET_OVERFLOW)) {
        int need[2] = {0, 0};
        CK(cudaMemcpyAsync(need, d.need, sizeof(int) * 2, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        CK(cudaMemsetAsync(d.need, 0, sizeof(int) * 2, e->stream));
        const size_t nr = (size_t)std::max(1, d.nrow);
        if (status & ST_SS_OVERFLOW) {
            // keep the spring history (the last successful list and the springs
            // its contact phase left): slot k of row r is element k * nrow + r,
            // so the old slots are a prefix of the new
            const int keep = e->par;
            const size_t old = (size_t)d.scap * nr;
            int* keepFwd = d.fwd[keep];
            float4* keepSpring[3] = {d.springOut[keep][0], d.springOut[keep][1], d.springOut[keep][2]};
            d.fwd[keep] = nullptr;
            for (int k = 0; k < 3; ++k) d.springOut[keep][k] = nullptr;
            void* ptrs[] = {d.rev, d.pF, d.pT, d.pTA, d.revF, d.revT, d.fwd[keep ^ 1], d.springIn[0], d.springIn[1], d.springIn[2],
                            d.springOut[keep ^ 1][0], d.springOut[keep ^ 1][1], d.springOut[keep ^ 1][2]};
            for (void* p : ptrs) freeOne(e, p);
            d.scap = std::max(d.scap * 2, need[0] + need[0] / 2 + 1);
            allocContactLists(e);
            CK(cudaMemcpyAsync(d.fwd[keep], keepFwd, sizeof(int) * old, cudaMemcpyDeviceToDevice, e->stream));
            for (int k = 0; k < 3; ++k)
                CK(cudaMemcpyAsync(d.springOut[keep][k], keepSpring[k], sizeof(float4) * old,
                                   cudaMemcpyDeviceToDevice, e->stream));
            void* olds[] = {keepFwd, keepSpring[0], keepSpring[1], keepSpring[2]};
            for (void* p : olds) freeOne(e, p);
        }
        if (status & ST_VERLET_OVERFLOW) {
            void* p = d.vcand;
            freeOne(e, p);
            d.vcap = std::max(d.vcap * 2, need[1] + need[1] / 2 + 1);
            d.vcand = dalloc<int>((size_t)d.vcap * nr, e->owned, e->stream, false);
            CK(cudaMemsetAsync(d.rebuild, 0xff, 2 * sizeof(int), e->stream));  // rebuild on the retry
        }
    }
    if (status & ST_FVERLET_OVERFLOW) {
        int need[4] = {0, 0, 0, 0};
        CK(cudaMemcpyAsync(need, d.need, sizeof(int) * 4, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        CK(cudaMemsetAsync(d.need + 2, 0, sizeof(int) * 2, e->stream));
        void* p = d.fvc;
        freeOne(e, p);
        p = d.fvsc;
        freeOne(e, p);
        d.kvf = std::max(d.kvf, need[2] + need[2] / 2 + 1);
        d.kvs = std::max(d.kvs, need[3] + need[3] / 2 + 1);
        allocFluidCandidates(e);
        CK(cudaMemsetAsync(d.frebuild, 0xff, sizeof(int), e->stream));  // rebuild on the retry
    }
    if (status & ST_COUPLE_OVERFLOW) {
        int need = 0;
        CK(cudaMemcpyAsync(&need, d.coupStart + d.ns, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        void* p = d.coupList;
        freeOne(e, p);
        d.coupCap = (int)std::min<long long>(2000000000LL, (long long)(need * 1.5) + 1024);
        d.coupList = dalloc<int>(d.coupCap, e->owned, e->stream);
    }
    if (status & ST_FBITS_OVERFLOW) {
        int need = 0;
        CK(cudaMemcpyAsync(&need, d.need + 4, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        CK(cudaMemsetAsync(d.need + 4, 0, sizeof(int), e->stream));
        void* p = d.fbits;
        freeOne(e, p);
        d.kbits = std::max(2 * d.kbits, (need + 31) / 32 + 1);
        d.fbits = dalloc<unsigned>((size_t)d.kbits * d.nf, e->owned, e->stream, false);
    }
    if (status & ST_SPLIT_CONTACTS) e->mergeContacts = false;  // the lists come from the walk from now on
    if ((status & ST_MODE_CHANGE) && d.fluidTiles) {
        // a particle left the domain: the lists come from the reference's walk
        // (the list kernels) from now on
        d.fluidTiles = 0;
        if (!d.ff) d.ff = dalloc<unsigned>((size_t)d.kff * d.nf, e->owned, e->stream, false);
        if (!d.fvc) allocFluidCandidates(e);
    }
    if (status & ST_MODE_CHANGE) {
        // the abandoned step may have counted some particles into cells
        CK(cudaMemsetAsync(d.scellCount, 0, sizeof(int) * d.grid.num, e->stream));
        if (d.nf > 0) CK(cudaMemsetAsync(d.fcellCount, 0, sizeof(int) * d.grid.num, e->stream));
    }
    CK(cudaMemsetAsync(d.status, 0, sizeof(int), e->stream));
    dropGraph(e);
}

constexpr int ALL_OVERFLOWS = ST_FF_OVERFLOW | ST_FS_OVERFLOW | ST_SS_OVERFLOW | ST_COUPLE_OVERFLOW |
                              ST_VERLET_OVERFLOW | ST_MODE_CHANGE | ST_FVERLET_OVERFLOW | ST_SPLIT_CONTACTS |
                              ST_FBITS_OVERFLOW;

// Neighbour search of the staged API: synchronises once, grows and retries.
int neighborSearchChecked(demsph_engine* e, int iStep, int gap)
{
    for (int attempt = 0; attempt < 16; ++attempt) {
        const int parBefore = e->par;
        stageNeighborSearch(e, iStep, gap);
        const int st = readStatus(e);
        if (st == 0) return DEMSPH_OK;
        e->par = parBefore;
        if (st & ST_BARRIER_TIMEOUT) return fail(e, DEMSPH_ERR_TIMEOUT, "a grid barrier of a cooperative launch gave up waiting");
        if (st & ~ALL_OVERFLOWS) return fail(e, DEMSPH_ERR_STATE, "unexpected device status " + std::to_string(st));
        grow(e, st);
    }
    return fail(e, DEMSPH_ERR_CAPACITY, "list overflow persists after growing");
}

}  // namespace

extern "C" {

const char* demsph_status_string(int s)
{
    switch (s) {
    case DEMSPH_OK: return "ok";
    case DEMSPH_ERR_ARGUMENT: return "invalid argument";
    case DEMSPH_ERR_STATE: return "call out of order";
    case DEMSPH_ERR_CUDA: return "CUDA error";
    case DEMSPH_ERR_NO_DEVICE: return "no usable CUDA device";
    case DEMSPH_ERR_CAPACITY: return "list capacity exceeded";
    case DEMSPH_ERR_OUT_OF_MEMORY: return "out of device memory";
    case DEMSPH_ERR_TIMEOUT: return "device wait timed out";
    case DEMSPH_ERR_IO: return "file error";
    default: return "unknown status";
    }
}

const char* demsph_last_error(const demsph_engine* e) { return e ? e->err.c_str() : ""; }
const char* demsph_version(void) { return "demsph_gb300 0.1 (sm_103a)"; }

int demsph_selftest_barrier(int device, int missing, int* status_out)
{
    if (!status_out || missing < 0 || missing > 1000) return DEMSPH_ERR_ARGUMENT;
    *status_out = 0;
    if (cudaSetDevice(device) != cudaSuccess) return DEMSPH_ERR_NO_DEVICE;
    return selftestBarrier(missing, status_out);
}

int demsph_create(const demsph_scene* sc, const demsph_options* opt, demsph_engine** out)
{
    if (!sc || !out) return DEMSPH_ERR_ARGUMENT;
    *out = nullptr;
    if (sc->n_fluid < 0 || sc->n_solid < 0 || sc->n_clump < 0 || sc->n_wall < 0 || sc->n_material < 1)
        return DEMSPH_ERR_ARGUMENT;
    if (sc->n_fluid >= MAX_LIST_INDEX || sc->n_solid >= MAX_LIST_INDEX) return DEMSPH_ERR_CAPACITY;
    if (opt && (opt->fluid_lanes < 0 || opt->fluid_lanes > 8 || (opt->fluid_lanes & (opt->fluid_lanes - 1)) != 0))
        return DEMSPH_ERR_ARGUMENT;
    if (opt && opt->contact_rows_per_warp != 0 && opt->contact_rows_per_warp != 4 && opt->contact_rows_per_warp != 8 &&
        opt->contact_rows_per_warp != 16 && opt->contact_rows_per_warp != 32)
        return DEMSPH_ERR_ARGUMENT;
    demsph_options o{};
    if (opt) o = *opt;
    // Material ids index the contact tables (getCombinedIndex, core/hostStructs.h:369-384);
    // the reference reads outside the table for ids >= n_material, so reject them here.
    for (int i = 0; i < sc->n_solid; ++i)
        if (sc->solid_material[i] < 0 || sc->solid_material[i] >= sc->n_material) return DEMSPH_ERR_ARGUMENT;
    for (int k = 0; k < sc->n_wall; ++k)
        if (sc->wall_material[k] < 0 || sc->wall_material[k] >= sc->n_material) return DEMSPH_ERR_ARGUMENT;
    for (int c = 0; c < sc->n_clump; ++c)
        if (sc->clump_pebble_start[c] < 0 || sc->clump_pebble_end[c] > sc->n_solid ||
            sc->clump_pebble_start[c] > sc->clump_pebble_end[c])
            return DEMSPH_ERR_ARGUMENT;
    demsph_engine* e = new demsph_engine();
    e->debug = o.debug;
    int rc = checkDevice(e, o.device);
    if (rc != DEMSPH_OK) {
        *out = e;  // keep the message readable
        return rc;
    }
    e->opt = o;
    try {
        e->device = o.device;
        CK(cudaSetDevice(o.device));
        keepPoolMemory(o.device);
        CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&e->forkEv, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&e->joinEv, cudaEventDisableTiming));
        DeviceState& d = e->d;
        d.fixes = o.fixes;
        d.nf = sc->n_fluid;
        d.ns = sc->n_solid;
        d.nc = sc->n_clump;
        d.nw = sc->n_wall;
        d.kff = o.fluid_neighbors_max > 0 ? o.fluid_neighbors_max : 160;
        d.kfs = o.fluid_solids_max > 0 ? o.fluid_solids_max : 96;
        d.lanes = o.fluid_lanes > 0 ? o.fluid_lanes : fluidLanes(d.nf);
        const int perParticle = o.solid_contacts_per_particle > 0 ? o.solid_contacts_per_particle : 16;

        // ---- grid: dataBase::setSpatialGrids (core/dataBase.cpp:415-432) ----
        double mf = 0, ms = 0;
        for (int i = 0; i < d.nf; ++i) mf = std::max(mf, sc->fluid_smoothing_length[i]);
        for (int i = 0; i < d.ns; ++i) ms = std::max(ms, sc->solid_effective_radius[i]);
        e->hmax = mf;
        const double cell = 2 * std::max(mf, ms);
        int g[3];
        for (int a = 0; a < 3; ++a) {
            const double L = sc->domain_size[a];
            g[a] = L > cell ? int(L / cell) : 1;
            d.minB[a] = sc->domain_origin[a];
            d.cs[a] = L / double(g[a]);
        }
        const long long ncell = (long long)g[0] * g[1] * g[2] + 1;
        if (ncell > 1500000000LL) throw CudaError{cudaErrorMemoryAllocation, "grid has too many cells"};
        d.grid.gx = g[0];
        d.grid.gy = g[1];
        d.grid.gz = g[2];
        d.grid.num = (int)ncell;
        d.grid.csx = df_from_double(d.cs[0]);
        d.grid.csy = df_from_double(d.cs[1]);
        d.grid.csz = df_from_double(d.cs[2]);
        d.grid.cs = make_float3((float)d.cs[0], (float)d.cs[1], (float)d.cs[2]);
        for (int a = 0; a < 3; ++a) d.g64[a] = sc->gravity[a];
        d.g = make_float3((float)sc->gravity[0], (float)sc->gravity[1], (float)sc->gravity[2]);

        // ---- contact tables ----
        const int nslot = sc->n_material * (sc->n_material + 1) / 2;
        e->hzF.assign(sc->hertzian, sc->hertzian + 8 * nslot);
        e->lnF.assign(sc->linear, sc->linear + 11 * nslot);
        e->bdF.assign(sc->bonded, sc->bonded + 6 * nslot);
        e->dampF.resize(nslot);
        for (int k = 0; k < nslot; ++k) {
            const double lr = std::log(sc->hertzian[8 * k + 2]);
            e->dampF[k] = (float)(-lr / std::sqrt(lr * lr + 3.1415926535897931 * 3.1415926535897931));
        }
        float* tab = dalloc<float>(26 * nslot, e->owned, e->stream);
        CK(cudaMemcpyAsync(tab, e->hzF.data(), sizeof(float) * 8 * nslot, cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(tab + 8 * nslot, e->lnF.data(), sizeof(float) * 11 * nslot, cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(tab + 19 * nslot, e->bdF.data(), sizeof(float) * 6 * nslot, cudaMemcpyHostToDevice, e->stream));
        CK(cudaMemcpyAsync(tab + 25 * nslot, e->dampF.data(), sizeof(float) * nslot, cudaMemcpyHostToDevice, e->stream));
        d.tab.nMat = sc->n_material;
        d.tab.hz = tab;
        d.tab.ln = tab + 8 * nslot;
        d.tab.bd = tab + 19 * nslot;
        d.tab.damp = tab + 25 * nslot;

        d.status = dalloc<int>(1, e->owned, e->stream);
        d.stepsDone = dalloc<int>(1, e->owned, e->stream);
        size_t wk = std::max({scanWorkspaceInts(d.grid.num), scanWorkspaceInts(std::max(1, d.ns)),
                              scanWorkspaceInts(std::max(1, d.nf))});
        d.scanWork = dalloc<int>(wk, e->owned, e->stream);

        // ---- fluid ----
        const int nf = d.nf;
        {
            std::vector<int4> cell(nf);
            std::vector<float4> ph(nf), pl(nf), vh(nf), vl(nf), acc(nf), par(nf);
            std::vector<float> drho(nf);
            std::vector<int> id(nf);
            for (int i = 0; i < nf; ++i) {
                splitPosition(d, v3(sc->fluid_position, i), cell[i], ph[i], pl[i]);
                const dfl h = df_from_double(sc->fluid_smoothing_length[i]);
                ph[i].w = h.hi;
                pl[i].w = h.lo;
                const double3 v = v3(sc->fluid_velocity, i);
                const dfl vx = df_from_double(v.x), vy = df_from_double(v.y), vz = df_from_double(v.z);
                vh[i] = make_float4(vx.hi, vy.hi, vz.hi, 0.f);
                vl[i] = make_float4(vx.lo, vy.lo, vz.lo, 0.f);
                const double3 a = v3(sc->fluid_acceleration, i);
                acc[i] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.f);
                const double rho0 = sc->fluid_rho0[i];
                const double m = std::pow(sc->fluid_smoothing_length[i] / 1.3, 3) * rho0;
                par[i] = make_float4((float)rho0, (float)sc->fluid_sound_speed[i], (float)sc->fluid_nu[i], (float)m);
                drho[i] = sc->fluid_drho ? (float)sc->fluid_drho[i] : 0.f;
                id[i] = i;
            }
            d.fcell = dalloc<int4>(nf, e->owned, e->stream);
            d.fcp = dalloc<float4>(nf, e->owned, e->stream);
            for (int b = 0; b < 2; ++b) {
                d.fph[b] = dalloc<float4>(nf, e->owned, e->stream);
                d.fpl[b] = dalloc<float4>(nf, e->owned, e->stream);
                d.fvh[b] = dalloc<float4>(nf, e->owned, e->stream);
                d.fvl[b] = dalloc<float4>(nf, e->owned, e->stream);
                d.fdrho[b] = dalloc<float>(nf, e->owned, e->stream);
            }
            for (int b = 0; b < 3; ++b) d.fpd[b] = dalloc<float4>(nf, e->owned, e->stream);
            d.facc = dalloc<float4>(nf, e->owned, e->stream);
            d.fpar = dalloc<float4>(nf, e->owned, e->stream);
            d.fsumW0 = dalloc<float2>(nf, e->owned, e->stream);
            d.fid = dalloc<int>(nf, e->owned, e->stream);
            d.fslot = dalloc<int>(nf, e->owned, e->stream);
            d.tcell = dalloc<int4>(nf, e->owned, e->stream);
            d.tacc = dalloc<float4>(nf, e->owned, e->stream);
            d.tpar = dalloc<float4>(nf, e->owned, e->stream);
            d.tsumW0 = dalloc<float2>(nf, e->owned, e->stream);
            d.tid = dalloc<int>(nf, e->owned, e->stream);
            d.fkey = dalloc<int>(nf, e->owned, e->stream);
            d.fslotInCell = dalloc<int>(nf, e->owned, e->stream);
            d.fsortTmp = dalloc<int>(nf, e->owned, e->stream);
            d.fcellCount = dalloc<int>(d.grid.num, e->owned, e->stream);
            d.fcellStart = dalloc<int>((size_t)d.grid.num + 1, e->owned, e->stream);
            d.ffc = dalloc<int>(nf, e->owned, e->stream);
            d.fsc = dalloc<int>(nf, e->owned, e->stream);
            d.fluidTiles = tileModeWanted(sc, d, o) ? 1 : 0;
            allocFluidLists(e);
            // Verlet candidates of the fluid lists (list mode)
            d.kvf = d.kff + d.kff / 2;
            d.kvs = d.kfs + d.kfs / 2;
            d.fvcn = dalloc<int>(nf, e->owned, e->stream);
            d.fvsn = dalloc<int>(nf, e->owned, e->stream);
            d.fvref = dalloc<float4>(nf, e->owned, e->stream);
            if (d.fluidTiles) {
                sizeTiles(e, cell);
                d.fbits = dalloc<unsigned>((size_t)d.kbits * nf, e->owned, e->stream, false);
                d.fwalk = dalloc<int>(nf, e->owned, e->stream);
            } else {
                allocFluidCandidates(e);
            }
            d.fhmax = (float)mf;
            d.fskin = (float)(o.fluid_verlet_skin > 0 ? o.fluid_verlet_skin : 0.2 * mf);
            d.frebuild = dalloc<int>(1, e->owned, e->stream);
            d.fslowMode = dalloc<int>(1, e->owned, e->stream);
            {
                const int one = 1;
                const bool walkOnly = o.fluid_verlet_skin < 0 || d.grid.gx < 3 || d.grid.gy < 3 || d.grid.gz < 3;
                CK(cudaMemcpyAsync(d.frebuild, &one, sizeof(int), cudaMemcpyHostToDevice, e->stream));
                if (walkOnly) CK(cudaMemcpyAsync(d.fslowMode, &one, sizeof(int), cudaMemcpyHostToDevice, e->stream));
            }
            if (nf > 0) {
                CK(cudaMemcpyAsync(d.fcell, cell.data(), sizeof(int4) * nf, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.fph[0], ph.data(), sizeof(float4) * nf, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.fpl[0], pl.data(), sizeof(float4) * nf, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.fvh[0], vh.data(), sizeof(float4) * nf, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.fvl[0], vl.data(), sizeof(float4) * nf, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.fdrho[0], drho.data(), sizeof(float) * nf, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.facc, acc.data(), sizeof(float4) * nf, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.fpar, par.data(), sizeof(float4) * nf, cudaMemcpyHostToDevice, e->stream));
                d.uniformFluid = 1;
                for (int i = 1; i < nf && d.uniformFluid; ++i)
                    d.uniformFluid = par[i].x == par[0].x && par[i].y == par[0].y && par[i].z == par[0].z &&
                                     par[i].w == par[0].w && ph[i].w == ph[0].w && pl[i].w == pl[0].w;
                d.fparU = par[0];
                d.cellPack = d.uniformFluid && !d.fluidTiles && d.grid.gx <= 2048 && d.grid.gy <= 2048 &&
                             d.grid.gz <= 1024 ? 1 : 0;
                {
                    const float h = ph[0].w;
                    const float kg = 5.f * 21.f / (16.f * 3.14159265358979323846f);
                    d.fconstU = make_float4(4.f * h * h, 0.5f / h, kg / (h * h * h * h * h), 1.f / par[0].y);
                }
                CK(cudaMemcpyAsync(d.fid, id.data(), sizeof(int) * nf, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.fslot, id.data(), sizeof(int) * nf, cudaMemcpyHostToDevice, e->stream));
            }
        }

        // ---- solids ----
        const int ns = d.ns;
        {
            std::vector<int4> cell(ns), flags(ns);
            std::vector<float4> ph(ns), pl(ns), vh(ns), vl(ns), wh(ns), wl(ns), acc(ns), tq(ns), nrm(ns), rad(ns);
            for (int i = 0; i < ns; ++i) {
                splitPosition(d, v3(sc->solid_position, i), cell[i], ph[i], pl[i]);
                const double im = sc->solid_inverse_mass[i];
                ph[i].w = (float)im;
                pl[i].w = 0.f;
                auto put = [&](const double* src, float4& hi, float4& lo) {
                    const double3 v = v3(src, i);
                    const dfl x = df_from_double(v.x), y = df_from_double(v.y), z = df_from_double(v.z);
                    hi = make_float4(x.hi, y.hi, z.hi, 0.f);
                    lo = make_float4(x.lo, y.lo, z.lo, 0.f);
                };
                put(sc->solid_velocity, vh[i], vl[i]);
                put(sc->solid_angular_velocity, wh[i], wl[i]);
                const double3 a = v3(sc->solid_acceleration, i), t = v3(sc->solid_torque, i), n = v3(sc->solid_normal, i);
                acc[i] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.f);
                tq[i] = make_float4((float)t.x, (float)t.y, (float)t.z, 0.f);
                nrm[i] = make_float4((float)n.x, (float)n.y, (float)n.z, 0.f);
                const dfl r = df_from_double(sc->solid_radius[i]), ef = df_from_double(sc->solid_effective_radius[i]);
                rad[i] = make_float4(r.hi, r.lo, ef.hi, ef.lo);
                int bits = 0;
                if (sc->solid_is_dummy[i] == 1) bits |= F_DUMMY;
                if (im < 1.e-10) bits |= F_FIXED;
                if (im > 1.e-10) bits |= F_MASSIVE;
                if (im > 0.) bits |= F_HASMASS;
                if (im > 0.) e->nMassive++;
                flags[i] = make_int4(sc->solid_material[i], sc->solid_cluster[i], sc->solid_clump[i], bits);
            }
            d.scell = dalloc<int4>(ns, e->owned, e->stream);
            d.sph = dalloc<float4>(ns, e->owned, e->stream);
            d.spl = dalloc<float4>(ns, e->owned, e->stream);
            d.sphE = dalloc<float4>(ns, e->owned, e->stream);
            d.splE = dalloc<float4>(ns, e->owned, e->stream);
            d.svh = dalloc<float4>(ns, e->owned, e->stream);
            d.svl = dalloc<float4>(ns, e->owned, e->stream);
            d.swh = dalloc<float4>(ns, e->owned, e->stream);
            d.swl = dalloc<float4>(ns, e->owned, e->stream);
            d.sacc = dalloc<float4>(ns, e->owned, e->stream);
            d.storque = dalloc<float4>(ns, e->owned, e->stream);
            d.snormal = dalloc<float4>(ns, e->owned, e->stream);
            d.sfcoup = dalloc<float4>(ns, e->owned, e->stream);
            d.srad = dalloc<float4>(ns, e->owned, e->stream);
            d.sflags = dalloc<int4>(ns, e->owned, e->stream);
            d.skey = dalloc<int>(ns, e->owned, e->stream);
            d.skeySearch = dalloc<int>(ns, e->owned, e->stream);
            d.sslotInCell = dalloc<int>(ns, e->owned, e->stream);
            d.ssorted = dalloc<int>(ns, e->owned, e->stream);
            d.ssortTmp = dalloc<int>(ns, e->owned, e->stream);
            d.scellCount = dalloc<int>(d.grid.num, e->owned, e->stream);
            d.scellStart = dalloc<int>((size_t)d.grid.num + 1, e->owned, e->stream);
            // contact rows: every solid but the dummy wall particles, in index order
            std::vector<int> srow(ns, -1), rowSolid;
            double rmin = 0, effMax = 0;
            for (int i = 0; i < ns; ++i) {
                if (flags[i].w & F_DUMMY) continue;
                srow[i] = (int)rowSolid.size();
                rowSolid.push_back(i);
                rmin = rowSolid.size() == 1 ? sc->solid_radius[i] : std::min(rmin, sc->solid_radius[i]);
                effMax = std::max(effMax, sc->solid_effective_radius[i]);
            }
            d.nrow = (int)rowSolid.size();
            // solids the integration advances (a dummy at rest never moves: it has no mass)
            {
                std::vector<int>& move = e->moveHost;
                e->moveKind.assign(ns, 1);
                for (int i = 0; i < ns; ++i) {
                    if (sc->solid_clump[i] >= 0) {
                        e->moveKind[i] = 0;
                        continue;
                    }
                    const double3 v = v3(sc->solid_velocity, i);
                    const bool moving = v.x != 0.0 || v.y != 0.0 || v.z != 0.0;
                    if (flags[i].w & F_DUMMY) {
                        e->moveKind[i] = 2;
                        e->dummyIdx.push_back(i);
                        e->dummyMoving.push_back(moving ? 1 : 0);
                    }
                    if (!(flags[i].w & F_DUMMY) || moving) move.push_back(i);
                }
                d.nmove = (int)move.size();
                d.moveList = dalloc<int>(move.size(), e->owned, e->stream);
                d.moveFirst = consecutiveFirst(move.data(), move.size());
                d.ndummy = (int)e->dummyIdx.size();
                e->movingDummies = (int)std::count(e->dummyMoving.begin(), e->dummyMoving.end(), (unsigned char)1);
                d.dummyIdx = dalloc<int>(std::max(1, d.ndummy), e->owned, e->stream);
                d.dummyMoving = dalloc<unsigned char>(std::max(1, d.ndummy), e->owned, e->stream);
                d.moveChanged = dalloc<int>(1, e->owned, e->stream);
                if (d.ndummy > 0) {
                    CK(cudaMemcpyAsync(d.dummyIdx, e->dummyIdx.data(), sizeof(int) * d.ndummy, cudaMemcpyHostToDevice,
                                       e->stream));
                    CK(cudaMemcpyAsync(d.dummyMoving, e->dummyMoving.data(), d.ndummy, cudaMemcpyHostToDevice,
                                       e->stream));
                }
                if (!move.empty())
                    CK(cudaMemcpyAsync(d.moveList, move.data(), sizeof(int) * move.size(), cudaMemcpyHostToDevice,
                                       e->stream));
            }
            d.srow = dalloc<int>(ns, e->owned, e->stream);
            d.rowSolid = dalloc<int>(d.nrow, e->owned, e->stream);
            d.rowsAreSolids = d.nrow == ns ? 1 : 0;
            for (int r = 0; r < d.nrow && d.rowsAreSolids; ++r) d.rowsAreSolids = rowSolid[r] == r;
            d.scentre = dalloc<int4>(d.nrow, e->owned, e->stream);
            d.scentreSearch = dalloc<int4>(d.nrow, e->owned, e->stream);
            if (ns > 0) CK(cudaMemcpyAsync(d.srow, srow.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, e->stream));
            if (d.nrow > 0)
                CK(cudaMemcpyAsync(d.rowSolid, rowSolid.data(), sizeof(int) * d.nrow, cudaMemcpyHostToDevice, e->stream));
            const size_t nr = (size_t)std::max(1, d.nrow);
            d.scap = perParticle;
            d.fcnt[0] = dalloc<int>(nr, e->owned, e->stream);
            d.fcnt[1] = dalloc<int>(nr, e->owned, e->stream);
            d.rcnt = dalloc<int>(nr, e->owned, e->stream);
            allocContactLists(e);
            // Verlet candidates
            d.skin = (float)(o.solid_verlet_skin > 0 ? o.solid_verlet_skin : 0.2 * rmin);
            d.vmaxEff = (float)effMax;
            d.vcap = 2 * perParticle;
            d.vcand = dalloc<int>((size_t)d.vcap * nr, e->owned, e->stream, false);
            d.vcnt = dalloc<int>(nr, e->owned, e->stream);
            d.vref = dalloc<float4>(ns, e->owned, e->stream);
            d.svref = dalloc<float4>(ns, e->owned, e->stream);
            d.rebuild = dalloc<int>(2, e->owned, e->stream);
            d.slowMode = dalloc<int>(1, e->owned, e->stream);
            d.need = dalloc<int>(5, e->owned, e->stream);
            d.rowStats = dalloc<int>(3, e->owned, e->stream);
            d.gridBar = dalloc<unsigned>(2, e->owned, e->stream);
            {
                const char* v = std::getenv("DEMSPH_COOPERATIVE_SORT");
                // at most two blocks per SM, and no more than two elements per
                // thread need: small scenes leave the GPU to the others
                const long long n = std::max<long long>(d.nf, ns);
                d.sortBlocks = (v && v[0] == '0') ? 0
                                                 : (int)std::min<long long>(cooperativeSortBlocks(),
                                                                            std::max<long long>(1, (n + 511) / 512));
            }
            {
                const char* v = std::getenv("DEMSPH_FUSE_INTEGRATION");
                e->fuseIntegration = !(v && v[0] == '0');
            }
            d.forceRows = o.contact_rows_per_warp > 0 ? o.contact_rows_per_warp : 32;
            e->adaptRows = o.contact_rows_per_warp == 0;
            const int one = 1;
            const bool walkOnly = o.solid_verlet_skin < 0 || d.grid.gx < 3 || d.grid.gy < 3 || d.grid.gz < 3;
            {
                const char* v = std::getenv("DEMSPH_MERGE_CONTACTS");
                e->mergeContacts = !(v && v[0] == '0') && !walkOnly;
            }
            {
                const char* v = std::getenv("DEMSPH_FOLD_INTEGRATION");
                e->foldIntegration = !(v && v[0] == '0');
            }
            const int both[2] = {1, 1};
            CK(cudaMemcpyAsync(d.rebuild, both, sizeof(both), cudaMemcpyHostToDevice, e->stream));
            if (walkOnly) CK(cudaMemcpyAsync(d.slowMode, &one, sizeof(int), cudaMemcpyHostToDevice, e->stream));
            d.coupCount = dalloc<int>(ns, e->owned, e->stream);
            d.coupStart = dalloc<int>((size_t)ns + 1, e->owned, e->stream);
            d.coupCap = std::max(1024, std::min(64 * e->nMassive + 1024, std::max(1, d.kfs * nf)));
            d.coupList = dalloc<int>(d.coupCap, e->owned, e->stream);
            if (ns > 0) {
                CK(cudaMemcpyAsync(d.scell, cell.data(), sizeof(int4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.sph, ph.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.spl, pl.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.svh, vh.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.svl, vl.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.swh, wh.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.swl, wl.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.sacc, acc.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.storque, tq.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.snormal, nrm.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.srad, rad.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.sflags, flags.data(), sizeof(int4) * ns, cudaMemcpyHostToDevice, e->stream));
            }
        }

        // ---- walls ----
        {
            const int nw = d.nw;
            std::vector<float4> nh(nw), nl(nw);
            std::vector<float2> P(nw);
            std::vector<int> mat(nw);
            for (int k = 0; k < nw; ++k) {
                const double3 p = v3(sc->wall_point, k), n = v3(sc->wall_normal, k);
                const dfl x = df_from_double(n.x), y = df_from_double(n.y), z = df_from_double(n.z);
                nh[k] = make_float4(x.hi, y.hi, z.hi, 0.f);
                nl[k] = make_float4(x.lo, y.lo, z.lo, 0.f);
                const dfl pp = df_from_double((p.x - d.minB[0]) * n.x + (p.y - d.minB[1]) * n.y + (p.z - d.minB[2]) * n.z);
                P[k] = make_float2(pp.hi, pp.lo);
                mat[k] = sc->wall_material[k];
            }
            d.wnh = dalloc<float4>(nw, e->owned, e->stream);
            d.wnl = dalloc<float4>(nw, e->owned, e->stream);
            d.wP = dalloc<float2>(nw, e->owned, e->stream);
            d.wmat = dalloc<int>(nw, e->owned, e->stream);
            for (int p = 0; p < 2; ++p) {
                for (int k = 0; k < 3; ++k) d.wspring[p][k] = dalloc<float4>((size_t)ns * nw, e->owned, e->stream);
                d.wmask[p] = dalloc<unsigned>(ns, e->owned, e->stream);
            }
            if (nw > 0) {
                CK(cudaMemcpyAsync(d.wnh, nh.data(), sizeof(float4) * nw, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.wnl, nl.data(), sizeof(float4) * nw, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.wP, P.data(), sizeof(float2) * nw, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.wmat, mat.data(), sizeof(int) * nw, cudaMemcpyHostToDevice, e->stream));
            }
        }

        // ---- clumps ----
        {
            const int nc = d.nc;
            d.cpH = dalloc<float4>(nc, e->owned, e->stream);
            d.cpL = dalloc<float4>(nc, e->owned, e->stream);
            d.cvH = dalloc<float4>(nc, e->owned, e->stream);
            d.cvL = dalloc<float4>(nc, e->owned, e->stream);
            d.cwH = dalloc<float4>(nc, e->owned, e->stream);
            d.cwL = dalloc<float4>(nc, e->owned, e->stream);
            d.cacc = dalloc<float4>(nc, e->owned, e->stream);
            d.ctorque = dalloc<float4>(nc, e->owned, e->stream);
            d.cIw = dalloc<float>(6 * (size_t)nc, e->owned, e->stream);
            d.cinvm = dalloc<float>(nc, e->owned, e->stream);
            d.cq = dalloc<double4>(nc, e->owned, e->stream);
            d.cinvI = dalloc<double>(6 * (size_t)nc, e->owned, e->stream);
            d.cstart = dalloc<int>(nc, e->owned, e->stream);
            d.cend = dalloc<int>(nc, e->owned, e->stream);
            int most = 1;
            for (int c = 0; c < nc; ++c) most = std::max(most, sc->clump_pebble_end[c] - sc->clump_pebble_start[c]);
            d.clumpLanes = 1;
            while (d.clumpLanes < most && d.clumpLanes < 32) d.clumpLanes *= 2;
            if (nc > 0) {
                std::vector<float4> pH(nc), pL(nc), vH(nc), vL(nc), wH(nc), wL(nc), acc(nc), tq(nc);
                std::vector<float> Iw(6 * (size_t)nc), im(nc);
                auto split = [](double3 v, float4& h, float4& l) {
                    const dfl x = df_from_double(v.x), y = df_from_double(v.y), z = df_from_double(v.z);
                    h = make_float4(x.hi, y.hi, z.hi, 0.f);
                    l = make_float4(x.lo, y.lo, z.lo, 0.f);
                };
                for (int c = 0; c < nc; ++c) {
                    const double3 p = v3(sc->clump_centroid, c);
                    split(make_double3(p.x - d.minB[0], p.y - d.minB[1], p.z - d.minB[2]), pH[c], pL[c]);
                    split(v3(sc->clump_velocity, c), vH[c], vL[c]);
                    split(v3(sc->clump_angular_velocity, c), wH[c], wL[c]);
                    const double3 a = v3(sc->clump_acceleration, c), t = v3(sc->clump_torque, c);
                    acc[c] = make_float4((float)a.x, (float)a.y, (float)a.z, 0.f);
                    tq[c] = make_float4((float)t.x, (float)t.y, (float)t.z, 0.f);
                    im[c] = (float)sc->clump_inverse_mass[c];
                    // world-frame inverse inertia R invI R^T (core/myMat.h:102-127)
                    const double* q = sc->clump_orientation + 4 * c;
                    const double q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
                    const double R[3][3] = {{1 - 2 * q2 * q2 - 2 * q3 * q3, 2 * q1 * q2 - 2 * q0 * q3, 2 * q1 * q3 + 2 * q0 * q2},
                                            {2 * q1 * q2 + 2 * q0 * q3, 1 - 2 * q1 * q1 - 2 * q3 * q3, 2 * q2 * q3 - 2 * q0 * q1},
                                            {2 * q1 * q3 - 2 * q0 * q2, 2 * q2 * q3 + 2 * q0 * q1, 1 - 2 * q1 * q1 - 2 * q2 * q2}};
                    const double* I = sc->clump_inverse_inertia + 6 * c;
                    const double B[3][3] = {{I[0], I[3], I[4]}, {I[3], I[1], I[5]}, {I[4], I[5], I[2]}};
                    double W[3][3];
                    for (int i = 0; i < 3; ++i)
                        for (int j = 0; j < 3; ++j) {
                            double sum = 0;
                            for (int k = 0; k < 3; ++k)
                                for (int m = 0; m < 3; ++m) sum += R[i][k] * B[k][m] * R[j][m];
                            W[i][j] = sum;
                        }
                    const double w6[6] = {W[0][0], W[1][1], W[2][2], W[0][1], W[0][2], W[1][2]};
                    for (int k = 0; k < 6; ++k) Iw[6 * c + k] = (float)w6[k];
                }
                CK(cudaMemcpyAsync(d.cpH, pH.data(), sizeof(float4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cpL, pL.data(), sizeof(float4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cvH, vH.data(), sizeof(float4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cvL, vL.data(), sizeof(float4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cwH, wH.data(), sizeof(float4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cwL, wL.data(), sizeof(float4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cacc, acc.data(), sizeof(float4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.ctorque, tq.data(), sizeof(float4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cIw, Iw.data(), sizeof(float) * 6 * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cinvm, im.data(), sizeof(float) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cq, sc->clump_orientation, sizeof(double4) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cinvI, sc->clump_inverse_inertia, sizeof(double) * 6 * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cstart, sc->clump_pebble_start, sizeof(int) * nc, cudaMemcpyHostToDevice, e->stream));
                CK(cudaMemcpyAsync(d.cend, sc->clump_pebble_end, sizeof(int) * nc, cudaMemcpyHostToDevice, e->stream));
            }
        }
        CK(cudaStreamSynchronize(e->stream));
    } catch (const CudaError& c) {
        rc = cudaFail(e, c);
        *out = e;
        return rc;
    }
    *out = e;
    return DEMSPH_OK;
}


int demsph_destroy(demsph_engine* e)
{
    if (!e) return DEMSPH_ERR_ARGUMENT;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    delete e;
    return DEMSPH_OK;
}

static void adaptRowsPerWarp(demsph_engine* e, const int* stats);

int demsph_initialize(demsph_engine* e)
{
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    // the initial list comes from the reference's walk, in its order, so bonds
    // are numbered as addBondData numbers them
    e->forceWalk = true;
    const int rc = neighborSearchChecked(e, 0, 1);
    e->forceWalk = false;
    if (rc != DEMSPH_OK) return rc;
    // bonds between touching spheres of one cluster
    const long long nslots = (long long)d.nrow * d.scap;
    if (nslots > 0) {
        if (nslots > 2000000000LL) return fail(e, DEMSPH_ERR_CAPACITY, "contact rows too large for bond creation");
        std::vector<Allocation> tmp;
        int* flag = dalloc<int>((size_t)nslots + 1, tmp, e->stream);
        int* pos = dalloc<int>((size_t)nslots + 1, tmp, e->stream);
        int* work = dalloc<int>(scanWorkspaceInts((int)nslots), tmp, e->stream);
        const int nb = launchBondFlags(d, e->par, flag, pos, work, e->stream);
        if (nb > 0) {
            d.nb = nb;
            d.bab = dalloc<int2>(nb, e->owned, e->stream);
            d.bon = dalloc<int>(nb, e->owned, e->stream);
            d.bFnTt = dalloc<float4>(nb, e->owned, e->stream);
            d.bFsH = dalloc<float4>(nb, e->owned, e->stream);
            d.bFsL = dalloc<float4>(nb, e->owned, e->stream);
            d.bTbH = dalloc<float4>(nb, e->owned, e->stream);
            d.bTbL = dalloc<float4>(nb, e->owned, e->stream);
            d.bN = dalloc<float4>(nb, e->owned, e->stream);
            d.bLever = dalloc<float4>(nb, e->owned, e->stream);
            d.bF = dalloc<float4>(nb, e->owned, e->stream);
            d.bTA = dalloc<float4>(nb, e->owned, e->stream);
            d.bTB = dalloc<float4>(nb, e->owned, e->stream);
            launchBondWrite(d, e->par, flag, pos, e->stream);
        }
        CK(cudaStreamSynchronize(e->stream));
        for (const auto& a : tmp) cudaFreeAsync(a.p, e->stream);
    }
    // bonds of each solid, in bond order (the per-solid force sums)
    {
        std::vector<int2> ab;
        if (d.nb > 0) {
            ab.resize(d.nb);
            CK(cudaMemcpyAsync(ab.data(), d.bab, sizeof(int2) * d.nb, cudaMemcpyDeviceToHost, e->stream));
            CK(cudaStreamSynchronize(e->stream));
        }
        std::vector<int> start((size_t)d.ns + 1, 0), list(2 * (size_t)d.nb);
        for (const int2& p : ab) {
            start[p.x + 1]++;
            start[p.y + 1]++;
        }
        for (int i = 0; i < d.ns; ++i) start[i + 1] += start[i];
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int b = 0; b < d.nb; ++b) {
            list[fill[ab[b].x]++] = b;
            list[fill[ab[b].y]++] = b;
        }
        d.bondStart = dalloc<int>((size_t)d.ns + 1, e->owned, e->stream);
        d.bondList = dalloc<int>(list.size(), e->owned, e->stream);
        if (d.ns > 0) CK(cudaMemcpyAsync(d.bondStart, start.data(), sizeof(int) * (d.ns + 1), cudaMemcpyHostToDevice, e->stream));
        if (!list.empty()) CK(cudaMemcpyAsync(d.bondList, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, e->stream));
    }
    // the contact-force rows per warp from the first contact lists
    if (d.nrow > 0 && e->adaptRows) {
        int stats[2] = {0, 0};
        launchRowStats(d, e->par, e->stream);
        CK(cudaMemcpyAsync(stats, d.rowStats, sizeof(stats), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        if (stats[1] > 0) adaptRowsPerWarp(e, stats);
    }
    // normals of walls and clump pebbles (setSolidNormal), kernel length = largest fluid h
    launchSolidNormals(d, e->hmax, e->stream);
    CK(cudaStreamSynchronize(e->stream));
    CK(cudaGetLastError());
    e->initialized = true;
    return DEMSPH_OK;
    ENGINE_END(e)
}

#define REQUIRE_INIT(e) \
    if (!(e)->initialized) return fail((e), DEMSPH_ERR_STATE, "demsph_initialize has not been called")

int demsph_neighbor_search(demsph_engine* e, int i_step, int gap)
{
    if (gap < 1) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    return neighborSearchChecked(e, i_step, gap);
    ENGINE_END(e)
}

int demsph_solid_integrate_before_contact(demsph_engine* e, double dt)
{
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    stageBefore(e, dt);
    CK(cudaGetLastError());
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_fluid_integrate(demsph_engine* e, double dt, int i_step, int gap)
{
    if (gap < 1) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    stageFluid(e, dt, i_step, gap);
    CK(cudaGetLastError());
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_solid_contact_after_fluid_integrate(demsph_engine* e, double dt)
{
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    stageContact(e, dt);
    CK(cudaGetLastError());
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_solid_integrate_after_contact(demsph_engine* e, double dt)
{
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    stageAfter(e, dt);
    CK(cudaGetLastError());
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_synchronize(demsph_engine* e)
{
    ENGINE_GUARD(e)
    CK(cudaStreamSynchronize(e->stream));
    CK(cudaGetLastError());
    const int st = readStatus(e);
    if (st) return fail(e, DEMSPH_ERR_CAPACITY, "a list overflowed (status " + std::to_string(st) + ")");
    return DEMSPH_OK;
    ENGINE_END(e)
}

// n_steps update() bodies without the driver hook.  With use_graph, steps run
// uncaptured until i_step is a multiple of the period (and > 1: step 1 stores
// the Shepard reference), whole periods replay one captured graph, the rest
// runs uncaptured.  One synchronisation at the end; on a list overflow the
// engine grows the list and resumes from the first incomplete step.
// Kind of step i: bit 0 a fluid step (every gap steps), bit 1 a Shepard
// re-initialisation (every 5 gap steps).  Steps of one kind launch the same
// kernels with the same arguments, apart from the contact-list parity.
static int stepKind(const DeviceState& d, int i, int gap)
{
    if (d.nf <= 0) return 0;
    return (i % gap == 0 ? 1 : 0) | (i % (5 * gap) == 0 ? 2 : 0);
}

// The graph of `length` steps of `kind` starting from the current parity,
// captured on first use.
static const demsph_engine::CachedGraph& graphFor(demsph_engine* e, int kind, int length, double dt, int step, int gap)
{
    for (const auto& g : e->graphs)
        if (g.kind == kind && g.parity == e->par && g.length == length) return g;
    const int parity = e->par;
    cudaGraph_t g;
    const long long before = t_kernelLaunches;
    // runs of plain DEM steps fuse each step's closing integration with the
    // next one's opening (fluid steps are captured one at a time)
    const bool fused = e->fuseIntegration && kind == 0 && length >= 2;
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    if (fused)
        fusedSteps(e, dt, step, length, gap);
    else
        for (int k = 0; k < length; ++k) fullStep(e, dt, step + k, gap);
    CK(cudaStreamEndCapture(e->stream, &g));
    e->par = parity;  // nothing ran: the parity is where it was
    demsph_engine::CachedGraph c{kind, parity, length, nullptr, t_kernelLaunches - before, fused};
    e->capturedLaunches += c.kernels;
    const cudaError_t ie = cudaGraphInstantiate(&c.exec, g, 0);
    cudaGraphDestroy(g);
    CK(ie);
    e->graphs.push_back(c);
    return e->graphs.back();
}

// Rows per warp of the contact kernels for about 192 items per warp (a warp
// also does per-row work for each of its rows, so fewer rows pay only when
// rows hold many items; measured on GB300 with 0.6 and ~12 items per row);
// kept while the current value is within a factor of the ideal one (a change
// re-captures the graphs).
static int rowsPerWarp(double itemsPerRow, int current)
{
    const double ideal = 192.0 / std::max(itemsPerRow, 0.25);
    if (ideal >= 0.75 * current && ideal <= 2.5 * current) return current;
    int r = 32;
    while (r > 4 && r > ideal) r >>= 1;
    return r;
}

static void adaptRowsPerWarp(demsph_engine* e, const int* stats)
{
    DeviceState& d = e->d;
    const int fr = rowsPerWarp((double)stats[0] / stats[1], d.forceRows);
    if (fr == d.forceRows) return;
    d.forceRows = fr;
    dropGraph(e);  // the launch shape and the state are baked into the graphs
}

// The steps of demsph_update; `afterSteps` (when given) is enqueued after the
// steps of every attempt, before the one synchronisation that reads the
// status, so a transfer it enqueues sees the state of the completed steps (an
// attempt that overflowed is followed by one that enqueues it again).
static int runUpdate(demsph_engine* e, double dt, int first_step, int n_steps, int gap, int use_graph,
                     const std::function<void()>* afterSteps)
{
    DeviceState& d = e->d;
    const int end = first_step + n_steps;
    int step = first_step;
    for (int attempt = 0; step < end; ++attempt) {
        if (attempt > 32) return fail(e, DEMSPH_ERR_CAPACITY, "list overflow persists after growing");
        CK(cudaMemsetAsync(d.stepsDone, 0, sizeof(int), e->stream));
        const int startPar = e->par;
        const bool startOpened = e->resumeOpened;
        const bool graphs = use_graph && !e->profiling;
        // profiled runs that ask for graphs launch the graphs' bodies directly
        // (the same fused runs, each stage timed): the stage times are those of
        // the steps the graphs run
        const bool eagerFused = use_graph && e->profiling;
        if (graphs && (e->graphDt != dt || e->graphGap != gap)) {
            dropGraph(e);
            e->graphDt = dt;
            e->graphGap = gap;
        }
        int s = step;
        // the first step of each fused graph launched: an overflow in the
        // search of any later step of it leaves that step opened
        std::vector<std::pair<int, int>> fusedRuns;
        while (s < end) {
            const int kind = stepKind(d, s, gap);
            if ((!graphs && !eagerFused) || s == 1 || e->resumeOpened) {  // step 1 stores the Shepard reference sums: run it as it is
                fullStep(e, dt, s++, gap, e->resumeOpened);
                e->resumeOpened = false;
                continue;
            }
            // a run of plain DEM steps replays 10- and 2-step graphs (parity
            // unchanged), an odd last step or a fluid step a 1-step graph
            int run = 1;
            if (kind == 0)
                while (s + run < end && stepKind(d, s + run, gap) == 0) ++run;
            while (run > 0) {
                const int len = kind != 0 ? 1 : (run >= 10 ? 10 : (run >= 2 ? 2 : 1));
                bool fusedRun;
                if (eagerFused) {
                    fusedRun = e->fuseIntegration && kind == 0 && len >= 2;
                    if (fusedRun)
                        fusedSteps(e, dt, s, len, gap);
                    else
                        for (int k = 0; k < len; ++k) fullStep(e, dt, s + k, gap);  // the steps flip the parity
                } else {
                    const auto& g = graphFor(e, kind, len, dt, s, gap);
                    CK(cudaGraphLaunch(g.exec, e->stream));
                    e->replayedKernels += g.kernels;
                    fusedRun = g.fused;
                    e->par ^= (len & 1);
                }
                if (fusedRun) {
                    fusedRuns.emplace_back(s, len);
                    e->runStats.fused_passes += len - 1;
                }
                s += len;
                run -= len;
            }
        }
        int rowStats[2] = {0, 0};
        if (graphs && d.nrow > 0 && e->adaptRows && n_steps >= 8) {  // long runs only
            launchRowStats(d, e->par, e->stream);
            CK(cudaMemcpyAsync(rowStats, d.rowStats, sizeof(rowStats), cudaMemcpyDeviceToHost, e->stream));
        }
        if (afterSteps) (*afterSteps)();
        int done = 0;
        const int st = readStatus(e, &done);
        if (st == 0) {
            step = s;
            if (rowStats[1] > 0) adaptRowsPerWarp(e, rowStats);
            continue;
        }
        if (st & ST_BARRIER_TIMEOUT) return fail(e, DEMSPH_ERR_TIMEOUT, "a grid barrier of a cooperative launch gave up waiting");
        if (st & ~ALL_OVERFLOWS) return fail(e, DEMSPH_ERR_STATE, "unexpected device status " + std::to_string(st));
        step += done;                        // steps before the failed one completed
        e->par = startPar ^ (done & 1);      // every step builds one contact list
        // every overflow is raised in a neighbour search or the contact list
        // of the contact stage; in a fused graph both run, for every step but
        // the first, after the pass that opened that step (and a resumed step
        // stays opened when its own search overflows again).  Nothing else of
        // a plain DEM step before the contact stage changes state.
        e->resumeOpened = done == 0 && startOpened;
        for (const auto& r : fusedRuns)
            if (step > r.first && step < r.first + r.second) e->resumeOpened = true;
        if (e->resumeOpened) ++e->runStats.resumed_steps;
        ++e->runStats.list_growths;
        grow(e, st);
    }
    if (afterSteps && n_steps == 0) {
        (*afterSteps)();
        CK(cudaStreamSynchronize(e->stream));
    }
    CK(cudaGetLastError());
    return DEMSPH_OK;
}

int demsph_update(demsph_engine* e, double dt, int first_step, int n_steps, int gap, int use_graph)
{
    if (gap < 1 || n_steps < 0) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    return runUpdate(e, dt, first_step, n_steps, gap, use_graph, nullptr);
    ENGINE_END(e)
}

int demsph_update_io(demsph_engine* e, double dt, int first_step, int n_steps, int gap, int use_graph,
                     const double* fluid_pos_in, const double* fluid_vel_in, const double* fluid_drho_in,
                     const double* solid_pos_in, const double* solid_vel_in, const double* solid_angvel_in,
                     double* fluid_pos_out, double* fluid_vel_out, double* fluid_drho_out, double* solid_pos_out,
                     double* solid_vel_out, double* solid_angvel_out)
{
    if (gap < 1 || n_steps < 0) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    const DeviceState& d = e->d;
    const bool fIn = fluid_pos_in || fluid_vel_in || fluid_drho_in, sIn = solid_pos_in || solid_vel_in || solid_angvel_in;
    const bool fOut = fluid_pos_out || fluid_vel_out || fluid_drho_out,
               sOut = solid_pos_out || solid_vel_out || solid_angvel_out;
    // the solids' transfers and conversions on the second stream beside the
    // fluids' (their own staging slot; the conversions touch disjoint arrays),
    // forked from and joined back into the engine's stream
    const bool split = d.nf > 0 && d.ns > 0 && ((fIn && sIn) || (fOut && sOut));
    cudaStream_t ss = split ? e->side : e->stream;
    const int sslot = split ? 1 : 0;
    if (split) {  // both slots exist before the fork (they are allocated on the engine's stream)
        scratchDoubles(e, 10 * (size_t)d.nf, 0);
        scratchDoubles(e, 18 * (size_t)d.ns, 1);
    }
    const auto fork = [&] {
        if (!split) return;
        CK(cudaEventRecord(e->forkEv, e->stream));
        CK(cudaStreamWaitEvent(e->side, e->forkEv, 0));
    };
    const auto join = [&] {
        if (!split) return;
        CK(cudaEventRecord(e->joinEv, e->side));
        CK(cudaStreamWaitEvent(e->stream, e->joinEv, 0));
    };
    fork();
    if (fIn) enqueueUploadFluids(e, fluid_pos_in, fluid_vel_in, fluid_drho_in);
    if (sIn) enqueueUploadSolids(e, solid_pos_in, solid_vel_in, solid_angvel_in, ss, sslot);
    join();
    const std::function<void()> download = [&] {
        fork();
        if (sOut) enqueueDownloadSolids(e, solid_pos_out, solid_vel_out, nullptr, nullptr, nullptr, solid_angvel_out, ss,
                                        sslot);
        if (fOut) enqueueDownloadFluids(e, fluid_pos_out, fluid_vel_out, nullptr, fluid_drho_out);
        join();
    };
    return runUpdate(e, dt, first_step, n_steps, gap, use_graph, &download);
    ENGINE_END(e)
}

int demsph_get_launch_shapes(const demsph_engine* e, demsph_launch_shapes* out)
{
    if (!e || !out) return DEMSPH_ERR_ARGUMENT;
    out->fluid_lanes = e->d.lanes;
    out->clump_lanes = e->d.clumpLanes;
    out->contact_force_rows = e->d.forceRows;
    out->fluid_bit_lists = e->d.fluidTiles ? 1 : 0;
    out->fluid_bit_words = e->d.fluidTiles ? e->d.kbits : 0;
    return DEMSPH_OK;
}

int demsph_get_run_stats(const demsph_engine* e, demsph_run_stats* out)
{
    if (!e || !out) return DEMSPH_ERR_ARGUMENT;
    *out = e->runStats;
    return DEMSPH_OK;
}

// Threads per fluid particle, chosen by timing: the first continuity pass
// (it reads the step's state and writes only buffers the next fluid step
// overwrites) is timed with 1, 2, 4 and 8 lanes, and the fastest is kept for
// every fluid list and pair kernel.
int demsph_autotune(demsph_engine* e, int* lanes_out)
{
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    DeviceState& d = e->d;
    if (d.nf > 0) {
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        float best = 0.f;
        int bestL = d.lanes;
        for (int L = 1; L <= 8; L *= 2) {
            d.lanes = L;
            launchContinuityPass(d, 0, 1.0e-9, e->stream);  // warm-up
            CK(cudaEventRecord(a, e->stream));
            for (int r = 0; r < 5; ++r) launchContinuityPass(d, 0, 1.0e-9, e->stream);
            CK(cudaEventRecord(b, e->stream));
            CK(cudaEventSynchronize(b));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, a, b));
            if (L == 1 || ms < best) {
                best = ms;
                bestL = L;
            }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        d.lanes = bestL;
        dropGraph(e);  // the lane count is baked into captured launches
    }
    if (lanes_out) *lanes_out = d.lanes;
    return DEMSPH_OK;
    ENGINE_END(e)
}

void* demsph_stream(demsph_engine* e) { return e ? (void*)e->stream : nullptr; }

long long demsph_device_bytes(const demsph_engine* e)
{
    if (!e) return -1;
    long long b = 0;
    for (const auto& a : e->owned) b += (long long)a.bytes;
    return b;
}

long long demsph_estimate_bytes(const demsph_scene* sc, const demsph_options* opt)
{
    if (!sc || sc->n_fluid < 0 || sc->n_solid < 0) return -1;
    demsph_options o{};
    if (opt) o = *opt;
    const long long kff = o.fluid_neighbors_max > 0 ? o.fluid_neighbors_max : 160;
    const long long kfs = o.fluid_solids_max > 0 ? o.fluid_solids_max : 96;
    const long long slots = o.solid_contacts_per_particle > 0 ? o.solid_contacts_per_particle : 16;
    double mf = 0, ms = 0;
    for (int i = 0; i < sc->n_fluid; ++i) mf = std::max(mf, sc->fluid_smoothing_length[i]);
    for (int i = 0; i < sc->n_solid; ++i) ms = std::max(ms, sc->solid_effective_radius[i]);
    const double cell = 2 * std::max(mf, ms);
    long long cells = 1;
    for (int a = 0; a < 3; ++a) cells *= sc->domain_size[a] > cell ? (long long)(sc->domain_size[a] / cell) : 1;
    long long rows = 0;
    for (int i = 0; i < sc->n_solid; ++i) rows += sc->solid_is_dummy[i] != 1;
    const long long nf = sc->n_fluid, ns = sc->n_solid;
    // per fluid particle: state, reorder buffers, both neighbour lists and their candidates; per
    // solid: state, sort and wall springs; per contact row: its slots, two
    // list parities, springs in and out, candidates; per cell: counts and starts
    const long long kvf = kff + kff / 2, kvs = kfs + kfs / 2;
    return nf * (380 + 4 * (kff + kfs) + 4 * (kvf + kvs)) + ns * (248 + 48LL * sc->n_wall) +
           rows * (72 + slots * 184 + 2 * slots * 4) + (cells + 1) * 16 + (long long)sc->n_clump * 160 +
           std::min(64 * rows + 1024, std::max(1LL, kfs * nf)) * 4 + (1 << 20);
}

long long demsph_kernel_launches(demsph_engine* e)
{
    if (!e) return -1;
    return e->launched - e->capturedLaunches + e->replayedKernels;
}

int demsph_set_profiling(demsph_engine* e, int enable)
{
    if (!e) return DEMSPH_ERR_ARGUMENT;
    e->profiling = enable != 0;
    return DEMSPH_OK;
}

int demsph_profile_report(demsph_engine* e, char* buf, int cap)
{
    if (!e || !buf || cap <= 0) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    CK(cudaStreamSynchronize(e->stream));
    std::vector<std::string> order;
    std::vector<std::pair<int, double>> acc;
    for (auto& t : e->timed) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, t.a, t.b));
        size_t k = 0;
        while (k < order.size() && order[k] != t.tag) ++k;
        if (k == order.size()) {
            order.push_back(t.tag);
            acc.push_back({0, 0.0});
        }
        acc[k].first += 1;
        acc[k].second += ms;
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    e->timed.clear();
    std::string out;
    for (size_t k = 0; k < order.size(); ++k)
        out += order[k] + " " + std::to_string(acc[k].first) + " " + std::to_string(acc[k].second) + "\n";
    const size_t n = std::min(out.size(), (size_t)cap - 1);
    std::memcpy(buf, out.data(), n);
    buf[n] = 0;
    return DEMSPH_OK;
    ENGINE_END(e)
}

}  // extern "C"

// ---- many engines advanced by one graph launch (demsph_batch_*) ----
//
// No counterpart in the reference, which runs one scene per process.  Each
// engine of a batch contributes a round: `n` steps from `first`, captured once
// as a graph of exactly the launches its own graph replays make (plain DEM
// runs fused, fluid steps one by one), so a scene's state after a batched
// round is bit for bit its state after the same steps alone.  The batch's
// graph holds every member's round as a child graph (independent branches:
// the scenes' kernels overlap on the device), then one report kernel that
// copies each member's status and completed-step count into mapped host
// memory.  The launch is re-instantiated only when a member's round changes
// (another length, phase or parity, or a member whose graphs were dropped by
// list growth); rounds that are whole multiples of the Shepard period (5 gap
// steps) and of even length keep their phase and parity, so a steady batch
// launches the same executable graph round after round.  A member whose round
// overflowed a list resumes alone after its lists grow (demsph_update's path),
// before the call returns.
namespace {

long long g_roundIds = 0;  // ids of captured rounds (batch keys); guarded by g_roundMutex
std::mutex g_roundMutex;

__global__ void kBatchReport(int* const* where, int n, int2* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_int2(*where[2 * i], *where[2 * i + 1]);
}

// The round of `n` steps of engine e from step `first` (captured on first use).
const demsph_engine::RoundGraph& roundFor(demsph_engine* e, double dt, int first, int n, int gap)
{
    const DeviceState& d = e->d;
    const int period = d.nf > 0 ? 5 * gap : 1;
    const int phase = first % period;
    for (const auto& r : e->rounds)
        if (r.phase == phase && r.length == n && r.parity == e->par && r.gap == gap && r.dt == dt) return r;
    demsph_engine::RoundGraph r{phase, n, e->par, gap, dt, nullptr, 0, 0, {}};
    {
        std::lock_guard<std::mutex> g(g_roundMutex);
        r.id = ++g_roundIds;
    }
    const int parity = e->par;
    const long long before = t_kernelLaunches;
    CK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    try {
        CK(cudaMemsetAsync(d.stepsDone, 0, sizeof(int), e->stream));
        for (int s = first, end = first + n; s < end;) {
            int run = 1;
            if (stepKind(d, s, gap) == 0)
                while (s + run < end && stepKind(d, s + run, gap) == 0) ++run;
            if (run >= 2 && e->fuseIntegration) {
                fusedSteps(e, dt, s, run, gap);
                r.fusedRuns.emplace_back(s - first, run);
            } else {
                for (int k = 0; k < run; ++k) fullStep(e, dt, s + k, gap);
            }
            s += run;
        }
    } catch (...) {
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(e->stream, &junk);
        if (junk) cudaGraphDestroy(junk);
        e->par = parity;
        throw;
    }
    CK(cudaStreamEndCapture(e->stream, &r.graph));
    e->par = parity;  // nothing ran
    r.kernels = t_kernelLaunches - before;
    e->capturedLaunches += r.kernels;
    e->rounds.push_back(std::move(r));
    return e->rounds.back();
}

}  // namespace

struct demsph_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    // the graph launched last, the mapped status array it writes (per member
    // {status, steps done}) and the device array of the members' status and
    // step-count addresses it reads
    cudaGraphExec_t exec = nullptr;
    int2* report = nullptr;
    int2* reportDev = nullptr;
    int** where = nullptr;
    // executable graphs of recent member sets (the current one first): a set
    // that comes back (rounds cycling through phases) is not instantiated again
    struct Cached {
        std::vector<long long> key;
        cudaGraphExec_t exec;
        int2* report;   // the mapped status array the graph writes
        int** where;    // the status addresses it reads
    };
    std::vector<Cached> cache;
    demsph_batch_info info{};
    std::string err;
};

extern "C" {

int demsph_batch_create(int device, demsph_batch** out)
{
    if (!out) return DEMSPH_ERR_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return DEMSPH_ERR_NO_DEVICE;
    auto* b = new demsph_batch;
    b->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return DEMSPH_ERR_CUDA;
    }
    *out = b;
    return DEMSPH_OK;
}

int demsph_batch_destroy(demsph_batch* b)
{
    if (!b) return DEMSPH_ERR_ARGUMENT;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto& c : b->cache) {
        cudaGraphExecDestroy(c.exec);
        cudaFreeHost(c.report);
        cudaFree(c.where);
    }
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return DEMSPH_OK;
}

const char* demsph_batch_last_error(const demsph_batch* b) { return b ? b->err.c_str() : "no batch"; }

int demsph_batch_get_info(const demsph_batch* b, demsph_batch_info* out)
{
    if (!b || !out) return DEMSPH_ERR_ARGUMENT;
    *out = b->info;
    return DEMSPH_OK;
}

int demsph_batch_update(demsph_batch* b, demsph_engine* const* engines, int count, const int* first_step,
                        const int* n_steps, const double* dt, const int* gap, int* status_out)
{
    if (!b || count < 0 || (count > 0 && (!engines || !first_step || !n_steps || !dt || !gap || !status_out)))
        return DEMSPH_ERR_ARGUMENT;
    struct Member {
        int i;
        demsph_engine* e;
        const demsph_engine::RoundGraph* r;
        int startPar;
    };
    {
        // an engine listed twice would have two rounds in one launch
        std::vector<demsph_engine*> sorted(engines, engines + count);
        std::sort(sorted.begin(), sorted.end());
        if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) {
            b->err = "batch: an engine is listed twice";
            return DEMSPH_ERR_ARGUMENT;
        }
    }
    std::vector<Member> members;
    auto engineFail = [&](int i, demsph_engine* e, const CudaError& c) { status_out[i] = cudaFail(e, c); };
    for (int i = 0; i < count; ++i) {
        demsph_engine* e = engines[i];
        status_out[i] = DEMSPH_OK;
        if (!e || !e->stream || gap[i] < 1 || n_steps[i] < 0 || first_step[i] < 1) {
            status_out[i] = DEMSPH_ERR_ARGUMENT;
            continue;
        }
        if (!e->initialized) {
            status_out[i] = fail(e, DEMSPH_ERR_STATE, "batch: engine not initialised");
            continue;
        }
        if (e->device != b->device) {
            status_out[i] = fail(e, DEMSPH_ERR_ARGUMENT, "batch: engine on another device");
            continue;
        }
        LaunchTally tally(e);
        try {
            CK(cudaSetDevice(e->device));
            int first = first_step[i], n = n_steps[i];
            if (e->graphDt != dt[i] || e->graphGap != gap[i]) {
                dropGraph(e);
                e->graphDt = dt[i];
                e->graphGap = gap[i];
            }
            // step 1 (it stores the Shepard reference sums), a step opened by a
            // fused pass before an overflow, and profiled runs go alone
            if (n > 0 && (first == 1 || e->resumeOpened || e->profiling)) {
                const int alone = e->profiling ? n : 1;
                const int rc = runUpdate(e, dt[i], first, alone, gap[i], 1, nullptr);
                if (rc != DEMSPH_OK) {
                    status_out[i] = rc;
                    continue;
                }
                first += alone;
                n -= alone;
            }
            if (n == 0) continue;
            CK(cudaStreamSynchronize(e->stream));  // the member's own work before the batch
            const auto tc = std::chrono::steady_clock::now();
            const auto& r = roundFor(e, dt[i], first, n, gap[i]);
            b->info.capture_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - tc).count();
            members.push_back({i, e, &r, e->par});
        } catch (const CudaError& c) {
            engineFail(i, e, c);
        }
    }
    if (members.empty()) return DEMSPH_OK;
    const int m = (int)members.size();
    try {
        CK(cudaSetDevice(b->device));
        std::vector<long long> key(m);
        for (int k = 0; k < m; ++k) key[k] = members[k].r->id;
        size_t hit = 0;
        while (hit < b->cache.size() && b->cache[hit].key != key) ++hit;
        if (hit < b->cache.size()) {
            std::rotate(b->cache.begin(), b->cache.begin() + hit, b->cache.begin() + hit + 1);
        } else {
            const auto ti = std::chrono::steady_clock::now();
            constexpr size_t KEEP = 4;
            while (b->cache.size() >= KEEP) {  // the least recently used goes
                auto& c = b->cache.back();
                CK(cudaGraphExecDestroy(c.exec));
                CK(cudaFreeHost(c.report));
                CK(cudaFree(c.where));
                b->cache.pop_back();
            }
            // each graph writes its own status array (mapped host memory)
            CK(cudaHostAlloc(reinterpret_cast<void**>(&b->report), sizeof(int2) * m, cudaHostAllocMapped));
            CK(cudaHostGetDevicePointer(reinterpret_cast<void**>(&b->reportDev), b->report, 0));
            CK(cudaMalloc(reinterpret_cast<void**>(&b->where), sizeof(int*) * 2 * m));
            std::vector<int*> where(2 * m);
            for (int k = 0; k < m; ++k) {
                where[2 * k] = members[k].e->d.status;
                where[2 * k + 1] = members[k].e->d.stepsDone;
            }
            CK(cudaMemcpy(b->where, where.data(), sizeof(int*) * 2 * m, cudaMemcpyHostToDevice));
            cudaGraph_t g;
            CK(cudaGraphCreate(&g, 0));
            std::vector<cudaGraphNode_t> nodes(m);
            size_t total = 0;
            for (int k = 0; k < m; ++k) {
                CK(cudaGraphAddChildGraphNode(&nodes[k], g, nullptr, 0, members[k].r->graph));
                size_t c = 0;
                CK(cudaGraphGetNodes(members[k].r->graph, nullptr, &c));
                total += c;
            }
            int** whereArg = b->where;
            int nArg = m;
            int2* outArg = b->reportDev;
            void* args[] = {&whereArg, &nArg, &outArg};
            cudaKernelNodeParams kp{};
            kp.func = reinterpret_cast<void*>(kBatchReport);
            kp.gridDim = dim3((unsigned)((m + 127) / 128));
            kp.blockDim = dim3(128);
            kp.kernelParams = args;
            cudaGraphNode_t rep;
            CK(cudaGraphAddKernelNode(&rep, g, nodes.data(), nodes.size(), &kp));
            cudaGraphExec_t exec = nullptr;
            const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) {
                cudaFreeHost(b->report);
                cudaFree(b->where);
            }
            CK(ie);
            b->cache.insert(b->cache.begin(), {key, exec, b->report, b->where});
            ++b->info.graph_builds;
            b->info.members = m;
            b->info.nodes = (long long)total + 1;
            b->info.instantiate_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - ti).count();
        }
        b->exec = b->cache.front().exec;
        b->report = b->cache.front().report;
        const auto tl = std::chrono::steady_clock::now();
        CK(cudaGraphLaunch(b->exec, b->stream));
        CK(cudaStreamSynchronize(b->stream));
        b->info.launch_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - tl).count();
        ++b->info.launches;
    } catch (const CudaError& c) {
        b->err = std::string(c.what) + ": " + cudaGetErrorString(c.e);
        for (const auto& mb : members) status_out[mb.i] = cudaFail(mb.e, c);
        return c.e == cudaErrorMemoryAllocation ? DEMSPH_ERR_OUT_OF_MEMORY : DEMSPH_ERR_CUDA;
    }
    for (int k = 0; k < m; ++k) {
        const Member& mb = members[k];
        demsph_engine* e = mb.e;
        const int i = mb.i;
        const int first = first_step[i] + (n_steps[i] - mb.r->length), n = mb.r->length, g = gap[i];
        const int st = b->report[k].x, done = b->report[k].y;
        e->replayedKernels += mb.r->kernels;
        for (const auto& fr : mb.r->fusedRuns) e->runStats.fused_passes += fr.second - 1;
        if (st == 0) {
            e->par = mb.startPar ^ (n & 1);
            continue;
        }
        LaunchTally tally(e);
        try {
            CK(cudaSetDevice(e->device));
            if (st & ST_BARRIER_TIMEOUT) {
                status_out[i] = fail(e, DEMSPH_ERR_TIMEOUT, "a grid barrier of a cooperative launch gave up waiting");
                continue;
            }
            if (st & ~ALL_OVERFLOWS) {
                status_out[i] = fail(e, DEMSPH_ERR_STATE, "unexpected device status " + std::to_string(st));
                continue;
            }
            // as demsph_update after an overflow: the steps before the failed
            // one completed; a step a fused pass opened resumes opened
            const int step = first + done;
            e->par = mb.startPar ^ (done & 1);
            e->resumeOpened = false;
            for (const auto& fr : mb.r->fusedRuns)
                if (step > first + fr.first && step < first + fr.first + fr.second) e->resumeOpened = true;
            if (e->resumeOpened) ++e->runStats.resumed_steps;
            ++e->runStats.list_growths;
            grow(e, st);
            status_out[i] = runUpdate(e, dt[i], step, first + n - step, g, 1, nullptr);
        } catch (const CudaError& c) {
            engineFail(i, e, c);
        }
    }
    return DEMSPH_OK;
}

}  // extern "C"

// ---- particles added while a simulation runs (demsph_append) ----
//
// dataBase::addFluidData / addSolidData after the start (core/dataBase.cpp:
// 226-268) re-upload the whole state with the new particles appended and
// recompute the spatial grid; addCluster then searches again and bonds the new
// cluster (core/dataBase.cpp:83-113, 307-343).  Here an engine for the whole
// scene is made on the same device and the old engine's histories are carried
// into it on the device: the contact list of the last step with its springs
// (as the previous list, so the first search remaps them pair by pair), the
// bonds and their states, the wall and pebble normals, and the Shepard
// reference sums.  As in the reference: the new particles come after the old
// ones in index order, the wall springs start again from zero (it rebuilds
// solid2InfiniteWall), new solids have zero normals (setSolidNormal runs only
// at the start), and only pairs of a new cluster above the last bonded index
// are bonded.  Two differences, both stated in the header: the neighbour lists
// are rebuilt at once for every kind of addition (the reference rebuilds them
// at the next search, or at once for a cluster), and the new fluids' Shepard
// reference sums are taken at the append (the reference leaves them zero, and
// its next re-initialisation divides by them).
namespace {

__global__ void kCarryContacts(DeviceState o, int op, DeviceState n, int np)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= o.nrow) return;
    const int a = solidOf(o, r);
    const int nr = rowOf(n, a);
    if (nr < 0) return;
    const int cnt = min(min(o.fcnt[op][r], o.scap), n.scap);
    for (int q = 0; q < cnt; ++q) {
        const size_t src = (size_t)q * o.nrow + r, dst = (size_t)q * n.nrow + nr;
        n.fwd[np][dst] = o.fwd[op][src];
        for (int j = 0; j < 3; ++j) n.springOut[np][j][dst] = o.springOut[op][j][src];
    }
    n.fcnt[np][nr] = cnt;
}

__global__ void kSlotOfId(DeviceState n, int* slotOf)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n.nf) slotOf[n.fid[s]] = s;
}

__global__ void kCarrySumW0(DeviceState o, DeviceState n, const int* slotOf)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < o.nf) n.fsumW0[slotOf[o.fid[s]]] = o.fsumW0[s];
}

template <class T>
std::vector<T> fetch(const T* p, size_t n, cudaStream_t s)
{
    std::vector<T> v(n);
    if (n) CK(cudaMemcpyAsync(v.data(), p, sizeof(T) * n, cudaMemcpyDeviceToHost, s));
    return v;
}

template <class T>
void put(T* p, const std::vector<T>& v, cudaStream_t s)
{
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
}

// The bonds of engine n: the old engine's bonds as they stand, then - when the
// addition holds a cluster - the bonds initialisation makes in n for pairs
// whose first solid is above the last bonded one (addBondData after the
// start, core/dataBase.cpp:307-343); and the per-solid bond lists.
void carryBonds(demsph_engine* old, demsph_engine* n, bool cluster)
{
    DeviceState& o = old->d;
    DeviceState& d = n->d;
    const cudaStream_t s = n->stream;
    const int nbOld = o.nb;
    std::vector<int2> ab = fetch(o.bab, nbOld, old->stream);
    std::vector<int> on = fetch(o.bon, nbOld, old->stream);
    std::vector<float4> st[7] = {fetch(o.bFnTt, nbOld, old->stream), fetch(o.bFsH, nbOld, old->stream),
                                 fetch(o.bFsL, nbOld, old->stream), fetch(o.bTbH, nbOld, old->stream),
                                 fetch(o.bTbL, nbOld, old->stream), fetch(o.bN, nbOld, old->stream),
                                 fetch(o.bLever, nbOld, old->stream)};
    CK(cudaStreamSynchronize(old->stream));
    const long long nslots = (long long)d.nrow * d.scap;
    if (cluster && nslots > 0 && nslots <= 2000000000LL) {
        // every bond initialisation would make, in n's arrays (then filtered)
        std::vector<Allocation> tmp;
        int* flag = dalloc<int>((size_t)nslots + 1, tmp, s);
        int* pos = dalloc<int>((size_t)nslots + 1, tmp, s);
        int* work = dalloc<int>(scanWorkspaceInts((int)nslots), tmp, s);
        const int nb = launchBondFlags(d, n->par, flag, pos, work, s);
        if (nb > 0) {
            DeviceState t = d;
            std::vector<Allocation> arr;
            t.bab = dalloc<int2>(nb, arr, s);
            t.bon = dalloc<int>(nb, arr, s);
            t.bFnTt = dalloc<float4>(nb, arr, s);
            t.bFsH = dalloc<float4>(nb, arr, s);
            t.bFsL = dalloc<float4>(nb, arr, s);
            t.bTbH = dalloc<float4>(nb, arr, s);
            t.bTbL = dalloc<float4>(nb, arr, s);
            t.bN = dalloc<float4>(nb, arr, s);
            t.bLever = dalloc<float4>(nb, arr, s);
            t.bF = dalloc<float4>(nb, arr, s);
            t.bTA = dalloc<float4>(nb, arr, s);
            t.bTB = dalloc<float4>(nb, arr, s);
            t.nb = nb;
            launchBondWrite(t, n->par, flag, pos, s);
            std::vector<int2> nab = fetch(t.bab, nb, s);
            std::vector<int> non = fetch(t.bon, nb, s);
            std::vector<float4> nst[7] = {fetch(t.bFnTt, nb, s), fetch(t.bFsH, nb, s), fetch(t.bFsL, nb, s),
                                          fetch(t.bTbH, nb, s), fetch(t.bTbL, nb, s), fetch(t.bN, nb, s),
                                          fetch(t.bLever, nb, s)};
            CK(cudaStreamSynchronize(s));
            const int last = nbOld > 0 ? ab.back().x : -1;
            for (int b = 0; b < nb; ++b) {
                if (nab[b].x <= last) continue;
                ab.push_back(nab[b]);
                on.push_back(non[b]);
                for (int k = 0; k < 7; ++k) st[k].push_back(nst[k][b]);
            }
            for (const auto& a : arr) cudaFreeAsync(a.p, s);
        }
        CK(cudaStreamSynchronize(s));
        for (const auto& a : tmp) cudaFreeAsync(a.p, s);
    }
    const int nb = (int)ab.size();
    d.nb = nb;
    if (nb > 0) {
        d.bab = dalloc<int2>(nb, n->owned, s);
        d.bon = dalloc<int>(nb, n->owned, s);
        d.bFnTt = dalloc<float4>(nb, n->owned, s);
        d.bFsH = dalloc<float4>(nb, n->owned, s);
        d.bFsL = dalloc<float4>(nb, n->owned, s);
        d.bTbH = dalloc<float4>(nb, n->owned, s);
        d.bTbL = dalloc<float4>(nb, n->owned, s);
        d.bN = dalloc<float4>(nb, n->owned, s);
        d.bLever = dalloc<float4>(nb, n->owned, s);
        d.bF = dalloc<float4>(nb, n->owned, s);
        d.bTA = dalloc<float4>(nb, n->owned, s);
        d.bTB = dalloc<float4>(nb, n->owned, s);
        put(d.bab, ab, s);
        put(d.bon, on, s);
        float4* dst[7] = {d.bFnTt, d.bFsH, d.bFsL, d.bTbH, d.bTbL, d.bN, d.bLever};
        for (int k = 0; k < 7; ++k) put(dst[k], st[k], s);
    }
    // bonds of each solid, in bond order (as demsph_initialize)
    std::vector<int> start((size_t)d.ns + 1, 0), list(2 * (size_t)nb);
    for (const int2& p : ab) {
        start[p.x + 1]++;
        start[p.y + 1]++;
    }
    for (int i = 0; i < d.ns; ++i) start[i + 1] += start[i];
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int b = 0; b < nb; ++b) {
        list[fill[ab[b].x]++] = b;
        list[fill[ab[b].y]++] = b;
    }
    d.bondStart = dalloc<int>((size_t)d.ns + 1, n->owned, s);
    d.bondList = dalloc<int>(list.size(), n->owned, s);
    put(d.bondStart, start, s);
    put(d.bondList, list, s);
    CK(cudaStreamSynchronize(s));
}

}  // namespace

extern "C" {

int demsph_append(demsph_engine* e, const demsph_scene* cur, const demsph_scene* add)
{
    if (!cur || !add) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    REQUIRE_INIT(e);
    DeviceState& d = e->d;
    if (cur->n_fluid != d.nf || cur->n_solid != d.ns || cur->n_clump != d.nc || cur->n_wall != d.nw)
        return fail(e, DEMSPH_ERR_ARGUMENT, "append: the current scene's counts differ from the engine's");
    if (add->n_clump != 0 || add->n_wall != 0)
        return fail(e, DEMSPH_ERR_ARGUMENT,
                    "append: walls and clumps can only be added before the simulation starts");
    if (add->n_fluid < 0 || add->n_solid < 0 || (add->n_fluid == 0 && add->n_solid == 0))
        return fail(e, DEMSPH_ERR_ARGUMENT, "append: nothing to add");
    if (add->n_fluid > 0 && (!add->fluid_position || !add->fluid_smoothing_length || !add->fluid_rho0 ||
                             !add->fluid_sound_speed || !add->fluid_nu))
        return fail(e, DEMSPH_ERR_ARGUMENT, "append: the added fluids need positions, smoothing lengths, densities, "
                                            "sound speeds and viscosities");
    if (add->n_solid > 0 && (!add->solid_position || !add->solid_radius || !add->solid_effective_radius ||
                             !add->solid_inverse_mass || !add->solid_material))
        return fail(e, DEMSPH_ERR_ARGUMENT, "append: the added solids need positions, radii, effective radii, "
                                            "inverse masses and materials");
    for (int i = 0; i < add->n_solid; ++i) {
        if (add->solid_material[i] < 0 || add->solid_material[i] >= cur->n_material)
            return fail(e, DEMSPH_ERR_ARGUMENT, "append: material index exceeds the number of materials");
        if (add->solid_clump && add->solid_clump[i] >= 0)
            return fail(e, DEMSPH_ERR_ARGUMENT,
                        "append: walls and clumps can only be added before the simulation starts");
    }
    CK(cudaStreamSynchronize(e->stream));
    const size_t nf0 = d.nf, ns0 = d.ns, nc = d.nc, af = add->n_fluid, as = add->n_solid;
    const size_t nf = nf0 + af, ns = ns0 + as;
    // the state as it stands, FP64 in original order
    std::vector<double> fpos(3 * nf), fvel(3 * nf), facc(3 * nf), fdr(nf);
    std::vector<double> spos(3 * ns), svel(3 * ns), sacc(3 * ns), snrm(3 * ns), stq(3 * ns), sw(3 * ns);
    enqueueDownloadFluids(e, fpos.data(), fvel.data(), facc.data(), fdr.data());
    enqueueDownloadSolids(e, spos.data(), svel.data(), sacc.data(), snrm.data(), stq.data(), sw.data());
    CK(cudaStreamSynchronize(e->stream));
    std::vector<double> cc(3 * nc), cv(3 * nc), ca(3 * nc), cw(3 * nc), ct(3 * nc), cq(4 * nc);
    if (nc) {
        const int rc = demsph_download_clumps(e, cc.data(), cv.data(), ca.data(), cw.data(), ct.data(), cq.data());
        if (rc != DEMSPH_OK) return rc;
    }
    // the whole scene: the current one's parameters and state, then the additions
    auto cat = [](std::vector<double>& v, size_t at, const double* src, size_t n, double fill) {
        for (size_t k = 0; k < n; ++k) v[at + k] = src ? src[k] : fill;
    };
    std::vector<double> fh(nf), rho0(nf), c(nf), nu(nf);
    cat(fh, 0, cur->fluid_smoothing_length, nf0, 0);
    cat(rho0, 0, cur->fluid_rho0, nf0, 0);
    cat(c, 0, cur->fluid_sound_speed, nf0, 0);
    cat(nu, 0, cur->fluid_nu, nf0, 0);
    cat(fpos, 3 * nf0, add->fluid_position, 3 * af, 0);
    cat(fvel, 3 * nf0, add->fluid_velocity, 3 * af, 0);
    cat(facc, 3 * nf0, add->fluid_acceleration, 3 * af, 0);
    cat(fdr, nf0, add->fluid_drho, af, 0);
    cat(fh, nf0, add->fluid_smoothing_length, af, 0);
    cat(rho0, nf0, add->fluid_rho0, af, 0);
    cat(c, nf0, add->fluid_sound_speed, af, 0);
    cat(nu, nf0, add->fluid_nu, af, 0);
    std::vector<double> seff(ns), srad(ns), sim(ns);
    std::vector<int> smat(ns), sclu(ns), sclump(ns), sdum(ns);
    cat(seff, 0, cur->solid_effective_radius, ns0, 0);
    cat(srad, 0, cur->solid_radius, ns0, 0);
    cat(sim, 0, cur->solid_inverse_mass, ns0, 0);
    cat(spos, 3 * ns0, add->solid_position, 3 * as, 0);
    cat(svel, 3 * ns0, add->solid_velocity, 3 * as, 0);
    cat(sacc, 3 * ns0, add->solid_acceleration, 3 * as, 0);
    cat(snrm, 3 * ns0, nullptr, 3 * as, 0);  // new solids: zero normals
    cat(stq, 3 * ns0, add->solid_torque, 3 * as, 0);
    cat(sw, 3 * ns0, add->solid_angular_velocity, 3 * as, 0);
    cat(seff, ns0, add->solid_effective_radius, as, 0);
    cat(srad, ns0, add->solid_radius, as, 0);
    cat(sim, ns0, add->solid_inverse_mass, as, 0);
    bool cluster = false;
    for (size_t i = 0; i < ns0; ++i) {
        smat[i] = cur->solid_material[i];
        sclu[i] = cur->solid_cluster ? cur->solid_cluster[i] : -1;
        sclump[i] = cur->solid_clump ? cur->solid_clump[i] : -1;
        sdum[i] = cur->solid_is_dummy ? cur->solid_is_dummy[i] : 0;
    }
    for (size_t i = 0; i < as; ++i) {
        smat[ns0 + i] = add->solid_material[i];
        sclu[ns0 + i] = add->solid_cluster ? add->solid_cluster[i] : -1;
        sclump[ns0 + i] = -1;
        sdum[ns0 + i] = add->solid_is_dummy ? add->solid_is_dummy[i] : 0;
        cluster |= sclu[ns0 + i] >= 0;
    }
    demsph_scene sc = *cur;
    for (int a = 0; a < 3; ++a) sc.gravity[a] = d.g64[a];  // as set at run time
    sc.n_fluid = (int)nf;
    sc.fluid_position = fpos.data();
    sc.fluid_velocity = fvel.data();
    sc.fluid_acceleration = facc.data();
    sc.fluid_smoothing_length = fh.data();
    sc.fluid_rho0 = rho0.data();
    sc.fluid_drho = fdr.data();
    sc.fluid_sound_speed = c.data();
    sc.fluid_nu = nu.data();
    sc.n_solid = (int)ns;
    sc.solid_position = spos.data();
    sc.solid_velocity = svel.data();
    sc.solid_acceleration = sacc.data();
    sc.solid_normal = snrm.data();
    sc.solid_torque = stq.data();
    sc.solid_angular_velocity = sw.data();
    sc.solid_effective_radius = seff.data();
    sc.solid_radius = srad.data();
    sc.solid_inverse_mass = sim.data();
    sc.solid_material = smat.data();
    sc.solid_cluster = sclu.data();
    sc.solid_clump = sclump.data();
    sc.solid_is_dummy = sdum.data();
    if (nc) {
        sc.clump_centroid = cc.data();
        sc.clump_velocity = cv.data();
        sc.clump_acceleration = ca.data();
        sc.clump_angular_velocity = cw.data();
        sc.clump_torque = ct.data();
        sc.clump_orientation = cq.data();
    }
    // the same options, with the lists as large as they have grown
    demsph_options o = e->opt;
    o.device = e->device;
    o.fluid_neighbors_max = std::max(o.fluid_neighbors_max, d.kff);
    o.fluid_solids_max = std::max(o.fluid_solids_max, d.kfs);
    o.solid_contacts_per_particle = std::max(o.solid_contacts_per_particle, d.scap);
    demsph_engine* n = nullptr;
    int rc = demsph_create(&sc, &o, &n);
    if (rc != DEMSPH_OK) {
        const std::string msg = n ? n->err : std::string(demsph_status_string(rc));
        if (n) demsph_destroy(n);
        return fail(e, rc, "append: " + msg);
    }
    try {
        DeviceState& nd = n->d;
        const cudaStream_t s = n->stream;
        // the last contact list and its springs as n's previous list
        if (d.nrow > 0 && nd.nrow > 0)
            ++t_kernelLaunches, kCarryContacts<<<blocksFor(d.nrow, 128), 128, 0, s>>>(d, e->par, nd, n->par);
        CK(cudaStreamSynchronize(s));
        n->forceWalk = true;  // the list in the reference's walk order (bonds are numbered in it)
        rc = neighborSearchChecked(n, 0, 1);
        n->forceWalk = false;
        if (rc != DEMSPH_OK) throw rc;
        carryBonds(e, n, cluster);
        if (nd.nrow > 0 && n->adaptRows) {
            int stats[2] = {0, 0};
            launchRowStats(nd, n->par, s);
            CK(cudaMemcpyAsync(stats, nd.rowStats, sizeof(stats), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (stats[1] > 0) adaptRowsPerWarp(n, stats);
        }
        // old solids keep their normals (the scene carried them), new ones zero
        if (ns) {
            std::vector<float4> nr(ns);
            for (size_t i = 0; i < ns; ++i)
                nr[i] = make_float4((float)snrm[3 * i], (float)snrm[3 * i + 1], (float)snrm[3 * i + 2], 0.f);
            put(nd.snormal, nr, s);
        }
        // Shepard reference sums: every fluid's at the append, then the old ones'
        if (nf) {
            launchDensityReinit(nd, 1, s);
            if (nf0) {
                std::vector<Allocation> tmp;
                int* slotOf = dalloc<int>(nf, tmp, s, false);
                ++t_kernelLaunches, kSlotOfId<<<blocksFor((long long)nf, 256), 256, 0, s>>>(nd, slotOf);
                CK(cudaStreamSynchronize(e->stream));
                ++t_kernelLaunches, kCarrySumW0<<<blocksFor((long long)nf0, 256), 256, 0, s>>>(d, nd, slotOf);
                CK(cudaStreamSynchronize(s));
                for (const auto& a : tmp) cudaFreeAsync(a.p, s);
            }
        }
        CK(cudaStreamSynchronize(s));
        CK(cudaGetLastError());
        n->initialized = true;
        n->profiling = e->profiling;
        n->runStats = e->runStats;
        n->launched = e->launched;
        n->capturedLaunches = e->capturedLaunches;
        n->replayedKernels = e->replayedKernels;
    } catch (int code) {
        const std::string msg = n->err;
        demsph_destroy(n);
        return fail(e, code, "append: " + msg);
    } catch (const CudaError& ce) {
        const std::string msg = std::string(ce.what) + ": " + cudaGetErrorString(ce.e);
        demsph_destroy(n);
        return fail(e, ce.e == cudaErrorMemoryAllocation ? DEMSPH_ERR_OUT_OF_MEMORY : DEMSPH_ERR_CUDA, "append: " + msg);
    }
    // the handle now holds the new engine; the old one's memory goes
    e->swapWith(*n);
    demsph_destroy(n);
    return DEMSPH_OK;
    ENGINE_END(e)
}

}  // extern "C"
