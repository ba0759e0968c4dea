// Host-side engine object shared by engine.cu (life cycle, step schedule,
// batching) and engine_io.cu (state transfer, setters, artefact export).
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "../../include/demsph_gb300.h"

namespace demsph {

struct CudaError {
    cudaError_t e;
    const char* what;
};

#define CK(call)                                           \
    do {                                                   \
        cudaError_t _e = (call);                           \
        if (_e != cudaSuccess) throw demsph::CudaError{_e, #call}; \
    } while (0)

// A device buffer and its size.
struct Allocation {
    void* p;
    size_t bytes;
};

// Stream-ordered allocation (cudaMallocAsync from the device's pool) on the
// engine's stream: creating, growing or freeing one engine never waits for
// the work of others on the same GPU.
template <class T>
inline T* dalloc(size_t n, std::vector<Allocation>& owned, cudaStream_t s, bool zero = true)
{
    T* p = nullptr;
    if (n == 0) n = 1;
    CK(cudaMallocAsync(reinterpret_cast<void**>(&p), sizeof(T) * n, s));
    if (zero) CK(cudaMemsetAsync(p, 0, sizeof(T) * n, s));
    owned.push_back({p, sizeof(T) * n});
    return p;
}

}  // namespace demsph

struct demsph_engine {
    demsph::DeviceState d{};
    demsph_options opt{};         // the options the engine was created with
    int device = 0;
    cudaStream_t stream = nullptr;
    // a second stream and two events: inside runs of plain DEM steps the
    // coupling force of a step runs beside its contact detection (a branch of
    // the captured graph, joined before the contact forces)
    cudaStream_t side = nullptr;
    cudaEvent_t forkEv = nullptr, joinEv = nullptr;
    std::vector<demsph::Allocation> owned;  // every device buffer of the engine
    std::string err;
    int par = 1;                  // parity of the last successful solid list build
    bool forceWalk = false;       // next contact list from the reference's 27-cell walk
    bool adaptRows = true;        // contact rows per warp follow the contacts per row
    bool solidSortStale = true;   // solid cells must be recomputed although no solid has mass
    std::vector<unsigned char> moveKind;  // per solid: 0 clump pebble, 1 integrated, 2 dummy (integrated when moving)
    std::vector<int> moveHost;            // the device move list
    std::vector<int> dummyIdx;            // the dummy particles (moveKind 2), and whether each is
    std::vector<unsigned char> dummyMoving;  // in the move list (given a velocity)
    bool walkOrder[2] = {true, true};  // list of each parity is in the reference's walk order
    bool initialized = false;
    int debug = 0;
    double hmax = 0;              // largest fluid smoothing length
    int nMassive = 0;
    int movingDummies = 0;  // dummy particles given a velocity (in the move list)
    // CUDA graphs of step runs, keyed by the kind of step, the contact-list
    // parity they start from and their length (all for one dt and gap)
    struct CachedGraph {
        int kind, parity, length;
        cudaGraphExec_t exec;
        long long kernels;
        bool fused;  // its steps after the first open with the previous step's closing integration
    };
    // Graphs of two or more plain DEM steps integrate the end of one step and
    // the start of the next in one pass (DEMSPH_FUSE_INTEGRATION=0 keeps two).
    bool fuseIntegration = true;
    // In those graphs the steps a fused pass opens build their contact list
    // and contact forces in one launch when the scene has no bonds and the
    // lists come from candidates (DEMSPH_MERGE_CONTACTS=0 keeps two launches;
    // off for good once the lists come from the walk).
    bool mergeContacts = true;
    // The per-solid sums run the solids' integration pass in the same launch
    // when the integrated solids are exactly the contact rows
    // (DEMSPH_FOLD_INTEGRATION=0 keeps the separate pass).
    bool foldIntegration = true;
    // The step the next attempt starts with already had its before-contact
    // half applied (a fused pass ran before its neighbour search overflowed).
    bool resumeOpened = false;
    // An integration has rehashed the solids since the last neighbour search:
    // the keys and walk centres of that search are in skeySearch /
    // scentreSearch (exports read them there)
    bool keysAdvanced = false;
    demsph_run_stats runStats{};
    std::vector<CachedGraph> graphs;
    // Step rounds captured for demsph_batch_update (graphs, not instantiated:
    // a batch takes them as child graphs), keyed like the cached graphs plus
    // the round's phase in the fluid and Shepard schedule.
    struct RoundGraph {
        int phase, length, parity, gap;
        double dt;
        cudaGraph_t graph;
        long long id;     // unique over all engines: batches key on it
        long long kernels;
        std::vector<std::pair<int, int>> fusedRuns;  // (offset from the round's first step, length)
    };
    std::vector<RoundGraph> rounds;
    int graphGap = 0;
    double graphDt = 0;
    // contact tables as uploaded (FP32)
    std::vector<float> hzF, lnF, bdF, dampF;
    // kernel launch accounting (demsph_kernel_launches)
    long long launched = 0;          // launch calls made by this engine's API calls (any thread)
    long long capturedLaunches = 0;  // launch calls recorded into graphs (not executed then)
    long long replayedKernels = 0;   // kernels executed by graph replays
    // stage timing (demsph_set_profiling)
    bool profiling = false;
    struct Timed {
        const char* tag;
        cudaEvent_t a, b;
    };
    std::vector<Timed> timed;
    // staging of FP64 transfers (device, grown on demand): [0] the fluids'
    // (and every transfer on the engine's stream), [1] the solids' when
    // demsph_update_io moves them on the second stream
    double* dscratch[2] = {nullptr, nullptr};
    size_t dscratchN[2] = {0, 0};

    // Exchanges everything two engines hold (device memory, stream, graphs,
    // state), field by field: demsph_append hands the caller's handle the
    // engine it made.  Every field must be listed here.
    void swapWith(demsph_engine& o)
    {
        using std::swap;
        swap(d, o.d);
        swap(opt, o.opt);
        swap(device, o.device);
        swap(stream, o.stream);
        swap(side, o.side);
        swap(forkEv, o.forkEv);
        swap(joinEv, o.joinEv);
        swap(owned, o.owned);
        swap(err, o.err);
        swap(par, o.par);
        swap(forceWalk, o.forceWalk);
        swap(adaptRows, o.adaptRows);
        swap(solidSortStale, o.solidSortStale);
        swap(moveKind, o.moveKind);
        swap(moveHost, o.moveHost);
        swap(dummyIdx, o.dummyIdx);
        swap(dummyMoving, o.dummyMoving);
        swap(walkOrder[0], o.walkOrder[0]);
        swap(walkOrder[1], o.walkOrder[1]);
        swap(initialized, o.initialized);
        swap(debug, o.debug);
        swap(hmax, o.hmax);
        swap(nMassive, o.nMassive);
        swap(movingDummies, o.movingDummies);
        swap(fuseIntegration, o.fuseIntegration);
        swap(mergeContacts, o.mergeContacts);
        swap(foldIntegration, o.foldIntegration);
        swap(resumeOpened, o.resumeOpened);
        swap(keysAdvanced, o.keysAdvanced);
        swap(runStats, o.runStats);
        swap(graphs, o.graphs);
        swap(rounds, o.rounds);
        swap(graphGap, o.graphGap);
        swap(graphDt, o.graphDt);
        swap(hzF, o.hzF);
        swap(lnF, o.lnF);
        swap(bdF, o.bdF);
        swap(dampF, o.dampF);
        swap(launched, o.launched);
        swap(capturedLaunches, o.capturedLaunches);
        swap(replayedKernels, o.replayedKernels);
        swap(profiling, o.profiling);
        swap(timed, o.timed);
        swap(dscratch[0], o.dscratch[0]);
        swap(dscratch[1], o.dscratch[1]);
        swap(dscratchN[0], o.dscratchN[0]);
        swap(dscratchN[1], o.dscratchN[1]);
    }

    ~demsph_engine()
    {
        for (auto& t : timed) {
            cudaEventDestroy(t.a);
            cudaEventDestroy(t.b);
        }
        for (const auto& g : graphs) cudaGraphExecDestroy(g.exec);
        for (const auto& r : rounds) cudaGraphDestroy(r.graph);
        for (const auto& a : owned) cudaFreeAsync(a.p, stream);
        if (side) {
            cudaStreamSynchronize(side);
            cudaStreamDestroy(side);
        }
        if (forkEv) cudaEventDestroy(forkEv);
        if (joinEv) cudaEventDestroy(joinEv);
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }
};

namespace demsph {

inline int fail(demsph_engine* e, int code, const std::string& msg)
{
    if (e) e->err = msg;
    return code;
}

inline int cudaFail(demsph_engine* e, const CudaError& c)
{
    return fail(e, c.e == cudaErrorMemoryAllocation ? DEMSPH_ERR_OUT_OF_MEMORY : DEMSPH_ERR_CUDA,
                std::string(c.what) + ": " + cudaGetErrorString(c.e));
}

void freeOne(demsph_engine* e, void*& p);
void dropGraph(demsph_engine* e);
int readStatus(demsph_engine* e, int* stepsDone = nullptr);
// Host transfers of the state enqueued on the engine's stream, without
// synchronising (engine_io.cu).
// The transfers run on stream s (the engine's stream when null) with staging
// slot `slot` of scratchDoubles.
void enqueueDownloadFluids(demsph_engine* e, double* pos, double* vel, double* acc, double* drho,
                           cudaStream_t s = nullptr, int slot = 0);
void enqueueDownloadSolids(demsph_engine* e, double* pos, double* vel, double* acc, double* normal, double* torque,
                           double* angvel, cudaStream_t s = nullptr, int slot = 0);
void enqueueUploadFluids(demsph_engine* e, const double* pos, const double* vel, const double* drho,
                         cudaStream_t s = nullptr, int slot = 0);
void enqueueUploadSolids(demsph_engine* e, const double* pos, const double* vel, const double* angvel,
                         cudaStream_t s = nullptr, int slot = 0);
// Staging slot `slot` with room for n doubles (allocated on the engine's stream).
double* scratchDoubles(demsph_engine* e, size_t n, int slot = 0);
void splitPosition(const DeviceState& d, double3 p, int4& c, float4& h, float4& l);

}  // namespace demsph

// Adds the launches one API call made (on its thread) to the engine's tally.
struct LaunchTally {
    demsph_engine* e;
    long long t0;
    explicit LaunchTally(demsph_engine* eng) : e(eng), t0(demsph::t_kernelLaunches) {}
    ~LaunchTally() { e->launched += demsph::t_kernelLaunches - t0; }
};

#define ENGINE_GUARD(e)                                   \
    if (!(e) || !(e)->stream) return DEMSPH_ERR_ARGUMENT; \
    LaunchTally _launch_tally(e);                         \
    try {                                                 \
        CK(cudaSetDevice((e)->device));

#define ENGINE_END(e)                   \
    }                                   \
    catch (const demsph::CudaError& c)  \
    {                                   \
        return demsph::cudaFail((e), c); \
    }
