// All device buffers of one scene, as a plain struct of pointers, and the
// launch functions of the step.  engine.cu owns the allocations; the kernel
// files (grid.cu, lists.cu, sph.cu, dem.cu) only read this struct.
#pragma once
#include <cuda_runtime.h>
#include "engine.cuh"
#include "../../include/demsph_gb300.h"

namespace demsph {

// Bits of a solid's flags word (sflags .w): a dummy wall particle, a solid
// with zero inverse mass (fixed), one with mass above 1e-10, one with any mass.
enum SolidFlagBits { F_DUMMY = 1, F_FIXED = 2, F_MASSIVE = 4, F_HASMASS = 8 };

// Kernel launches issued by this thread (every launch site increments it);
// the engine turns deltas of it into the launch count of a run.
inline thread_local long long t_kernelLaunches = 0;

// Programmatic dependent launch.  The step's kernels are launched with
// programmatic stream serialisation, so a kernel's blocks may be scheduled
// while the kernel before it on the stream is still running, hiding the
// launch gap between the ~10 short kernels of a step.  Every such kernel
// therefore opens with stepKernelBegin(): griddepcontrol.wait holds the block
// until the previous grid has completed and its writes are visible (before
// this block reads or writes anything), then launch_dependents lets the next
// kernel be scheduled.  A kernel launched without the attribute passes both
// instructions at once.
__device__ __forceinline__ void stepKernelBegin()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Whether step kernels overlap their launch with the previous kernel
// (default on; DEMSPH_OVERLAP_LAUNCHES=0 in the environment turns it off).
bool overlapLaunches();

// Launches a step kernel whose blocks wait on one another (grid barriers) as
// a cooperative launch: all its blocks are resident at once, or the launch
// fails.  Returns false when the launch was refused.
template <typename... KArgs, typename... Args>
inline bool launchCooperative(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args)
{
    ++t_kernelLaunches;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...) == cudaSuccess;
}

// Barrier over all blocks of a cooperative launch.  bar[0] counts arrivals
// (the last of `expected` resets it), bar[1] is the generation; `gen` is the
// generation this block waits past (read from bar[1] when the launch began,
// before any barrier of the launch could complete).  The wait is bounded:
// after spinLimit polls (about 0.5 s for gridBarrier's limit) it records
// ST_BARRIER_TIMEOUT and returns false, and the block should return.
__device__ __forceinline__ bool gridBarrierN(unsigned* bar, unsigned& gen, int* status, unsigned expected,
                                             int spinLimit)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        __threadfence();
        if (atomicAdd(&bar[0], 1u) + 1u == expected) {
            bar[0] = 0u;
            __threadfence();
            atomicExch(&bar[1], gen + 1u);
        } else {
            int spins = 0;
            while (((volatile unsigned*)bar)[1] == gen) {
                if (++spins > spinLimit) {
                    atomicOr(status, ST_BARRIER_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
    }
    __syncthreads();
    ++gen;
    return ok != 0;
}
__device__ __forceinline__ bool gridBarrier(unsigned* bar, unsigned& gen, int* status)
{
    return gridBarrierN(bar, gen, status, gridDim.x, 1 << 22);
}

// Block-wide exclusive scan of one value per thread (THREADS threads);
// returns the thread's prefix and sets the block total.  Safe to call again
// right away (it ends with a barrier).
template <int THREADS>
__device__ __forceinline__ int blockScan(int v, int& total)
{
    __shared__ int warpSums[THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int t = lane < THREADS / 32 ? warpSums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < THREADS / 32) warpSums[lane] = t;
    }
    __syncthreads();
    const int before = warp ? warpSums[warp - 1] : 0;
    total = warpSums[THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// Launches a step kernel (one that opens with stepKernelBegin) on stream s.
template <typename... KArgs, typename... Args>
inline void launchStep(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args)
{
    ++t_kernelLaunches;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = overlapLaunches() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

// launchStep with dynamic shared memory.
template <typename... KArgs, typename... Args>
inline void launchStepSmem(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                           Args... args)
{
    ++t_kernelLaunches;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = overlapLaunches() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

struct DeviceState {
    GridDev grid;
    double minB[3], cs[3];   // FP64 grid, for import and export
    float3 g;                // gravity
    double g64[3];
    Tables tab;
    int fixes;
    int* status;             // StatusBits, sticky until the host clears it
    int* stepsDone;          // steps completed since the last reset
    int* scanWork;

    // ---- fluid (slots in cell order) ----
    int nf, kff, kfs;
    int lanes;               // threads per fluid particle in the list and pair loops
    int uniformFluid;        // every fluid particle has the parameters fparU (rest density, sound
    float4 fparU;            // speed, viscosity, mass) and the same smoothing length
    float4 fconstU;          // with them: 4 h^2, 0.5 / h, KG / h^5, 1 / sound speed
    int4* fcell;
    // filter records of uniform fluids on grids of at most 2048 x 2048 x 1024
    // cells (cellPack): the position offset of fph[0] and the cell packed in w
    // (packCell), as each fluid step's hash or reorder leaves them
    float4* fcp;
    int cellPack;
    float4* fph[2];
    float4* fpl[2];
    float4* fvh[2];
    float4* fvl[2];
    float* fdrho[2];
    // partner records of the uniform-fluid pair loops (position offset xyz,
    // density w: one 16-byte gather): [0] position 0 with density 0 (the
    // first continuity pass), [1] position 1 with density 1 (momentum), [2]
    // position 0 with density 1 (the second continuity pass)
    float4* fpd[3];
    float4* facc;
    float4* fpar;
    float2* fsumW0;          // Shepard reference sum / sigma(h), double-float
    int* fid;                // slot -> original index
    int* fslot;              // original index -> slot
    // reorder temporaries
    int4* tcell;
    float4* tacc;
    float4* tpar;
    float2* tsumW0;
    int* tid;
    int* fkey;
    int* fslotInCell;
    int* fsortTmp;
    int* fcellCount;         // grid.num
    int* fcellStart;         // grid.num + 1
    // Verlet candidates of the fluid lists (slots as of the last reorder):
    // partners within the list cut + fskin at the last rebuild
    int kvf, kvs;            // fluid / solid candidates per fluid particle
    unsigned* fvc;           // [k * nf + i]
    int* fvcn;
    int* fvsc;               // [k * nf + i] solid indices
    int* fvsn;
    float4* fvref;           // per fluid slot: position (from the grid origin) at the rebuild
    float4* svref;           // per solid (those with a contact row or moved): the same
    float fskin;
    float fhmax;             // largest fluid smoothing length
    int* frebuild;           // 1: fluid candidates are stale (a fluid or solid moved fskin / 2)
    int* fslowMode;          // 1: fluid lists from the 27-cell walk every fluid step
    // Membership bits (sph_tiles.cu, opt-in): with fluidTiles set the fluids
    // are sorted by cell every fluid step and list membership is kept as one
    // bit per candidate of each particle's 27-cell walk ([w * nf + i], kbits
    // words); the pair loops iterate the bits
    int fluidTiles;
    unsigned* fbits;
    int* fwalk;              // candidates of each fluid slot's walk
    int kbits;
    // lists (column-major, stride nf); with membership bits ff is made from
    // the bits for exports only
    unsigned* ff;
    int* ffc;
    int* fs;
    int* fsc;
    // fluid partners of each solid (for the coupling force), CSR over solids
    int coupCap;
    int* coupCount;          // ns
    int* coupStart;          // ns + 1
    int* coupList;           // coupCap fluid slots

    // ---- solids (original order) ----
    int ns;
    int4* scell;
    float4* sph;             // offset hi, w = inverse mass
    float4* spl;
    // End-of-step offsets (hi, lo) while sph/spl already hold the next step's
    // midpoint: the integration that closes a step and opens the next one in
    // one pass (INTEGRATE_FUSED) leaves them here for the neighbour search
    // between the two halves, which then reads these in place of sph/spl.
    float4* sphE;
    float4* splE;
    float4* svh;
    float4* svl;
    float4* swh;
    float4* swl;
    float4* sacc;
    float4* storque;
    float4* snormal;
    float4* sfcoup;
    float4* srad;            // r hi, r lo, eff hi, eff lo
    int4* sflags;            // material, cluster, clump, dummy
    int* skey;
    int* sslotInCell;
    int* ssorted;            // solid indices in (cell, index) order
    int* ssortTmp;
    int* scellCount;
    int* scellStart;
    // ---- contact lists: fixed slots per non-dummy solid ("row") ----
    // Slot k of row r is element [k * nrow + r] (a warp of consecutive rows
    // reads one line per slot).  Forward contacts (A, B) with B > A live in A's
    // row; two parities alternate between steps so each step's springs are
    // remapped from the previous list.  Reverse entries list the partners
    // A < B of row B.
    int nrow;                // solids that can be in contact (not dummy wall particles)
    int* srow;               // solid -> row, -1 for dummy particles
    int rowsAreSolids;       // 1: every solid has a row, row r is solid r (no dummy particles)
    int nmove;               // solids the integration advances: all but clump pebbles (their clump
    int* moveList;           // moves them) and dummy particles at rest (they never gain velocity)
    int moveFirst;           // >= 0: the list is moveFirst, moveFirst + 1, ... (moveList is not read)
    int* rowSolid;           // row -> solid
    int4* scentre;           // per row: centre cell of the reference's 27-cell walk at the last hash (exports)
    // The keys and walk centres the last neighbour search used: the closing
    // integration of a step rehashes the solids it moved (keys for the next
    // search) and keeps the previous values here, which the reference's
    // objectHash and list order of that step are (exports)
    int* skeySearch;
    int4* scentreSearch;
    int scap;                // slots per row
    int* fwd[2];             // partner id B of each forward slot
    int* fcnt[2];            // forward slots used per row
    int* rev;                // partner id A of each reverse slot
    int* rcnt;
    // sliding, rolling, torsion springs per forward slot: as remapped from the
    // previous list (In) and after the contact forces of the step whose list
    // has parity p (Out[p]); a step reads only the other parity's Out, so a
    // step abandoned after an overflow leaves the history it started from
    float4* springIn[3];
    float4* springOut[2][3];
    float4* pF;              // pair contact force on A, as the reference stores it (exports)
    float4* pT;              // pair contact torque (rolling + torsion), as the reference stores it (exports)
    float4* pTA;             // torque of the pair's contact on A, with its lever arm
    // per reverse slot: minus the pair's force and minus its torque on B (with
    // its lever arm); w 1 once the forward row's pair force wrote it, 0 as the
    // detection leaves it
    float4* revF;
    float4* revT;
    // Verlet candidates: partners within cut + skin at the last rebuild, by id
    int vcap;
    int* vcand;              // [k * nrow + r]
    int* vcnt;
    float4* vref;            // per solid (those with a contact row): position (relative to the
                             // grid origin) at the last rebuild
    float skin;              // candidate margin; a rebuild follows once a solid moved skin / 2
    float vmaxEff;           // largest effective radius of a non-dummy solid
    int* rebuild;            // [p] 1: the candidates are stale for the step whose list has parity p;
                             // set by the drift that ends the step before, cleared after the step
    int* slowMode;           // 1: lists come from the 27-cell walk every step (grid too small, or a solid left the domain)
    // dummy particles (index order) and whether each is in the move list
    // (given a velocity): an upload of the solids' velocities compares them on
    // the device and raises moveChanged when one starts or stops moving
    int ndummy;
    int* dummyIdx;
    unsigned char* dummyMoving;
    int* moveChanged;
    int* need;               // [0] most contacts of a row, [1] most candidates of a row,
                             // [2] / [3] most fluid / solid candidates of a fluid particle,
                             // [4] most walk candidates of a fluid particle in tile mode (for growing)
    // rows per warp of the contact-force kernel (4..32): fewer rows when rows
    // hold many items, so that busy scenes still fill the GPU; results do not
    // depend on it
    int forceRows;
    int* rowStats;           // [0] contact items, [1] rows, over a sample of rows
    unsigned* gridBar;       // [2]: grid barrier of the cooperative sort (arrivals, generation)
    int sortBlocks;          // blocks of the cooperative sort (0: the four-launch sort)

    // ---- infinite walls ----
    int nw;
    float4* wnh;             // normal hi
    float4* wnl;             // normal lo
    float2* wP;              // (p - min) . n, double-float
    int* wmat;
    // wall springs after the contact phase of the step whose list has parity
    // p (the step reads the other parity): [p][j][k * ns + a], wall k, solid a
    float4* wspring[2][3];
    unsigned* wmask[2];      // [p] per solid: bit k (k < 32) set while the springs of wall k may be non-zero

    // ---- bonds ----
    int nb;
    int2* bab;
    int* bon;
    float4* bFnTt;           // normal force hi lo, torsion torque hi lo
    float4* bFsH;
    float4* bFsL;
    float4* bTbH;
    float4* bTbL;
    float4* bN;              // contact normal
    float4* bLever;          // contact point - position of A
    float4* bF;              // this step's bond force on i
    float4* bTA;             // ... torque on i (with lever arm)
    float4* bTB;             // ... torque on j (with lever arm, to subtract)
    int* bondStart;          // bonds of each solid: bondList[bondStart[s] .. bondStart[s + 1])
    int* bondList;
    float4* fsPairForce;     // optional: per fluid-solid pair coupling force of the last step (column-major)

    // ---- clumps ----
    // Centroid (relative to the grid minimum), velocity and spin in
    // double-float; forces in FP32.  GB300's FP64 pipe is two orders of
    // magnitude slower than FP32, so FP64 is left to the orientation and the
    // body-frame inertia, which the step only reads through cIw.
    int nc;
    float4* cpH;
    float4* cpL;
    float4* cvH;
    float4* cvL;
    float4* cwH;
    float4* cwL;
    float4* cacc;
    float4* ctorque;
    float* cIw;              // world-frame inverse inertia R invI R^T, 6 per clump (xx yy zz xy xz yz)
    float* cinvm;
    double4* cq;             // orientation (q0 q1 q2 q3)
    double* cinvI;           // body-frame inverse inertia, 6 per clump (xx yy zz xy xz yz)
    int* cstart;
    int* cend;
    int clumpLanes;          // lanes per clump in the clump kernels: a power of two <= 32 covering most pebbles
};

// Device-side launch condition: a kernel given one does its work when
// `always` is set or either flag is non-zero, and otherwise returns at once
// (work a CUDA graph holds on every step but needs only on some).
struct RunIf {
    int always = 1;
    const int* a = nullptr;
    const int* b = nullptr;
    const int* c = nullptr;
    const int* e = nullptr;
    const int* unless = nullptr;  // when set and non-zero, the kernel does nothing
    const int* unless2 = nullptr;
    __device__ __forceinline__ bool active() const
    {
        if ((unless && *unless) || (unless2 && *unless2)) return false;
        return always || (a && *a) || (b && *b) || (c && *c) || (e && *e);
    }
};

// Lanes per fluid particle in the fluid pair loops and list builder: enough
// threads for every SM (152 SMs x 2048) when the scene is small, one lane per
// particle when it is large.
int fluidLanes(int nf);

// Launches kernel<L> (L in 1, 2, 4, 8) over n items x L lanes.
#define LAUNCH_LANES(kernel, L, n, threads, s, ...)                                                    \
    do {                                                                                               \
        const unsigned blocks_ = (unsigned)blocksFor((long long)(n) * (L), threads);                  \
        switch (L) {                                                                                   \
        case 8: launchStep(kernel<8>, blocks_, threads, s, __VA_ARGS__); break;                        \
        case 4: launchStep(kernel<4>, blocks_, threads, s, __VA_ARGS__); break;                        \
        case 2: launchStep(kernel<2>, blocks_, threads, s, __VA_ARGS__); break;                        \
        default: launchStep(kernel<1>, blocks_, threads, s, __VA_ARGS__); break;                       \
        }                                                                                              \
    } while (0)

// kernel<L, U> for a compile-time flag U.
#define LAUNCH_LANES_U(kernel, U, L, n, threads, s, ...)                                               \
    do {                                                                                               \
        const unsigned blocks_ = (unsigned)blocksFor((long long)(n) * (L), threads);                  \
        switch (L) {                                                                                   \
        case 8: launchStep(kernel<8, U>, blocks_, threads, s, __VA_ARGS__); break;                     \
        case 4: launchStep(kernel<4, U>, blocks_, threads, s, __VA_ARGS__); break;                     \
        case 2: launchStep(kernel<2, U>, blocks_, threads, s, __VA_ARGS__); break;                     \
        default: launchStep(kernel<1, U>, blocks_, threads, s, __VA_ARGS__); break;                    \
        }                                                                                              \
    } while (0)

// scan.cu
size_t scanWorkspaceInts(int n);
void scanExclusive(const int* in, int* out, int n, int* work, cudaStream_t s, RunIf when = RunIf{});

// grid.cu
// Fluid cell keys every fluid step (launchFluidHash); the reorder by cell
// (launchFluidReorder) only when `force`, when the fluid candidates are
// rebuilt, or when the lists come from the walk.
void launchFluidHash(const DeviceState& d, bool force, cudaStream_t s);
void launchFluidReorder(const DeviceState& d, bool force, cudaStream_t s);
// Solid cell keys every step (launchSolidHash); the sort by cell
// (launchSolidSort) only when `force`, when the contact candidates are stale,
// when lists come from the 27-cell walk, or - on fluid steps (fluidStep) -
// when the fluid lists walk the cells.
// par: the parity of the contact list the step builds (its rebuild flag).
void launchSolidHash(const DeviceState& d, bool force, bool fluidStep, int par, cudaStream_t s);
void launchSolidSort(const DeviceState& d, bool force, bool fluidStep, int par, cudaStream_t s);
// Blocks of the one-launch cooperative sort on this device (0 when it cannot
// be used); DEMSPH_COOPERATIVE_SORT=0 in the environment keeps the four-launch
// sort.
int cooperativeSortBlocks();
// Runs two blocks of a cooperative launch at a grid barrier that waits for
// 2 + missing of them, with a short wait limit; stores the status bits.
int selftestBarrier(int missing, int* statusOut);

// lists.cu
// Fluid lists of a fluid step: the reference's walk (walk = true, or once a
// particle has left the domain) or Verlet candidates rebuilt when stale, in
// one launch (launchFluidWalk); otherwise the candidates are filtered every
// fluid step (launchFluidFilter).
void launchFluidWalk(const DeviceState& d, bool walk, cudaStream_t s);
void launchFluidFilter(const DeviceState& d, cudaStream_t s);
void launchCouplingLists(const DeviceState& d, cudaStream_t s);

// sph_tiles.cu: the fluid lists as membership bits and the pair loops over
// them (opt-in).  launchFluidTileLists (fluid steps, after the reorder and
// the solid sort): the membership bits and the solid partner lists.
void launchFluidTileLists(const DeviceState& d, cudaStream_t s);
void launchTileContinuity(const DeviceState& d, int which, double dtf, cudaStream_t s, bool countStep);
void launchTileMomentum(const DeviceState& d, double dtf, cudaStream_t s);
void launchTileShepard(const DeviceState& d, int iStep, cudaStream_t s);
// The reference's fluid list (entries in walk order, as the list kernels
// write them) from the membership bits, for exports.
void launchBitsToLists(const DeviceState& d, cudaStream_t s);
// The contact rows of the step, each row first rebuilding its candidates when
// they are stale (launchContactDetect; forceWalk: from the reference's 27-cell
// walk, in the reference's order).
void launchContactDetect(const DeviceState& d, int parity, bool forceWalk, cudaStream_t s);
// Contact items over a sample of rows, into rowStats.
void launchRowStats(const DeviceState& d, int parity, cudaStream_t s);
int launchBondFlags(const DeviceState& d, int parity, int* flag, int* pos, int* work, cudaStream_t s);
void launchBondWrite(const DeviceState& d, int parity, const int* flag, const int* pos, cudaStream_t s);
void launchSolidNormals(const DeviceState& d, double h, cudaStream_t s);

// sph.cu
void launchDensityReinit(const DeviceState& d, int iStep, cudaStream_t s);
// which = 0: first half step (densities 0 -> 1, positions drift 0 -> 1);
// which = 1: second half step (densities 1 -> 0, velocities 1 -> 0).
// countStep: the pass counts the step in stepsDone (the last kernel of a step)
void launchContinuityPass(const DeviceState& d, int which, double dtf, cudaStream_t s, bool countStep = false);
// momentum + kick (dt_f) + drift (dt_f / 2): reads buffers [1], writes velocity [1], position [0].
void launchMomentumPass(const DeviceState& d, double dtf, cudaStream_t s);
void launchCoupling(const DeviceState& d, int src, cudaStream_t s);
void launchCouplingPairForces(const DeviceState& d, int src, float4* out, cudaStream_t s);

// dem.cu
// The step's contact forces, once per contact, and the bonds.
void launchPairForces(const DeviceState& d, int parity, float dt, cudaStream_t s);
// Contact, bond, wall, coupling and gravity forces of every solid, summed
// from the pair results of launchPairForces.  integrate (INTEGRATE_AFTER or
// INTEGRATE_FUSED; -1 none): each row's thread then runs its solid's
// integration pass (only when the integrated solids are exactly the rows);
// countStep as launchSolidIntegrate's.
void launchSolidForces(const DeviceState& d, int parity, double dt, cudaStream_t s, int integrate = -1,
                       bool countStep = false);
// The contact list of a plain DEM step opened by a fused integration pass and
// its contact forces in one launch (no bonds; candidates, not the walk):
// each row filters its candidates on the end-of-step offsets (sphE/splE) and
// the contact forces then act at the midpoint (sph/spl), springs remapped by
// both sides of a pair from the previous list.  Raises ST_SPLIT_CONTACTS,
// before any write, when the lists must come from the walk.
void launchContactForces(const DeviceState& d, int parity, float dt, cudaStream_t s);
void launchClumpForce(const DeviceState& d, cudaStream_t s);
// Kinds of solid integration pass: the half step after the contact forces
// (closing a step), the half step before them (opening one), or both in one
// pass - the closing half of step n, then the opening half of step n + 1 from
// the same forces (the neighbour search of step n + 1, which moves nothing,
// runs after it on the end-of-step offsets in sphE/splE).
enum IntegrateMode { INTEGRATE_AFTER = 0, INTEGRATE_BEFORE = 1, INTEGRATE_FUSED = 2 };
// Half-step integration of all solids; clumpForce: sum the clumps' pebble
// forces first (instead of launchClumpForce); countStep: count the step.
// par: the parity of the contact list of the step a closing half ends (its
// margin check raises d.rebuild[par ^ 1], the next step's flag).
void launchSolidIntegrate(const DeviceState& d, double dt, int mode, int par, bool clumpForce, bool countStep,
                          cudaStream_t s);

// Absolute FP64 position of solid i (cell origin + double-float offset).
__device__ __forceinline__ double3 solidAbsPos(const DeviceState& d, int i)
{
    const int4 c = d.scell[i];
    const float4 h = d.sph[i], l = d.spl[i];
    return make_double3(d.minB[0] + c.x * d.cs[0] + ((double)h.x + (double)l.x),
                        d.minB[1] + c.y * d.cs[1] + ((double)h.y + (double)l.y),
                        d.minB[2] + c.z * d.cs[2] + ((double)h.z + (double)l.z));
}

// Row of solid a (-1 for a dummy particle) and solid of row r: the identity,
// without a read, when every solid has a row.
__device__ __forceinline__ int rowOf(const DeviceState& d, int a) { return d.rowsAreSolids ? a : d.srow[a]; }
__device__ __forceinline__ int solidOf(const DeviceState& d, int r) { return d.rowsAreSolids ? r : d.rowSolid[r]; }

// After the last drift of a step: once a solid that can touch others (row >=
// 0) has moved half the candidate margin since the candidates were built, the
// next step rebuilds them (stale: that step's flag, d.rebuild[next parity]);
// once any moved solid (a dummy particle given a velocity too) has moved half
// the fluid candidates' margin, the fluid candidates are rebuilt.  c, h: its
// cell and offset after the drift; p0, q0: vref and svref of the solid.
__device__ __forceinline__ void checkDisplacementOf(const DeviceState& d, int* stale, int row, int4 c, float4 h,
                                                    float4 p0, float4 q0)
{
    if (row >= 0) {
        const float dx = (float)c.x * d.grid.cs.x + h.x - p0.x, dy = (float)c.y * d.grid.cs.y + h.y - p0.y,
                    dz = (float)c.z * d.grid.cs.z + h.z - p0.z;
        const float half = 0.5f * d.skin;
        if (!(dx * dx + dy * dy + dz * dz <= half * half)) *(volatile int*)stale = 1;
    }
    if (d.nf > 0) {  // the fluid candidates' solid partners
        const float ex = (float)c.x * d.grid.cs.x + h.x - q0.x, ey = (float)c.y * d.grid.cs.y + h.y - q0.y,
                    ez = (float)c.z * d.grid.cs.z + h.z - q0.z;
        const float fh = 0.5f * d.fskin;
        if (!(ex * ex + ey * ey + ez * ez <= fh * fh)) *(volatile int*)d.frebuild = 1;
    }
}
__device__ __forceinline__ void checkDisplacement(const DeviceState& d, int* stale, int i)
{
    const int r = rowOf(d, i);
    if (r < 0) return;
    checkDisplacementOf(d, stale, r, d.scell[i], d.sph[i], d.vref[i],
                        d.nf > 0 ? d.svref[i] : make_float4(0, 0, 0, 0));
}

// Cell key of solid i for the next step's neighbour search, at the end of
// this step (the position it starts from): the offset is renormalised into its
// cell, the key and the walk centre stored; a solid that can touch others and
// has left the domain sends the next lists to the reference's walk.  c, h, l:
// the solid's cell and offset after its last drift.
// rehashSolidTo leaves the renormalised offset in h, l and stores it to
// outH, outL (sph, spl; sphE, splE when the next step's first half is
// integrated in the same pass).
__device__ __forceinline__ void rehashSolidTo(const DeviceState& d, int i, int row, int4 c, float4& h, float4& l,
                                              float4* outH, float4* outL)
{
    renormAxis(c.x, h.x, l.x, d.grid.csx);
    renormAxis(c.y, h.y, l.y, d.grid.csy);
    renormAxis(c.z, h.z, l.z, d.grid.csz);
    const int key = cellKey(c.x, c.y, c.z, d.grid);
    c.w = key;
    d.scell[i] = c;
    outH[i] = h;
    outL[i] = l;
    d.skeySearch[i] = d.skey[i];
    d.skey[i] = key;
    if (row >= 0) {
        d.scentreSearch[row] = d.scentre[row];
        d.scentre[row] = make_int4(truncAxis(c.x, h.x, l.x), truncAxis(c.y, h.y, l.y), truncAxis(c.z, h.z, l.z), 0);
        if (key == d.grid.num - 1) *(volatile int*)d.slowMode = 1;
    }
}
__device__ __forceinline__ void rehashSolidOf(const DeviceState& d, int i, int row, int4 c, float4 h, float4 l)
{
    rehashSolidTo(d, i, row, c, h, l, d.sph, d.spl);
}
// withEnd: the end-of-step offset also goes to sphE, splE.
__device__ __forceinline__ void rehashSolid(const DeviceState& d, int i, bool withEnd = false)
{
    float4 h = d.sph[i], l = d.spl[i];
    rehashSolidTo(d, i, rowOf(d, i), d.scell[i], h, l, d.sph, d.spl);
    if (withEnd) {
        d.sphE[i] = h;
        d.splE[i] = l;
    }
}


// The fluid counterpart for fluid slot i: renormalised offset, cell key, the
// walk once a fluid leaves the domain, and stale list candidates once it has
// moved half their margin.
__device__ __forceinline__ void rehashFluid(const DeviceState& d, int i)
{
    int4 c = d.fcell[i];
    float4 h = d.fph[0][i], l = d.fpl[0][i];
    renormAxis(c.x, h.x, l.x, d.grid.csx);
    renormAxis(c.y, h.y, l.y, d.grid.csy);
    renormAxis(c.z, h.z, l.z, d.grid.csz);
    c.w = cellKey(c.x, c.y, c.z, d.grid);
    d.fcell[i] = c;
    d.fph[0][i] = h;
    d.fpl[0][i] = l;
    if (c.w == d.grid.num - 1) *(volatile int*)d.fslowMode = 1;
    const float4 p0 = d.fvref[i];
    const float dx = (float)c.x * d.grid.cs.x + h.x - p0.x, dy = (float)c.y * d.grid.cs.y + h.y - p0.y,
                dz = (float)c.z * d.grid.cs.z + h.z - p0.z;
    const float half = 0.5f * d.fskin;
    if (!(dx * dx + dy * dy + dz * dz <= half * half)) *(volatile int*)d.frebuild = 1;
}

// First entry of a list of consecutive solid indices, or -1.
inline int consecutiveFirst(const int* v, size_t n)
{
    for (size_t k = 1; k < n; ++k)
        if (v[k] != v[0] + (int)k) return -1;
    return n ? v[0] : 0;
}

inline int blocksFor(long long n, int threads) { return (int)((n + threads - 1) / threads > 0 ? (n + threads - 1) / threads : 1); }

}  // namespace demsph
