// Hashed grid: cell keys, counting sort by cell, cell spans.
//
// The reference hashes every particle each step (calculatePointHash,
// core/neighborSearch.cu:19-36), sorts (key, index) pairs with thrust (a
// stable radix sort) and finds cellStart/cellEnd (:38-113).  Here:
//   1. one pass renormalises each position into its cell, computes the key and
//      takes a slot in its cell with an atomic counter;
//   2. an exclusive scan of the counts gives every cell's start;
//   3. each particle is scattered to start + slot;
//   4. within a cell the atomic slots are arbitrary, so each particle's final
//      place is start + (number of particles of the same cell with a smaller
//      original index) - the same (key, index) order as the reference's stable
//      sort, deterministically.
// Fluids are then physically reordered (gathered) into that order; solids keep
// their original order and use the sorted index.  The solid hash also checks
// how far each solid has moved since its contact candidates were built.
#include <algorithm>

#include "kernels.cuh"

namespace demsph {

namespace {

constexpr int T = 256;

// Cell key of fluid slot i every fluid step; on reorder steps the whole
// particle is copied into the gather sources and takes a slot in its cell.
__device__ __forceinline__ void fluidHashOne(const DeviceState& d, int i, const RunIf& sortNow)
{
    int4 c = d.fcell[i];
    float4 h = d.fph[0][i];
    float4 l = d.fpl[0][i];
    renormAxis(c.x, h.x, l.x, d.grid.csx);
    renormAxis(c.y, h.y, l.y, d.grid.csy);
    renormAxis(c.z, h.z, l.z, d.grid.csz);
    const int key = cellKey(c.x, c.y, c.z, d.grid);
    c.w = key;
    if (key == d.grid.num - 1 && !*d.fslowMode) {
        // a fluid particle left the domain: from now on its lists come from the
        // reference's walk (which reaches it through the overflow cell); redo the step
        *(volatile int*)d.fslowMode = 1;
        atomicOr(d.status, ST_MODE_CHANGE);
    }
    if (!sortNow.active()) {
        d.fcell[i] = c;
        d.fph[0][i] = h;
        d.fpl[0][i] = l;
        if (d.cellPack) d.fcp[i] = make_float4(h.x, h.y, h.z, packCell(c));
        return;
    }
    // copy the whole particle into the gather sources
    d.tcell[i] = c;
    d.fph[1][i] = h;
    d.fpl[1][i] = l;
    d.fvh[1][i] = d.fvh[0][i];
    d.fvl[1][i] = d.fvl[0][i];
    d.fdrho[1][i] = d.fdrho[0][i];
    d.tacc[i] = d.facc[i];
    d.tpar[i] = d.fpar[i];
    d.tsumW0[i] = d.fsumW0[i];
    d.tid[i] = d.fid[i];
    d.fkey[i] = key;
    d.fslotInCell[i] = atomicAdd(&d.fcellCount[key], 1);
}

__global__ void kFluidHash(DeviceState d, RunIf sortNow)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nf || *d.status) return;
    fluidHashOne(d, i, sortNow);
}

__global__ void kScatter(int n, const int* __restrict__ key, const int* __restrict__ slotInCell,
                         const int* __restrict__ cellStart, int* __restrict__ out, const int* status, RunIf when)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || *status || !when.active()) return;
    out[cellStart[key[i]] + slotInCell[i]] = i;
}

// Final slot of the element at sorted position p: its cell start plus the
// number of elements of the same cell with a smaller original index.
__device__ __forceinline__ int stableRank(int p, const int* __restrict__ sorted, const int* __restrict__ key,
                                          const int* __restrict__ cellStart, const int* __restrict__ ident, int& e)
{
    e = sorted[p];
    const int k = key[e];
    const int s = cellStart[k], t = cellStart[k + 1];
    const int me = ident ? ident[e] : e;
    int rank = 0;
    for (int q = s; q < t; ++q) {
        const int o = sorted[q];
        rank += (ident ? ident[o] : o) < me;
    }
    return s + rank;
}

__device__ __forceinline__ void fluidGatherOne(const DeviceState& d, int p)
{
    int e;
    const int q = stableRank(p, d.fsortTmp, d.fkey, d.fcellStart, d.tid, e);
    const int4 c = d.tcell[e];
    const float4 h = d.fph[1][e];
    d.fcell[q] = c;
    d.fph[0][q] = h;
    if (d.cellPack) d.fcp[q] = make_float4(h.x, h.y, h.z, packCell(c));
    d.fpl[0][q] = d.fpl[1][e];
    d.fvh[0][q] = d.fvh[1][e];
    d.fvl[0][q] = d.fvl[1][e];
    d.fdrho[0][q] = d.fdrho[1][e];
    d.facc[q] = d.tacc[e];
    d.fpar[q] = d.tpar[e];
    d.fsumW0[q] = d.tsumW0[e];
    const int id = d.tid[e];
    d.fid[q] = id;
    d.fslot[id] = q;
    d.fcellCount[d.fkey[e]] = 0;  // the counts are consumed: clear them for the next reorder
}

__global__ void kFluidGather(DeviceState d, RunIf when)
{
    stepKernelBegin();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.nf || *d.status || !when.active()) return;
    fluidGatherOne(d, p);
}

// Cell keys of the solids every step (they are exported in the reference's
// objectHash); the atomic slots only when the sort follows.
__global__ void kSolidHash(DeviceState d, RunIf sortNow)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.ns || *d.status) return;
    int4 c = d.scell[i];
    float4 h = d.sph[i];
    float4 l = d.spl[i];
    renormAxis(c.x, h.x, l.x, d.grid.csx);
    renormAxis(c.y, h.y, l.y, d.grid.csy);
    renormAxis(c.z, h.z, l.z, d.grid.csz);
    const int key = cellKey(c.x, c.y, c.z, d.grid);
    c.w = key;
    d.scell[i] = c;
    d.sph[i] = h;
    d.spl[i] = l;
    d.skey[i] = key;
    d.skeySearch[i] = key;  // this search uses these keys
    if (sortNow.active()) d.sslotInCell[i] = atomicAdd(&d.scellCount[key], 1);
    const int row = d.srow[i];
    if (row >= 0) {
        const int4 centre = make_int4(truncAxis(c.x, h.x, l.x), truncAxis(c.y, h.y, l.y), truncAxis(c.z, h.z, l.z), 0);
        d.scentre[row] = centre;
        d.scentreSearch[row] = centre;
    }
    if (key == d.grid.num - 1 && row >= 0 && !*d.slowMode) {
        // a solid that can touch others left the domain: from now on the lists
        // come from the reference's walk, which finds it through the overflow
        // cell; this step is redone in that mode
        *(volatile int*)d.slowMode = 1;
        atomicOr(d.status, ST_MODE_CHANGE);
    }
}

// Each solid's slot in its cell, on steps that sort (keys computed at the end
// of the previous step).
__global__ void kSolidSlots(DeviceState d, RunIf when)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.ns || *d.status || !when.active()) return;
    d.sslotInCell[i] = atomicAdd(&d.scellCount[d.skey[i]], 1);
}

__global__ void kSolidRank(DeviceState d, RunIf when)
{
    stepKernelBegin();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.ns || *d.status || !when.active()) return;
    int e;
    const int q = stableRank(p, d.ssortTmp, d.skey, d.scellStart, nullptr, e);
    d.ssorted[q] = e;
    d.scellCount[d.skey[e]] = 0;  // the counts are consumed: clear them for the next sort
}

// The sort by cell of a step in ONE launch (keys from the last integration):
// the slots in the cells, the scan of the counts into the cell starts, the
// scatter and the stable rank of kSolidSlots, scanExclusive, kScatter and
// kSolidRank, as phases of a cooperative launch separated by grid barriers.
// Steps that do not sort pay one launch that returns at once instead of four.
constexpr int SORT_THREADS = 256;
constexpr int SORT_TILE = SORT_THREADS * 16;

// Exclusive scan of counts[0..num) into starts[0..num] by all blocks of a
// cooperative launch: tile sums, a grid barrier, then each tile scanned from
// the sum of the tiles before it, and a closing barrier.  False when a
// barrier gave up (the caller returns).
__device__ bool cooperativeScan(const int* __restrict__ counts, int* __restrict__ starts, int num, int* tileSum,
                                unsigned* bar, unsigned& gen, int* status)
{
    const int tiles = (num + SORT_TILE - 1) / SORT_TILE;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
        const int first = t * SORT_TILE + threadIdx.x * 16;
        int sum = 0;
        for (int k = 0; k < 16; ++k)
            if (first + k < num) sum += counts[first + k];
        int total;
        blockScan<SORT_THREADS>(sum, total);
        if (threadIdx.x == 0) tileSum[t] = total;
    }
    if (!gridBarrier(bar, gen, status)) return false;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
        int before = 0;
        for (int q = threadIdx.x; q < t; q += blockDim.x) before += tileSum[q];
        int offset;
        blockScan<SORT_THREADS>(before, offset);
        const int first = t * SORT_TILE + threadIdx.x * 16;
        int v[16];
        int sum = 0;
        for (int k = 0; k < 16; ++k) {
            v[k] = first + k < num ? counts[first + k] : 0;
            sum += v[k];
        }
        int total;
        int run = offset + blockScan<SORT_THREADS>(sum, total);
        for (int k = 0; k < 16; ++k) {
            if (first + k < num) starts[first + k] = run;
            run += v[k];
        }
        if (t == tiles - 1 && threadIdx.x == 0) starts[num] = offset + total;
    }
    return gridBarrier(bar, gen, status);
}

__global__ void __launch_bounds__(SORT_THREADS) kSolidSortCoop(DeviceState d, RunIf when)
{
    stepKernelBegin();
    // uniform over the blocks: no phase changes these flags or the status
    if (*d.status || !when.active()) return;
    unsigned gen = ((volatile unsigned*)d.gridBar)[1];
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.ns; i += stride)
        d.sslotInCell[i] = atomicAdd(&d.scellCount[d.skey[i]], 1);
    if (!gridBarrier(d.gridBar, gen, d.status)) return;
    if (!cooperativeScan(d.scellCount, d.scellStart, d.grid.num, d.scanWork, d.gridBar, gen, d.status)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.ns; i += stride)
        d.ssortTmp[d.scellStart[d.skey[i]] + d.sslotInCell[i]] = i;
    if (!gridBarrier(d.gridBar, gen, d.status)) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < d.ns; p += stride) {
        int e;
        const int q = stableRank(p, d.ssortTmp, d.skey, d.scellStart, nullptr, e);
        d.ssorted[q] = e;
        d.scellCount[d.skey[e]] = 0;  // the counts are consumed: clear them for the next sort
    }
}

// The fluid hash of a fluid step and, when the fluids are reordered, the
// reorder (scan of the counts, scatter, stable gather) in ONE cooperative
// launch.  Whether to reorder is decided after the hash, from flags and a
// status no later phase changes: a fluid leaving the domain in the hash sets
// the status (the step is redone) and every block returns.
__global__ void __launch_bounds__(SORT_THREADS) kFluidReorderCoop(DeviceState d, RunIf when)
{
    stepKernelBegin();
    if (*d.status) return;
    unsigned gen = ((volatile unsigned*)d.gridBar)[1];
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nf; i += stride) fluidHashOne(d, i, when);
    if (!gridBarrier(d.gridBar, gen, d.status)) return;
    if (*(volatile int*)d.status || !when.active()) return;
    if (!cooperativeScan(d.fcellCount, d.fcellStart, d.grid.num, d.scanWork, d.gridBar, gen, d.status)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.nf; i += stride)
        d.fsortTmp[d.fcellStart[d.fkey[i]] + d.fslotInCell[i]] = i;
    if (!gridBarrier(d.gridBar, gen, d.status)) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < d.nf; p += stride) fluidGatherOne(d, p);
}

}  // namespace

namespace {
// The barrier self-test: the blocks wait for `expected` arrivals with a short
// limit (a missing block makes the wait run out, nothing else).
__global__ void kBarrierProbe(unsigned* bar, int* status, unsigned expected, int spinLimit)
{
    unsigned gen = ((volatile unsigned*)bar)[1];
    gridBarrierN(bar, gen, status, expected, spinLimit);
}
}  // namespace

int selftestBarrier(int missing, int* statusOut)
{
    unsigned* bar = nullptr;
    int* status = nullptr;
    int rc = DEMSPH_OK;
    if (cudaMalloc(&bar, 2 * sizeof(unsigned)) != cudaSuccess || cudaMalloc(&status, sizeof(int)) != cudaSuccess ||
        cudaMemset(bar, 0, 2 * sizeof(unsigned)) != cudaSuccess || cudaMemset(status, 0, sizeof(int)) != cudaSuccess) {
        rc = DEMSPH_ERR_CUDA;
    } else if (!launchCooperative(kBarrierProbe, 2, 32, (cudaStream_t)0, bar, status, 2u + (unsigned)missing,
                                  1 << 16) ||
               cudaDeviceSynchronize() != cudaSuccess ||
               cudaMemcpy(statusOut, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
        rc = DEMSPH_ERR_CUDA;
    }
    cudaFree(bar);
    cudaFree(status);
    return rc;
}

int cooperativeSortBlocks()
{
    int dev = 0, sms = 0, perSm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kSolidSortCoop, SORT_THREADS, 0) != cudaSuccess)
        return 0;
    // two blocks per SM at most: room for other scenes' kernels beside it
    return std::max(0, sms * std::min(perSm, 2));
}

static RunIf fluidReorderWhen(const DeviceState& d, bool force)
{
    RunIf when;
    when.always = force ? 1 : 0;
    when.a = d.frebuild;
    when.b = d.fslowMode;
    return when;
}

void launchFluidHash(const DeviceState& d, bool force, cudaStream_t s)
{
    if (d.nf <= 0) return;
    if (d.sortBlocks > 0) {  // hash and reorder in one cooperative launch
        launchCooperative(kFluidReorderCoop, (unsigned)d.sortBlocks, SORT_THREADS, s, d, fluidReorderWhen(d, force));
        return;
    }
    launchStep(kFluidHash, blocksFor(d.nf, T), T, s, d, fluidReorderWhen(d, force));
}

void launchFluidReorder(const DeviceState& d, bool force, cudaStream_t s)
{
    if (d.nf <= 0 || d.sortBlocks > 0) return;
    // fcellCount is zero here: cleared at creation, by kFluidGather after every
    // reorder, and by the host after a step abandoned in kFluidHash
    const RunIf when = fluidReorderWhen(d, force);
    scanExclusive(d.fcellCount, d.fcellStart, d.grid.num, d.scanWork, s, when);
    launchStep(kScatter, blocksFor(d.nf, T), T, s, d.nf, d.fkey, d.fslotInCell, d.fcellStart, d.fsortTmp, d.status, when);
    launchStep(kFluidGather, blocksFor(d.nf, T), T, s, d, when);
}

static RunIf solidSortWhen(const DeviceState& d, bool force, bool fluidStep, int par)
{
    RunIf when;
    when.always = force ? 1 : 0;
    when.a = d.rebuild + par;
    when.b = d.slowMode;
    if (fluidStep) {
        when.c = d.frebuild;
        when.e = d.fslowMode;
    }
    return when;
}

void launchSolidHash(const DeviceState& d, bool force, bool fluidStep, int par, cudaStream_t s)
{
    if (d.ns <= 0) return;
    if (force)  // positions that no integration has hashed (creation, an upload)
        launchStep(kSolidHash, blocksFor(d.ns, T), T, s, d, solidSortWhen(d, true, fluidStep, par));
    else if (d.sortBlocks <= 0)  // keys come from the last integration of the previous step
        launchStep(kSolidSlots, blocksFor(d.ns, T), T, s, d, solidSortWhen(d, false, fluidStep, par));
}

void launchSolidSort(const DeviceState& d, bool force, bool fluidStep, int par, cudaStream_t s)
{
    if (d.ns <= 0) return;
    if (!force && d.sortBlocks > 0) {
        // the slots were not taken by launchSolidHash: the cooperative launch does everything
        launchCooperative(kSolidSortCoop, (unsigned)d.sortBlocks, SORT_THREADS, s, d,
                          solidSortWhen(d, false, fluidStep, par));
        return;
    }
    // scellCount is zero here: cleared at creation, by kSolidRank after every
    // sort, and by the host after a step abandoned in kSolidHash
    const RunIf when = solidSortWhen(d, force, fluidStep, par);
    scanExclusive(d.scellCount, d.scellStart, d.grid.num, d.scanWork, s, when);
    launchStep(kScatter, blocksFor(d.ns, T), T, s, d.ns, d.skey, d.sslotInCell, d.scellStart, d.ssortTmp, d.status, when);
    launchStep(kSolidRank, blocksFor(d.ns, T), T, s, d, when);
}

}  // namespace demsph
