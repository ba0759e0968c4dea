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
#include "kernels.cuh"

namespace demsph {

namespace {

constexpr int T = 256;

// Cell keys of the fluids every fluid step; on reorder steps the whole
// particle is copied into the gather sources and takes a slot in its cell.
__global__ void kFluidHash(DeviceState d, RunIf sortNow)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nf || *d.status) return;
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

__global__ void kFluidGather(DeviceState d, RunIf when)
{
    stepKernelBegin();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.nf || *d.status || !when.active()) return;
    int e;
    const int q = stableRank(p, d.fsortTmp, d.fkey, d.fcellStart, d.tid, e);
    d.fcell[q] = d.tcell[e];
    d.fph[0][q] = d.fph[1][e];
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
    if (sortNow.active()) d.sslotInCell[i] = atomicAdd(&d.scellCount[key], 1);
    const int row = d.srow[i];
    if (row >= 0) d.scentre[row] = make_int4(truncAxis(c.x, h.x, l.x), truncAxis(c.y, h.y, l.y), truncAxis(c.z, h.z, l.z), 0);
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

}  // namespace

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
    launchStep(kFluidHash, blocksFor(d.nf, T), T, s, d, fluidReorderWhen(d, force));
}

void launchFluidReorder(const DeviceState& d, bool force, cudaStream_t s)
{
    if (d.nf <= 0) return;
    // fcellCount is zero here: cleared at creation, by kFluidGather after every
    // reorder, and by the host after a step abandoned in kFluidHash
    const RunIf when = fluidReorderWhen(d, force);
    scanExclusive(d.fcellCount, d.fcellStart, d.grid.num, d.scanWork, s, when);
    launchStep(kScatter, blocksFor(d.nf, T), T, s, d.nf, d.fkey, d.fslotInCell, d.fcellStart, d.fsortTmp, d.status, when);
    launchStep(kFluidGather, blocksFor(d.nf, T), T, s, d, when);
}

static RunIf solidSortWhen(const DeviceState& d, bool force, bool fluidStep)
{
    RunIf when;
    when.always = force ? 1 : 0;
    when.a = d.rebuild;
    when.b = d.slowMode;
    if (fluidStep) {
        when.c = d.frebuild;
        when.e = d.fslowMode;
    }
    return when;
}

void launchSolidHash(const DeviceState& d, bool force, bool fluidStep, cudaStream_t s)
{
    if (d.ns <= 0) return;
    if (force)  // positions that no integration has hashed (creation, an upload)
        launchStep(kSolidHash, blocksFor(d.ns, T), T, s, d, solidSortWhen(d, true, fluidStep));
    else        // keys come from the last integration of the previous step
        launchStep(kSolidSlots, blocksFor(d.ns, T), T, s, d, solidSortWhen(d, false, fluidStep));
}

void launchSolidSort(const DeviceState& d, bool force, bool fluidStep, cudaStream_t s)
{
    if (d.ns <= 0) return;
    // scellCount is zero here: cleared at creation, by kSolidRank after every
    // sort, and by the host after a step abandoned in kSolidHash
    const RunIf when = solidSortWhen(d, force, fluidStep);
    scanExclusive(d.scellCount, d.scellStart, d.grid.num, d.scanWork, s, when);
    launchStep(kScatter, blocksFor(d.ns, T), T, s, d.ns, d.skey, d.sslotInCell, d.scellStart, d.ssortTmp, d.status, when);
    launchStep(kSolidRank, blocksFor(d.ns, T), T, s, d, when);
}

}  // namespace demsph
