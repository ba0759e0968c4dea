// Cell sort that allocates nothing: demsph_cell_sort_noalloc.
//
// Some callers cannot allocate device memory at the moment they need this
// sort: a host application whose own allocator has already reserved the
// GPU's memory (so cudaMalloc fails), or a time-critical loop that must not
// take the implicit device synchronisation of cudaMalloc and cudaFree.  For
// them this entry point keeps all of its scratch memory - the per-cell
// counters, the per-particle slots, the scatter buffer and the prefix-sum
// workspace - in one fixed array in device memory, declared below, which
// every GPU that loads this library holds until the process exits.  The call
// reads its bad-key flag back to the host and waits for its stream.
//
// The sort itself is the engine's counting sort by cell (grid.cu): count keys
// with atomic slots, exclusive prefix sum of the counts, scatter, then order
// each cell by original index, which reproduces the reference's stable
// (key, index) sort and its cellStart / cellEnd (core/neighborSearch.cu:38-87).
// Ordering a cell costs each of its elements one pass over the cell, so the
// work grows with the square of the elements per cell: meant for particle
// cell keys (tens per cell); a few thousand per cell still take
// microseconds, but all 524,288 keys in one cell would take seconds.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.cuh"

namespace demsph {
namespace {

// Largest sizes one call accepts: particles and cells.
constexpr int NOALLOC_MAX_N = 1 << 19;
constexpr int NOALLOC_MAX_CELLS = 1 << 19;
// counters (cells + 1) + starts (cells + 1) + slots (n) + scatter (n) + scan workspace
constexpr size_t NOALLOC_SCRATCH_INTS = 2 * (size_t)(NOALLOC_MAX_CELLS + 1) + 2 * (size_t)NOALLOC_MAX_N + 1024;

// The scratch.  In host code this name is only a host-side stand-in for the
// symbol; kernels get its device address, looked up once per device below.
static __device__ __align__(256) int g_noallocScratch[NOALLOC_SCRATCH_INTS];

// Device addresses of the scratch, looked up once per device and context.
// The key is the CUDA context's unique id, not the device alone: after a
// cudaDeviceReset, or in a context a caller made with the driver API, the
// array lives at an address of that context, and a cached address of another
// context would point at freed or foreign memory.
struct ScratchEntry {
    int device;
    unsigned long long context;
    int* address;
};
constexpr int SCRATCH_ENTRIES = 16;
ScratchEntry g_scratchAddr[SCRATCH_ENTRIES] = {};
int g_scratchNext = 0;
std::mutex g_scratchMutex;

typedef int (*CtxGetCurrentFn)(void**);                   // cuCtxGetCurrent
typedef int (*CtxGetIdFn)(void*, unsigned long long*);    // cuCtxGetId
CtxGetCurrentFn g_ctxGetCurrent = nullptr;
CtxGetIdFn g_ctxGetId = nullptr;
std::once_flag g_ctxOnce;

// Unique id of the calling thread's current context; 0 when there is none
// yet (or the driver cannot tell).
unsigned long long currentContextId()
{
    std::call_once(g_ctxOnce, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctxGetCurrent = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctxGetId = reinterpret_cast<CtxGetIdFn>(p);
    });
    void* ctx = nullptr;
    if (!g_ctxGetCurrent || g_ctxGetCurrent(&ctx) != 0 || !ctx) return 0;
    unsigned long long id = 0;
    if (!g_ctxGetId || g_ctxGetId(ctx, &id) != 0) return 0;
    return id;
}

// Device address of the scratch in the current device's current context
// (cudaGetSymbolAddress the first time, with that device current).
cudaError_t scratchAddress(int** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long ctx = currentContextId();
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    if (ctx != 0)
        for (const ScratchEntry& s : g_scratchAddr)
            if (s.address && s.device == dev && s.context == ctx) {
                *out = s.address;
                return cudaSuccess;
            }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noallocScratch);  // makes the device's primary context if there is none
    if (e != cudaSuccess) return e;
    const unsigned long long now = currentContextId();
    if (now != 0) {
        g_scratchAddr[g_scratchNext] = ScratchEntry{dev, now, static_cast<int*>(p)};
        g_scratchNext = (g_scratchNext + 1) % SCRATCH_ENTRIES;
    }
    *out = static_cast<int*>(p);
    return cudaSuccess;
}

__global__ void kCountKeys(const int* __restrict__ keys, int n, int nCells, int* __restrict__ counts,
                           int* __restrict__ slots, int* __restrict__ bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = keys[i];
    if (k < 0 || k >= nCells) {  // reported to the host; the element is left out
        atomicOr(bad, 1);
        slots[i] = -1;
        return;
    }
    slots[i] = atomicAdd(&counts[k], 1);
}

__global__ void kScatterKeys(const int* __restrict__ keys, int n, const int* __restrict__ slots,
                             const int* __restrict__ starts, int* __restrict__ tmp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || slots[i] < 0) return;
    tmp[starts[keys[i]] + slots[i]] = i;
}

// element at scatter position p goes to its cell start + #(same-cell elements with a smaller index)
__global__ void kOrderWithinCells(const int* __restrict__ keys, int n, const int* __restrict__ starts,
                                  const int* __restrict__ tmp, int* __restrict__ sorted)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int e = tmp[p];
    if (e < 0) return;
    const int k = keys[e];
    const int s = starts[k], t = starts[k + 1];
    int rank = 0;
    for (int q = s; q < t; ++q) rank += tmp[q] < e;
    sorted[s + rank] = e;
}

__global__ void kCellSpans(int nCells, const int* __restrict__ starts, int* __restrict__ cellStart,
                           int* __restrict__ cellEnd)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nCells) return;
    const int s = starts[k], t = starts[k + 1];
    cellStart[k] = s == t ? -1 : s;
    cellEnd[k] = s == t ? -1 : t;
}

}  // namespace
}  // namespace demsph

using namespace demsph;

extern "C" int demsph_cell_sort_noalloc(const int* keys, int n, int num_cells, int* sorted_index, int* cell_start,
                                        int* cell_end, void* stream)
{
    if (n < 0 || num_cells < 1 || (n > 0 && (!keys || !sorted_index)) || !cell_start || !cell_end)
        return DEMSPH_ERR_ARGUMENT;
    if (n > NOALLOC_MAX_N || num_cells > NOALLOC_MAX_CELLS) return DEMSPH_ERR_ARGUMENT;
    int* base = nullptr;
    if (scratchAddress(&base) != cudaSuccess) return DEMSPH_ERR_CUDA;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    int* counts = base;                       // num_cells + 1 (last entry: the bad-key flag)
    int* starts = counts + (num_cells + 1);   // num_cells + 1
    int* slots = starts + (num_cells + 1);    // n
    int* tmp = slots + n;                     // n
    int* work = tmp + n;                      // prefix-sum workspace
    if ((size_t)(work - base) + scanWorkspaceInts(num_cells) > NOALLOC_SCRATCH_INTS) return DEMSPH_ERR_ARGUMENT;
    int* bad = counts + num_cells;
    // the array keeps the previous call's contents: clear the counters and flag
    if (cudaMemsetAsync(counts, 0, sizeof(int) * (num_cells + 1), s) != cudaSuccess) return DEMSPH_ERR_CUDA;
    const int T = 256;
    if (n > 0) {
        ++t_kernelLaunches, kCountKeys<<<blocksFor(n, T), T, 0, s>>>(keys, n, num_cells, counts, slots, bad);
        if (cudaMemsetAsync(tmp, 0xff, sizeof(int) * n, s) != cudaSuccess) return DEMSPH_ERR_CUDA;
    }
    scanExclusive(counts, starts, num_cells, work, s);
    if (n > 0) {
        ++t_kernelLaunches, kScatterKeys<<<blocksFor(n, T), T, 0, s>>>(keys, n, slots, starts, tmp);
        ++t_kernelLaunches, kOrderWithinCells<<<blocksFor(n, T), T, 0, s>>>(keys, n, starts, tmp, sorted_index);
    }
    ++t_kernelLaunches, kCellSpans<<<blocksFor(num_cells, T), T, 0, s>>>(num_cells, starts, cell_start, cell_end);
    int flag = 0;
    if (cudaMemcpyAsync(&flag, bad, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return DEMSPH_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return DEMSPH_ERR_CUDA;
    if (cudaGetLastError() != cudaSuccess) return DEMSPH_ERR_CUDA;
    return flag ? DEMSPH_ERR_ARGUMENT : DEMSPH_OK;
}
