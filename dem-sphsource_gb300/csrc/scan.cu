// Exclusive prefix sums over int arrays (cell counts -> cell starts, per-
// particle list counts -> CSR offsets).  Up to 524,288 elements one block
// does it in one launch (kTileScan up to 4096, kScanBlock beyond); longer
// arrays reduce-then-scan in three launches (block sums, scan of block sums,
// block scans plus offsets).  No inter-block waiting, so
// nothing can spin.  Replaces the reference's thrust::inclusive_scan
// (core/neighborSearch.cu:11-17).
#include <cuda_runtime.h>
#include "kernels.cuh"

namespace demsph {

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ int blockExclusiveScan(int v, int& total)
{
    __shared__ int warpSums[SCAN_THREADS / 32];
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
        int s = lane < (int)(blockDim.x >> 5) ? warpSums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warpSums[lane] = s;  // inclusive scan of warp sums
    }
    __syncthreads();
    const int warpOffset = warp ? warpSums[warp - 1] : 0;
    total = warpSums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warpOffset + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) kTileSums(const int* __restrict__ in, int n, int* __restrict__ sums,
                                                          RunIf when)
{
    stepKernelBegin();
    if (!when.active()) return;
    const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) s += in[base + k];
    int total;
    blockExclusiveScan(s, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Scans in[0..n) into out[0..n] (out[n] = total), adding offsets[blockIdx].
__global__ void __launch_bounds__(SCAN_THREADS) kTileScan(const int* __restrict__ in, int n, int* __restrict__ out,
                                                          const int* __restrict__ offsets, RunIf when)
{
    stepKernelBegin();
    if (!when.active()) return;
    const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    int total;
    int run = blockExclusiveScan(s, total) + (offsets ? offsets[blockIdx.x] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = (offsets ? offsets[blockIdx.x] : 0) + total;
}

// The whole scan in one block, for up to SINGLE_MAX elements: tiles of
// 1024 x 16 consecutive elements in turn, each thread scanning its 16 and the
// block its thread totals, with the running total carried between tiles.
// One launch instead of three (most launches of the sort by cell return at
// once: the launch count is what costs).
constexpr int SINGLE_ITEMS = 16;
constexpr int SINGLE_TILE = SCAN_THREADS * SINGLE_ITEMS;
constexpr int SINGLE_MAX = 32 * SINGLE_TILE;

__global__ void __launch_bounds__(SCAN_THREADS) kScanBlock(const int* __restrict__ in, int n, int* __restrict__ out,
                                                           RunIf when)
{
    stepKernelBegin();
    if (!when.active()) return;
    int carry = 0;
    for (int base = 0; base < n; base += SINGLE_TILE) {
        const int first = base + threadIdx.x * SINGLE_ITEMS;
        int v[SINGLE_ITEMS];
        int sum = 0;
#pragma unroll
        for (int k = 0; k < SINGLE_ITEMS; ++k) {
            v[k] = first + k < n ? in[first + k] : 0;
            sum += v[k];
        }
        int total;
        int run = carry + blockExclusiveScan(sum, total);
#pragma unroll
        for (int k = 0; k < SINGLE_ITEMS; ++k) {
            if (first + k < n) out[first + k] = run;
            run += v[k];
        }
        carry += total;
    }
    if (threadIdx.x == 0) out[n] = carry;
}

}  // namespace

size_t scanWorkspaceInts(int n)
{
    size_t tiles = ((size_t)n + SCAN_TILE - 1) / SCAN_TILE;
    size_t w = 0;
    while (tiles > 1) {
        w += 2 * tiles + 1;  // tile sums + their scan (tiles + 1)
        tiles = (tiles + SCAN_TILE - 1) / SCAN_TILE;
    }
    return w + 1;
}

void scanExclusive(const int* in, int* out, int n, int* work, cudaStream_t s, RunIf when)
{
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(int), s);
        return;
    }
    if (n <= SINGLE_MAX && n > SCAN_TILE) {
        launchStep(kScanBlock, 1, SCAN_THREADS, s, in, n, out, when);
        return;
    }
    const int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        launchStep(kTileScan, 1, SCAN_THREADS, s, in, n, out, nullptr, when);
        return;
    }
    int* sums = work;
    int* offs = work + tiles;  // tiles + 1 entries
    launchStep(kTileSums, tiles, SCAN_THREADS, s, in, n, sums, when);
    scanExclusive(sums, offs, tiles, offs + tiles + 1, s, when);
    launchStep(kTileScan, tiles, SCAN_THREADS, s, in, n, out, offs, when);
}

}  // namespace demsph
