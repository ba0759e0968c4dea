// Per-warp schedule of variable-length row work.
//
// Lane l of a warp owns one row holding total(l) items (contacts, candidates).
// Looping over them lane by lane leaves most lanes idle when the counts are
// small and uneven, so the warp instead numbers all its items level by level
// (item 0 of every row, then item 1 of every row, ...: neighbouring items are
// neighbouring rows of the same slot, whose slot arrays [k * nrow + row] are
// then read and written in whole lines) and hands them out 32 at a time, one
// per lane.  Each lane's results go to shared memory; the owning lane then
// takes its own items of the chunk back in item order, so per-row sums and
// list order are exactly those of a lane-by-lane loop.
#pragma once
#include <cuda_runtime.h>

namespace demsph {

// Position of the r-th (from 0) set bit of m; m has more than r set bits.
__device__ __forceinline__ int nthSetBit(unsigned m, int r)
{
    int p = 0;
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) {
        const unsigned low = m & ((1u << w) - 1u);
        const int c = __popc(low);
        if (r >= c) {
            r -= c;
            m >>= w;
            p += w;
        } else {
            m = low;
        }
    }
    return p;
}

// Runs the items of the warp's rows.  Every lane of the warp calls it (the
// lanes of rows that do not exist with total 0).
//   eval(owner, q, valid): evaluates item q of the row of lane `owner` and
//     stores its result in the calling lane's shared slot; called by every
//     lane (valid false on lanes without an item this round), so it may use
//     warp shuffles - with the full mask - before testing `valid`.
//   take(q, pos): called on the owning lane for each of its items q, in
//     increasing q, with the shared slot pos (0..31) holding its result.
// Without take (warpItems(total, eval)) the items only share out the work:
// eval stores its results itself.
template <bool WithTake, typename Eval, typename Take>
__device__ __forceinline__ void warpItemsImpl(int total, Eval&& eval, Take&& take)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int levels = __reduce_max_sync(FULL, total);
    for (int L0 = 0; L0 < levels; L0 += 32) {
        // lane j describes level L0 + j: the lanes holding an item there and
        // the number of the level's first item
        unsigned rows = 0;
        for (int q = L0; q < min(L0 + 32, levels); ++q) {
            const unsigned m = __ballot_sync(FULL, total > q);
            if (lane == q - L0) rows = m;
        }
        const int cnt = __popc(rows);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        const int first = incl - cnt, items = __shfl_sync(FULL, incl, 31);
        for (int c0 = 0; c0 < items; c0 += 32) {
            const int idx = c0 + lane;
            // the item's level: the last lane whose first item is at or before it
            int lv = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (__shfl_sync(FULL, first, lv + step) <= idx) lv += step;
            const unsigned lrows = __shfl_sync(FULL, rows, lv);
            const int owner = nthSetBit(lrows, idx - __shfl_sync(FULL, first, lv)) & 31;
            eval(owner, L0 + lv, idx < items);
            if constexpr (WithTake) {
                __syncwarp();
                // each lane takes its items of this chunk, level by level
                const int lvLo = __shfl_sync(FULL, lv, 0), lvHi = __shfl_sync(FULL, lv, min(31, items - 1 - c0));
                for (int l = lvLo; l <= lvHi; ++l) {
                    const unsigned m = __shfl_sync(FULL, rows, l);
                    const int pos = __shfl_sync(FULL, first, l) + __popc(m & below) - c0;
                    if ((m >> lane & 1u) && pos >= 0 && pos < 32) take(L0 + l, pos);
                }
                __syncwarp();
            }
        }
    }
}

template <typename Eval, typename Take>
__device__ __forceinline__ void warpItems(int total, Eval&& eval, Take&& take)
{
    warpItemsImpl<true>(total, eval, take);
}
template <typename Eval>
__device__ __forceinline__ void warpItems(int total, Eval&& eval)
{
    warpItemsImpl<false>(total, eval, [](int, int) {});
}

}  // namespace demsph
