// Neighbour and contact lists.
//
// Reference: setFluidInteractionsKernel (core/neighborSearch.cu:115-220) and
// setSolid2SolidInteractionsKernel (:222-312) walk the 27 cells around each
// particle in (z, y, x) order and, within a cell, in (index) order, and keep
// HALF lists (i < j) in CSR form, evaluated from both sides later through
// reverse spans.  Pair membership is decided once per rebuild, on the
// positions of that moment, with FP64 distances.
//
// Here the same walk, the same order and the same membership test (a FP32
// distance with a 1e-5 margin, and a double-float distance inside the margin,
// so decisions agree with the FP64 reference), but:
//   * fluid lists are FULL lists (both directions) per fluid slot, column-major
//     ([k * n + i]) so a warp reads one coalesced 128-byte line per entry, and
//     each entry carries the cell delta of the pair so the SPH loops never
//     load the partner's cell;
//   * solid contacts are a forward CSR (A < B, by original index - the
//     reference's list exactly) plus a per-particle reverse CSR of the lower
//     partners, both filled in walk order; spring history is remapped by
//     looking the pair (A, B) up in A's previous forward segment, which holds
//     the same springs the reference finds through B's reverse span.
#include "kernels.cuh"
#include "contact_rows.cuh"

namespace demsph {

namespace {

constexpr int T = 128;


__device__ __forceinline__ unsigned deltaCode(int dx, int dy, int dz)
{
    if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) return 27u;
    return (unsigned)((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1));
}

__device__ __forceinline__ dfl dfMax(dfl a, dfl b) { return (a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo)) ? a : b; }

// Stencil walk shared by all list builders: calls f(hash, regular, hx, hy, hz)
// for the 27 cells around the (truncated) cell of a point, in the reference's
// order, skipping hashes outside [0, num).  "regular" means the hash is an
// in-domain cell whose coordinates are (hx, hy, hz); otherwise (aliased rows,
// overflow bucket) members carry their own cells.
template <class F>
__device__ __forceinline__ void forStencil(int4 c, float4 h, float4 l, const GridDev& g, F&& f)
{
    const int sx = truncAxis(c.x, h.x, l.x), sy = truncAxis(c.y, h.y, l.y), sz = truncAxis(c.z, h.z, l.z);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int hx = sx + dx, hy = sy + dy, hz = sz + dz;
                const int hash = hz * g.gy * g.gx + hy * g.gx + hx;
                if (hash < 0 || hash >= g.num) continue;
                f(hash, inDomain(hx, hy, hz, g), hx, hy, hz);
            }
}

// ---- fluid lists (full) ----
// One particle's 27-cell walk split over a group of L lanes: lane l takes the
// walk positions t = l, l + L, ...  The group advances in lockstep, one
// candidate per lane per round; the accepted entries of a round are written
// in lane order after the entries of earlier rounds (a warp ballot gives each
// its slot), so the list is complete and its order fixed, though not the
// walk order (exports restore that from the walk positions in the entries).
struct LaneWalk {
    int t, p, pe, hx, hy, hz, hash;
    bool regular;
};

// Next candidate in lane's share of the walk over the cell ranges `start`
// (fluid or solid cells); returns false when the share is exhausted.
template <int L>
__device__ __forceinline__ bool nextCandidate(LaneWalk& w, const int* __restrict__ start, int sx, int sy, int sz,
                                              const GridDev& g, int& idx)
{
    while (w.p >= w.pe) {
        w.t += L;
        if (w.t >= 27) return false;
        const int dx = w.t % 3 - 1, dy = (w.t / 3) % 3 - 1, dz = w.t / 9 - 1;
        w.hx = sx + dx;
        w.hy = sy + dy;
        w.hz = sz + dz;
        w.hash = w.hz * g.gy * g.gx + w.hy * g.gx + w.hx;
        if (w.hash < 0 || w.hash >= g.num) continue;
        w.regular = inDomain(w.hx, w.hy, w.hz, g);
        w.p = start[w.hash];
        w.pe = start[w.hash + 1];
    }
    idx = w.p++;
    return true;
}

// Next cell member in lane's share of a box of cells (x0..x1, y0..y1, z0..z1,
// all inside the domain), cells taken round-robin by the lanes.  Cells whose
// nearest point is beyond the reach (the box's corners and edges) are
// skipped: no particle in them can be a candidate.
struct LaneBox {
    int u, p, pe, x0, y0, z0, nx, ny, nz, hx, hy, hz, hash;
    int ix, iy, iz;  // box-local index of cell u, advanced without dividing
    int4 c;        // the particle's cell
    float4 h;      // and its offset in it
    float reach2;  // squared reach, widened past the FP32 rounding of the cell gaps
};
__device__ __forceinline__ float cellGap(int k, int c, float h, float cs)
{
    const float lo = (float)(k - c) * cs - h, hi = h - (float)(k - c + 1) * cs;
    return fmaxf(0.f, fmaxf(lo, hi));
}
template <int L>
__device__ __forceinline__ bool nextBoxMember(LaneBox& b, const int* __restrict__ start, const GridDev& g, int& idx)
{
    while (b.p >= b.pe) {
        b.u += L;
        if (b.u >= b.nx * b.ny * b.nz) return false;
        b.ix += L;
        while (b.ix >= b.nx) {
            b.ix -= b.nx;
            ++b.iy;
        }
        while (b.iy >= b.ny) {
            b.iy -= b.ny;
            ++b.iz;
        }
        b.hx = b.x0 + b.ix;
        b.hy = b.y0 + b.iy;
        b.hz = b.z0 + b.iz;
        const float gx = cellGap(b.hx, b.c.x, b.h.x, g.cs.x), gy = cellGap(b.hy, b.c.y, b.h.y, g.cs.y),
                    gz = cellGap(b.hz, b.c.z, b.h.z, g.cs.z);
        if (gx * gx + gy * gy + gz * gz > b.reach2) continue;
        b.hash = (b.hz * g.gy + b.hy) * g.gx + b.hx;
        b.p = start[b.hash];
        b.pe = start[b.hash + 1];
    }
    idx = b.p++;
    return true;
}

// The cells within `reach` of a particle at cell c, offset h (clamped to the domain).
__device__ __forceinline__ LaneBox boxAround(int lane, int L, int4 c, float4 h, float reach, const GridDev& g)
{
    LaneBox b;
    b.u = lane - L;
    b.p = b.pe = 0;
    b.x0 = max(0, c.x + (int)floorf((h.x - reach) / g.cs.x));
    b.y0 = max(0, c.y + (int)floorf((h.y - reach) / g.cs.y));
    b.z0 = max(0, c.z + (int)floorf((h.z - reach) / g.cs.z));
    const int x1 = min(g.gx - 1, c.x + (int)floorf((h.x + reach) / g.cs.x));
    const int y1 = min(g.gy - 1, c.y + (int)floorf((h.y + reach) / g.cs.y));
    const int z1 = min(g.gz - 1, c.z + (int)floorf((h.z + reach) / g.cs.z));
    b.nx = max(0, x1 - b.x0 + 1);
    b.ny = max(0, y1 - b.y0 + 1);
    b.nz = max(0, z1 - b.z0 + 1);
    b.hx = b.hy = b.hz = b.hash = 0;
    b.ix = lane - L;  // cell u = lane - L: one advance of L reaches the lane's first cell
    b.iy = b.iz = 0;
    b.c = c;
    b.h = h;
    // the candidate test keeps partners up to 1e-4 past the reach (squared);
    // the gaps carry a few FP32 roundings of the cell size
    const float wide = reach * 1.001f + 1.e-5f * (g.cs.x + g.cs.y + g.cs.z);
    b.reach2 = wide * wide;
    return b;
}

// The walk writes either the lists themselves (BUILD_LISTS: the reference's
// walk every fluid step) or Verlet candidates (within the cut + fskin) that
// kFluidFilter turns into the lists on the following fluid steps.
enum WalkMode { BUILD_LISTS = 0, BUILD_CANDIDATES = 1 };

template <int L, int MODE>
__device__ __forceinline__ void fluidWalk(const DeviceState& d, RunIf when)
{
    const int th = blockIdx.x * blockDim.x + threadIdx.x;
    if ((th & ~31) >= d.nf * L || *d.status || !when.active()) return;
    const int i = th / L, lane = th % L;
    const bool live = i < d.nf;
    const int groupShift = (threadIdx.x & 31) & ~(L - 1);
    const unsigned groupBits = L == 32 ? 0xffffffffu : ((1u << L) - 1u);
    const unsigned below = (1u << lane) - 1u;
    const int n = d.nf;
    const float skin = MODE == BUILD_CANDIDATES ? d.fskin : 0.f;
    const int capF = MODE == BUILD_CANDIDATES ? d.kvf : d.kff;
    const int capS = MODE == BUILD_CANDIDATES ? d.kvs : d.kfs;
    int4 ci = make_int4(0, 0, 0, 0);
    float4 hi = make_float4(0, 0, 0, 0), li = hi;
    dfl hI = df_make(0.f), cutS = hI;
    int sx = 0, sy = 0, sz = 0;
    if (live) {
        ci = d.fcell[i];
        hi = d.fph[0][i];
        li = d.fpl[0][i];
        hI = df_make(hi.w, li.w);
        cutS = df_add(hI, hI);  // fluid-solid: 2 h_i
        sx = truncAxis(ci.x, hi.x, li.x);
        sy = truncAxis(ci.y, hi.y, li.y);
        sz = truncAxis(ci.z, hi.z, li.z);
    }
    // a walk position gives the partner's cell offset from the particle's own
    // cell only when the walk is centred on that cell
    const bool centred = sx == ci.x && sy == ci.y && sz == ci.z;
    // candidates: every cell within the largest cut + skin, all inside the
    // domain (particles outside it send the lists back to the walk)
    LaneBox boxF, boxS;
    if (MODE == BUILD_CANDIDATES) {
        boxF = boxAround(lane, L, ci, hi, 2.f * fmaxf(hi.w, d.fhmax) + skin, d.grid);
        boxS = boxAround(lane, L, ci, hi, 2.f * hi.w + skin, d.grid);
        if (!live) boxF.nx = boxS.nx = 0;
    }
    // fluid partners
    int nff = 0;
    {
        LaneWalk w{lane - L, 0, 0, 0, 0, 0, 0, false};
        while (true) {
            int j = 0;
            const bool has = live && (MODE == BUILD_CANDIDATES ? nextBoxMember<L>(boxF, d.fcellStart, d.grid, j)
                                                               : nextCandidate<L>(w, d.fcellStart, sx, sy, sz, d.grid, j));
            if (MODE == BUILD_CANDIDATES) {
                w.regular = true;
                w.hx = boxF.hx;
                w.hy = boxF.hy;
                w.hz = boxF.hz;
                w.hash = boxF.hash;
            }
            bool take = false;
            int4 cj = make_int4(0, 0, 0, 0);
            if (has && j != i) {
                cj = w.regular ? make_int4(w.hx, w.hy, w.hz, w.hash) : d.fcell[j];
                const float4 hj = d.fph[0][j];
                // FP32 decision away from the cut (most candidates); the exact
                // double-float test within 1e-5 of it
                const float3 r = relF(ci, hi, cj, hj, d.grid);
                const float c = 2.f * fmaxf(hi.w, hj.w) + skin;
                const float d2 = dot3(r, r), c2 = c * c;
                if (MODE == BUILD_CANDIDATES) {
                    take = d2 <= c2 * (1.f + 1.e-4f);
                } else if (d2 < c2 * (1.f - 1.e-5f)) {
                    take = true;
                } else if (d2 <= c2 * (1.f + 1.e-5f)) {
                    const dfl hJ = df_make(hj.w, d.fpl[0][j].w);
                    const dfl rad = dfMax(hI, hJ);
                    take = withinCut(ci, hi, li, cj, hj, d.fpl[0], j, df_add(rad, rad), d.grid);
                }
            }
            const unsigned mine = (__ballot_sync(0xffffffffu, take) >> groupShift) & groupBits;
            if (take) {
                const int slot = nff + __popc(mine & below);
                if (slot < capF) {
                    if (MODE == BUILD_CANDIDATES) d.fvc[(size_t)slot * n + i] = (unsigned)j;
                    else d.ff[(size_t)slot * n + i] = ffEntry(j, w.t, w.regular && centred);
                }
            }
            nff += __popc(mine);
            if (!__any_sync(0xffffffffu, has)) break;
        }
    }
    // solid partners
    int nfs = 0;
    {
        LaneWalk w{lane - L, 0, 0, 0, 0, 0, 0, false};
        while (true) {
            int p = 0;
            const bool has = live && (MODE == BUILD_CANDIDATES ? nextBoxMember<L>(boxS, d.scellStart, d.grid, p)
                                                               : nextCandidate<L>(w, d.scellStart, sx, sy, sz, d.grid, p));
            if (MODE == BUILD_CANDIDATES) {
                w.regular = true;
                w.hx = boxS.hx;
                w.hy = boxS.hy;
                w.hz = boxS.hz;
                w.hash = boxS.hash;
            }
            bool take = false;
            int a = 0;
            if (has) {
                a = d.ssorted[p];
                const int4 ca = w.regular ? make_int4(w.hx, w.hy, w.hz, w.hash) : d.scell[a];
                const float4 ha = d.sph[a];
                const float3 r = relF(ci, hi, ca, ha, d.grid);
                const float c = 2.f * hi.w + skin;
                const float d2 = dot3(r, r), c2 = c * c;
                if (MODE == BUILD_CANDIDATES) take = d2 <= c2 * (1.f + 1.e-4f);
                else if (d2 < c2 * (1.f - 1.e-5f)) take = true;
                else if (d2 <= c2 * (1.f + 1.e-5f)) take = withinCut(ci, hi, li, ca, ha, d.spl, a, cutS, d.grid);
            }
            const unsigned mine = (__ballot_sync(0xffffffffu, take) >> groupShift) & groupBits;
            if (take) {
                const int slot = nfs + __popc(mine & below);
                if (slot < capS) {
                    if (MODE == BUILD_CANDIDATES) d.fvsc[(size_t)slot * n + i] = a;
                    else d.fs[(size_t)slot * n + i] = fsEntry(a, w.t);
                }
            }
            nfs += __popc(mine);
            if (!__any_sync(0xffffffffu, has)) break;
        }
    }
    if (!live || lane != 0) return;
    if (MODE == BUILD_CANDIDATES) {
        d.fvcn[i] = nff;
        d.fvsn[i] = nfs;
        d.fvref[i] = make_float4((float)ci.x * d.grid.cs.x + hi.x, (float)ci.y * d.grid.cs.y + hi.y,
                                 (float)ci.z * d.grid.cs.z + hi.z, 0.f);
        if (nff > capF || nfs > capS) {
            atomicOr(d.status, ST_FVERLET_OVERFLOW);
            atomicMax(&d.need[2], nff);
            atomicMax(&d.need[3], nfs);
        }
    } else {
        d.ffc[i] = nff;
        d.fsc[i] = nfs;
        if (nff > d.kff) atomicOr(d.status, ST_FF_OVERFLOW);
        if (nfs > d.kfs) atomicOr(d.status, ST_FS_OVERFLOW);
    }
}

// Walk position (0..26) of cell cj in the 27-cell walk centred on ci, or -1.
__device__ __forceinline__ int walkPosition(int4 ci, int4 cj)
{
    const int dx = cj.x - ci.x, dy = cj.y - ci.y, dz = cj.z - ci.z;
    if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) return -1;
    return (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
}

// The lists of this fluid step from the candidates (setFluidInteractionsKernel,
// core/neighborSearch.cu:115-220, on positions the candidates cover): the
// reference's test on the current positions, for partners in the 27 cells
// around the particle's current cell (all particles are inside the domain
// here, so those are the cells the reference walks).  The rebuild flag is
// cleared: the last position update of the step raises it again.
//
// P (cellPack): a candidate's cell and position offset come from its filter
// record (one 16-byte read); the smoothing length is every particle's.
#ifndef DEMSPH_FILTER_UNROLL
#define DEMSPH_FILTER_UNROLL 4  // rounds of candidate reads in flight with one lane per particle
#endif
template <int L, bool P>
__device__ __forceinline__ void fluidFilter(const DeviceState& d)
{
    // one lane per particle walks a long candidate list: 4 rounds of reads in
    // flight; with 4 or 8 lanes a round already covers many candidates
    constexpr int FILTER_UNROLL = L == 1 ? DEMSPH_FILTER_UNROLL : (L == 2 ? 2 : 1);
    stepKernelBegin();
    const int th = blockIdx.x * blockDim.x + threadIdx.x;
    if ((th & ~31) >= d.nf * L || *d.status || *d.fslowMode || *d.slowMode) return;
    if (th == 0) *(volatile int*)d.frebuild = 0;
    const int i = th / L, lane = th % L;
    const bool live = i < d.nf;
    const int groupShift = (threadIdx.x & 31) & ~(L - 1);
    const unsigned groupBits = L == 32 ? 0xffffffffu : ((1u << L) - 1u);
    const unsigned below = (1u << lane) - 1u;
    const int n = d.nf;
    int4 ci = make_int4(0, 0, 0, 0);
    float4 hi = make_float4(0, 0, 0, 0), li = hi;
    dfl hI = df_make(0.f), cutS = hI;
    int nc = 0, ns = 0;
    if (live) {
        ci = d.fcell[i];
        hi = d.fph[0][i];
        li = d.fpl[0][i];
        hI = df_make(hi.w, li.w);
        cutS = df_add(hI, hI);
        nc = min(d.fvcn[i], d.kvf);
        ns = min(d.fvsn[i], d.kvs);
    }
    // candidates are taken FILTER_UNROLL rounds of L at a time: the rounds'
    // reads are issued together, their results compacted round by round (the
    // list order of one round per iteration)
    int nff = 0;
    // the next rounds' candidate ids are read while this round's partners are
    // gathered and tested
    int jn[FILTER_UNROLL];
#pragma unroll
    for (int u = 0; u < FILTER_UNROLL; ++u) {
        const int k = u * L + lane;
        jn[u] = k < nc ? (int)d.fvc[(size_t)k * n + i] : -1;
    }
    for (int base = 0; __any_sync(0xffffffffu, base < nc); base += FILTER_UNROLL * L) {
        int j[FILTER_UNROLL];
        int4 cj[FILTER_UNROLL];
        float4 hj[FILTER_UNROLL];
#pragma unroll
        for (int u = 0; u < FILTER_UNROLL; ++u) {
            j[u] = jn[u];
            const int k = base + (FILTER_UNROLL + u) * L + lane;
            jn[u] = k < nc ? (int)d.fvc[(size_t)k * n + i] : -1;
        }
#pragma unroll
        for (int u = 0; u < FILTER_UNROLL; ++u) {
            if (j[u] >= 0) {
                if constexpr (P) {
                    const float4 r = __ldg(d.fcp + j[u]);
                    cj[u] = unpackCell(r.w);
                    hj[u] = make_float4(r.x, r.y, r.z, hi.w);
                } else {
                    cj[u] = d.fcell[j[u]];
                    hj[u] = d.fph[0][j[u]];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < FILTER_UNROLL; ++u) {
            bool take = false;
            int t = -1;
            if (j[u] >= 0) {
                t = walkPosition(ci, cj[u]);
                if (t >= 0) {
                    const float3 r = relF(ci, hi, cj[u], hj[u], d.grid);
                    const float c = 2.f * fmaxf(hi.w, hj[u].w);
                    const float d2 = dot3(r, r), c2 = c * c;
                    if (d2 < c2 * (1.f - 1.e-5f)) {
                        take = true;
                    } else if (d2 <= c2 * (1.f + 1.e-5f)) {
                        const dfl hJ = P ? hI : df_make(hj[u].w, d.fpl[0][j[u]].w);
                        const dfl rad = dfMax(hI, hJ);
                        take = withinCut(ci, hi, li, cj[u], hj[u], d.fpl[0], j[u], df_add(rad, rad), d.grid);
                    }
                }
            }
            const unsigned mine = (__ballot_sync(0xffffffffu, take) >> groupShift) & groupBits;
            if (take) {
                const int slot = nff + __popc(mine & below);
                if (slot < d.kff) d.ff[(size_t)slot * n + i] = ffEntry(j[u], t, true);
            }
            nff += __popc(mine);
        }
    }
    int nfs = 0;
    for (int base = 0; __any_sync(0xffffffffu, base < ns); base += L) {
        const int k = base + lane;
        bool take = false;
        int a = 0, t = -1;
        if (k < ns) {
            a = d.fvsc[(size_t)k * n + i];
            const int4 ca = d.scell[a];
            t = walkPosition(ci, ca);
            if (t >= 0) {
                const float4 ha = d.sph[a];
                const float3 r = relF(ci, hi, ca, ha, d.grid);
                const float d2 = dot3(r, r), c2 = 4.f * hi.w * hi.w;
                if (d2 < c2 * (1.f - 1.e-5f)) take = true;
                else if (d2 <= c2 * (1.f + 1.e-5f)) take = withinCut(ci, hi, li, ca, ha, d.spl, a, cutS, d.grid);
            }
        }
        const unsigned mine = (__ballot_sync(0xffffffffu, take) >> groupShift) & groupBits;
        if (take) {
            const int slot = nfs + __popc(mine & below);
            if (slot < d.kfs) d.fs[(size_t)slot * n + i] = fsEntry(a, t);
        }
        nfs += __popc(mine);
    }
    if (!live || lane != 0) return;
    d.ffc[i] = nff;
    d.fsc[i] = nfs;
    if (nff > d.kff) atomicOr(d.status, ST_FF_OVERFLOW);
    if (nfs > d.kfs) atomicOr(d.status, ST_FS_OVERFLOW);
}
template <int L>
__global__ void __launch_bounds__(T) kFluidFilter(DeviceState d)
{
    fluidFilter<L, false>(d);
}
template <int L>
__global__ void __launch_bounds__(T) kFluidFilterPacked(DeviceState d)
{
    fluidFilter<L, true>(d);
}

// ---- fluid partners of each massive solid (coupling force) ----
__global__ void kCoupCount(DeviceState d)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nf || *d.status) return;
    const int m = min(d.fsc[i], d.kfs);
    for (int k = 0; k < m; ++k) {
        const int a = fsPartner(d.fs[(size_t)k * d.nf + i]);
        if (d.sflags[a].w & F_HASMASS) atomicAdd(&d.coupCount[a], 1);
    }
}
__global__ void kCoupFill(DeviceState d)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nf || *d.status) return;
    if (d.coupStart[d.ns] > d.coupCap) {
        if (i == 0) atomicOr(d.status, ST_COUPLE_OVERFLOW);
        return;
    }
    const int m = min(d.fsc[i], d.kfs);
    for (int k = 0; k < m; ++k) {
        const int a = fsPartner(d.fs[(size_t)k * d.nf + i]);
        if (d.sflags[a].w & F_HASMASS) d.coupList[d.coupStart[a] + atomicAdd(&d.coupCount[a], 1)] = i;
    }
}
// atomics leave each solid's fluid partners in arbitrary order: sort them
__global__ void kCoupSort(DeviceState d)
{
    stepKernelBegin();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= d.ns || *d.status) return;
    const int s = d.coupStart[a], e = d.coupStart[a + 1];
    for (int p = s + 1; p < e; ++p) {
        const int v = d.coupList[p];
        int q = p - 1;
        while (q >= s && d.coupList[q] > v) {
            d.coupList[q + 1] = d.coupList[q];
            --q;
        }
        d.coupList[q + 1] = v;
    }
}

// ---- solid contact lists ----
// One row's contacts of this step (setSolid2SolidInteractionsKernel,
// core/neighborSearch.cu:222-312): the partners that pass the reference's
// test, either from the Verlet candidates or - for grids under 3 cells on an
// axis, or once a solid has left the domain - from the reference's own 27-cell
// walk.  Forward partners (B > A) and reverse partners (B < A) are kept in
// index order, whichever way they were found, so the forces - and their sums
// per solid - do not depend on the candidate margin; the reference's pair
// order (walk order) matters only to exports, which restore it.  Each forward
// pair then takes the springs of the same pair in the previous list (the exact
// history remap of the reference, from the springs the last contact phase
// left in the previous list's slots).  At initialisation (forceWalk) the list
// stays in walk order: bonds are numbered in it.
// The spring history of the forward pairs q = first, first + step, ... of row
// r from the previous list (the pair's springs there, or zeros).
__device__ __forceinline__ void remapSprings(const DeviceState& d, int par, int r, int nf, int first, int step)
{
    const int prev = par ^ 1;
    const size_t nr = (size_t)d.nrow;
    const int prevCnt = min(d.fcnt[prev][r], d.scap);
    for (int q = first; q < nf; q += step) {
        const size_t slot = (size_t)q * nr + r;
        const int b = d.fwd[par][slot];
        float4 s0 = make_float4(0, 0, 0, 0), s1 = s0, s2 = s0;
        for (int k = 0; k < prevCnt; ++k) {
            const size_t ps = (size_t)k * nr + r;
            if (d.fwd[prev][ps] == b) {
                s0 = d.springOut[prev][0][ps];
                s1 = d.springOut[prev][1][ps];
                s2 = d.springOut[prev][2][ps];
                break;
            }
        }
        d.springIn[0][slot] = s0;
        d.springIn[1][slot] = s1;
        d.springIn[2][slot] = s2;
    }
}

__device__ __forceinline__ void detectRow(const DeviceState& d, int par, int forceWalk, bool walk, int r)
{
    // stale candidates are rebuilt first, row by row (the contact force
    // kernel clears the flag once every row has read it)
    if (!walk && d.rebuild[par]) verletBuildRow(d, r);
    const int a = solidOf(d, r);
    const int4 fa = d.sflags[a];
    const int C = d.scap;
    const size_t nr = (size_t)d.nrow;
    int nf = 0, nb = 0;
    auto emit = [&](int b) {
        if (b > a) {
            if (nf < C) d.fwd[par][(size_t)nf * nr + r] = b;
            ++nf;
        } else {
            if (nb < C) d.rev[(size_t)nb * nr + r] = b;
            ++nb;
        }
    };
    if (walk) {
        const int4 ca = d.scell[a];
        const float4 ha = d.sph[a], la = d.spl[a];
        forStencil(ca, ha, la, d.grid, [&](int hash, bool, int, int, int) {
            for (int p = d.scellStart[hash], pe = d.scellStart[hash + 1]; p < pe; ++p) {
                const int b = d.ssorted[p];
                if (solidPairCandidate(d, a, fa, b) && solidsTouch(d, a, b)) emit(b);
            }
        });
    } else {
        const int n = min(d.vcnt[r], d.vcap);
        for (int k = 0; k < n; ++k) {
            const int b = d.vcand[(size_t)k * nr + r];
            if (solidsTouch(d, a, b)) emit(b);
        }
    }
    d.fcnt[par][r] = nf;
    d.rcnt[r] = nb;
    if (nf > C || nb > C) {
        atomicOr(d.status, ST_SS_OVERFLOW);
        atomicMax(&d.need[0], max(nf, nb));
        return;
    }
    if (walk && !forceWalk) {
        sortSlots(d.fwd[par], r, d.nrow, nf);
        sortSlots(d.rev, r, d.nrow, nb);
    }
    for (int q = 0; q < nb; ++q) d.revF[(size_t)q * nr + r].w = 0.f;  // until a forward row's pair force writes it
    remapSprings(d, par, r, nf, 0, 1);
}


// L lanes per row (rows with many candidates): the lanes test the candidates
// in turn and a ballot keeps the lists in candidate order, exactly the lists
// of one lane per row; each lane then remaps the history of every L-th
// forward pair.  The reference's walk (at initialisation, or once a solid has
// left the domain) and stale candidates (their rebuild) run on the row's
// first lane.
template <int L>
__global__ void __launch_bounds__(T) kContactDetect(DeviceState d, int par, int forceWalk)
{
    stepKernelBegin();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if ((t & ~31) >= d.nrow * L || *d.status) return;  // whole warps: the ballots take every lane
    const int r = t / L, lane = t % L;
    const bool live = r < d.nrow;
    const bool walk = forceWalk || *d.slowMode;
    if (L == 1 || walk) {
        if (live && lane == 0) detectRow(d, par, forceWalk, walk, r);
        return;
    }
    // stale candidates are rebuilt first (the contact force kernel clears the
    // flag once every row has read it)
    if (live && lane == 0 && d.rebuild[par]) verletBuildRow(d, r);
    __syncwarp();  // the rebuilt candidates, for the row's other lanes
    const unsigned FULL = 0xffffffffu;
    const int groupShift = (threadIdx.x & 31) & ~(L - 1);
    const unsigned groupBits = (1u << L) - 1u;
    const unsigned below = (1u << lane) - 1u;
    const int C = d.scap;
    const size_t nr = (size_t)d.nrow;
    const int a = live ? solidOf(d, r) : 0;
    const int n = live ? min(d.vcnt[r], d.vcap) : 0;
    int nf = 0, nb = 0;
    for (int base = 0; __any_sync(FULL, base < n); base += L) {
        const int k = base + lane;
        int b = 0;
        bool tf = false, tb = false;
        if (k < n) {
            b = d.vcand[(size_t)k * nr + r];
            if (solidsTouch(d, a, b)) {
                tf = b > a;
                tb = !tf;
            }
        }
        const unsigned mf = (__ballot_sync(FULL, tf) >> groupShift) & groupBits;
        const unsigned mb = (__ballot_sync(FULL, tb) >> groupShift) & groupBits;
        if (tf) {
            const int q = nf + __popc(mf & below);
            if (q < C) d.fwd[par][(size_t)q * nr + r] = b;
        }
        if (tb) {
            const int q = nb + __popc(mb & below);
            if (q < C) {
                d.rev[(size_t)q * nr + r] = b;
                d.revF[(size_t)q * nr + r].w = 0.f;  // until the forward row's pair force writes it
            }
        }
        nf += __popc(mf);
        nb += __popc(mb);
    }
    __syncwarp();  // the list entries, for the lanes that remap them
    if (!live) return;
    if (lane == 0) {
        d.fcnt[par][r] = nf;
        d.rcnt[r] = nb;
    }
    if (nf > C || nb > C) {
        if (lane == 0) {
            atomicOr(d.status, ST_SS_OVERFLOW);
            atomicMax(&d.need[0], max(nf, nb));
        }
        return;
    }
    remapSprings(d, par, r, nf, lane, L);
}

// Contact items (forward and reverse contacts, bonds) per row over at most
// 4096 evenly spaced rows, one row per thread, summed into rowStats (zeroed by
// the caller): the host sizes the rows per warp of the contact force kernel
// from them.
constexpr int ROW_SAMPLES = 4096;
__global__ void kRowStats(DeviceState d, int par)
{
    stepKernelBegin();
    __shared__ int sums[2][8];
    const int stride = max(1, d.nrow / ROW_SAMPLES);
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) * stride;
    int items = 0, rows = 0;
    if (r < d.nrow) {
        const int a = solidOf(d, r);
        items = min(d.fcnt[par][r], d.scap) + min(d.rcnt[r], d.scap) + d.bondStart[a + 1] - d.bondStart[a];
        rows = 1;
    }
    items = __reduce_add_sync(0xffffffffu, items);
    rows = __reduce_add_sync(0xffffffffu, rows);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        sums[0][w] = items;
        sums[1][w] = rows;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        int t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sums[threadIdx.x][k];
        atomicAdd(&d.rowStats[threadIdx.x], t);
    }
}

// ---- bonds at initialisation (addBondData, core/dataBase.cpp:270-308) ----
// Flags over (row, slot) in row-major order: rows ascend with the solid index
// and the initial list is in walk order, so the exclusive scan numbers the new
// bonds in the reference's list order.
__global__ void kBondFlags(DeviceState d, int par, int* flag)
{
    stepKernelBegin();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)d.nrow * d.scap) return;
    const int r = (int)(i / d.scap), k = (int)(i % d.scap);
    int ok = 0;
    if (k < min(d.fcnt[par][r], d.scap)) {
        const int a = solidOf(d, r), b = d.fwd[par][(size_t)k * d.nrow + r];
        const float4 ra = d.srad[a], rb = d.srad[b];
        const dfl dist = dfNorm(relDF(d.scell[a], d.sph[a], d.spl[a], d.scell[b], d.sph[b], d.spl[b], d.grid));
        // skip when r_a + r_b + 1e-10 <= |x_a - x_b|
        const dfl gap = df_sub(df_add_f(df_add(df_make(ra.x, ra.y), df_make(rb.x, rb.y)), 1.e-10f), dist);
        if (df_ge0(gap) && !(gap.hi == 0.f && gap.lo == 0.f)) {
            const int4 fa = d.sflags[a], fb = d.sflags[b];
            const int slot = tableSlot(d.tab, fa.x, fb.x);
            if (slot >= 0 && d.tab.bd[6 * slot + 1] > 1.e-10f && fa.y >= 0 && fa.y == fb.y) ok = 1;
        }
    }
    flag[i] = ok;
}
__global__ void kBondWrite(DeviceState d, int par, const int* flag, const int* pos)
{
    stepKernelBegin();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)d.nrow * d.scap || !flag[i]) return;
    const int r = (int)(i / d.scap), k = (int)(i % d.scap);
    const int b = pos[i];
    const int ii = solidOf(d, r), j = d.fwd[par][(size_t)k * d.nrow + r];
    const DF3 rr = relDF(d.scell[ii], d.sph[ii], d.spl[ii], d.scell[j], d.sph[j], d.spl[j], d.grid);
    const dfl dist = dfNorm(rr);
    const float dd = dist.hi;
    const float3 n = toF3(rr) / dd;
    const float4 ri = d.srad[ii], rj = d.srad[j];
    // contact point - x_i = -(d + r_i - r_j) / 2 * n
    const float lever = -0.5f * (dd + ri.x - rj.x);
    d.bab[b] = make_int2(ii, j);
    d.bon[b] = 1;
    d.bFnTt[b] = make_float4(0, 0, 0, 0);
    d.bFsH[b] = d.bFsL[b] = d.bTbH[b] = d.bTbL[b] = make_float4(0, 0, 0, 0);
    d.bN[b] = f4(n);
    d.bLever[b] = f4(n * lever);
}

// ---- solid normals at initialisation (setSolidNormal, core/dataBase.cpp:348-413) ----
// FP64, once per scene: inside a three-layer wall the kernel-gradient sum of
// the middle layer cancels exactly, and the reference's absolute 1e-10
// threshold then sees an FP64 residue (~1e-15: zero normal) where FP32 would
// leave ~1e-6 (a spurious unit normal).
__global__ void kSolidNormals(DeviceState d, double h)
{
    stepKernelBegin();
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= d.ns) return;
    const int4 ca = d.scell[a];
    const float4 ha = d.sph[a], la = d.spl[a];
    const int4 fa = d.sflags[a];
    const double3 pa = solidAbsPos(d, a);
    const double PI = 3.1415926535897931;
    const double sigma = 21.0 / (16.0 * PI * h * h * h);
    const double hf = h / 1.3;
    const double vFixed = hf * hf * hf;
    // FP32 pre-test: candidates clearly beyond 2h skip the FP64 arithmetic
    // (GB300's FP64 rate is a small fraction of its FP32 rate)
    const float far2 = (float)(4.0 * h * h) * (1.f + 1.e-4f);
    double tx = 0, ty = 0, tz = 0;
    forStencil(ca, ha, la, d.grid, [&](int hash, bool, int, int, int) {
        for (int p = d.scellStart[hash], pe = d.scellStart[hash + 1]; p < pe; ++p) {
            const int b = d.ssorted[p];
            const int4 fb = d.sflags[b];
            const bool fixedPair = !(fa.w & F_MASSIVE) && !(fb.w & F_MASSIVE);  // both inverse mass <= 1e-10
            const bool sameClump = fa.z >= 0 && fa.z == fb.z;
            if (!fixedPair && !sameClump) continue;
            const float3 r32 = relF(ca, ha, d.scell[b], d.sph[b], d.grid);
            if (dot3(r32, r32) > far2) continue;
            const double3 pb = solidAbsPos(d, b);
            const double rx = pa.x - pb.x, ry = pa.y - pb.y, rz = pa.z - pb.z;
            const double rr = sqrt(rx * rx + ry * ry + rz * rz);
            if (rr > 2 * h) continue;
            double vol;
            if (fixedPair) {
                vol = vFixed;
            } else {
                const double s2 = 2.0 * (double)d.srad[b].x + 2.0 * (double)d.srad[b].y;
                vol = s2 * s2 * s2;
            }
            if (rr < 1.e-10 || rr >= 2.0 * h) continue;  // gradient of W is zero
            const double q = rr / h, t = 1.0 - 0.5 * q;
            const double t3 = t * t * t;
            const double dWdq = -2.0 * t3 * (1.0 + 2.0 * q) + 2.0 * t3 * t;
            const double f = sigma * dWdq / h / rr;
            tx -= vol * f * rx;
            ty -= vol * f * ry;
            tz -= vol * f * rz;
        }
    });
    const double l = sqrt(tx * tx + ty * ty + tz * tz);
    d.snormal[a] = l > 1.e-10 ? make_float4((float)(tx / l), (float)(ty / l), (float)(tz / l), 0.f)
                              : make_float4(0, 0, 0, 0);
}

}  // namespace

// The fluid walk of a fluid step in one launch: the reference's walk (at
// initialisation, and every fluid step once a fluid or a solid has left the
// domain), else the Verlet candidates when they are stale - with the contact
// rows' positions at the rebuild (a solid moving half the fluid margin since
// then makes the candidates stale) - else nothing.
template <int L>
__global__ void __launch_bounds__(T) kFluidWalk(DeviceState d, RunIf lists, RunIf cands)
{
    stepKernelBegin();
    if (lists.active()) {
        fluidWalk<L, BUILD_LISTS>(d, lists);
        return;
    }
    if (!cands.active()) return;
    fluidWalk<L, BUILD_CANDIDATES>(d, cands);
    if (*d.status) return;
    const auto ref = [&](int a) {
        const int4 c = d.scell[a];
        const float4 h = d.sph[a];
        d.svref[a] = make_float4((float)c.x * d.grid.cs.x + h.x, (float)c.y * d.grid.cs.y + h.y,
                                 (float)c.z * d.grid.cs.z + h.z, 0.f);
    };
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < d.nrow; r += gridDim.x * blockDim.x) ref(solidOf(d, r));
    // dummy particles given a velocity move too
    if (d.ndummy > 0)
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.nmove; k += gridDim.x * blockDim.x) {
            const int a = d.moveFirst >= 0 ? d.moveFirst + k : d.moveList[k];
            if (rowOf(d, a) < 0) ref(a);
        }
}

void launchFluidWalk(const DeviceState& d, bool walk, cudaStream_t s)
{
    if (d.nf <= 0) return;
    RunIf lists;  // the reference's walk every fluid step (a fluid or a solid left the domain)
    lists.always = walk ? 1 : 0;
    lists.a = d.fslowMode;
    lists.b = d.slowMode;
    RunIf cands;  // Verlet candidates, when stale
    cands.always = 0;
    cands.a = d.frebuild;
    cands.unless = d.fslowMode;
    cands.unless2 = d.slowMode;
    LAUNCH_LANES(kFluidWalk, d.lanes, d.nf, T, s, d, lists, cands);
}

void launchFluidFilter(const DeviceState& d, cudaStream_t s)
{
    if (d.nf <= 0) return;
    if (d.cellPack) LAUNCH_LANES(kFluidFilterPacked, d.lanes, d.nf, T, s, d);
    else LAUNCH_LANES(kFluidFilter, d.lanes, d.nf, T, s, d);
}

void launchCouplingLists(const DeviceState& d, cudaStream_t s)
{
    if (d.nf <= 0 || d.ns <= 0) return;
    cudaMemsetAsync(d.coupCount, 0, sizeof(int) * d.ns, s);
    launchStep(kCoupCount, blocksFor(d.nf, 256), 256, s, d);
    scanExclusive(d.coupCount, d.coupStart, d.ns, d.scanWork, s);
    cudaMemsetAsync(d.coupCount, 0, sizeof(int) * d.ns, s);
    launchStep(kCoupFill, blocksFor(d.nf, 256), 256, s, d);
    launchStep(kCoupSort, blocksFor(d.ns, 256), 256, s, d);
}

void launchContactDetect(const DeviceState& d, int par, bool forceWalk, cudaStream_t s)
{
    if (d.nrow <= 0) return;
    // rows holding many contacts and bonds (the force kernel's rows per warp
    // adapted down to 16 or fewer) have many candidates: four lanes per row
    if (d.forceRows <= 16)
        launchStep(kContactDetect<4>, blocksFor((long long)d.nrow * 4, T), T, s, d, par, forceWalk ? 1 : 0);
    else
        launchStep(kContactDetect<1>, blocksFor(d.nrow, T), T, s, d, par, forceWalk ? 1 : 0);
}

void launchRowStats(const DeviceState& d, int par, cudaStream_t s)
{
    if (d.nrow <= 0) return;
    cudaMemsetAsync(d.rowStats, 0, 2 * sizeof(int), s);
    launchStep(kRowStats, ROW_SAMPLES / 256, 256, s, d, par);
}

// Bond creation from the contact list (addBondData at initialisation,
// core/dataBase.cpp:270-308), in two launches: flags + exclusive scan give each
// new bond its index in list order; returns the bond count (synchronises).
// flag and pos hold nrow * scap + 1 ints.
int launchBondFlags(const DeviceState& d, int par, int* flag, int* pos, int* work, cudaStream_t s)
{
    const long long n = (long long)d.nrow * d.scap;
    if (n <= 0) return 0;
    launchStep(kBondFlags, (unsigned)((n + 255) / 256), 256, s, d, par, flag);
    scanExclusive(flag, pos, (int)n, work, s);
    int nb = 0;
    cudaMemcpyAsync(&nb, pos + n, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return nb;
}

void launchBondWrite(const DeviceState& d, int par, const int* flag, const int* pos, cudaStream_t s)
{
    const long long n = (long long)d.nrow * d.scap;
    if (n <= 0 || d.nb <= 0) return;
    launchStep(kBondWrite, (unsigned)((n + 255) / 256), 256, s, d, par, flag, pos);
}

void launchSolidNormals(const DeviceState& d, double h, cudaStream_t s)
{
    if (d.ns <= 0 || !(h > 0.0)) return;
    launchStep(kSolidNormals, blocksFor(d.ns, T), T, s, d, h);
}

}  // namespace demsph
