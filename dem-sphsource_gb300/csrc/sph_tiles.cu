// Fluid lists as membership bits and the WCSPH pair loops over them ("tile
// mode", an alternative to the list kernels of lists.cu / sph.cu; selected
// with DEMSPH_FLUID_TILES=1).
//
// The fluids are sorted by (cell, original index) at every fluid step, so the
// 27 cells a particle's list walks (core/neighborSearch.cu:135-149: z, y, x
// loops; cells in index order) are nine runs of consecutive slots.
// Membership of the reference's lists is decided once per fluid step, where
// the reference builds them (kWalkBuild, in the neighbour search): the test
// 2 max(h_i, h_j) - |x_i - x_j| >= 0 on the positions of that moment (FP32
// away from the cut, double-float within 1e-5 of it), kept as one bit per
// candidate of the particle's walk, in walk order.  Those bits are the
// reference's list (both halves of it), 4 B per 32 candidates instead of 4 B
// per partner, and no candidate filter runs on later steps.  Every pass of
// the step (Shepard, continuity, momentum, continuity) then iterates the set
// bits only, each thread walking its own cells through the cell starts and
// reading its partners in place (consecutive particles share their walks'
// lines in L1).  Solid partners stay an explicit list (fs), written by the
// same kernel in walk order, because only particles near walls or grains
// have any.
//
// Measured against the list kernels on GB300 it is slower (the per-step walk
// over all 27 cells costs more than filtering the Verlet candidates, and the
// passes are not faster), so the list kernels stay the default; a variant
// that staged each pencil of cells in shared memory measured slower still and
// was not kept.
#include <algorithm>

#include "contact_rows.cuh"
#include "sph_common.cuh"

namespace demsph {

namespace {

using namespace sph;

constexpr int TT = 128;  // threads per block

// Solid partners of fluid slot p (setFluidInteractionsKernel's second list,
// core/neighborSearch.cu:115-220): the solids within 2 h of it, in the
// reference's walk order over the solid cells, as list entries (fs).  Aliased
// cells (a walk position outside the domain) are skipped: they hold no
// partner when every axis has three cells or more and every solid is inside
// the domain (tile mode).
__device__ __forceinline__ void buildSolidPartners(const DeviceState& d, int p, int4 ci, float4 hi, float4 li,
                                                   dfl cutDF, float c2)
{
    const int n = d.nf;
    int nfs = 0;
    for (int t = 0; t < 27; ++t) {
        const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
        const int x = ci.x + dx, y = ci.y + dy, z = ci.z + dz;
        if (!inDomain(x, y, z, d.grid)) continue;
        const int key = (z * d.grid.gy + y) * d.grid.gx + x;
        for (int q = d.scellStart[key], e = d.scellStart[key + 1]; q < e; ++q) {
            const int a = d.ssorted[q];
            const int4 ca = d.scell[a];
            const float4 ha = d.sph[a];
            const float3 r = relF(ci, hi, ca, ha, d.grid);
            const float d2 = dot3(r, r);
            bool take = false;
            if (d2 < c2 * (1.f - 1.e-5f)) take = true;
            else if (d2 <= c2 * (1.f + 1.e-5f)) take = withinCut(ci, hi, li, ca, ha, d.spl, a, cutDF, d.grid);
            if (take) {
                if (nfs < d.kfs) d.fs[(size_t)nfs * n + p] = fsEntry(a, t);
                ++nfs;
            }
        }
    }
    d.fsc[p] = nfs;
    if (nfs > d.kfs) atomicOr(d.status, ST_FS_OVERFLOW);
}

// ---- pair terms and per-particle epilogues ----

// Continuity term of fluid partner j (uniform fluid; kContinuity's U branch):
// false when j is beyond the kernel's support.
__device__ __forceinline__ bool continuityTerm(const DeviceState& d, const Self& o, float negTwoRhoM, float3 r,
                                               float drj, float3 vj, float& term)
{
    const float r2 = dot3(r, r);
    if (r2 >= d.fconstU.x) return false;
    const float rhoj = d.fparU.x + drj;
    const float Pj = drj * d.fparU.y * d.fparU.y;
    const float rr = sqrtf(r2);
    const float tt = 1.f - rr * d.fconstU.y;
    const float G = d.fconstU.z * tt * tt * tt;
    const float3 vij = o.v - vj;
    term = negTwoRhoM * G / (rhoj * (o.rho + rhoj)) * (rhoj * dot3(vij, r) + (o.P - Pj) * rr * d.fconstU.w);
    return true;
}

// Momentum term of fluid partner j (kMomentum's U branch).
__device__ __forceinline__ bool momentumTerm(const DeviceState& d, const Self& o, float twoNuRhoI, float twoVi,
                                             float3 r, float drj, float3 vj, float3& term)
{
    const float r2 = dot3(r, r);
    if (r2 >= d.fconstU.x) return false;
    const float c = d.fparU.y;
    const float rhoj = d.fparU.x + drj;
    const float Pj = drj * c * c;
    const float rr = sqrtf(r2);
    const float tt = 1.f - rr * d.fconstU.y;
    const float G = d.fconstU.z * tt * tt * tt;
    const float3 vij = o.v - vj;
    const float dU = -dot3(vij, r) / rr;  // U_L - U_R
    const float beta = fminf(3.f * fmaxf(dU, 0.f), c);
    const float invSum = 1.f / (o.rho + rhoj);
    const float Ps = (o.rho * Pj + rhoj * o.P + o.rho * rhoj * beta * dU) * invSum;
    const float gbar = twoNuRhoI * rhoj * invSum;  // 2 g_i g_j / (g_i + g_j), g = nu rho
    const float w = twoVi * G / rhoj;              // 2 V_i V_j G / m, V_j = m / rho_j
    term = (r * Ps - vij * gbar) * w;
    return true;
}

// Solid partners (the fs list) of the continuity and momentum passes.
__device__ __forceinline__ void continuitySolids(const DeviceState& d, const Self& o, int p, KahanF& acc)
{
    const int nfs = min(d.fsc[p], d.kfs);
    const float ci2 = o.cs * o.cs;
    for (int k = 0; k < nfs; ++k) {
        const int sa = fsPartner(d.fs[(size_t)k * d.nf + p]);
        const SolidPartner sp = solidPartner(d, o.c, o.p, o.h, o.P, o.rho, o.rho0, ci2, sa);
        if (!sp.inside) continue;
        acc.add(-2.f * o.rho * sp.Va * sp.G / (o.rho + sp.rhoa) *
                (2.f * sp.rhoa * dot3(o.v - sp.v, sp.r) + (o.P - sp.Pa) * sp.rr / o.cs));
    }
}
__device__ __forceinline__ void momentumSolids(const DeviceState& d, const Self& o, int p, KahanF3& acc)
{
    const int nfs = min(d.fsc[p], d.kfs);
    const float ci2 = o.cs * o.cs;
    for (int k = 0; k < nfs; ++k) {
        const int sa = fsPartner(d.fs[(size_t)k * d.nf + p]);
        const SolidPartner sp = solidPartner(d, o.c, o.p, o.h, o.P, o.rho, o.rho0, ci2, sa);
        if (!sp.inside) continue;
        const float3 via = o.v - sp.v;
        const float dU = -2.f * dot3(via, xyz(d.snormal[sa]));
        const float beta = fminf(3.f * fmaxf(dU, 0.f), o.cs);
        const float Ps = (o.rho * sp.Pa + sp.rhoa * o.P + o.rho * sp.rhoa * beta * dU) / (o.rho + sp.rhoa);
        const float w = 2.f * o.V * sp.Va * sp.G / o.m;
        acc.add((sp.r * Ps - via * (2.f * o.gam)) * w);
    }
}

struct TileContinuityArgs {
    int ps, vs, ds, dd, driftTo, velCopyTo, countStep;
    float dt;
    dfl drift;
};

__device__ __forceinline__ void continuityFinish(const DeviceState& d, const TileContinuityArgs& a, int p, float sum)
{
    d.fdrho[a.dd][p] = d.fdrho[a.ds][p] + a.dt * sum;
    if (a.driftTo >= 0) {
        float4 xh = d.fph[a.ps][p], xl = d.fpl[a.ps][p];
        dfAxpy(xh, xl, d.fvh[a.vs][p], d.fvl[a.vs][p], a.drift);
        d.fph[a.driftTo][p] = xh;
        d.fpl[a.driftTo][p] = xl;
    }
    if (a.velCopyTo >= 0) {
        d.fvh[a.velCopyTo][p] = d.fvh[a.vs][p];
        d.fvl[a.velCopyTo][p] = d.fvl[a.vs][p];
    }
}

// Kick (dt_f) and drift (dt_f / 2) after momentum: reads velocity [0] and
// position [1], writes acc, velocity [1] and position [0].
__device__ __forceinline__ void momentumFinish(const DeviceState& d, int p, float3 sum, dfl dtf, dfl halfDtf)
{
    const float3 acl = sum + d.g;
    d.facc[p] = f4(acl);
    const float4 vh0 = d.fvh[0][p], vl0 = d.fvl[0][p];
    const dfl vx = df_add(df_make(vh0.x, vl0.x), df_mul_f(dtf, acl.x));
    const dfl vy = df_add(df_make(vh0.y, vl0.y), df_mul_f(dtf, acl.y));
    const dfl vz = df_add(df_make(vh0.z, vl0.z), df_mul_f(dtf, acl.z));
    const float4 vhN = make_float4(vx.hi, vy.hi, vz.hi, 0.f), vlN = make_float4(vx.lo, vy.lo, vz.lo, 0.f);
    d.fvh[1][p] = vhN;
    d.fvl[1][p] = vlN;
    float4 xh = d.fph[1][p], xl = d.fpl[1][p];
    dfAxpy(xh, xl, vhN, vlN, halfDtf);
    d.fph[0][p] = xh;
    d.fpl[0][p] = xl;
}

// Shepard sums (kDensityReinit): the solid partners, then the update.
__device__ __forceinline__ void shepardFinish(const DeviceState& d, int p, int4 ci, float4 pi, float4 li, dfl invh,
                                              dfl twoH, dfl S, int storeReference)
{
    const dfl k26 = df_from_double(2.6);
    const int nfs = min(d.fsc[p], d.kfs);
    for (int k = 0; k < nfs; ++k) {
        const int a = fsPartner(d.fs[(size_t)k * d.nf + p]);
        const dfl r = dfNorm(relDF(ci, pi, li, d.scell[a], d.sph[a], d.spl[a], d.grid));
        if (df_ge0(df_sub(r, twoH))) continue;
        const float4 ra = d.srad[a];
        const dfl x = df_mul(df_mul(k26, df_make(ra.x, ra.y)), invh);
        const dfl vr = df_mul(df_mul(x, x), x);
        S = df_add(S, df_mul(shepardTerm(r, invh), vr));
    }
    if (storeReference) {
        d.fsumW0[p] = make_float2(S.hi, S.lo);
    } else {
        const float2 s0 = d.fsumW0[p];
        const dfl diff = df_sub(S, df_make(s0.x, s0.y));
        const float rho0 = d.fpar[p].x;
        const float cand = rho0 * ((diff.hi + diff.lo) / s0.x);
        d.fdrho[0][p] = fmaxf(d.fdrho[0][p], cand);
    }
}

// Shepard term of fluid partner j (double-float distance from the cells).
__device__ __forceinline__ void shepardFluid(const DeviceState& d, int4 ci, float4 pi, float4 li, int ddx, int ddy,
                                             int ddz, float4 hj, float4 lj, dfl invh, dfl twoH, dfl& S)
{
    DF3 rv;
    rv.x = relAxis(ci.x, pi.x, li.x, ci.x + ddx, hj.x, lj.x, d.grid.csx);
    rv.y = relAxis(ci.y, pi.y, li.y, ci.y + ddy, hj.y, lj.y, d.grid.csy);
    rv.z = relAxis(ci.z, pi.z, li.z, ci.z + ddz, hj.z, lj.z, d.grid.csz);
    const dfl r = dfNorm(rv);
    if (df_ge0(df_sub(r, twoH))) return;  // q >= 2
    S = df_add(S, shepardTerm(r, invh));
}

// ---- the walks: one thread per particle in slot order ----
// Walks a particle's cells in the reference's order (z, y, x loops) through
// the cell starts; candidate k lies in the cell whose range [bStart, bEnd)
// holds it.
struct WalkCursor {
    int dx, dy, dz;
    int bStart, bEnd;
    int slotBase;          // slot of candidate k = slotBase + k
    float3 oi;             // x_i - x_j = oi - o_j for partners in the current cell
    __device__ __forceinline__ void start()
    {
        dx = 1;
        dy = 1;
        dz = -2;
        bStart = bEnd = 0;
    }
    __device__ __forceinline__ bool seek(int k, int4 ci, float3 o, const int* __restrict__ cellStart, const GridDev& g)
    {
        while (k >= bEnd) {
            if (++dx > 1) {
                dx = -1;
                if (++dy > 1) {
                    dy = -1;
                    ++dz;
                }
            }
            if (dz > 1) return false;
            const int x = ci.x + dx, y = ci.y + dy, z = ci.z + dz;
            int first = 0, n = 0;
            if (inDomain(x, y, z, g)) {
                const int key = (z * g.gy + y) * g.gx + x;
                first = cellStart[key];
                n = cellStart[key + 1] - first;
            }
            bStart = bEnd;
            bEnd += n;
            slotBase = first - bStart;
            oi = make_float3(o.x - (float)dx * g.cs.x, o.y - (float)dy * g.cs.y, o.z - (float)dz * g.cs.z);
        }
        return true;
    }
};

template <class F>
__device__ __forceinline__ void forWalkMembers(const DeviceState& d, int p, int4 ci, float3 o, F&& f)
{
    WalkCursor cur;
    cur.start();
    const int words = (d.fwalk[p] + 31) >> 5;
    const size_t stride = (size_t)d.nf;
    const unsigned* bits = d.fbits + p;
    int w = 0;
    unsigned m = words > 0 ? bits[0] : 0u;
    unsigned next = words > 1 ? bits[stride] : 0u;
    while (true) {
        while (m == 0u) {
            if (++w >= words) return;
            m = next;
            next = w + 1 < words ? bits[(size_t)(w + 1) * stride] : 0u;
        }
        const int k = (w << 5) + __ffs(m) - 1;
        m &= m - 1;
        if (!cur.seek(k, ci, o, d.fcellStart, d.grid)) return;
        f(cur.slotBase + k, cur);
    }
}

__global__ void __launch_bounds__(TT) kWalkBuild(DeviceState d)
{
    stepKernelBegin();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.nf || *d.status) return;
    const int n = d.nf;
    const GridDev& g = d.grid;
    const int4 ci = d.fcell[p];
    const float4 hi = d.fph[0][p];
    const float4 li = d.fpl[0][p];
    const dfl hI = df_make(hi.w, li.w);
    const dfl cutDF = df_add(hI, hI);
    const float c2 = 4.f * hi.w * hi.w;
    unsigned word = 0;
    int members = 0, k = 0;
    bool over = false;
    for (int dz = -1; dz <= 1 && !over; ++dz)
        for (int dy = -1; dy <= 1 && !over; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int x = ci.x + dx, y = ci.y + dy, z = ci.z + dz;
                if (!inDomain(x, y, z, g)) continue;
                const int key = (z * g.gy + y) * g.gx + x;
                const int first = d.fcellStart[key], last = d.fcellStart[key + 1];
                if (k + (last - first) > 32 * d.kbits) {
                    over = true;
                    k += last - first;
                    break;
                }
                const float3 oi = make_float3(hi.x - (float)dx * g.cs.x, hi.y - (float)dy * g.cs.y,
                                              hi.z - (float)dz * g.cs.z);
                for (int j = first; j < last; ++j, ++k) {
                    bool take = false;
                    if (j != p) {
                        const float4 pj = d.fph[0][j];
                        const float3 rv = make_float3(oi.x - pj.x, oi.y - pj.y, oi.z - pj.z);
                        const float d2 = dot3(rv, rv);
                        if (d2 < c2 * (1.f - 1.e-5f)) {
                            take = true;
                        } else if (d2 <= c2 * (1.f + 1.e-5f)) {
                            const int4 cj = make_int4(x, y, z, 0);
                            take = withinCut(ci, hi, li, cj, pj, d.fpl[0], j, cutDF, g);
                        }
                    }
                    if (take) word |= 1u << (k & 31);
                    if ((k & 31) == 31) {
                        d.fbits[(size_t)(k >> 5) * n + p] = word;
                        members += __popc(word);
                        word = 0;
                    }
                }
            }
    if (over) {
        // count the rest of the walk for the capacity the retry needs
        int total = 0;
        for (int t = 0; t < 27; ++t) {
            const int x = ci.x + t % 3 - 1, y = ci.y + (t / 3) % 3 - 1, z = ci.z + t / 9 - 1;
            if (!inDomain(x, y, z, g)) continue;
            const int key = (z * g.gy + y) * g.gx + x;
            total += d.fcellStart[key + 1] - d.fcellStart[key];
        }
        atomicOr(d.status, ST_FBITS_OVERFLOW);
        atomicMax(&d.need[4], total);
        return;
    }
    if (k & 31) {
        d.fbits[(size_t)(k >> 5) * n + p] = word;
        members += __popc(word);
    }
    d.ffc[p] = members;
    d.fwalk[p] = k;
    buildSolidPartners(d, p, ci, hi, li, cutDF, c2);
}

__global__ void __launch_bounds__(TT) kWalkContinuity(DeviceState d, TileContinuityArgs a)
{
    stepKernelBegin();
    if (a.countStep && blockIdx.x == 0 && threadIdx.x == 0 && *d.status == 0) atomicAdd(d.stepsDone, 1);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.nf || *d.status) return;
    const float4* __restrict__ ph = d.fph[a.ps];
    const float4* __restrict__ vh = d.fvh[a.vs];
    const float* __restrict__ dr = d.fdrho[a.ds];
    const Self o = loadSelf(d, p, a.ps, a.vs, a.ds);
    const float negTwoRhoM = -2.f * o.rho * d.fparU.w;
    KahanF acc;
    forWalkMembers(d, p, o.c, make_float3(o.p.x, o.p.y, o.p.z), [&](int j, const WalkCursor& cur) {
        const float4 pj = __ldg(ph + j);
        const float4 vj = __ldg(vh + j);
        float term;
        if (continuityTerm(d, o, negTwoRhoM, make_float3(cur.oi.x - pj.x, cur.oi.y - pj.y, cur.oi.z - pj.z),
                           __ldg(dr + j), xyz(vj), term))
            acc.add(term);
    });
    continuitySolids(d, o, p, acc);
    continuityFinish(d, a, p, acc.value());
}

__global__ void __launch_bounds__(TT) kWalkMomentum(DeviceState d, dfl dtf, dfl halfDtf)
{
    stepKernelBegin();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.nf || *d.status) return;
    const float4* __restrict__ ph = d.fph[1];
    const float4* __restrict__ vh = d.fvh[0];
    const float* __restrict__ dr = d.fdrho[1];
    const Self o = loadSelf(d, p, 1, 0, 1);
    const float twoNuRhoI = 2.f * d.fparU.z * o.rho, twoVi = 2.f * o.V;
    KahanF3 acc;
    forWalkMembers(d, p, o.c, make_float3(o.p.x, o.p.y, o.p.z), [&](int j, const WalkCursor& cur) {
        const float4 pj = __ldg(ph + j);
        const float4 vj = __ldg(vh + j);
        float3 term;
        if (momentumTerm(d, o, twoNuRhoI, twoVi, make_float3(cur.oi.x - pj.x, cur.oi.y - pj.y, cur.oi.z - pj.z),
                         __ldg(dr + j), xyz(vj), term))
            acc.add(term);
    });
    momentumSolids(d, o, p, acc);
    momentumFinish(d, p, acc.sum(), dtf, halfDtf);
}

__global__ void __launch_bounds__(TT) kWalkShepard(DeviceState d, int storeReference)
{
    stepKernelBegin();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.nf || *d.status) return;
    const int4 ci = d.fcell[p];
    const float4 pi = d.fph[0][p], li = d.fpl[0][p];
    const dfl h = df_make(pi.w, li.w);
    const dfl invh = df_div(df_make(1.f), h);
    const dfl twoH = df_add(h, h);
    dfl S = df_make(1.f);
    forWalkMembers(d, p, ci, make_float3(pi.x, pi.y, pi.z), [&](int j, const WalkCursor& cur) {
        shepardFluid(d, ci, pi, li, cur.dx, cur.dy, cur.dz, d.fph[0][j], d.fpl[0][j], invh, twoH, S);
    });
    shepardFinish(d, p, ci, pi, li, invh, twoH, S, storeReference);
}

// ---- the reference's list from the bits (exports) ----
// Writes slot p's fluid partners as list entries (partner slot, walk position)
// in walk order, as the list kernels do.
__global__ void kBitsToLists(DeviceState d)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.nf) return;
    const GridDev& g = d.grid;
    const int4 ci = d.fcell[p];
    int cnt = 0, k = 0;
    for (int t = 0; t < 27; ++t) {
        const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
        const int x = ci.x + dx, y = ci.y + dy, z = ci.z + dz;
        if (!inDomain(x, y, z, g)) continue;
        const int key = (z * g.gy + y) * g.gx + x;
        for (int j = d.fcellStart[key], e = d.fcellStart[key + 1]; j < e; ++j, ++k) {
            if (k >= 32 * d.kbits) return;
            if (!((d.fbits[(size_t)(k >> 5) * d.nf + p] >> (k & 31)) & 1u)) continue;
            if (cnt < d.kff) d.ff[(size_t)cnt * d.nf + p] = ffEntry(j, t, true);
            ++cnt;
        }
    }
}

}  // namespace

void launchFluidTileLists(const DeviceState& d, cudaStream_t s)
{
    if (d.nf <= 0) return;
    launchStep(kWalkBuild, blocksFor(d.nf, TT), TT, s, d);
}

void launchTileContinuity(const DeviceState& d, int which, double dtf, cudaStream_t s, bool countStep)
{
    TileContinuityArgs a;
    a.countStep = countStep ? 1 : 0;
    a.dt = (float)(0.5 * dtf);
    a.drift = df_from_double(0.5 * dtf);
    if (which == 0) {  // first half step: densities 0 -> 1, drift positions 0 -> 1
        a.ps = 0; a.vs = 0; a.ds = 0; a.dd = 1; a.driftTo = 1; a.velCopyTo = -1;
    } else {           // second half step: densities 1 -> 0, velocity 1 -> 0
        a.ps = 0; a.vs = 1; a.ds = 1; a.dd = 0; a.driftTo = -1; a.velCopyTo = 0;
    }
    launchStep(kWalkContinuity, blocksFor(d.nf, TT), TT, s, d, a);
}

void launchTileMomentum(const DeviceState& d, double dtf, cudaStream_t s)
{
    launchStep(kWalkMomentum, blocksFor(d.nf, TT), TT, s, d, df_from_double(dtf), df_from_double(0.5 * dtf));
}

void launchTileShepard(const DeviceState& d, int iStep, cudaStream_t s)
{
    launchStep(kWalkShepard, blocksFor(d.nf, TT), TT, s, d, iStep == 1 ? 1 : 0);
}

void launchBitsToLists(const DeviceState& d, cudaStream_t s)
{
    if (d.nf <= 0) return;
    ++t_kernelLaunches, kBitsToLists<<<blocksFor(d.nf, 128), 128, 0, s>>>(d);
}

}  // namespace demsph
