// WCSPH pair loops: Riemann continuity, Riemann momentum, Shepard density
// re-initialisation and the SPH->DEM coupling force.
//
// Physics restated from core/integrate.cu:3-330 (reference) with the Wendland
// C2 kernel of core/SPHKernelDEMContactModel.h:5-32.  Algebraic forms used
// here (equal to the reference's expressions, with fewer operations and no
// cancellation of the Riemann averages):
//   grad W(r, h)   = -G r,  G = 5 sigma t^3 / h^2,  t = 1 - |r| / (2h),
//                    sigma = 21 / (16 pi h^3)        (zero for |r| >= 2h)
//   continuity, fluid partner j (integrate.cu:75-103):
//     dRho/dt += -2 rho_i V_j G / (rho_i + rho_j)
//                * [rho_j (v_i - v_j).r + (P_i - P_j) |r| / c_ij]
//   continuity, solid partner a (integrate.cu:139-158), with the mirrored
//   velocity 2 v_a - v_i and the hydrostatic wall pressure P_a:
//     dRho/dt += -2 rho_i V_a G / (rho_i + rho_a)
//                * [2 rho_a (v_i - v_a).r + (P_i - P_a) |r| / c_i]
//   momentum, fluid partner (integrate.cu:185-213):
//     dv/dt += 2 V_i V_j G / m_i [P* r - gamma_ij (v_i - v_j)]
//   momentum, solid partner (integrate.cu:251-277) and the per-pair coupling
//   force (integrate.cu:282-329, = m_i times the same term):
//     dv/dt += 2 V_i V_a G / m_i [P* r - 2 gamma_i (v_i - v_a)]
// Sums are Kahan-compensated FP32; positions and velocities are integrated
// in double-float.  The continuity pass reads every partner's density as of
// the pass start (dRho is double-buffered).
#include "sph_common.cuh"

namespace demsph {

namespace {

constexpr int T = 128;
using namespace sph;

#ifndef DEMSPH_WALK_TABLE
#define DEMSPH_WALK_TABLE 1  // 1: the 27 cell offsets come from a table in shared memory
#endif

// Offset of walk cell `code` (dx, dy, dz in -1..1, code = (dz+1) 9 + (dy+1) 3 + dx+1)
// times the cell size.
__device__ __forceinline__ float4 walkOffsetOf(unsigned code, float3 cs)
{
    const int dx = (int)(code % 3u) - 1, dy = (int)((code / 3u) % 3u) - 1, dz = (int)(code / 9u) - 1;
    return make_float4((float)dx * cs.x, (float)dy * cs.y, (float)dz * cs.z, 0.f);
}

// The table of the 27 offsets in a block's shared memory (filled before the
// block's first early return).
__device__ __forceinline__ void fillWalkTable(float4* tab, float3 cs)
{
    if (DEMSPH_WALK_TABLE) {
        if (threadIdx.x < 27) tab[threadIdx.x] = walkOffsetOf(threadIdx.x, cs);
        __syncthreads();
    }
}

// Relative position of fluid partner entry e of slot i (tab: the offsets'
// table; the products are exact, so the table changes no bit).
__device__ __forceinline__ float3 fluidRel(const DeviceState& d, const float4* tab, int4 ci, float4 pi, unsigned e,
                                           int j, float4 pj)
{
    if (ffRegular(e)) {
        const float4 o = DEMSPH_WALK_TABLE ? tab[entryWalk(e)] : walkOffsetOf((unsigned)entryWalk(e), d.grid.cs);
        return make_float3((pi.x - pj.x) - o.x, (pi.y - pj.y) - o.y, (pi.z - pj.z) - o.z);
    }
    return relF(ci, pi, d.fcell[j], pj, d.grid);
}

// ---- batched partner loops ----
// Entries per lane read before any of their partners is used: a lane reads
// B list entries, then the B partners' state, then adds the B pair terms in
// list order.  B gathers per lane are in flight instead of one (the loop is
// bound by the latency of the list stream and the dependent gathers, not by
// bandwidth), and every sum is that of the one-by-one loop, bit for bit.
// Depths and block counts measured on GB300 (ms per fluid period of the 1.0M
// coupled dam break, one lane per particle; depth 1 = the one-by-one loop):
// depth 1 with 12 continuity blocks 3.889, depth 2 with 8 continuity and 6
// momentum blocks 3.829, depth 4 3.89-4.15 (continuity spills at 8 blocks),
// depth 8 4.43.  The 48k dam break (eight lanes) is flat within 3 %.
#ifndef DEMSPH_PAIR_BATCH
#define DEMSPH_PAIR_BATCH 2       // entries per batch, one or two lanes per particle
#endif
#ifndef DEMSPH_PAIR_BATCH_WIDE
#define DEMSPH_PAIR_BATCH_WIDE 2  // entries per batch, four or more lanes per particle
#endif
#ifndef DEMSPH_CONTINUITY_BLOCKS
#define DEMSPH_CONTINUITY_BLOCKS 8  // resident blocks of T per SM the registers allow
#endif
#ifndef DEMSPH_MOMENTUM_BLOCKS
#define DEMSPH_MOMENTUM_BLOCKS 6
#endif
#ifndef DEMSPH_PAIR_AHEAD
#define DEMSPH_PAIR_AHEAD 1  // 1: the next batch's entries are read while this batch computes
#endif
#ifndef DEMSPH_PAIR_L2_AHEAD
#define DEMSPH_PAIR_L2_AHEAD 0  // > 0: the list line that many batches ahead is prefetched into L2
#endif
template <int L>
constexpr int batchDepth() { return L >= 4 ? DEMSPH_PAIR_BATCH_WIDE : DEMSPH_PAIR_BATCH; }

template <int L, int B, class Gather, class Term>
__device__ __forceinline__ void forFluidPartners(const unsigned* __restrict__ ff, int n, int i, int lane, int m,
                                                 Gather gather, Term term)
{
    const size_t stride = (size_t)L * n;  // from entry k of slot i to entry k + L
    const unsigned* p = ff + (size_t)lane * n + i;
    unsigned next[B];
    if (DEMSPH_PAIR_AHEAD) {
#pragma unroll
        for (int u = 0; u < B; ++u) next[u] = lane + u * L < m ? __ldcs(p + u * stride) : 0u;
    }
    for (int k0 = lane; k0 < m; k0 += B * L) {
        unsigned e[B];
#pragma unroll
        for (int u = 0; u < B; ++u) e[u] = DEMSPH_PAIR_AHEAD ? next[u] : (k0 + u * L < m ? __ldcs(p + u * stride) : 0u);
        p += B * stride;
        if (DEMSPH_PAIR_AHEAD) {
#pragma unroll
            for (int u = 0; u < B; ++u) next[u] = k0 + (B + u) * L < m ? __ldcs(p + u * stride) : 0u;
        }
        if (DEMSPH_PAIR_L2_AHEAD > 0 && k0 + DEMSPH_PAIR_L2_AHEAD * B * L < m)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(p + (size_t)(DEMSPH_PAIR_L2_AHEAD - 1) * B * stride));
        decltype(gather(0u)) g[B];
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (k0 + u * L < m) g[u] = gather(e[u]);
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (k0 + u * L < m) term(e[u], g[u]);
    }
}

// A fluid partner's state read by the continuity and momentum terms (the
// buffers a pass reads are not written by it: read-only loads).  Uniform
// fluids (U) read the position and density as one partner record (pd, the
// pass's fpd); par only for scenes whose fluids differ (U false).
template <bool U>
struct FluidPartner {
    float4 p, v, par;
    float dr;
};

template <bool U>
__device__ __forceinline__ FluidPartner<U> gatherFluid(const DeviceState& d, int j, const float4* __restrict__ ph,
                                                       const float4* __restrict__ vh, const float* __restrict__ dr,
                                                       const float4* __restrict__ pd)
{
    FluidPartner<U> q;
    if constexpr (U) {
        q.p = __ldg(pd + j);
        q.dr = q.p.w;
    } else {
        q.p = __ldg(ph + j);
        q.dr = __ldg(dr + j);
        q.par = __ldg(d.fpar + j);
    }
    q.v = __ldg(vh + j);
    return q;
}

// ---- lane groups ----
// A fluid particle's neighbour loop is split over a group of L lanes (L a
// power of two <= 32, chosen per scene so that small scenes still fill the
// GPU); the lanes' compensated partial sums are added in a fixed tree, so the
// result does not depend on timing.  Kernels return early only for whole
// warps: the shuffles take every lane.
template <int L>
__device__ __forceinline__ dfl groupSum(dfl v)
{
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
        const dfl u = df_make(__shfl_xor_sync(0xffffffffu, v.hi, o, L), __shfl_xor_sync(0xffffffffu, v.lo, o, L));
        v = (threadIdx.x & o) ? df_add(u, v) : df_add(v, u);
    }
    return v;
}
template <int L>
__device__ __forceinline__ float groupSum(const KahanF& k)
{
    if (L == 1) return k.value();
    const dfl v = groupSum<L>(df_two_sum(k.s, -k.c));
    return v.hi + v.lo;
}

// ---- continuity (+ optional drift) ----
struct ContinuityArgs {
    int ps, vs, ds, dd;  // position / velocity / density source, density destination
    int rec;             // partner records read (uniform fluids): fpd[rec] holds position ps, density ds
    int recOut;          // -1: none; else fpd[recOut] receives the drifted position and density dd
    int driftTo;         // -1: no drift; else position buffer receiving x + v * drift
    int velCopyTo;       // -1: none; else velocity buffer receiving a copy of this particle's velocity
    int countStep;       // 1: the pass ends the step (nothing after it can raise a status): count it
    float dt;
    dfl drift;
};

template <int L, bool U>
__global__ void __launch_bounds__(T, DEMSPH_CONTINUITY_BLOCKS) kContinuity(DeviceState d, ContinuityArgs a)
{
    stepKernelBegin();
    __shared__ float4 walkTab[27];
    fillWalkTable(walkTab, d.grid.cs);
    if (a.countStep && blockIdx.x == 0 && threadIdx.x == 0 && *d.status == 0) atomicAdd(d.stepsDone, 1);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if ((t & ~31) >= d.nf * L || *d.status) return;
    const int i = t / L, lane = t % L;
    const bool live = i < d.nf;
    KahanF acc;
    Self o;
    if (live) {
        o = loadSelf(d, i, a.ps, a.vs, a.ds);
        const int n = d.nf;
        const int nff = min(d.ffc[i], d.kff);
        // U: every fluid particle has the same rest density, sound speed,
        // viscosity, mass and smoothing length - one gather fewer per
        // neighbour, and the kernel's constants and the shared sound speed
        // taken out of the loop (one division per pair instead of five)
        const float negTwoRhoM = -2.f * o.rho * d.fparU.w;
        const float4* __restrict__ ph = d.fph[a.ps];
        const float4* __restrict__ vh = d.fvh[a.vs];
        const float* __restrict__ drh = d.fdrho[a.ds];
        const float4* __restrict__ pd = d.fpd[a.rec];
        forFluidPartners<L, batchDepth<L>()>(
            d.ff, n, i, lane, nff, [&](unsigned e) { return gatherFluid<U>(d, ffPartner(e), ph, vh, drh, pd); },
            [&](unsigned e, const FluidPartner<U>& q) {
                const float3 r = fluidRel(d, walkTab, o.c, o.p, e, ffPartner(e), q.p);
                const float r2 = dot3(r, r);
                if constexpr (U) {
                    // the shared constants are read from the kernel parameters
                    if (r2 >= d.fconstU.x) return;
                    const float rhoj = d.fparU.x + q.dr;
                    const float Pj = q.dr * d.fparU.y * d.fparU.y;
                    const float rr = sqrtf(r2);
                    const float tt = 1.f - rr * d.fconstU.y;
                    const float G = d.fconstU.z * tt * tt * tt;
                    const float3 vij = o.v - xyz(q.v);
                    acc.add(negTwoRhoM * G / (rhoj * (o.rho + rhoj)) *
                            (rhoj * dot3(vij, r) + (o.P - Pj) * rr * d.fconstU.w));
                } else {
                    const float h = 0.5f * (o.h + q.p.w);
                    if (r2 >= 4.f * h * h) return;
                    const float rhoj = q.par.x + q.dr;
                    const float Pj = q.dr * q.par.y * q.par.y;
                    const float Vj = q.par.w / rhoj;
                    const float rr = sqrtf(r2);
                    const float tt = 1.f - 0.5f * rr / h;
                    const float h2 = h * h;
                    const float G = KG * tt * tt * tt / (h2 * h2 * h);
                    const float c = 0.5f * (o.cs + q.par.y);
                    const float3 vij = o.v - xyz(q.v);
                    acc.add(-2.f * o.rho * Vj * G / (o.rho + rhoj) * (rhoj * dot3(vij, r) + (o.P - Pj) * rr / c));
                }
            });
        const int nfs = min(d.fsc[i], d.kfs);
        const float ci2 = o.cs * o.cs;
        for (int k = lane; k < nfs; k += L) {
            const int sa = fsPartner(d.fs[(size_t)k * n + i]);
            const SolidPartner sp = solidPartner(d, o.c, o.p, o.h, o.P, o.rho, o.rho0, ci2, sa);
            if (!sp.inside) continue;
            acc.add(-2.f * o.rho * sp.Va * sp.G / (o.rho + sp.rhoa) *
                    (2.f * sp.rhoa * dot3(o.v - sp.v, sp.r) + (o.P - sp.Pa) * sp.rr / o.cs));
        }
    }
    const float sum = groupSum<L>(acc);
    if (!live || lane != 0) return;
    const float drho = d.fdrho[a.ds][i] + a.dt * sum;
    d.fdrho[a.dd][i] = drho;
    if (a.driftTo >= 0) {
        float4 xh = d.fph[a.ps][i], xl = d.fpl[a.ps][i];
        dfAxpy(xh, xl, d.fvh[a.vs][i], d.fvl[a.vs][i], a.drift);
        d.fph[a.driftTo][i] = xh;
        d.fpl[a.driftTo][i] = xl;
        if (U && a.recOut >= 0) d.fpd[a.recOut][i] = make_float4(xh.x, xh.y, xh.z, drho);
    }
    if (a.velCopyTo >= 0) {
        d.fvh[a.velCopyTo][i] = d.fvh[a.vs][i];
        d.fvl[a.velCopyTo][i] = d.fvl[a.vs][i];
    }
}

// ---- momentum + kick (dt_f) + drift (dt_f / 2) ----
// Reads position [1], velocity [0], density [1]; writes acc, velocity [1] and
// position [0] (the buffers no other thread reads in this pass).
template <int L, bool U>
__global__ void __launch_bounds__(T, DEMSPH_MOMENTUM_BLOCKS) kMomentum(DeviceState d, dfl dtf, dfl halfDtf)
{
    stepKernelBegin();
    __shared__ float4 walkTab[27];
    fillWalkTable(walkTab, d.grid.cs);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if ((t & ~31) >= d.nf * L || *d.status) return;
    const int i = t / L, lane = t % L;
    const bool live = i < d.nf;
    KahanF3 acc;
    if (live) {
        const Self o = loadSelf(d, i, 1, 0, 1);
        const int n = d.nf;
        const int nff = min(d.ffc[i], d.kff);
        // U: the same parameters and smoothing length for every particle (see
        // kContinuity): three divisions per pair instead of seven
        const float twoNuRhoI = 2.f * d.fparU.z * o.rho, twoVi = 2.f * o.V;
        forFluidPartners<L, batchDepth<L>()>(
            d.ff, n, i, lane, nff,
            [&](unsigned e) { return gatherFluid<U>(d, ffPartner(e), d.fph[1], d.fvh[0], d.fdrho[1], d.fpd[1]); },
            [&](unsigned e, const FluidPartner<U>& q) {
                const float3 r = fluidRel(d, walkTab, o.c, o.p, e, ffPartner(e), q.p);
                const float r2 = dot3(r, r);
                if constexpr (U) {
                    if (r2 >= d.fconstU.x) return;
                    const float rhoj = d.fparU.x + q.dr;
                    const float Pj = q.dr * d.fparU.y * d.fparU.y;
                    const float rr = sqrtf(r2);
                    const float tt = 1.f - rr * d.fconstU.y;
                    const float G = d.fconstU.z * tt * tt * tt;
                    const float3 vij = o.v - xyz(q.v);
                    const float dU = -dot3(vij, r) / rr;  // U_L - U_R
                    const float beta = fminf(3.f * fmaxf(dU, 0.f), d.fparU.y);
                    const float invSum = 1.f / (o.rho + rhoj);
                    const float Ps = (o.rho * Pj + rhoj * o.P + o.rho * rhoj * beta * dU) * invSum;
                    const float gbar = twoNuRhoI * rhoj * invSum;  // 2 g_i g_j / (g_i + g_j), g = nu rho
                    const float w = twoVi * G / rhoj;              // 2 V_i V_j G / m, V_j = m / rho_j
                    acc.add((r * Ps - vij * gbar) * w);
                } else {
                    const float h = 0.5f * (o.h + q.p.w);
                    if (r2 >= 4.f * h * h) return;
                    const float rhoj = q.par.x + q.dr;
                    const float Pj = q.dr * q.par.y * q.par.y;
                    const float Vj = q.par.w / rhoj;
                    const float gj = q.par.z * rhoj;
                    const float rr = sqrtf(r2);
                    const float tt = 1.f - 0.5f * rr / h;
                    const float h2 = h * h;
                    const float G = KG * tt * tt * tt / (h2 * h2 * h);
                    const float c = 0.5f * (o.cs + q.par.y);
                    const float3 vij = o.v - xyz(q.v);
                    const float dU = -dot3(vij, r) / rr;  // U_L - U_R
                    const float beta = fminf(3.f * fmaxf(dU, 0.f), c);
                    const float Ps = (o.rho * Pj + rhoj * o.P + o.rho * rhoj * beta * dU) / (o.rho + rhoj);
                    const float gbar = 2.f * o.gam * gj / (o.gam + gj);
                    const float w = 2.f * o.V * Vj * G / o.m;
                    acc.add((r * Ps - vij * gbar) * w);
                }
            });
        const int nfs = min(d.fsc[i], d.kfs);
        const float ci2 = o.cs * o.cs;
        for (int k = lane; k < nfs; k += L) {
            const int sa = fsPartner(d.fs[(size_t)k * n + i]);
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
    const float3 sum = make_float3(groupSum<L>(acc.x), groupSum<L>(acc.y), groupSum<L>(acc.z));
    if (!live || lane != 0) return;
    const float3 acl = sum + d.g;
    d.facc[i] = f4(acl);
    // kick: v += a dt_f
    const float4 vh0 = d.fvh[0][i], vl0 = d.fvl[0][i];
    const dfl vx = df_add(df_make(vh0.x, vl0.x), df_mul_f(dtf, acl.x));
    const dfl vy = df_add(df_make(vh0.y, vl0.y), df_mul_f(dtf, acl.y));
    const dfl vz = df_add(df_make(vh0.z, vl0.z), df_mul_f(dtf, acl.z));
    const float4 vh = make_float4(vx.hi, vy.hi, vz.hi, 0.f), vl = make_float4(vx.lo, vy.lo, vz.lo, 0.f);
    d.fvh[1][i] = vh;
    d.fvl[1][i] = vl;
    // drift: x += v dt_f / 2
    float4 xh = d.fph[1][i], xl = d.fpl[1][i];
    dfAxpy(xh, xl, vh, vl, halfDtf);
    d.fph[0][i] = xh;
    d.fpl[0][i] = xl;
    if (U) d.fpd[2][i] = make_float4(xh.x, xh.y, xh.z, d.fdrho[1][i]);  // the second continuity pass's partners
    // the fluid candidates go stale once a particle has moved half the margin
    const int4 c = d.fcell[i];
    const float4 p0 = d.fvref[i];
    const float dx = (float)c.x * d.grid.cs.x + xh.x - p0.x, dy = (float)c.y * d.grid.cs.y + xh.y - p0.y,
                dz = (float)c.z * d.grid.cs.z + xh.z - p0.z;
    const float half = 0.5f * d.fskin;
    if (!(dx * dx + dy * dy + dz * dz <= half * half)) *(volatile int*)d.frebuild = 1;
}

// The first continuity pass's partner records: position 0 and density 0 as
// the step's search and Shepard re-initialisation leave them.
__global__ void kPackPartners(DeviceState d)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nf || *d.status) return;
    const float4 x = d.fph[0][i];
    d.fpd[0][i] = make_float4(x.x, x.y, x.z, d.fdrho[0][i]);
}

template <int L>
__global__ void __launch_bounds__(T) kDensityReinit(DeviceState d, int storeReference)
{
    stepKernelBegin();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if ((t & ~31) >= d.nf * L || *d.status) return;
    const int i = t / L, lane = t % L;
    const bool live = i < d.nf;
    dfl S = df_make(lane == 0 ? 1.f : 0.f);
    if (live) {
        const int4 ci = d.fcell[i];
        const float4 pi = d.fph[0][i], li = d.fpl[0][i];
        const dfl h = df_make(pi.w, li.w);
        const dfl invh = df_div(df_make(1.f), h);
        const dfl twoH = df_add(h, h);
        const int n = d.nf;
        const int nff = min(d.ffc[i], d.kff);
        struct PartnerPosition {
            float4 h, l;
        };
        forFluidPartners<L, batchDepth<L>()>(
            d.ff, n, i, lane, nff,
            [&](unsigned e) {
                const int j = ffPartner(e);
                return PartnerPosition{__ldg(d.fph[0] + j), __ldg(d.fpl[0] + j)};
            },
            [&](unsigned e, const PartnerPosition& q) {
                const unsigned code = (unsigned)entryWalk(e);
                int4 cj;
                if (ffRegular(e))
                    cj = make_int4(ci.x + (int)(code % 3u) - 1, ci.y + (int)((code / 3u) % 3u) - 1,
                                   ci.z + (int)(code / 9u) - 1, 0);
                else
                    cj = d.fcell[ffPartner(e)];
                const dfl r = dfNorm(relDF(ci, pi, li, cj, q.h, q.l, d.grid));
                if (df_ge0(df_sub(r, twoH))) return;  // q >= 2
                S = df_add(S, shepardTerm(r, invh));
            });
        // V0_a / V0_i = (2 r_a / (h_i / 1.3))^3 = (2.6 r_a / h_i)^3
        const dfl k26 = df_from_double(2.6);
        const int nfs = min(d.fsc[i], d.kfs);
        for (int k = lane; k < nfs; k += L) {
            const int a = fsPartner(d.fs[(size_t)k * n + i]);
            const dfl r = dfNorm(relDF(ci, pi, li, d.scell[a], d.sph[a], d.spl[a], d.grid));
            if (df_ge0(df_sub(r, twoH))) continue;
            const float4 ra = d.srad[a];
            const dfl x = df_mul(df_mul(k26, df_make(ra.x, ra.y)), invh);
            const dfl vr = df_mul(df_mul(x, x), x);
            S = df_add(S, df_mul(shepardTerm(r, invh), vr));
        }
    }
    S = groupSum<L>(S);
    if (!live || lane != 0) return;
    if (storeReference) {
        d.fsumW0[i] = make_float2(S.hi, S.lo);
    } else {
        const float2 s0 = d.fsumW0[i];
        const dfl diff = df_sub(S, df_make(s0.x, s0.y));
        const float rho0 = d.fpar[i].x;
        // max(rho*, rho0 S / S0) - rho0 = max(dRho, rho0 (S - S0) / S0)
        const float cand = rho0 * ((diff.hi + diff.lo) / s0.x);
        d.fdrho[0][i] = fmaxf(d.fdrho[0][i], cand);
    }
}

// ---- coupling force, per massive solid: sum over its fluid partners of
// m_i x (solid term of momentum) (integrate.cu:282-330, gathered per solid
// as calSolidForceTorque does through fluidSolidRange, :847-854) ----
__device__ __forceinline__ float3 couplingPairForce(const DeviceState& d, int src, int i, int a, bool& inside)
{
    const Self o = loadSelf(d, i, src, 0, src);
    const SolidPartner s = solidPartner(d, o.c, o.p, o.h, o.P, o.rho, o.rho0, o.cs * o.cs, a);
    inside = s.inside;
    if (!s.inside) return make_float3(0.f, 0.f, 0.f);
    const float3 via = o.v - s.v;
    const float dU = -2.f * dot3(via, xyz(d.snormal[a]));
    const float beta = fminf(3.f * fmaxf(dU, 0.f), o.cs);
    const float Ps = (o.rho * s.Pa + s.rhoa * o.P + o.rho * s.rhoa * beta * dU) / (o.rho + s.rhoa);
    return (s.r * Ps - via * (2.f * o.gam)) * (2.f * o.V * s.Va * s.G);
}

// Only contact rows can hold solids with mass, the only solids with fluid
// partners here (the coupling lists take no others); L lanes of a row take
// its partners in turn, each Kahan-summing its share, and the shares are
// added in a fixed tree (groupSum).
template <int L>
__global__ void kCoupling(DeviceState d, int src)
{
    stepKernelBegin();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if ((t & ~31) >= d.nrow * L || *d.status) return;  // whole warps: the group sums shuffle
    const int row = t / L, lane = t % L;
    const bool live = row < d.nrow;
    const int a = live ? solidOf(d, row) : 0;
    KahanF3 f;
    if (live)
        for (int p = d.coupStart[a] + lane, e = d.coupStart[a + 1]; p < e; p += L) {
            bool inside;
            const float3 fi = couplingPairForce(d, src, d.coupList[p], a, inside);
            if (inside) f.add(fi);
        }
    const float x = groupSum<L>(f.x), y = groupSum<L>(f.y), z = groupSum<L>(f.z);
    if (live && lane == 0) d.sfcoup[a] = make_float4(x, y, z, 0.f);
}

// Per-pair coupling force in the fluid's list order (for export only).
__global__ void kCouplingPairs(DeviceState d, int src, float4* out)
{
    stepKernelBegin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nf) return;
    const int m = min(d.fsc[i], d.kfs);
    for (int k = 0; k < m; ++k) {
        bool inside;
        const float3 f = couplingPairForce(d, src, i, fsPartner(d.fs[(size_t)k * d.nf + i]), inside);
        out[(size_t)k * d.nf + i] = f4(f);
    }
}

}  // namespace

void launchDensityReinit(const DeviceState& d, int iStep, cudaStream_t s)
{
    if (d.nf <= 0) return;
    if (d.fluidTiles) return launchTileShepard(d, iStep, s);
    LAUNCH_LANES(kDensityReinit, d.lanes, d.nf, T, s, d, iStep == 1 ? 1 : 0);
}

int fluidLanes(int nf)
{
    int L = 1;
    while (L < 8 && (long long)nf * L < 152LL * 2048) L *= 2;
    return L;
}

void launchContinuityPass(const DeviceState& d, int which, double dtf, cudaStream_t s, bool countStep)
{
    if (d.nf <= 0) return;
    if (d.fluidTiles) return launchTileContinuity(d, which, dtf, s, countStep);
    ContinuityArgs a;
    a.countStep = countStep ? 1 : 0;
    a.dt = (float)(0.5 * dtf);
    a.drift = df_from_double(0.5 * dtf);
    if (which == 0) {  // first half step: densities 0 -> 1, drift positions 0 -> 1
        a.ps = 0; a.vs = 0; a.ds = 0; a.dd = 1; a.driftTo = 1; a.velCopyTo = -1; a.rec = 0; a.recOut = 1;
        if (d.uniformFluid) launchStep(kPackPartners, blocksFor(d.nf, 256), 256, s, d);
    } else {           // second half step: densities 1 -> 0, velocity 1 -> 0
        a.ps = 0; a.vs = 1; a.ds = 1; a.dd = 0; a.driftTo = -1; a.velCopyTo = 0; a.rec = 2; a.recOut = -1;
    }
    if (d.uniformFluid) LAUNCH_LANES_U(kContinuity, true, d.lanes, d.nf, T, s, d, a);
    else LAUNCH_LANES_U(kContinuity, false, d.lanes, d.nf, T, s, d, a);
}

void launchMomentumPass(const DeviceState& d, double dtf, cudaStream_t s)
{
    if (d.nf <= 0) return;
    if (d.fluidTiles) return launchTileMomentum(d, dtf, s);
    if (d.uniformFluid) LAUNCH_LANES_U(kMomentum, true, d.lanes, d.nf, T, s, d, df_from_double(dtf), df_from_double(0.5 * dtf));
    else LAUNCH_LANES_U(kMomentum, false, d.lanes, d.nf, T, s, d, df_from_double(dtf), df_from_double(0.5 * dtf));
}

void launchCoupling(const DeviceState& d, int src, cudaStream_t s)
{
    if (d.nf <= 0 || d.ns <= 0 || d.nrow <= 0) return;
    constexpr int L = 8;  // lanes per row: rows hold tens of fluid partners
    launchStep(kCoupling<L>, blocksFor((long long)d.nrow * L, 256), 256, s, d, src);
}

void launchCouplingPairForces(const DeviceState& d, int src, float4* out, cudaStream_t s)
{
    if (d.nf <= 0 || d.ns <= 0) return;
    launchStep(kCouplingPairs, blocksFor(d.nf, 128), 128, s, d, src, out);
}

}  // namespace demsph
