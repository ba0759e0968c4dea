// DEM contact phase and the solid / clump integrators.
//
// Reference: calSolidContactForceTorque (core/integrate.cu:423-512), the
// contact laws of core/SPHKernelDEMContactModel.h:170-326, the parallel bond
// (:115-168, integrate.cu:717-804), calSolidForceTorque (:806-858),
// calInfiniteWallForceTorque (:514-610), calClumpForceTorque (:860-881) and the
// half-step integrators (:883-998).
//
// Precision: the overlap delta = r_i + r_j - |x_i - x_j| and the wall overlap
// are computed in double-float (they are 1e-4..1e-3 of the radius); the laws
// themselves run in FP32; bond forces/torques accumulate in double-float;
// positions, velocities and spins integrate in double-float; the clump rigid
// body (a handful of clumps) is FP64.
//
// The per-particle gather adds forward pairs and subtracts reverse pairs in
// list order - no atomics, so results are bit-reproducible run to run.
#include "kernels.cuh"
#include "contact_rows.cuh"
#include "warp_items.cuh"

namespace demsph {

namespace {

constexpr int T = 128;
constexpr float SQRT56 = 0.912870929175276855f;  // sqrt(5/6)

// Tangential (sliding / rolling) spring with Coulomb cap (SPHKernelDEMContactModel.h:170-193).
__device__ __forceinline__ float3 slideRollSpring(float3 prev, float3 vel, float3 n, float aN, float mu, float k, float c,
                                                 float dt)
{
    float3 s = make_float3(0.f, 0.f, 0.f);
    if (mu > 0.f) {
        float3 p1 = prev - n * dot3(prev, n);
        const float a = len3(p1);
        if (a > 1.e-10f) p1 = p1 * (len3(prev) / a);
        s = p1 + vel * dt;
        float3 F = s * (-k) - vel * c;
        const float aF = len3(F);
        if (aF > mu * aN) {
            F = F * (mu * aN / aF);
            s = (F + vel * c) * (-1.f / k);
        }
    }
    return s;
}
// Torsion spring (SPHKernelDEMContactModel.h:195-212).
__device__ __forceinline__ float3 torsionSpring(float3 prev, float3 vel, float3 n, float aN, float mu, float k, float c,
                                               float dt)
{
    float3 s = make_float3(0.f, 0.f, 0.f);
    if (mu > 0.f) {
        s = n * dot3(prev + vel * dt, n);
        float3 F = s * (-k) - vel * c;
        const float aF = len3(F);
        if (aF > mu * aN) {
            F = F * (mu * aN / aF);
            s = (F + vel * c) * (-1.f / k);
        }
    }
    return s;
}

// Linear / Hertz-Mindlin dispatch (integrate.cu:463-505).  Also returns the
// tangential (sliding) part Ft of F: a lever arm along n turns F into the
// torque s (n x Ft) exactly, without the FP32 residue of n x (Fn n).
__device__ __forceinline__ void contactLaw(const Tables& tab, int slot, float3& F, float3& Ft, float3& T, float3& es,
                                           float3& er, float3& et, float3 vc, float3 wr, float3 n, float delta, float m,
                                           float R, float dt)
{
    if (!(delta > 0.f)) {
        es = er = et = make_float3(0.f, 0.f, 0.f);
        return;
    }
    const float* L = tab.ln + 11 * slot;
    float kn, ks, kr, kt, cn, cs, cr, ct, mus, mur, mut;
    if (L[0] > 1.e-10f) {  // LinearContact (SPHKernelDEMContactModel.h:214-268)
        kn = L[0]; ks = L[1]; kr = L[2]; kt = L[3];
        cn = 2.f * L[4] * sqrtf(m * kn);
        cs = 2.f * L[5] * sqrtf(m * ks);
        cr = 2.f * L[6] * sqrtf(m * kr);
        ct = 2.f * L[7] * sqrtf(m * kt);
        mus = L[8]; mur = L[9]; mut = L[10];
    } else {               // HertzianMindlinContact (SPHKernelDEMContactModel.h:270-326)
        const float* H = tab.hz + 8 * slot;
        const float D = tab.damp[slot];
        const float sRd = sqrtf(R * delta);
        kn = 4.f / 3.f * H[0] * sRd;
        ks = 8.f * H[1] * sRd;
        kr = ks * H[3];
        kt = ks * H[4];
        const float c0 = 2.f * SQRT56 * D;
        cn = c0 * sqrtf(m * kn);
        cs = c0 * sqrtf(m * ks);
        cr = c0 * sqrtf(m * kr);
        ct = c0 * sqrtf(m * kt);
        mus = H[5]; mur = H[6]; mut = H[7];
    }
    const float3 vn = n * dot3(vc, n);
    const float3 Fn = n * (kn * delta) - vn * cn;
    const float aN = len3(Fn);
    const float3 vs = vc - vn;
    es = slideRollSpring(es, vs, n, aN, mus, ks, cs, dt);
    const float3 Fs = es * (-ks) - vs * cs;
    const float3 vr = cross3(n, wr) * (-R);
    er = slideRollSpring(er, vr, n, aN, mur, kr, cr, dt);
    const float3 Fr = er * (-kr) - vr * cr;
    const float3 Tr = cross3(n, Fr) * R;
    const float Dm = 2.f * R;
    const float3 vt = n * (Dm * dot3(wr, n));
    et = torsionSpring(et, vt, n, aN, mut, kt, ct, dt);
    const float3 Fto = et * (-kt) - vt * ct;
    F = Fn + Fs;
    Ft = Fs;
    T = Tr + Fto * Dm;
}

struct PairGeom {
    float3 n;        // unit vector from B to A
    float delta;     // overlap r_A + r_B - |x_A - x_B|
    float dist;
    float sA, sB;    // contact point - x_A = sA n, contact point - x_B = sB n
    float3 leverA;
    float3 leverB;
};
__device__ __forceinline__ PairGeom pairGeometry(const DeviceState& d, int a, int b)
{
    PairGeom g;
    const DF3 r = relDF(d.scell[a], d.sph[a], d.spl[a], d.scell[b], d.sph[b], d.spl[b], d.grid);
    const dfl dist = dfNorm(r);
    const float4 ra = d.srad[a], rb = d.srad[b];
    const dfl del = df_sub(df_add(df_make(ra.x, ra.y), df_make(rb.x, rb.y)), dist);
    g.delta = del.hi + del.lo;
    g.dist = dist.hi + dist.lo;
    g.n = g.dist > 0.f ? toF3(r) / g.dist : make_float3(0.f, 0.f, 0.f);
    g.sA = -0.5f * (g.dist + ra.x - rb.x);
    g.sB = 0.5f * (g.dist + rb.x - ra.x);
    g.leverA = g.n * g.sA;
    g.leverB = g.n * g.sB;
    return g;
}

// (v_a - v_b) from the double-float velocities: grains moving together have
// nearly equal velocities, whose float parts alone would cancel.
__device__ __forceinline__ float3 velDiff(const DeviceState& d, int a, int b)
{
    const float4 ha = d.svh[a], la = d.svl[a], hb = d.svh[b], lb = d.svl[b];
    return make_float3((ha.x - hb.x) + (la.x - lb.x), (ha.y - hb.y) + (la.y - lb.y), (ha.z - hb.z) + (la.z - lb.z));
}
__device__ __forceinline__ float3 spinDiff(const DeviceState& d, int a, int b)
{
    const float4 ha = d.swh[a], la = d.swl[a], hb = d.swh[b], lb = d.swl[b];
    return make_float3((ha.x - hb.x) + (la.x - lb.x), (ha.y - hb.y) + (la.y - lb.y), (ha.z - hb.z) + (la.z - lb.z));
}
// velocity of b's contact point relative to a's: v_a + w_a x lever_a - (v_b + w_b x lever_b)
__device__ __forceinline__ float3 contactVel(const DeviceState& d, int a, int b, float3 leverA, float3 leverB)
{
    return velDiff(d, a, b) + cross3(xyz(d.swh[a]), leverA) - cross3(xyz(d.swh[b]), leverB);
}

// One contact (calSolidContactForceTorque, core/integrate.cu:423-512) of the
// pair (A, B), A < B, with the springs es, er, et (updated in place): the
// force on A, the contact torque as the reference stores it, and the torques
// on A and B with their lever arms.
struct PairForce {
    float3 F, T, TA, TB;
};
__device__ __forceinline__ PairForce pairForce(const DeviceState& d, int a, int b, float3& es, float3& er,
                                               float3& et, float dt)
{
    const PairGeom g = pairGeometry(d, a, b);
    const float4 ra = d.srad[a], rb = d.srad[b];
    const float R = ra.x * rb.x / (ra.x + rb.x);
    const float m = 1.f / (d.sph[a].w + d.sph[b].w);
    const float3 vc = contactVel(d, a, b, g.leverA, g.leverB);
    const float3 wr = spinDiff(d, a, b);
    float3 F = make_float3(0.f, 0.f, 0.f), Ft = F, Tq = F;
    const int slot = tableSlot(d.tab, d.sflags[a].x, d.sflags[b].x);
    contactLaw(d.tab, slot, F, Ft, Tq, es, er, et, vc, wr, g.n, g.delta, m, R, dt);
    const float3 nxF = cross3(g.n, Ft);
    PairForce p;
    p.F = F;
    p.T = Tq;
    p.TA = Tq + nxF * g.sA;
    p.TB = Tq + nxF * g.sB;
    return p;
}

// Slot (index into the per-slot arrays) of the forward contact (a, b), b > a,
// or -1 when the pair is not in a's row.
__device__ __forceinline__ long long forwardSlot(const DeviceState& d, int par, int a, int b)
{
    const int r = rowOf(d, a);
    if (r < 0) return -1;
    const int n = min(d.fcnt[par][r], d.scap);
    for (int q = 0; q < n; ++q) {
        const size_t k = (size_t)q * d.nrow + r;
        if (d.fwd[par][k] == b) return (long long)k;
    }
    return -1;
}

// Adds the small rotation (R(theta) - I) v to a double-float vector.
__device__ __forceinline__ void rotateDF(float4& h, float4& l, float3 th)
{
    const float a = len3(th);
    if (a < 1.e-10f) return;
    const float3 k = th / a;
    const float s = sinf(a), sh = sinf(0.5f * a);
    const float omc = 2.f * sh * sh;  // 1 - cos a
    const float3 v = xyz(h);
    const float3 dv = cross3(k, v) * s + (k * dot3(k, v) - v) * omc;
    dfl x = df_add_f(df_make(h.x, l.x), dv.x), y = df_add_f(df_make(h.y, l.y), dv.y),
        z = df_add_f(df_make(h.z, l.z), dv.z);
    h = make_float4(x.hi, y.hi, z.hi, h.w);
    l = make_float4(x.lo, y.lo, z.lo, l.w);
}
__device__ __forceinline__ void addDF3(float4& h, float4& l, float3 dv)
{
    dfl x = df_add_f(df_make(h.x, l.x), dv.x), y = df_add_f(df_make(h.y, l.y), dv.y),
        z = df_add_f(df_make(h.z, l.z), dv.z);
    h = make_float4(x.hi, y.hi, z.hi, h.w);
    l = make_float4(x.lo, y.lo, z.lo, l.w);
}

// One parallel bond's update (integrate.cu:717-804): its state, force and
// torques on both solids.
__device__ __forceinline__ void bondUpdate(const DeviceState& d, int par, float dt, int b)
{
    // Every load the update needs is issued before the bond's checks (a broken
    // bond, a pair that left the contact list), which end in stores: the
    // loads then wait for one another only through the pair's indices, not
    // behind the search of the contact list.
    const int2 ab = d.bab[b];
    const int bonded = d.bon[b];
    const float4 FnTt0 = d.bFnTt[b], FsH0 = d.bFsH[b], FsL0 = d.bFsL[b], TbH0 = d.bTbH[b], TbL0 = d.bTbL[b];
    const float3 n0 = xyz(d.bN[b]);
    const int i = ab.x, j = ab.y;
    const PairGeom g = pairGeometry(d, i, j);
    const float3 wi = xyz(d.swh[i]), wj = xyz(d.swh[j]);
    const float3 vc = contactVel(d, i, j, g.leverA, g.leverB);
    const float3 wr = spinDiff(d, i, j);
    const float4 ri = d.srad[i], rj = d.srad[j];
    const int ms = tableSlot(d.tab, d.sflags[i].x, d.sflags[j].x);
    const long long slot = forwardSlot(d, par, i, j);
    if (bonded == 0) {
        d.bFnTt[b] = make_float4(0, 0, 0, 0);
        d.bFsH[b] = d.bFsL[b] = d.bTbH[b] = d.bTbL[b] = make_float4(0, 0, 0, 0);
        d.bN[b] = make_float4(0, 0, 0, 0);
        d.bF[b] = d.bTA[b] = d.bTB[b] = make_float4(0, 0, 0, 0);
        return;
    }
    if (slot < 0) {  // the pair left the contact list: the bond breaks
        d.bon[b] = 0;
        d.bF[b] = d.bTA[b] = d.bTB[b] = make_float4(0, 0, 0, 0);
        return;
    }
    const float3 n = g.n;
    const float* B = d.tab.bd + 6 * ms;  // gamma E knks sigma C mu
    const float4 FnTt = FnTt0;
    float4 FsH = FsH0, FsL = FsL0, TbH = TbH0, TbL = TbL0;
    // rotate shear force / bending torque with the normal, then about it
    const float3 th1 = cross3(n0, n);
    rotateDF(FsH, FsL, th1);
    rotateDF(TbH, TbL, th1);
    const float3 th2 = n * dot3((wi + wj) * (0.5f * dt), n);
    rotateDF(FsH, FsL, th2);
    rotateDF(TbH, TbL, th2);
    const float rmin = ri.x < rj.x ? ri.x : rj.x;
    const float br = B[0] * rmin;
    const float Ab = br * br * 3.14159265358979323846f;
    const float Ib = br * br * br * br / 4.f * 3.14159265358979323846f;
    const float Jb = 2.f * Ib;
    const float kn = B[1] / (ri.x + rj.x);
    const float ks = kn / B[2];
    const float3 dn = n * (dot3(vc, n) * dt);
    const float3 dtg = vc * dt - dn;
    dfl Fn = df_add_f(df_make(FnTt.x, FnTt.y), -dot3(dn * (kn * Ab), n));
    addDF3(FsH, FsL, dtg * (-ks * Ab));
    const float3 dn2 = n * (dot3(wr, n) * dt);
    const float3 dt2 = wr * dt - dn2;
    dfl Tt = df_add_f(df_make(FnTt.z, FnTt.w), -dot3(dn2 * (ks * Jb), n));
    addDF3(TbH, TbL, dt2 * (-kn * Ib));
    const float fn = Fn.hi + Fn.lo, tt = Tt.hi + Tt.lo;
    const float3 Fs = xyz(FsH) + xyz(FsL), Tb = xyz(TbH) + xyz(TbL);
    const float sN = -fn / Ab + len3(Tb) / Ib * br;
    const float sS = len3(Fs) / Ab + fabsf(tt) / Jb * br;
    int on = 1;
    if (B[3] > 0.f && sN > B[3]) on = 0;
    else if (B[4] > 0.f && sS > B[4] - B[5] * sN) on = 0;
    d.bon[b] = on;
    d.bFnTt[b] = make_float4(Fn.hi, Fn.lo, Tt.hi, Tt.lo);
    d.bFsH[b] = FsH;
    d.bFsL[b] = FsL;
    d.bTbH[b] = TbH;
    d.bTbL[b] = TbL;
    d.bN[b] = f4(n);
    d.bLever[b] = f4(g.leverA);
    // the bond's share of the pair's force and torque (integrate.cu:802-803),
    // added per solid by kSolidForces
    const float3 F = n * fn + Fs;
    const float3 Tq = n * tt + Tb;
    const float3 nxF = cross3(n, Fs);  // the lever is along n: n x (fn n) = 0
    d.bF[b] = f4(F);
    d.bTA[b] = f4(Tq + nxF * g.sA);
    d.bTB[b] = f4(Tq + nxF * g.sB);
}

// Wall overlap r - ((x - p) . n) in double-float.
__device__ __forceinline__ float wallOverlap(const DeviceState& d, int4 c, float4 h, float4 l, int k, float r,
                                             float rlo)
{
    const float4 nh = d.wnh[k], nl = d.wnl[k];
    const dfl px = df_add(df_mul_f(d.grid.csx, (float)c.x), df_make(h.x, l.x));
    const dfl py = df_add(df_mul_f(d.grid.csy, (float)c.y), df_make(h.y, l.y));
    const dfl pz = df_add(df_mul_f(d.grid.csz, (float)c.z), df_make(h.z, l.z));
    dfl s = df_mul(df_make(nh.x, nl.x), px);
    s = df_add(s, df_mul(df_make(nh.y, nl.y), py));
    s = df_add(s, df_mul(df_make(nh.z, nl.z), pz));
    const float2 P = d.wP[k];
    s = df_sub(s, df_make(P.x, P.y));
    const dfl del = df_sub(df_make(r, rlo), s);
    return del.hi + del.lo;
}

// The rest of a row's force and torque once its contact and bond items are
// summed: the coupling force, gravity and the infinite walls
// (integrate.cu:514-610); stores the acceleration and torque.  Wall springs
// come from the previous contact phase's parity and go to this step's
// (wmask bit k, walls below 32: wall k's springs may be non-zero), so a step
// abandoned after an overflow leaves the springs it started from.
__device__ __forceinline__ void solidRowTail(const DeviceState& d, int par, int a, KahanF3& F, KahanF3& Tq,
                                             int withCoupling, float dt)
{
    const int prev = par ^ 1;
    const int4 fa = d.sflags[a];
    if (withCoupling) F.add(-xyz(d.sfcoup[a]));
    const float4 ph = d.sph[a];
    const float im = ph.w;
    float3 acc = F.sum() * im;
    if ((fa.w & F_HASMASS) && fa.z < 0) acc = acc + d.g;
    float3 tq = Tq.sum();
    if (d.nw > 0 && !(fa.w & F_DUMMY) && !(fa.w & F_FIXED)) {
        const int4 ca = d.scell[a];
        const float4 pl = d.spl[a];
        const float4 rad = d.srad[a];
        const float3 v = xyz(d.svh[a]), w = xyz(d.swh[a]);
        const unsigned held0 = d.wmask[prev][a];
        unsigned mask = 0;
        const float3 pf = make_float3((float)ca.x * d.grid.cs.x + ph.x, (float)ca.y * d.grid.cs.y + ph.y,
                                      (float)ca.z * d.grid.cs.z + ph.z);
        int k = 0;
        for (; k < d.nw; ++k) {
            const size_t h = (size_t)k * d.ns + a;  // wall-major: a warp's solids are adjacent
            const bool held = k >= 32 || ((held0 >> k) & 1u);
            // FP32 pre-test: a sphere clearly off the wall (by far more than
            // the FP32 rounding of this estimate) has a negative exact overlap
            const float3 nf = xyz(d.wnh[k]);
            const float Pf = d.wP[k].x;
            const float est = rad.x - (dot3(nf, pf) - Pf);
            const float tol = 4.e-6f * (fabsf(pf.x) + fabsf(pf.y) + fabsf(pf.z) + fabsf(Pf) + rad.x);
            const float delta = est < -tol ? -1.f : wallOverlap(d, ca, ph, pl, k, rad.x, rad.y);
            if (delta < 0.f) {
                // no contact: the springs are zero (bit k stays clear; walls
                // from 32 on have no bit and store the zeros)
                if (k >= 32) d.wspring[par][0][h] = d.wspring[par][1][h] = d.wspring[par][2][h] = make_float4(0, 0, 0, 0);
                if (d.fixes & DEMSPH_FIX_WALL_LOOP) continue;
                break;
            }
            const float3 n = xyz(d.wnh[k]);
            const float3 lever = n * (-(rad.x - delta));
            const float3 vc = v + cross3(w, lever);
            float3 es = make_float3(0.f, 0.f, 0.f), er = es, et = es;
            if (held) {
                es = xyz(d.wspring[prev][0][h]);
                er = xyz(d.wspring[prev][1][h]);
                et = xyz(d.wspring[prev][2][h]);
            }
            float3 Fw = make_float3(0.f, 0.f, 0.f), Fwt = Fw, Tw = Fw;
            const int slot = tableSlot(d.tab, fa.x, d.wmat[k]);
            contactLaw(d.tab, slot, Fw, Fwt, Tw, es, er, et, vc, w, n, delta, 1.f / im, rad.x, dt);
            d.wspring[par][0][h] = f4(es);
            d.wspring[par][1][h] = f4(er);
            d.wspring[par][2][h] = f4(et);
            if (k < 32) mask |= 1u << k;
            acc = acc + Fw * im;
            tq = tq + Tw + cross3(n, Fwt) * (-(rad.x - delta));
        }
        // the walls after the first one not touched keep their springs (the
        // reference returns from its wall loop there)
        for (++k; k < d.nw; ++k) {
            if (k < 32 && !((held0 >> k) & 1u)) continue;
            const size_t h = (size_t)k * d.ns + a;
            d.wspring[par][0][h] = d.wspring[prev][0][h];
            d.wspring[par][1][h] = d.wspring[prev][1][h];
            d.wspring[par][2][h] = d.wspring[prev][2][h];
            if (k < 32) mask |= 1u << k;
        }
        d.wmask[par][a] = mask;
    }
    d.sacc[a] = f4(acc);
    d.storque[a] = f4(tq);
}

// The contact forces of a step (calSolidContactForceTorque,
// core/integrate.cu:423-512), each contact evaluated once, by the row of its
// lower solid A (forward slot k): the springs advance, the slot keeps the
// force on A, the contact torque as the reference stores it and the torque on
// A with its lever arm, and the pair's slot in B's reverse list (found by
// its id, while the force is evaluated) gets minus the force and minus the
// torque on B with its lever arm.  The bonds (blocks from contactBlocks on)
// are updated in the same launch: kSolidForces reads both.
//
// Rows hold few contacts and their counts vary: a warp shares its rows'
// forward contacts out through warpItems, one lane per contact.
#ifndef DEMSPH_PAIR_FORCE_BLOCKS
#define DEMSPH_PAIR_FORCE_BLOCKS 6  // resident blocks of T per SM the registers allow
#endif
__global__ void __launch_bounds__(T, DEMSPH_PAIR_FORCE_BLOCKS) kPairForces(DeviceState d, int par, float dt, int rowsPerWarp,
                                                    int contactBlocks)
{
    stepKernelBegin();
    if (*d.status) return;
    if ((int)blockIdx.x >= contactBlocks) {
        const int b = ((int)blockIdx.x - contactBlocks) * blockDim.x + threadIdx.x;
        if (b < d.nb) bondUpdate(d, par, dt, b);
        return;
    }
    // this step's flag has been read by every row's contact detection (the
    // launch before); the step before's flag is free for this step's closing
    // drift to raise
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *(volatile int*)&d.rebuild[par] = 0;
        *(volatile int*)&d.rebuild[par ^ 1] = 0;
    }
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // lanes 0 .. rowsPerWarp - 1 of each warp own a row
    const int row0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * rowsPerWarp;
    const int row = row0 + lane;
    const bool live = lane < rowsPerWarp && row < d.nrow;
    const int a = live ? solidOf(d, row) : 0;
    const size_t nr = (size_t)d.nrow;
    const int n = live ? min(d.fcnt[par][row], d.scap) : 0;
    warpItems(n, [&](int owner, int q, bool valid) {
        const int A = __shfl_sync(FULL, a, owner);
        if (!valid) return;
        const size_t k = (size_t)q * nr + (row0 + owner);
        const int B = d.fwd[par][k];
        const float3 es0 = xyz(d.springIn[0][k]), er0 = xyz(d.springIn[1][k]), et0 = xyz(d.springIn[2][k]);
        // B's reverse slot of the pair (a reverse list has no entry for it
        // when B's detection did not find it)
        const int rb = rowOf(d, B);
        long long kr = -1;
        if (rb >= 0)
            for (int m = min(d.rcnt[rb], d.scap), u = 0; u < m; ++u)
                if (d.rev[(size_t)u * nr + rb] == A) {
                    kr = (long long)u * nr + rb;
                    break;
                }
        float3 es = es0, er = er0, et = et0;
        const PairForce p = pairForce(d, A, B, es, er, et, dt);
        d.springOut[par][0][k] = f4(es);
        d.springOut[par][1][k] = f4(er);
        d.springOut[par][2][k] = f4(et);
        d.pF[k] = f4(p.F);
        d.pT[k] = f4(p.T);
        d.pTA[k] = f4(p.TA);
        if (kr >= 0) {
            const float3 mF = -p.F;
            d.revF[kr] = make_float4(mF.x, mF.y, mF.z, 1.f);
            d.revT[kr] = f4(-p.TB);
        }
    });
}

// Force and torque on every solid that can touch others (calSolidForceTorque,
// core/integrate.cu:806-858, with the walls of :514-610), one thread per row,
// from the pair results of kPairForces: the forward contacts (the force on A
// and its torque), then the reverse ones (minus the force, minus the torque
// on B; a reverse slot that no forward row holds was left marked by the
// detection and adds nothing), then the bonds.  Sums are Kahan-compensated,
// in that order - no atomics.  Every item is a few loads: they are issued
// GATHER_BATCH at a time before their sums (the slots [k * nrow + row] of
// neighbouring rows are neighbouring words).
constexpr int GATHER_BATCH = 4;
// Row `row`'s sums and tail; returns its solid.
__device__ __forceinline__ int solidForcesRow(const DeviceState& d, int par, float dt, int withCoupling, int row)
{
    const int a = solidOf(d, row);
    const size_t nr = (size_t)d.nrow;
    const int n = min(d.fcnt[par][row], d.scap), m = min(d.rcnt[row], d.scap);
    const int b0 = d.bondStart[a], b1 = d.bondStart[a + 1];
    KahanF3 F, Tq;
    for (int q0 = 0; q0 < n; q0 += GATHER_BATCH) {
        float4 f[GATHER_BATCH], t[GATHER_BATCH];
#pragma unroll
        for (int u = 0; u < GATHER_BATCH; ++u)
            if (q0 + u < n) {
                const size_t k = (size_t)(q0 + u) * nr + row;
                f[u] = d.pF[k];
                t[u] = d.pTA[k];
            }
#pragma unroll
        for (int u = 0; u < GATHER_BATCH; ++u)
            if (q0 + u < n) {
                F.add(xyz(f[u]));
                Tq.add(xyz(t[u]));
            }
    }
    for (int q0 = 0; q0 < m; q0 += GATHER_BATCH) {
        float4 f[GATHER_BATCH], t[GATHER_BATCH];
#pragma unroll
        for (int u = 0; u < GATHER_BATCH; ++u)
            if (q0 + u < m) {
                const size_t k = (size_t)(q0 + u) * nr + row;
                f[u] = d.revF[k];
                t[u] = d.revT[k];
            }
#pragma unroll
        for (int u = 0; u < GATHER_BATCH; ++u)
            if (q0 + u < m && f[u].w != 0.f) {  // w 0: a reverse pair the forward row does not hold
                F.add(xyz(f[u]));
                Tq.add(xyz(t[u]));
            }
    }
    for (int q0 = b0; q0 < b1; q0 += GATHER_BATCH) {
        int bi[GATHER_BATCH];
#pragma unroll
        for (int u = 0; u < GATHER_BATCH; ++u) bi[u] = q0 + u < b1 ? d.bondList[q0 + u] : 0;
        float4 f[GATHER_BATCH], t[GATHER_BATCH];
        bool sideA[GATHER_BATCH];
#pragma unroll
        for (int u = 0; u < GATHER_BATCH; ++u)
            if (q0 + u < b1) {
                f[u] = d.bF[bi[u]];
                sideA[u] = d.bab[bi[u]].x == a;
                t[u] = sideA[u] ? d.bTA[bi[u]] : d.bTB[bi[u]];
            }
#pragma unroll
        for (int u = 0; u < GATHER_BATCH; ++u)
            if (q0 + u < b1) {
                F.add(sideA[u] ? xyz(f[u]) : -xyz(f[u]));
                Tq.add(sideA[u] ? xyz(t[u]) : -xyz(t[u]));
            }
    }
    solidRowTail(d, par, a, F, Tq, withCoupling, dt);
    return a;
}

__global__ void __launch_bounds__(T) kSolidForces(DeviceState d, int par, float dt, int withCoupling)
{
    stepKernelBegin();
    if (*d.status) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row < d.nrow) solidForcesRow(d, par, dt, withCoupling, row);
}

// The contact list of a plain DEM step opened by a fused integration pass
// and its contact forces in one launch (no bonds; 32 rows per warp): each
// lane first builds its row's list from the candidates (rebuilt when stale)
// on the end-of-step offsets sphE/splE, exactly as kContactDetect does; a
// warp then runs its rows' contacts through warpItems, one lane per contact,
// each contact evaluated by both of its solids with its springs from the
// previous list (springOut of the other parity - the values kContactDetect's
// remap would hand them): the same instructions on the same inputs give both
// sides the bits kPairForces gives the pair, and the per-row sums are those
// of kSolidForces, in the same order.  The candidates and the contact test
// are symmetric in the two solids, so the forward row of every reverse pair
// holds it.  In the walk mode they need not be: the launch then raises
// ST_SPLIT_CONTACTS before writing anything, and the step is redone with the
// separate launches.
__global__ void __launch_bounds__(T, 6) kContactForces(DeviceState d, int par, float dt, int withCoupling)
{
    stepKernelBegin();
    __shared__ float4 itemF[T], itemT[T];  // 32 items per warp
    if (*d.status) return;
    if (*d.slowMode) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(d.status, ST_SPLIT_CONTACTS);
        return;
    }
    const int prev = par ^ 1;
    // this step's flag is cleared by the next step's launch (this launch's
    // rows read it); the step before's flag is free for this step's closing
    // drift to raise
    if (blockIdx.x == 0 && threadIdx.x == 0) *(volatile int*)&d.rebuild[prev] = 0;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int row0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
    const int row = row0 + lane;
    const bool live = row < d.nrow;
    const int a = live ? solidOf(d, row) : 0;
    const size_t nr = (size_t)d.nrow;
    // forward contacts (a, b) come first, then reverse ones (b, a)
    int n = 0, contacts = 0;
    if (live) {
        DeviceState atEnd = d;  // the end-of-step offsets
        atEnd.sph = d.sphE;
        atEnd.spl = d.splE;
        if (d.rebuild[par]) verletBuildRow(atEnd, row);
        const int C = d.scap;
        int nf = 0, nb = 0;
        const int nc = min(d.vcnt[row], d.vcap);
        for (int k = 0; k < nc; ++k) {
            const int b = d.vcand[(size_t)k * nr + row];
            if (!solidsTouch(atEnd, a, b)) continue;
            if (b > a) {
                if (nf < C) d.fwd[par][(size_t)nf * nr + row] = b;
                ++nf;
            } else {
                if (nb < C) d.rev[(size_t)nb * nr + row] = b;
                ++nb;
            }
        }
        d.fcnt[par][row] = nf;
        d.rcnt[row] = nb;
        if (nf > C || nb > C) {
            atomicOr(d.status, ST_SS_OVERFLOW);
            atomicMax(&d.need[0], max(nf, nb));
            nf = nb = 0;
        }
        n = nf;
        contacts = nf + nb;
    }
    __syncwarp();  // the row's list entries, for the lanes that evaluate them
    float4* resF = itemF + (threadIdx.x & ~31);
    float4* resT = itemT + (threadIdx.x & ~31);
    KahanF3 F, Tq;
    warpItems(
        contacts,
        [&](int owner, int q, bool valid) {
            const int oa = __shfl_sync(FULL, a, owner), on = __shfl_sync(FULL, n, owner);
            const int orow = row0 + owner;
            float4 rF = make_float4(0.f, 0.f, 0.f, 0.f), rT = rF;
            if (valid) {
                // through ONE inlined copy of pairForce: a pair's two solids run
                // the same instructions on the same inputs and get the same bits
                const bool fwdSide = q < on;
                int A = oa, B;
                size_t k = 0;
                if (fwdSide) {
                    k = (size_t)q * nr + orow;
                    B = d.fwd[par][k];
                } else {
                    A = d.rev[(size_t)(q - on) * nr + orow];
                    B = oa;
                }
                float3 es = make_float3(0.f, 0.f, 0.f), er = es, et = es;
                const long long ko = forwardSlot(d, prev, A, B);  // the pair in the previous list
                if (ko >= 0) {
                    es = xyz(d.springOut[prev][0][ko]);
                    er = xyz(d.springOut[prev][1][ko]);
                    et = xyz(d.springOut[prev][2][ko]);
                }
                const PairForce p = pairForce(d, A, B, es, er, et, dt);
                if (fwdSide) {
                    d.springOut[par][0][k] = f4(es);
                    d.springOut[par][1][k] = f4(er);
                    d.springOut[par][2][k] = f4(et);
                    d.pF[k] = f4(p.F);
                    d.pT[k] = f4(p.T);
                    rF = make_float4(p.F.x, p.F.y, p.F.z, 1.f);
                    rT = f4(p.TA);
                } else {
                    const float3 mF = -p.F, mT = -p.TB;
                    rF = make_float4(mF.x, mF.y, mF.z, 1.f);
                    rT = f4(mT);
                }
            }
            resF[lane] = rF;
            resT[lane] = rT;
        },
        [&](int, int pos) {
            const float4 f = resF[pos];
            if (f.w != 0.f) {
                F.add(xyz(f));
                Tq.add(xyz(resT[pos]));
            }
        });
    if (!live) return;
    solidRowTail(d, par, a, F, Tq, withCoupling, dt);
}

// x_i - centroid of pebble i as double-float per axis, then float.
__device__ __forceinline__ float3 pebbleLever(const DeviceState& d, int i, float4 cH, float4 cL)
{
    const int4 c = d.scell[i];
    const float4 h = d.sph[i], l = d.spl[i];
    const dfl x = df_sub(df_add(df_mul_f(d.grid.csx, (float)c.x), df_make(h.x, l.x)), df_make(cH.x, cL.x));
    const dfl y = df_sub(df_add(df_mul_f(d.grid.csy, (float)c.y), df_make(h.y, l.y)), df_make(cH.y, cL.y));
    const dfl z = df_sub(df_add(df_mul_f(d.grid.csz, (float)c.z), df_make(h.z, l.z)), df_make(cH.z, cL.z));
    return make_float3(x.hi + x.lo, y.hi + y.lo, z.hi + z.lo);
}

// Double-float sum over the `width` lanes of a group (width a power of two
// <= 32), in a fixed tree: every lane gets the same bits.
__device__ __forceinline__ dfl groupSumDF(dfl v, int width)
{
    for (int o = width >> 1; o > 0; o >>= 1) {
        const dfl u = df_make(__shfl_xor_sync(0xffffffffu, v.hi, o, width), __shfl_xor_sync(0xffffffffu, v.lo, o, width));
        // the same operand order on both lanes of a pair: lower lane first
        v = (threadIdx.x & o) ? df_add(u, v) : df_add(v, u);
    }
    return v;
}

// calClumpForceTorque (integrate.cu:860-881): a group of `width` lanes per
// clump over its pebbles; the pebbles' forces (a m) and torques about the
// centroid are summed in double-float, reduced in a fixed tree.
__device__ __forceinline__ void clumpForceGroup(const DeviceState& d, int width, int t)
{
    const int c = t / width, lane = t % width;
    // whole warps only: the shuffles below take every lane of the warp
    if ((t & ~31) >= d.nc * width || *d.status) return;
    const bool live = c < d.nc;
    dfl Fx = df_make(0.f, 0.f), Fy = Fx, Fz = Fx, Tx = Fx, Ty = Fx, Tz = Fx;
    if (live) {
        const float4 cH = d.cpH[c], cL = d.cpL[c];
        for (int i = d.cstart[c] + lane; i < d.cend[c]; i += width) {
            float3 fi = make_float3(0.f, 0.f, 0.f);
            if (d.sflags[i].w & F_MASSIVE) fi = xyz(d.sacc[i]) / d.sph[i].w;
            const float3 ti = xyz(d.storque[i]) + cross3(pebbleLever(d, i, cH, cL), fi);
            Fx = df_add_f(Fx, fi.x);
            Fy = df_add_f(Fy, fi.y);
            Fz = df_add_f(Fz, fi.z);
            Tx = df_add_f(Tx, ti.x);
            Ty = df_add_f(Ty, ti.y);
            Tz = df_add_f(Tz, ti.z);
            d.sacc[i] = make_float4(0, 0, 0, 0);
            d.storque[i] = make_float4(0, 0, 0, 0);
        }
    }
    Fx = groupSumDF(Fx, width);
    Fy = groupSumDF(Fy, width);
    Fz = groupSumDF(Fz, width);
    Tx = groupSumDF(Tx, width);
    Ty = groupSumDF(Ty, width);
    Tz = groupSumDF(Tz, width);
    if (live && lane == 0) {
        const float im = d.cinvm[c];
        float3 a = make_float3(Fx.hi + Fx.lo, Fy.hi + Fy.lo, Fz.hi + Fz.lo) * im;
        if (im > 0.f) a = a + d.g;
        d.cacc[c] = f4(a);
        d.ctorque[c] = make_float4(Tx.hi + Tx.lo, Ty.hi + Ty.lo, Tz.hi + Tz.lo, 0.f);
    }
}

// Double-float x += v dt for one position (hi/lo float4 pairs, w kept).
__device__ __forceinline__ void driftRegs(float4& h, float4& l, float4 vh, float4 vl, dfl dt)
{
    const dfl x = df_add(df_make(h.x, l.x), df_mul(df_make(vh.x, vl.x), dt));
    const dfl y = df_add(df_make(h.y, l.y), df_mul(df_make(vh.y, vl.y), dt));
    const dfl z = df_add(df_make(h.z, l.z), df_mul(df_make(vh.z, vl.z), dt));
    h = make_float4(x.hi, y.hi, z.hi, h.w);
    l = make_float4(x.lo, y.lo, z.lo, l.w);
}

// double-float x += v dt for one particle's position (solid arrays).
__device__ __forceinline__ void driftSolid(const DeviceState& d, int i, dfl dt)
{
    float4 h = d.sph[i], l = d.spl[i];
    driftRegs(h, l, d.svh[i], d.svl[i], dt);
    d.sph[i] = h;
    d.spl[i] = l;
}

// solidVelocityAngularVelocityIntegrate (integrate.cu:883-897) for one
// particle: v += a dt, and w += T / (0.4 m r^2) dt unless it is fixed or has
// no radius (spin false).
__device__ __forceinline__ void kickRegs(float4& vh, float4& vl, float4& wh, float4& wl, float3 a, float3 tq, float r,
                                         float im, bool spin, dfl dt)
{
    {
        const dfl x = df_add(df_make(vh.x, vl.x), df_mul_f(dt, a.x));
        const dfl y = df_add(df_make(vh.y, vl.y), df_mul_f(dt, a.y));
        const dfl z = df_add(df_make(vh.z, vl.z), df_mul_f(dt, a.z));
        vh = make_float4(x.hi, y.hi, z.hi, vh.w);
        vl = make_float4(x.lo, y.lo, z.lo, vl.w);
    }
    if (!spin) return;
    const float3 alpha = tq * (im / (0.4f * r * r));
    const dfl x = df_add(df_make(wh.x, wl.x), df_mul_f(dt, alpha.x));
    const dfl y = df_add(df_make(wh.y, wl.y), df_mul_f(dt, alpha.y));
    const dfl z = df_add(df_make(wh.z, wl.z), df_mul_f(dt, alpha.z));
    wh = make_float4(x.hi, y.hi, z.hi, wh.w);
    wl = make_float4(x.lo, y.lo, z.lo, wl.w);
}

// One half-step of a solid that is not a clump pebble (integrate.cu:964-1027):
// before contact kick then drift; after contact drift, kick, the displacement
// check and the cell key of the next step; fused, the after-contact half, its
// end-of-step offset to sphE/splE, then the next step's before-contact half
// from the same registers (the same operations on the same values as the two
// separate passes).  Every input is read before anything is written: the
// compiler cannot tell the arrays apart, so a read placed after a write would
// wait for it.
template <int MODE>
__device__ __forceinline__ void solidIntegrateOne(const DeviceState& d, int i, dfl half, int* stale)
{
    const int4 f = d.sflags[i];
    float4 ph = d.sph[i], pl = d.spl[i], vh = d.svh[i], vl = d.svl[i], wh = d.swh[i], wl = d.swl[i];
    const float3 a = xyz(d.sacc[i]), tq = xyz(d.storque[i]);
    const float r = d.srad[i].x;
    int row = -1;
    int4 c = make_int4(0, 0, 0, 0);
    float4 p0 = make_float4(0, 0, 0, 0), q0 = p0;
    if (MODE != INTEGRATE_BEFORE) {
        row = rowOf(d, i);
        c = d.scell[i];
        p0 = d.vref[i];
        if (d.nf > 0) q0 = d.svref[i];
    }
    if (f.z >= 0) return;  // clump pebbles: clumpIntegrateGroup
    const bool spin = !((f.w & F_FIXED) || r < 1.e-10f);
    if (MODE != INTEGRATE_BEFORE) {
        driftRegs(ph, pl, vh, vl, half);
        kickRegs(vh, vl, wh, wl, a, tq, r, ph.w, spin, half);
        checkDisplacementOf(d, stale, row, c, ph, p0, q0);
        rehashSolidTo(d, i, row, c, ph, pl, MODE == INTEGRATE_FUSED ? d.sphE : d.sph,
                      MODE == INTEGRATE_FUSED ? d.splE : d.spl);
    }
    if (MODE != INTEGRATE_AFTER) {
        kickRegs(vh, vl, wh, wl, a, tq, r, ph.w, spin, half);
        driftRegs(ph, pl, vh, vl, half);
        d.sph[i] = ph;
        d.spl[i] = pl;
    }
    d.svh[i] = vh;
    d.svl[i] = vl;
    if (spin) {
        d.swh[i] = wh;
        d.swl[i] = wl;
    }
}

// Symmetric 3x3 (xx yy zz xy xz yz) times a vector.
__device__ __forceinline__ float3 symTimes(const float* I, float3 t)
{
    return make_float3(I[0] * t.x + I[3] * t.y + I[4] * t.z, I[3] * t.x + I[1] * t.y + I[5] * t.z,
                       I[4] * t.x + I[5] * t.y + I[2] * t.z);
}

__device__ __forceinline__ void addDF(float4& h, float4& l, float3 dv)
{
    const dfl x = df_add_f(df_make(h.x, l.x), dv.x), y = df_add_f(df_make(h.y, l.y), dv.y),
              z = df_add_f(df_make(h.z, l.z), dv.z);
    h = make_float4(x.hi, y.hi, z.hi, 0.f);
    l = make_float4(x.lo, y.lo, z.lo, 0.f);
}

// x += v dt in double-float (x, v as hi/lo float4 pairs).
__device__ __forceinline__ void axpyDF(float4& xh, float4& xl, float4 vh, float4 vl, dfl dt)
{
    const dfl x = df_add(df_make(xh.x, xl.x), df_mul(df_make(vh.x, vl.x), dt));
    const dfl y = df_add(df_make(xh.y, xl.y), df_mul(df_make(vh.y, vl.y), dt));
    const dfl z = df_add(df_make(xh.z, xl.z), df_mul(df_make(vh.z, vl.z), dt));
    xh = make_float4(x.hi, y.hi, z.hi, 0.f);
    xl = make_float4(x.lo, y.lo, z.lo, 0.f);
}

// First-order quaternion update with the mean spin, renormalised, and the
// world-frame inverse inertia from the new orientation (only with
// DEMSPH_FIX_CLUMP_ROTATION; the reference never turns a clump's orientation).
__device__ void clumpRotate(const DeviceState& d, int c, float3 w0, float3 w, float dt)
{
    const double vx = 0.5 * ((double)w0.x + w.x) * dt, vy = 0.5 * ((double)w0.y + w.y) * dt,
                 vz = 0.5 * ((double)w0.z + w.z) * dt;
    const double4 q = d.cq[c];
    double4 n = make_double4(q.x + 0.5 * (-q.y * vx - q.z * vy - q.w * vz), q.y + 0.5 * (q.x * vx + q.w * vy - q.z * vz),
                             q.z + 0.5 * (-q.w * vx + q.x * vy + q.y * vz), q.w + 0.5 * (q.z * vx - q.y * vy + q.x * vz));
    const double l = sqrt(n.x * n.x + n.y * n.y + n.z * n.z + n.w * n.w);
    if (l > 0) n = make_double4(n.x / l, n.y / l, n.z / l, n.w / l);
    d.cq[c] = n;
    // R invI R^T (core/myMat.h:102-127)
    const double q0 = n.x, q1 = n.y, q2 = n.z, q3 = n.w;
    const double R[3][3] = {{1 - 2 * q2 * q2 - 2 * q3 * q3, 2 * q1 * q2 - 2 * q0 * q3, 2 * q1 * q3 + 2 * q0 * q2},
                            {2 * q1 * q2 + 2 * q0 * q3, 1 - 2 * q1 * q1 - 2 * q3 * q3, 2 * q2 * q3 - 2 * q0 * q1},
                            {2 * q1 * q3 - 2 * q0 * q2, 2 * q2 * q3 + 2 * q0 * q1, 1 - 2 * q1 * q1 - 2 * q2 * q2}};
    const double* I = d.cinvI + 6 * c;
    const double B[3][3] = {{I[0], I[3], I[4]}, {I[3], I[1], I[5]}, {I[4], I[5], I[2]}};
    double W[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k)
                for (int m = 0; m < 3; ++m) s += R[i][k] * B[k][m] * R[j][m];
            W[i][j] = s;
        }
    float* o = d.cIw + 6 * c;
    o[0] = (float)W[0][0];
    o[1] = (float)W[1][1];
    o[2] = (float)W[2][2];
    o[3] = (float)W[0][1];
    o[4] = (float)W[0][2];
    o[5] = (float)W[1][2];
}

// The rigid-body motion handed to pebble i (clumpVelocityAngularVelocityIntegrate,
// integrate.cu:908-929): acceleration a + a x r + w x (w x r) (the reference's
// form), velocity v + w x r, spin w, and the normal turned by the mean spin.
__device__ __forceinline__ void pebbleKick(const DeviceState& d, int i, float3 a, float4 vH, float4 vL, float4 wH,
                                           float4 wL, float4 cH, float4 cL, float3 rotn)
{
    const float3 r = pebbleLever(d, i, cH, cL);
    const float3 w = xyz(wH);
    d.sacc[i] = f4(a + cross3(a, r) + cross3(w, cross3(w, r)));
    addDF(vH, vL, cross3(w, r));
    d.svh[i] = vH;
    d.svl[i] = vL;
    d.swh[i] = wH;
    d.swl[i] = wL;
    d.snormal[i] = f4(rotateF(xyz(d.snormal[i]), rotn));
}

// Half-step clump integration (clumpVelocityAngularVelocityIntegrate and
// clumpPositionIntegrate, integrate.cu:908-938, in the order of
// integrate.cu:964-1027), a group of `width` lanes per clump: the group's
// first lane advances the clump's state, the lanes then move the pebbles.
//   before contact: kick, pebbles from the kicked state, centroid and pebble drift;
//   after contact:  pebble and centroid drift, kick, pebbles from the kicked state.
//   withEnd (after contact): the pebbles' end-of-step offsets also go to
//   sphE/splE (a fused pass, whose before-contact half follows).
__device__ __forceinline__ void clumpIntegrateGroup(const DeviceState& d, dfl halfDF, int before, int width, int t,
                                                    int* stale, bool withEnd = false)
{
    const int c = t / width, lane = t % width;
    // whole warps only: the shuffles below take every lane of the warp
    if ((t & ~31) >= d.nc * width || *d.status) return;
    const bool live = c < d.nc;
    const int s = live ? d.cstart[c] : 0, e = live ? d.cend[c] : 0;
    if (!before)
        for (int i = s + lane; i < e; i += width) driftSolid(d, i, halfDF);
    float4 v[6];  // centroid hi lo, velocity hi lo, spin hi lo
    float3 a = make_float3(0.f, 0.f, 0.f), w0 = a;
    if (live && lane == 0) {
        float4 cH = d.cpH[c], cL = d.cpL[c], vH = d.cvH[c], vL = d.cvL[c], wH = d.cwH[c], wL = d.cwL[c];
        if (!before) axpyDF(cH, cL, vH, vL, halfDF);
        a = xyz(d.cacc[c]);
        w0 = xyz(wH);
        const float hdt = halfDF.hi;
        addDF(vH, vL, a * hdt);
        if (d.cinvm[c] > 0.f) addDF(wH, wL, symTimes(d.cIw + 6 * c, xyz(d.ctorque[c])) * hdt);
        v[0] = cH; v[1] = cL; v[2] = vH; v[3] = vL; v[4] = wH; v[5] = wL;
        d.cvH[c] = vH;
        d.cvL[c] = vL;
        d.cwH[c] = wH;
        d.cwL[c] = wL;
        if (before) axpyDF(cH, cL, vH, vL, halfDF);
        d.cpH[c] = cH;
        d.cpL[c] = cL;
        if (d.fixes & DEMSPH_FIX_CLUMP_ROTATION) clumpRotate(d, c, w0, xyz(wH), hdt);
    }
    // hand the state (centroid before this half step's drift when before
    // contact, after it when after contact) to the group
#pragma unroll
    for (int k = 0; k < 6; ++k)
        v[k] = make_float4(__shfl_sync(0xffffffffu, v[k].x, 0, width), __shfl_sync(0xffffffffu, v[k].y, 0, width),
                           __shfl_sync(0xffffffffu, v[k].z, 0, width), 0.f);
    a = make_float3(__shfl_sync(0xffffffffu, a.x, 0, width), __shfl_sync(0xffffffffu, a.y, 0, width),
                    __shfl_sync(0xffffffffu, a.z, 0, width));
    w0 = make_float3(__shfl_sync(0xffffffffu, w0.x, 0, width), __shfl_sync(0xffffffffu, w0.y, 0, width),
                     __shfl_sync(0xffffffffu, w0.z, 0, width));
    const float3 rotn = (w0 + xyz(v[4])) * (0.5f * halfDF.hi);
    for (int i = s + lane; i < e; i += width) {
        pebbleKick(d, i, a, v[2], v[3], v[4], v[5], v[0], v[1], rotn);
        if (before) {
            driftSolid(d, i, halfDF);
        } else {
            checkDisplacement(d, stale, i);
            rehashSolid(d, i, withEnd);
        }
    }
}

__global__ void kClumpForce(DeviceState d, int width)
{
    stepKernelBegin();
    clumpForceGroup(d, width, blockIdx.x * blockDim.x + threadIdx.x);
}

// One half-step integration of all solids (integrate.cu:964-1027), or, fused,
// the closing half of one step and the opening half of the next: the first
// clumpBlocks blocks take a group of `width` lanes per clump (first, so their
// longer chains of dependent reads overlap the rest), the others one solid
// each per thread.  clumpForce: each clump group first sums its pebbles'
// forces (kClumpForce's work, for runs of whole steps where nothing happens
// between the contact phase and this integration); countStep: the step has
// completed (the status can no longer change) and is counted.
template <int MODE>
__global__ void kIntegrate(DeviceState d, dfl half, int width, int clumpBlocks, int clumpForce, int countStep,
                           int par)
{
    stepKernelBegin();
    int* stale = d.rebuild + (par ^ 1);  // the next step's candidate flag
    if (countStep && blockIdx.x == 0 && threadIdx.x == 0 && *d.status == 0) atomicAdd(d.stepsDone, 1);
    if ((int)blockIdx.x >= clumpBlocks) {
        const int k = (blockIdx.x - clumpBlocks) * blockDim.x + threadIdx.x;
        if (k >= d.nmove || *d.status) return;
        solidIntegrateOne<MODE>(d, d.moveFirst >= 0 ? d.moveFirst + k : d.moveList[k], half, stale);
        return;
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (clumpForce) clumpForceGroup(d, width, t);
    if (MODE == INTEGRATE_FUSED) {
        // the group's lanes take the same pebbles in both halves, and lane 0
        // re-reads the clump state it wrote: each reads its own writes
        clumpIntegrateGroup(d, half, 0, width, t, stale, true);
        clumpIntegrateGroup(d, half, 1, width, t, stale);
    } else {
        clumpIntegrateGroup(d, half, MODE == INTEGRATE_BEFORE ? 1 : 0, width, t, stale);
    }
}

// The per-solid sums of kSolidForces and, in the same thread, the solid's
// integration pass (MODE after or fused, kIntegrate's work for one solid),
// for scenes whose integrated solids are exactly the contact rows (no clumps,
// no moving dummy particles): no other thread of the launch reads the state
// a row's integration writes.  countStep as kIntegrate's.
template <int MODE>
__global__ void __launch_bounds__(T) kSolidForcesIntegrate(DeviceState d, int par, float dt, int withCoupling,
                                                           dfl half, int countStep)
{
    stepKernelBegin();
    if (countStep && blockIdx.x == 0 && threadIdx.x == 0 && *d.status == 0) atomicAdd(d.stepsDone, 1);
    if (*d.status) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= d.nrow) return;
    const int a = solidForcesRow(d, par, dt, withCoupling, row);
    solidIntegrateOne<MODE>(d, a, half, d.rebuild + (par ^ 1));
}



}  // namespace

void launchPairForces(const DeviceState& d, int par, float dt, cudaStream_t s)
{
    const int cb = d.nrow > 0 ? blocksFor(d.nrow, d.forceRows * (T / 32)) : 0;
    const int bb = d.nb > 0 ? blocksFor(d.nb, T) : 0;
    if (cb + bb == 0) return;
    launchStep(kPairForces, cb + bb, T, s, d, par, dt, d.forceRows, cb);
}
void launchSolidForces(const DeviceState& d, int par, double dt, cudaStream_t s, int integrate, bool countStep)
{
    if (d.nrow <= 0) return;
    const int blocks = blocksFor(d.nrow, T), cpl = d.nf > 0 ? 1 : 0, cs = countStep ? 1 : 0;
    const dfl h = df_from_double(0.5 * dt);
    if (integrate == INTEGRATE_FUSED)
        launchStep(kSolidForcesIntegrate<INTEGRATE_FUSED>, blocks, T, s, d, par, (float)dt, cpl, h, cs);
    else if (integrate == INTEGRATE_AFTER)
        launchStep(kSolidForcesIntegrate<INTEGRATE_AFTER>, blocks, T, s, d, par, (float)dt, cpl, h, cs);
    else
        launchStep(kSolidForces, blocks, T, s, d, par, (float)dt, cpl);
}
void launchContactForces(const DeviceState& d, int par, float dt, cudaStream_t s)
{
    if (d.nrow <= 0) return;
    launchStep(kContactForces, blocksFor(d.nrow, T), T, s, d, par, dt, d.nf > 0 ? 1 : 0);
}
void launchClumpForce(const DeviceState& d, cudaStream_t s)
{
    if (d.nc <= 0) return;
    const int w = d.clumpLanes;
    launchStep(kClumpForce, blocksFor((long long)d.nc * w, 256), 256, s, d, w);
}
void launchSolidIntegrate(const DeviceState& d, double dt, int mode, int par, bool clumpForce, bool countStep,
                          cudaStream_t s)
{
    const dfl h = df_from_double(0.5 * dt);
    const int sb = d.nmove > 0 ? blocksFor(d.nmove, 256) : 0;
    const int cb = d.nc > 0 ? blocksFor((long long)d.nc * d.clumpLanes, 256) : 0;
    if (sb + cb == 0 && !countStep) return;
    const int blocks = std::max(1, sb + cb), cf = clumpForce ? 1 : 0, cs = countStep ? 1 : 0;
    if (mode == INTEGRATE_FUSED)
        launchStep(kIntegrate<INTEGRATE_FUSED>, blocks, 256, s, d, h, d.clumpLanes, cb, cf, cs, par);
    else if (mode == INTEGRATE_BEFORE)
        launchStep(kIntegrate<INTEGRATE_BEFORE>, blocks, 256, s, d, h, d.clumpLanes, cb, cf, cs, par);
    else
        launchStep(kIntegrate<INTEGRATE_AFTER>, blocks, 256, s, d, h, d.clumpLanes, cb, cf, cs, par);
}


}  // namespace demsph
