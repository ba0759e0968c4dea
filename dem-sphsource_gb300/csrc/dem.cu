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

namespace demsph {

namespace {

constexpr int T = 128;
enum FlagBits { F_DUMMY = 1, F_FIXED = 2, F_MASSIVE = 4, F_HASMASS = 8 };
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

// Contact forces of every forward slot (calSolidContactForceTorque,
// core/integrate.cu:423-512), one thread per row.
__global__ void __launch_bounds__(T) kPairContacts(DeviceState d, int par, float dt)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= d.nrow || *d.status) return;
    const int a = d.rowSolid[r];
    const int n = min(d.fcnt[par][r], d.scap);
    if (n == 0) return;
    const float4 ra = d.srad[a];
    const float ima = d.sph[a].w;
    const int mata = d.sflags[a].x;
    for (int q = 0; q < n; ++q) {
        const size_t k = (size_t)q * d.nrow + r;
        const int b = d.fwd[par][k];
        const PairGeom g = pairGeometry(d, a, b);
        const float4 rb = d.srad[b];
        const float R = ra.x * rb.x / (ra.x + rb.x);
        const float m = 1.f / (ima + d.sph[b].w);
        const float3 vc = contactVel(d, a, b, g.leverA, g.leverB);
        const float3 wr = spinDiff(d, a, b);
        float3 es = xyz(d.spring[par][0][k]), er = xyz(d.spring[par][1][k]), et = xyz(d.spring[par][2][k]);
        float3 F = make_float3(0.f, 0.f, 0.f), Ft = F, Tq = F;
        const int slot = tableSlot(d.tab, mata, d.sflags[b].x);
        contactLaw(d.tab, slot, F, Ft, Tq, es, er, et, vc, wr, g.n, g.delta, m, R, dt);
        d.spring[par][0][k] = f4(es);
        d.spring[par][1][k] = f4(er);
        d.spring[par][2][k] = f4(et);
        d.pF[k] = f4(F);
        d.pT[k] = f4(Tq);
        const float3 nxF = cross3(g.n, Ft);
        d.pTA[k] = f4(Tq + nxF * g.sA);
        d.pTB[k] = f4(Tq + nxF * g.sB);
    }
}

// Slot (index into the per-slot arrays) of the forward contact (a, b), b > a,
// or -1 when the pair is not in a's row.
__device__ __forceinline__ long long forwardSlot(const DeviceState& d, int par, int a, int b)
{
    const int r = d.srow[a];
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

__global__ void __launch_bounds__(T) kBonds(DeviceState d, int par, float dt)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.nb || *d.status) return;
    if (d.bon[b] == 0) {
        d.bFnTt[b] = make_float4(0, 0, 0, 0);
        d.bFsH[b] = d.bFsL[b] = d.bTbH[b] = d.bTbL[b] = make_float4(0, 0, 0, 0);
        d.bN[b] = make_float4(0, 0, 0, 0);
        return;
    }
    const int2 ab = d.bab[b];
    const int i = ab.x, j = ab.y;
    const long long slot = forwardSlot(d, par, i, j);
    if (slot < 0) {  // the pair left the contact list: the bond breaks
        d.bon[b] = 0;
        return;
    }
    const PairGeom g = pairGeometry(d, i, j);
    const float3 n = g.n;
    const float3 n0 = xyz(d.bN[b]);
    const float3 wi = xyz(d.swh[i]), wj = xyz(d.swh[j]);
    const float3 vc = contactVel(d, i, j, g.leverA, g.leverB);
    const float4 ri = d.srad[i], rj = d.srad[j];
    const int ms = tableSlot(d.tab, d.sflags[i].x, d.sflags[j].x);
    const float* B = d.tab.bd + 6 * ms;  // gamma E knks sigma C mu
    float4 FnTt = d.bFnTt[b];
    float4 FsH = d.bFsH[b], FsL = d.bFsL[b], TbH = d.bTbH[b], TbL = d.bTbL[b];
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
    const float3 wr = spinDiff(d, i, j);
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
    // add onto the pair's force and torque (integrate.cu:802-803)
    const float3 F = n * fn + Fs;
    const float3 Tq = n * tt + Tb;
    const float3 nxF = cross3(n, Fs);  // the lever is along n: n x (fn n) = 0
    d.pF[slot] = f4(xyz(d.pF[slot]) + F);
    d.pT[slot] = f4(xyz(d.pT[slot]) + Tq);
    d.pTA[slot] = f4(xyz(d.pTA[slot]) + Tq + nxF * g.sA);
    d.pTB[slot] = f4(xyz(d.pTB[slot]) + Tq + nxF * g.sB);
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

__global__ void __launch_bounds__(T) kGatherWalls(DeviceState d, int par, float dt, int withCoupling)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= d.ns || *d.status) return;
    const int4 fa = d.sflags[a];
    KahanF3 F, Tq;
    const int row = d.srow[a];
    if (row >= 0) {
        // forward slots (+), then the reverse partners' slots of this pair (-)
        const int n = min(d.fcnt[par][row], d.scap);
        for (int q = 0; q < n; ++q) {
            const size_t k = (size_t)q * d.nrow + row;
            F.add(xyz(d.pF[k]));
            Tq.add(xyz(d.pTA[k]));
        }
        const int m = min(d.rcnt[row], d.scap);
        for (int q = 0; q < m; ++q) {
            const int b = d.rev[(size_t)q * d.nrow + row];
            const long long k = forwardSlot(d, par, b, a);
            if (k >= 0) {
                F.add(-xyz(d.pF[k]));
                Tq.add(-xyz(d.pTB[k]));
            }
        }
    }
    if (withCoupling) F.add(-xyz(d.sfcoup[a]));
    const float4 ph = d.sph[a];
    const float im = ph.w;
    float3 acc = F.sum() * im;
    if ((fa.w & F_HASMASS) && fa.z < 0) acc = acc + d.g;
    float3 tq = Tq.sum();
    // infinite walls (integrate.cu:514-610)
    if (d.nw > 0 && !(fa.w & F_DUMMY) && !(fa.w & F_FIXED)) {
        const int4 ca = d.scell[a];
        const float4 pl = d.spl[a];
        const float4 rad = d.srad[a];
        const float3 v = xyz(d.svh[a]), w = xyz(d.swh[a]);
        for (int k = 0; k < d.nw; ++k) {
            const size_t h = (size_t)a * d.nw + k;
            const float delta = wallOverlap(d, ca, ph, pl, k, rad.x, rad.y);
            if (delta < 0.f) {
                d.wspring[0][h] = d.wspring[1][h] = d.wspring[2][h] = make_float4(0, 0, 0, 0);
                if (d.fixes & DEMSPH_FIX_WALL_LOOP) continue;
                break;
            }
            const float3 n = xyz(d.wnh[k]);
            const float3 lever = n * (-(rad.x - delta));
            const float3 vc = v + cross3(w, lever);
            float3 es = xyz(d.wspring[0][h]), er = xyz(d.wspring[1][h]), et = xyz(d.wspring[2][h]);
            float3 Fw = make_float3(0.f, 0.f, 0.f), Fwt = Fw, Tw = Fw;
            const int slot = tableSlot(d.tab, fa.x, d.wmat[k]);
            contactLaw(d.tab, slot, Fw, Fwt, Tw, es, er, et, vc, w, n, delta, 1.f / im, rad.x, dt);
            d.wspring[0][h] = f4(es);
            d.wspring[1][h] = f4(er);
            d.wspring[2][h] = f4(et);
            acc = acc + Fw * im;
            tq = tq + Tw + cross3(n, Fwt) * (-(rad.x - delta));
        }
    }
    d.sacc[a] = f4(acc);
    d.storque[a] = f4(tq);
}

__device__ __forceinline__ double3 dadd(double3 a, double3 b) { return make_double3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ double3 dsub(double3 a, double3 b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double3 dscale(double3 a, double s) { return make_double3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double3 dcross(double3 a, double3 b)
{
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double3 toD3(float4 v) { return make_double3(v.x, v.y, v.z); }
__device__ __forceinline__ double3 absPos(const DeviceState& d, int i)
{
    const int4 c = d.scell[i];
    const float4 h = d.sph[i], l = d.spl[i];
    return make_double3(d.minB[0] + c.x * d.cs[0] + ((double)h.x + (double)l.x),
                        d.minB[1] + c.y * d.cs[1] + ((double)h.y + (double)l.y),
                        d.minB[2] + c.z * d.cs[2] + ((double)h.z + (double)l.z));
}

// Sum over the `width` lanes of a group (width a power of two <= 32), in a
// fixed tree: every lane gets the same bits.
__device__ __forceinline__ double groupSumD(double v, int width)
{
    for (int o = width >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, width);
    return v;
}

// calClumpForceTorque (integrate.cu:860-881): a group of `width` lanes per
// clump over its pebbles, FP64 sums reduced in a fixed tree (deterministic).
__global__ void kClumpForce(DeviceState d, int width)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = t / width, lane = t % width;
    // whole warps only: the shuffles below take every lane of the warp
    if ((t & ~31) >= d.nc * width || *d.status) return;
    const bool live = c < d.nc;
    double3 F = make_double3(0, 0, 0), Tq = F;
    if (live) {
        const double3 cp = d.cpos[c];
        for (int i = d.cstart[c] + lane; i < d.cend[c]; i += width) {
            double3 fi = make_double3(0, 0, 0);
            if (d.sflags[i].w & F_MASSIVE) fi = dscale(toD3(d.sacc[i]), 1.0 / (double)d.sph[i].w);
            F = dadd(F, fi);
            Tq = dadd(Tq, dadd(toD3(d.storque[i]), dcross(dsub(absPos(d, i), cp), fi)));
            d.sacc[i] = make_float4(0, 0, 0, 0);
            d.storque[i] = make_float4(0, 0, 0, 0);
        }
    }
    F = make_double3(groupSumD(F.x, width), groupSumD(F.y, width), groupSumD(F.z, width));
    Tq = make_double3(groupSumD(Tq.x, width), groupSumD(Tq.y, width), groupSumD(Tq.z, width));
    if (live && lane == 0) {
        const double im = d.cinvm[c];
        double3 a = dscale(F, im);
        if (im > 0.) a = dadd(a, make_double3(d.g64[0], d.g64[1], d.g64[2]));
        d.cacc[c] = a;
        d.ctorque[c] = Tq;
    }
}

// double-float x += v dt for one particle's position (solid arrays).
__device__ __forceinline__ void driftSolid(const DeviceState& d, int i, dfl dt)
{
    float4 h = d.sph[i], l = d.spl[i];
    const float4 vh = d.svh[i], vl = d.svl[i];
    const dfl x = df_add(df_make(h.x, l.x), df_mul(df_make(vh.x, vl.x), dt));
    const dfl y = df_add(df_make(h.y, l.y), df_mul(df_make(vh.y, vl.y), dt));
    const dfl z = df_add(df_make(h.z, l.z), df_mul(df_make(vh.z, vl.z), dt));
    d.sph[i] = make_float4(x.hi, y.hi, z.hi, h.w);
    d.spl[i] = make_float4(x.lo, y.lo, z.lo, l.w);
}

// solidVelocityAngularVelocityIntegrate (integrate.cu:883-897) for one particle.
__device__ __forceinline__ void kickSolid(const DeviceState& d, int i, dfl dt, int4 f)
{
    const float3 a = xyz(d.sacc[i]);
    const float4 vh = d.svh[i], vl = d.svl[i];
    {
        const dfl x = df_add(df_make(vh.x, vl.x), df_mul_f(dt, a.x));
        const dfl y = df_add(df_make(vh.y, vl.y), df_mul_f(dt, a.y));
        const dfl z = df_add(df_make(vh.z, vl.z), df_mul_f(dt, a.z));
        d.svh[i] = make_float4(x.hi, y.hi, z.hi, vh.w);
        d.svl[i] = make_float4(x.lo, y.lo, z.lo, vl.w);
    }
    const float r = d.srad[i].x;
    const float im = d.sph[i].w;
    if ((f.w & F_FIXED) || r < 1.e-10f) return;
    const float3 alpha = xyz(d.storque[i]) * (im / (0.4f * r * r));
    float4 wh = d.swh[i], wl = d.swl[i];
    const dfl x = df_add(df_make(wh.x, wl.x), df_mul_f(dt, alpha.x));
    const dfl y = df_add(df_make(wh.y, wl.y), df_mul_f(dt, alpha.y));
    const dfl z = df_add(df_make(wh.z, wl.z), df_mul_f(dt, alpha.z));
    d.swh[i] = make_float4(x.hi, y.hi, z.hi, wh.w);
    d.swl[i] = make_float4(x.lo, y.lo, z.lo, wl.w);
}

// After the last drift of a step: once a solid that can touch others has
// moved half the candidate margin since the candidates were built, the next
// step rebuilds them.
__device__ __forceinline__ void checkDisplacement(const DeviceState& d, int i)
{
    const int r = d.srow[i];
    if (r < 0) return;
    const int4 c = d.scell[i];
    const float4 h = d.sph[i];
    const float4 p0 = d.vref[r];
    const float dx = (float)c.x * d.grid.cs.x + h.x - p0.x, dy = (float)c.y * d.grid.cs.y + h.y - p0.y,
                dz = (float)c.z * d.grid.cs.z + h.z - p0.z;
    const float half = 0.5f * d.skin;
    if (!(dx * dx + dy * dy + dz * dz <= half * half)) *(volatile int*)d.rebuild = 1;
}

__global__ void kSolidIntegrate(DeviceState d, dfl half, int before)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.ns || *d.status) return;
    const int4 f = d.sflags[i];
    if (f.z >= 0) return;  // clump pebbles: kClumpIntegrate
    if (before) {
        kickSolid(d, i, half, f);
        driftSolid(d, i, half);
    } else {
        driftSolid(d, i, half);
        kickSolid(d, i, half, f);
        checkDisplacement(d, i);
    }
}

__device__ __forceinline__ double3 rotInvInertiaTimes(double4 q, const double* I, double3 t)
{
    // R(q) invI R(q)^T t  (core/myMat.h:102-127 applied to a vector)
    const double q0 = q.x, q1 = q.y, q2 = q.z, q3 = q.w;
    const double R00 = 1 - 2 * q2 * q2 - 2 * q3 * q3, R01 = 2 * q1 * q2 - 2 * q0 * q3, R02 = 2 * q1 * q3 + 2 * q0 * q2;
    const double R10 = 2 * q1 * q2 + 2 * q0 * q3, R11 = 1 - 2 * q1 * q1 - 2 * q3 * q3, R12 = 2 * q2 * q3 - 2 * q0 * q1;
    const double R20 = 2 * q1 * q3 - 2 * q0 * q2, R21 = 2 * q2 * q3 + 2 * q0 * q1, R22 = 1 - 2 * q1 * q1 - 2 * q2 * q2;
    // body frame: u = R^T t
    const double ux = R00 * t.x + R10 * t.y + R20 * t.z;
    const double uy = R01 * t.x + R11 * t.y + R21 * t.z;
    const double uz = R02 * t.x + R12 * t.y + R22 * t.z;
    // I = (xx, yy, zz, xy, xz, yz)
    const double wx = I[0] * ux + I[3] * uy + I[4] * uz;
    const double wy = I[3] * ux + I[1] * uy + I[5] * uz;
    const double wz = I[4] * ux + I[5] * uy + I[2] * uz;
    return make_double3(R00 * wx + R01 * wy + R02 * wz, R10 * wx + R11 * wy + R12 * wz,
                        R20 * wx + R21 * wy + R22 * wz);
}

// clumpVelocityAngularVelocityIntegrate (integrate.cu:908-929): the clump's
// new velocity v and spin w (from w0) after a kick of dt.
__device__ __forceinline__ void clumpKickState(const DeviceState& d, int c, double dt, double3& a, double3& v,
                                               double3& w0, double3& w)
{
    a = d.cacc[c];
    w0 = d.cw[c];
    v = dadd(d.cvel[c], dscale(a, dt));
    w = w0;
    if (d.cinvm[c] > 0.) w = dadd(w0, dscale(rotInvInertiaTimes(d.cq[c], d.cinvI + 6 * c, d.ctorque[c]), dt));
}

// The rigid-body motion handed to pebble i (clump centroid cp): acceleration,
// velocity, spin and the normal turned by the mean spin.
__device__ __forceinline__ void pebbleKick(const DeviceState& d, int i, double3 a, double3 v, double3 w, double3 cp,
                                           float3 rotn)
{
    const double3 r = dsub(absPos(d, i), cp);
    const double3 ai = dadd(dadd(a, dcross(a, r)), dcross(w, dcross(w, r)));
    const double3 vi = dadd(v, dcross(w, r));
    d.sacc[i] = make_float4((float)ai.x, (float)ai.y, (float)ai.z, 0.f);
    const dfl vx = df_from_double(vi.x), vy = df_from_double(vi.y), vz = df_from_double(vi.z);
    d.svh[i] = make_float4(vx.hi, vy.hi, vz.hi, 0.f);
    d.svl[i] = make_float4(vx.lo, vy.lo, vz.lo, 0.f);
    const dfl wx = df_from_double(w.x), wy = df_from_double(w.y), wz = df_from_double(w.z);
    d.swh[i] = make_float4(wx.hi, wy.hi, wz.hi, 0.f);
    d.swl[i] = make_float4(wx.lo, wy.lo, wz.lo, 0.f);
    d.snormal[i] = f4(rotateF(xyz(d.snormal[i]), rotn));
}

// First-order quaternion update with the mean spin, renormalised (only with
// DEMSPH_FIX_CLUMP_ROTATION; the reference never turns a clump's orientation).
__device__ __forceinline__ void clumpRotate(const DeviceState& d, int c, double3 w0, double3 w, double dt)
{
    const double3 v = dscale(dadd(w0, w), 0.5 * dt);
    const double4 q = d.cq[c];
    double4 n = make_double4(q.x + 0.5 * (-q.y * v.x - q.z * v.y - q.w * v.z),
                             q.y + 0.5 * (q.x * v.x + q.w * v.y - q.z * v.z),
                             q.z + 0.5 * (-q.w * v.x + q.x * v.y + q.y * v.z),
                             q.w + 0.5 * (q.z * v.x - q.y * v.y + q.x * v.z));
    const double l = sqrt(n.x * n.x + n.y * n.y + n.z * n.z + n.w * n.w);
    if (l > 0) n = make_double4(n.x / l, n.y / l, n.z / l, n.w / l);
    d.cq[c] = n;
}

__device__ __forceinline__ double3 shflD3(double3 v, int src, int width)
{
    return make_double3(__shfl_sync(0xffffffffu, v.x, src, width), __shfl_sync(0xffffffffu, v.y, src, width),
                        __shfl_sync(0xffffffffu, v.z, src, width));
}

// Half-step clump integration (clumpVelocityAngularVelocityIntegrate and
// clumpPositionIntegrate, integrate.cu:908-938, in the order of
// integrate.cu:964-1027), a group of `width` lanes per clump: the group's
// first lane computes the clump's new state in FP64 and hands it to the
// others, the lanes move the pebbles.
//   before contact: kick, pebbles from the kicked state, centroid and pebble drift;
//   after contact:  pebble and centroid drift, kick, pebbles from the kicked state.
__global__ void kClumpIntegrate(DeviceState d, double half, dfl halfDF, int before, int width)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = t / width, lane = t % width;
    // whole warps only: the shuffles below take every lane of the warp
    if ((t & ~31) >= d.nc * width || *d.status) return;
    const bool live = c < d.nc;
    const int s = live ? d.cstart[c] : 0, e = live ? d.cend[c] : 0;
    if (!before)
        for (int i = s + lane; i < e; i += width) driftSolid(d, i, halfDF);
    double3 a = make_double3(0, 0, 0), v = a, w0 = a, w = a, cp = a;
    if (live && lane == 0) {
        cp = before ? d.cpos[c] : dadd(d.cpos[c], dscale(d.cvel[c], half));
        clumpKickState(d, c, half, a, v, w0, w);
        d.cvel[c] = v;
        d.cw[c] = w;
        d.cpos[c] = before ? dadd(cp, dscale(v, half)) : cp;
        if (d.fixes & DEMSPH_FIX_CLUMP_ROTATION) clumpRotate(d, c, w0, w, half);
    }
    const int src = 0;  // lane 0 of the group
    a = shflD3(a, src, width);
    v = shflD3(v, src, width);
    w0 = shflD3(w0, src, width);
    w = shflD3(w, src, width);
    cp = shflD3(cp, src, width);
    const float3 rotn = make_float3((float)(0.5 * (w0.x + w.x) * half), (float)(0.5 * (w0.y + w.y) * half),
                                    (float)(0.5 * (w0.z + w.z) * half));
    for (int i = s + lane; i < e; i += width) {
        pebbleKick(d, i, a, v, w, cp, rotn);
        if (before) driftSolid(d, i, halfDF);
        else checkDisplacement(d, i);
    }
}

__global__ void kStepDone(int* status, int* steps)
{
    if (*status == 0) atomicAdd(steps, 1);
}

}  // namespace

void launchPairContacts(const DeviceState& d, int par, float dt, cudaStream_t s)
{
    if (d.nrow <= 0) return;
    ++t_kernelLaunches, kPairContacts<<<blocksFor(d.nrow, T), T, 0, s>>>(d, par, dt);
}
void launchBonds(const DeviceState& d, int par, float dt, cudaStream_t s)
{
    if (d.nb <= 0) return;
    ++t_kernelLaunches, kBonds<<<blocksFor(d.nb, T), T, 0, s>>>(d, par, dt);
}
void launchGatherWalls(const DeviceState& d, int par, float dt, cudaStream_t s)
{
    if (d.ns <= 0) return;
    ++t_kernelLaunches, kGatherWalls<<<blocksFor(d.ns, T), T, 0, s>>>(d, par, dt, d.nf > 0 ? 1 : 0);
}
void launchClumpForce(const DeviceState& d, cudaStream_t s)
{
    if (d.nc <= 0) return;
    const int w = d.clumpLanes;
    ++t_kernelLaunches, kClumpForce<<<blocksFor((long long)d.nc * w, 256), 256, 0, s>>>(d, w);
}
void launchSolidIntegrate(const DeviceState& d, double dt, bool before, cudaStream_t s)
{
    const double half = 0.5 * dt;
    const dfl h = df_from_double(half);
    if (d.ns > 0) ++t_kernelLaunches, kSolidIntegrate<<<blocksFor(d.ns, 256), 256, 0, s>>>(d, h, before ? 1 : 0);
    if (d.nc > 0) {
        const int w = d.clumpLanes;
        ++t_kernelLaunches,
            kClumpIntegrate<<<blocksFor((long long)d.nc * w, 256), 256, 0, s>>>(d, half, h, before ? 1 : 0, w);
    }
}
void launchStepDone(const DeviceState& d, cudaStream_t s)
{
    ++t_kernelLaunches, kStepDone<<<1, 1, 0, s>>>(d.status, d.stepsDone);
}

}  // namespace demsph
