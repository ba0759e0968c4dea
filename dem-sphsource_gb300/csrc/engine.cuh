// Device data layout of the engine and the geometry helpers every kernel uses.
//
// Positions are split as an integer grid cell plus a double-float offset from
// that cell's origin (origin = domain min + cell * cellSize, per axis), so a
// relative vector x_i - x_j = (c_i - c_j) * cellSize + (o_i - o_j) is exact to
// ~48 bits however far the particles are from the origin.  The cell is the
// reference's hashing cell (core/neighborSearch.h:44-53): offsets are brought
// back into [0, cellSize) whenever a particle set is re-hashed.
//
// Fluid particles are stored in cell order (sorted by (cell key, original
// index) at every fluid list rebuild); solids stay in their original order and
// are reached through a per-step sorted index, so clump pebble ranges, bond
// endpoints and contact history keep stable indices.
#pragma once
#include <cstdint>
#include "dfloat.cuh"

namespace demsph {

enum StatusBits : int {
    ST_FF_OVERFLOW = 1,      // a fluid particle has more fluid partners than the list holds
    ST_FS_OVERFLOW = 2,      // ... more solid partners
    ST_SS_OVERFLOW = 4,      // a solid has more contacts (forward or reverse) than its row holds
    ST_COUPLE_OVERFLOW = 8,  // fluid-solid coupling reverse list over capacity
    ST_VERLET_OVERFLOW = 16, // a solid has more contact candidates than its row holds
    ST_MODE_CHANGE = 32,     // a particle left the domain: lists switch to the 27-cell walk; redo the step
    ST_FVERLET_OVERFLOW = 64,// a fluid particle has more list candidates than it holds
    ST_BARRIER_TIMEOUT = 128,// a grid barrier of a cooperative launch gave up waiting (an error)
    ST_SPLIT_CONTACTS = 256, // the one-launch contact list + forces met the walk mode: redo the step in two
    ST_FBITS_OVERFLOW = 512, // a fluid particle's walk has more candidates than its membership bits hold
};

// Neighbour list entries.  A fluid partner entry holds the partner's slot j,
// the position t (0..26) of its cell in the reference's 27-cell walk around
// the particle (z, y, x loops: t = 9 (dz+1) + 3 (dy+1) + (dx+1)) and whether
// that cell is a plain in-domain cell, whose offset from the particle's cell
// t then gives.  A solid partner entry holds the solid's index and t.  The
// walk position restores the reference's list order on export.
__host__ __device__ __forceinline__ unsigned ffEntry(int j, int t, bool regular)
{
    return ((unsigned)j << 6) | (regular ? 32u : 0u) | (unsigned)t;
}
__host__ __device__ __forceinline__ int ffPartner(unsigned e) { return (int)(e >> 6); }
__host__ __device__ __forceinline__ int entryWalk(unsigned e) { return (int)(e & 31u); }
__host__ __device__ __forceinline__ bool ffRegular(unsigned e) { return (e & 32u) != 0u; }
__host__ __device__ __forceinline__ int fsEntry(int a, int t) { return (a << 5) | t; }
__host__ __device__ __forceinline__ int fsPartner(int e) { return e >> 5; }
constexpr int MAX_LIST_INDEX = 1 << 26;  // slots / solid indices the entries can hold

struct GridDev {
    int gx, gy, gz, num;  // num = gx*gy*gz + 1; the last cell holds out-of-domain particles
    float3 cs;            // cell size, float part
    dfl csx, csy, csz;    // cell size, double-float
};

struct Tables {          // contact model per material-pair slot
    int nMat;
    const float* hz;     // 8 per slot: E G res krks ktks mus mur mut
    const float* ln;     // 11 per slot: kn ks kr kt dn ds dr dt mus mur mut
    const float* bd;     // 6 per slot: gamma E knks sigma C mu
    const float* damp;   // 1 per slot: Hertz dissipation D = -ln e / sqrt(ln^2 e + pi^2)
};

__device__ __forceinline__ int tableSlot(const Tables& t, int a, int b)
{
    if (a >= t.nMat || b >= t.nMat) return -1;
    const int i = a < b ? a : b, j = a < b ? b : a;
    return (i * (2 * t.nMat - i + 1)) / 2 + j - i;
}

// ---- cells and keys ----

__device__ __forceinline__ bool inDomain(int x, int y, int z, const GridDev& g)
{
    return x >= 0 && x < g.gx && y >= 0 && y < g.gy && z >= 0 && z < g.gz;
}
// calculatePointHash (core/neighborSearch.cu:19-36): linear cell key, or the
// overflow bucket num-1 for particles outside the domain.
__device__ __forceinline__ int cellKey(int x, int y, int z, const GridDev& g)
{
    return inDomain(x, y, z, g) ? (z * g.gy + y) * g.gx + x : g.num - 1;
}

__device__ __forceinline__ dfl cellSizeAxis(const GridDev& g, int axis)
{
    return axis == 0 ? g.csx : (axis == 1 ? g.csy : g.csz);
}

// Brings one offset component back into [0, cs) and moves the cell.
__device__ __forceinline__ void renormAxis(int& c, float& hi, float& lo, dfl cs)
{
    dfl o = df_make(hi, lo);
    for (int it = 0; it < 4; ++it) {
        int k = (int)floorf(__fdiv_rn(o.hi, cs.hi));
        if (k == 0) {
            if (df_lt0(o)) k = -1;
            else if (df_ge0(df_sub(o, cs))) k = 1;
            else break;
        }
        o = df_sub(o, df_mul_f(cs, (float)k));
        c += k;
    }
    hi = o.hi;
    lo = o.lo;
}

// Cell used as the centre of the 27-cell stencil.  The reference truncates
// (p - min) / cs toward zero (core/neighborSearch.h:44-49), which differs from
// the stored (floor) cell only outside the domain on the low side.
__device__ __forceinline__ int truncAxis(int c, float hi, float lo)
{
    return (c < 0 && (hi > 0.f || (hi == 0.f && lo > 0.f))) ? c + 1 : c;
}

// x_a - x_b as double-float per axis.
__device__ __forceinline__ dfl relAxis(int ca, float ha, float la, int cb, float hb, float lb, dfl cs)
{
    const dfl d = df_sub(df_make(ha, la), df_make(hb, lb));
    const int dc = ca - cb;
    return dc == 0 ? d : df_add(d, df_mul_f(cs, (float)dc));
}
struct DF3 {
    dfl x, y, z;
};
__device__ __forceinline__ DF3 relDF(int4 ca, float4 ha, float4 la, int4 cb, float4 hb, float4 lb, const GridDev& g)
{
    DF3 r;
    r.x = relAxis(ca.x, ha.x, la.x, cb.x, hb.x, lb.x, g.csx);
    r.y = relAxis(ca.y, ha.y, la.y, cb.y, hb.y, lb.y, g.csy);
    r.z = relAxis(ca.z, ha.z, la.z, cb.z, hb.z, lb.z, g.csz);
    return r;
}
__device__ __forceinline__ dfl dfNorm(DF3 r)
{
    dfl s = df_mul(r.x, r.x);
    s = df_add(s, df_mul(r.y, r.y));
    s = df_add(s, df_mul(r.z, r.z));
    return df_sqrt(s);
}
__device__ __forceinline__ float3 toF3(DF3 r)
{
    return make_float3(r.x.hi + r.x.lo, r.y.hi + r.y.lo, r.z.hi + r.z.lo);
}
// x_a - x_b in FP32 (hi parts only): exact cell term, ~1e-7 relative.
// A cell inside the grid (x < 2048, y < 2048, z < 1024) as the bits of one
// float, and back (the key, w, is not kept).
__device__ __forceinline__ float packCell(int4 c)
{
    return __uint_as_float((unsigned)c.x | ((unsigned)c.y << 11) | ((unsigned)c.z << 22));
}
__device__ __forceinline__ int4 unpackCell(float w)
{
    const unsigned b = __float_as_uint(w);
    return make_int4((int)(b & 2047u), (int)((b >> 11) & 2047u), (int)(b >> 22), 0);
}

__device__ __forceinline__ float3 relF(int4 ca, float4 ha, int4 cb, float4 hb, const GridDev& g)
{
    return make_float3((ha.x - hb.x) + (float)(ca.x - cb.x) * g.cs.x, (ha.y - hb.y) + (float)(ca.y - cb.y) * g.cs.y,
                       (ha.z - hb.z) + (float)(ca.z - cb.z) * g.cs.z);
}

// ---- float3 helpers ----
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ float3 unit3(float3 a)
{
    const float l = len3(a);
    return l > 0.f ? a / l : a;
}
__device__ __forceinline__ float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float4 f4(float3 a, float w = 0.f) { return make_float4(a.x, a.y, a.z, w); }

// Rodrigues rotation of v by the rotation vector w (core/myVec.h:98-109).
__device__ __forceinline__ float3 rotateF(float3 v, float3 w)
{
    const float a = len3(w);
    if (a < 1.e-10f) return v;
    const float3 k = w / a;
    float s, c;
    sincosf(a, &s, &c);
    return v * c + cross3(k, v) * s + k * (dot3(k, v) * (1.f - c));
}

// ---- device views ----

struct FluidDev {
    int n;
    const int4* cell;       // home cell (x, y, z, key) at the last rebuild
    float4* ph[2];          // offset hi (xyz) + smoothing length hi (w); [0] step state, [1] mid-step
    float4* pl[2];          // offset lo (xyz) + smoothing length lo (w)
    float4* vh[2];          // velocity hi
    float4* vl[2];          // velocity lo
    float* drho[2];         // density minus rest density
    float4* acc;            // last momentum result (incl. gravity)
    const float4* par;      // rest density, sound speed, kinematic viscosity, mass
    float* sumW0;           // Shepard reference sum
    const int* id;          // original index of each slot
    // neighbour lists, column-major: entry k of slot i at [k * n + i]
    int kff, kfs;
    const unsigned* ff;     // (partner slot << 5) | cell-delta code (27 = look up cells)
    const int* ffc;         // partners found (may exceed kff on overflow)
    const int* fs;          // solid partner index
    const int* fsc;
};

struct SolidDev {
    int n;
    int4* cell;             // (x, y, z, key)
    float4* ph;             // offset hi (xyz), w: inverse mass
    float4* pl;             // offset lo
    float4* vh;             // velocity hi
    float4* vl;             // velocity lo
    float4* wh;             // angular velocity hi
    float4* wl;             // angular velocity lo
    float4* acc;
    float4* torque;
    float4* normal;
    float4* fcoup;          // total coupling force from the fluid this step
    const float4* rad;      // radius hi, radius lo, effective radius hi, lo
    const int4* flags;      // material, cluster, clump, dummy
};

}  // namespace demsph
