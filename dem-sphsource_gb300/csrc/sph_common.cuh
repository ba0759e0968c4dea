// Pair terms of the WCSPH loops shared by the list kernels (sph.cu) and the
// cell-tile kernels (sph_tiles.cu): the solid partner quantities, a fluid
// particle's own state, the double-float drift and the Shepard term.  The
// physics and its algebraic forms are described at the top of sph.cu.
#pragma once
#include "kernels.cuh"

namespace demsph {
namespace sph {

constexpr float KG = 5.f * 21.f / (16.f * 3.14159265358979323846f);  // G = KG t^3 / h^5
constexpr float SIG = 21.f / (16.f * 3.14159265358979323846f);       // sigma h^3

struct SolidPartner {
    float3 r;      // x_i - x_a
    float3 v;      // v_a
    float Pa, rhoa, Va, G, rr;
    bool inside;
};

// Wall/solid partner quantities shared by continuity, momentum and coupling.
__device__ __forceinline__ SolidPartner solidPartner(const DeviceState& d, int4 ci, float4 pi, float hi, float Pi,
                                                     float rhoi, float rho0i, float ci2, int a)
{
    SolidPartner s;
    const float4 pa = d.sph[a];
    s.r = relF(ci, pi, d.scell[a], pa, d.grid);
    const float ra = d.srad[a].x;
    const float h = 0.5f * (hi + 2.6f * ra);
    const float r2 = dot3(s.r, s.r);
    s.inside = r2 < 4.f * h * h;
    if (!s.inside) return s;
    s.rr = sqrtf(r2);
    const float t = 1.f - 0.5f * s.rr / h;
    const float h2 = h * h;
    s.G = KG * t * t * t / (h2 * h2 * h);
    s.v = xyz(d.svh[a]);
    const float3 na = xyz(d.snormal[a]);
    const float3 aa = xyz(d.sacc[a]);
    s.Pa = Pi + rhoi * fmaxf(0.f, dot3(d.g - aa, na)) * dot3(s.r, na);
    s.rhoa = s.Pa / ci2 + rho0i;
    s.Va = 8.f * ra * ra * ra;
    return s;
}

struct Self {
    int4 c;
    float4 p;
    float3 v;
    float h, rho0, cs, nu, m, rho, P, V, gam;
};

__device__ __forceinline__ Self loadSelf(const DeviceState& d, int i, int ps, int vs, int ds)
{
    Self o;
    o.c = d.fcell[i];
    o.p = d.fph[ps][i];
    o.v = xyz(d.fvh[vs][i]);
    const float dr = d.fdrho[ds][i];
    const float4 par = d.fpar[i];
    o.h = o.p.w;
    o.rho0 = par.x;
    o.cs = par.y;
    o.nu = par.z;
    o.m = par.w;
    o.rho = o.rho0 + dr;
    o.P = dr * o.cs * o.cs;
    o.V = o.m / o.rho;
    o.gam = o.nu * o.rho;
    return o;
}

// Position/velocity update in double-float: x += v dt.
__device__ __forceinline__ void dfAxpy(float4& xh, float4& xl, float4 vh, float4 vl, dfl dt)
{
    dfl x = df_add(df_make(xh.x, xl.x), df_mul(df_make(vh.x, vl.x), dt));
    dfl y = df_add(df_make(xh.y, xl.y), df_mul(df_make(vh.y, vl.y), dt));
    dfl z = df_add(df_make(xh.z, xl.z), df_mul(df_make(vh.z, vl.z), dt));
    xh.x = x.hi; xl.x = x.lo;
    xh.y = y.hi; xl.y = y.lo;
    xh.z = z.hi; xl.z = z.lo;
}


// ---- Shepard density re-initialisation (integrate.cu:3-53) ----
// sumW = sigma(h_i) S with S = 1 + sum_j f(q_j) + sum_a f(q_a) V0_a / V0_i,
// f(q) = (1 - q/2)^4 (1 + 2q).  The update rho0 S / S0 - rho0 is a difference
// of two nearly equal sums (1e-3 apart), so S is carried in double-float from
// double-float distances, and S - S0 is formed before dividing.
__device__ __forceinline__ dfl shepardTerm(dfl r, dfl invh)
{
    const dfl q = df_mul(r, invh);
    const dfl t = df_add_f(df_mul_f(q, -0.5f), 1.0f);
    const dfl t2 = df_mul(t, t);
    return df_mul(df_mul(t2, t2), df_add_f(df_mul_f(q, 2.0f), 1.0f));
}

}  // namespace sph
}  // namespace demsph
