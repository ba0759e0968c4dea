// Contact-row helpers shared by the contact detection (lists.cu) and the
// one-launch contact list + forces (dem.cu): the reference's pair filters and
// contact test, the insertion sort of a row's slots, and the Verlet candidate
// rebuild of one row.  Each reads positions through the DeviceState it is
// given (sph/spl, or the end-of-step offsets when the caller passes a copy
// whose sph/spl point at sphE/splE).
#pragma once
#include "kernels.cuh"

namespace demsph {

// |x_a - x_b| <= cut (cut in double-float): FP32 decision outside a 1e-5
// relative band, double-float inside it.
__device__ __forceinline__ bool withinCut(int4 ca, float4 ha, float4 la, int4 cb, float4 hb, const float4* lbPtr,
                                          int jb, dfl cut, const GridDev& g)
{
    const float3 r = relF(ca, ha, cb, hb, g);
    const float d2 = dot3(r, r);
    const float c2 = cut.hi * cut.hi;
    if (d2 > c2 * (1.f + 1.e-5f)) return false;
    if (d2 < c2 * (1.f - 1.e-5f)) return true;
    const float4 lb = lbPtr[jb];
    const dfl dist = dfNorm(relDF(ca, ha, la, cb, hb, lb, g));
    return df_ge0(df_sub(cut, dist));
}

// Filters of core/neighborSearch.cu:246-263 for candidate b of particle a.
__device__ __forceinline__ bool solidPairCandidate(const DeviceState& d, int a, int4 fa, int b)
{
    if (b == a) return false;
    const int4 fb = d.sflags[b];
    if (fb.w & F_DUMMY) return false;
    if (fa.z >= 0 && fa.z == fb.z) return false;           // same clump
    if ((fa.w & F_FIXED) && (fb.w & F_FIXED)) return false;  // both fixed
    return true;
}

// The reference's contact test |x_a - x_b| <= eff_a + eff_b
// (core/neighborSearch.cu:264-270), always evaluated with the lower index
// first, so that the rows of both solids reach the same decision bit for bit.
__device__ __forceinline__ bool solidsTouch(const DeviceState& d, int a, int b)
{
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const float4 rl = d.srad[lo], rh = d.srad[hi];
    const dfl cut = df_add(df_make(rl.z, rl.w), df_make(rh.z, rh.w));
    return withinCut(d.scell[lo], d.sph[lo], d.spl[lo], d.scell[hi], d.sph[hi], d.spl, hi, cut, d.grid);
}

// Insertion sort of the n slots [k * nrow + r] of one row (n is small).
__device__ __forceinline__ void sortSlots(int* v, int r, int nrow, int n)
{
    const size_t nr = (size_t)nrow;
    for (int k = 1; k < n; ++k) {
        const int x = v[(size_t)k * nr + r];
        int q = k - 1;
        while (q >= 0 && v[(size_t)q * nr + r] > x) {
            v[(size_t)(q + 1) * nr + r] = v[(size_t)q * nr + r];
            --q;
        }
        v[(size_t)(q + 1) * nr + r] = x;
    }
}

__device__ __forceinline__ float3 gridPos(int4 c, float4 h, const GridDev& g)
{
    return make_float3((float)c.x * g.cs.x + h.x, (float)c.y * g.cs.y + h.y, (float)c.z * g.cs.z + h.z);
}

// Verlet candidates of one row: every solid passing the reference's filters
// within eff_a + eff_b + skin, found in the cells that box overlaps.  Runs only
// on steps where the hash found a solid displaced by more than skin / 2 since
// the last rebuild (so every pair within eff_a + eff_b now was within
// eff_a + eff_b + skin then).  All non-dummy solids are inside the domain
// here (otherwise the lists come from the 27-cell walk), so the cells are
// plain (x, y, z) cells.
__device__ __forceinline__ void verletBuildRow(const DeviceState& d, int r)
{
    const int a = solidOf(d, r);
    const int4 fa = d.sflags[a];
    const int4 ca = d.scell[a];
    const float4 ha = d.sph[a];
    const float effA = d.srad[a].z;
    const float reach = effA + d.vmaxEff + d.skin;
    const GridDev& g = d.grid;
    const int x0 = max(0, ca.x + (int)floorf((ha.x - reach) / g.cs.x)), x1 = min(g.gx - 1, ca.x + (int)floorf((ha.x + reach) / g.cs.x));
    const int y0 = max(0, ca.y + (int)floorf((ha.y - reach) / g.cs.y)), y1 = min(g.gy - 1, ca.y + (int)floorf((ha.y + reach) / g.cs.y));
    const int z0 = max(0, ca.z + (int)floorf((ha.z - reach) / g.cs.z)), z1 = min(g.gz - 1, ca.z + (int)floorf((ha.z + reach) / g.cs.z));
    int n = 0;
    for (int z = z0; z <= z1; ++z)
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                const int hash = (z * g.gy + y) * g.gx + x;
                for (int p = d.scellStart[hash], pe = d.scellStart[hash + 1]; p < pe; ++p) {
                    const int b = d.ssorted[p];
                    if (!solidPairCandidate(d, a, fa, b)) continue;
                    const float3 rr = relF(ca, ha, make_int4(x, y, z, hash), d.sph[b], g);
                    const float c = (effA + d.srad[b].z + d.skin) * 1.0001f;
                    if (dot3(rr, rr) > c * c) continue;
                    if (n < d.vcap) d.vcand[(size_t)n * d.nrow + r] = b;
                    ++n;
                }
            }
    // by index: the contact list filtered from them is then in index order
    sortSlots(d.vcand, r, d.nrow, min(n, d.vcap));
    d.vcnt[r] = n;
    d.vref[a] = f4(gridPos(ca, ha, g));
    if (n > d.vcap) {
        atomicOr(d.status, ST_VERLET_OVERFLOW);
        atomicMax(&d.need[1], n);
    }
}

}  // namespace demsph
