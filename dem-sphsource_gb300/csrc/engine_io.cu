// State transfer, run-time setters and artefact export - the I/O half of the
// C ABI in include/demsph_gb300.h.
//
// Downloads return the reference's host layout (FP64, original particle
// order): positions are rebuilt as cell origin + double-float offset in FP64
// on the device, then copied.  Exports rebuild the reference's artefacts
// (objectHash, half pair lists in CSR order, springs, bonds) from the
// engine's own structures, in the reference's order (core/neighborSearch.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine_impl.cuh"

using namespace demsph;

namespace {

__device__ __forceinline__ double cellOrigin(const DeviceState& d, int a, int c) { return d.minB[a] + (double)c * d.cs[a]; }

// Planar FP64 output in original order: pos[3n] vel[3n] acc[3n] drho[n].
__global__ void kFluidOut(DeviceState d, double* out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.nf) return;
    const size_t n = d.nf;
    const int id = d.fid[s];
    const int4 c = d.fcell[s];
    const float4 h = d.fph[0][s], l = d.fpl[0][s];
    const float4 vh = d.fvh[0][s], vl = d.fvl[0][s];
    const float4 a = d.facc[s];
    double* p = out + 3 * (size_t)id;
    double* v = out + 3 * n + 3 * (size_t)id;
    double* ac = out + 6 * n + 3 * (size_t)id;
    p[0] = cellOrigin(d, 0, c.x) + ((double)h.x + (double)l.x);
    p[1] = cellOrigin(d, 1, c.y) + ((double)h.y + (double)l.y);
    p[2] = cellOrigin(d, 2, c.z) + ((double)h.z + (double)l.z);
    v[0] = (double)vh.x + (double)vl.x;
    v[1] = (double)vh.y + (double)vl.y;
    v[2] = (double)vh.z + (double)vl.z;
    ac[0] = a.x;
    ac[1] = a.y;
    ac[2] = a.z;
    out[9 * n + id] = d.fdrho[0][s];
}

// Planar FP64 output: pos vel acc normal torque angvel, 3n each.
// The solid state in FP64 for export: position, velocity, acceleration,
// normal, torque, spin, each 3 x ns at out + k * 3 ns, for the outputs whose
// bit k is set in `want`.
__global__ void kSolidOut(DeviceState d, double* out, unsigned want)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.ns) return;
    const size_t n3 = 3 * (size_t)d.ns;
    double* o = out + 3 * (size_t)i;
    if (want & 1u) {
        const int4 c = d.scell[i];
        const float4 h = d.sph[i], l = d.spl[i];
        o[0] = cellOrigin(d, 0, c.x) + ((double)h.x + (double)l.x);
        o[1] = cellOrigin(d, 1, c.y) + ((double)h.y + (double)l.y);
        o[2] = cellOrigin(d, 2, c.z) + ((double)h.z + (double)l.z);
    }
    o += n3;
    if (want & 2u) {
        const float4 vh = d.svh[i], vl = d.svl[i];
        o[0] = (double)vh.x + vl.x; o[1] = (double)vh.y + vl.y; o[2] = (double)vh.z + vl.z;
    }
    o += n3;
    if (want & 4u) {
        const float4 a = d.sacc[i];
        o[0] = a.x; o[1] = a.y; o[2] = a.z;
    }
    o += n3;
    if (want & 8u) {
        const float4 nr = d.snormal[i];
        o[0] = nr.x; o[1] = nr.y; o[2] = nr.z;
    }
    o += n3;
    if (want & 16u) {
        const float4 t = d.storque[i];
        o[0] = t.x; o[1] = t.y; o[2] = t.z;
    }
    o += n3;
    if (want & 32u) {
        const float4 wh = d.swh[i], wl = d.swl[i];
        o[0] = (double)wh.x + wl.x; o[1] = (double)wh.y + wl.y; o[2] = (double)wh.z + wl.z;
    }
}

// Writes the state given in original order (FP64) into the engine.
__global__ void kFluidIn(DeviceState d, const double* pos, const double* vel, const double* drho)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.nf) return;
    const int id = d.fid[s];
    if (pos) {
        int4 c = d.fcell[s];
        float4 h = d.fph[0][s], l = d.fpl[0][s];
        const double p[3] = {pos[3 * id], pos[3 * id + 1], pos[3 * id + 2]};
        float hh[3], ll[3];
        const int cc[3] = {c.x, c.y, c.z};
        for (int a = 0; a < 3; ++a) {
            const dfl o = df_from_double(p[a] - cellOrigin(d, a, cc[a]));
            hh[a] = o.hi;
            ll[a] = o.lo;
        }
        h.x = hh[0]; h.y = hh[1]; h.z = hh[2];
        l.x = ll[0]; l.y = ll[1]; l.z = ll[2];
        d.fph[0][s] = h;
        d.fpl[0][s] = l;
        rehashFluid(d, s);
    }
    if (vel) {
        const dfl x = df_from_double(vel[3 * id]), y = df_from_double(vel[3 * id + 1]), z = df_from_double(vel[3 * id + 2]);
        d.fvh[0][s] = make_float4(x.hi, y.hi, z.hi, 0.f);
        d.fvl[0][s] = make_float4(x.lo, y.lo, z.lo, 0.f);
    }
    if (drho) d.fdrho[0][s] = (float)drho[id];
}

__global__ void kSolidIn(DeviceState d, const double* pos, const double* vel, const double* w, int* stale)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.ns) return;
    if (pos) {
        const int4 c = d.scell[i];
        float4 h = d.sph[i], l = d.spl[i];
        const dfl x = df_from_double(pos[3 * i] - cellOrigin(d, 0, c.x));
        const dfl y = df_from_double(pos[3 * i + 1] - cellOrigin(d, 1, c.y));
        const dfl z = df_from_double(pos[3 * i + 2] - cellOrigin(d, 2, c.z));
        d.sph[i] = make_float4(x.hi, y.hi, z.hi, h.w);
        d.spl[i] = make_float4(x.lo, y.lo, z.lo, l.w);
        // new key; candidates stale only if the solid moved half a margin
        checkDisplacement(d, stale, i);
        rehashSolid(d, i);
    }
    if (vel) {
        const dfl x = df_from_double(vel[3 * i]), y = df_from_double(vel[3 * i + 1]), z = df_from_double(vel[3 * i + 2]);
        d.svh[i] = make_float4(x.hi, y.hi, z.hi, 0.f);
        d.svl[i] = make_float4(x.lo, y.lo, z.lo, 0.f);
    }
    if (w) {
        const dfl x = df_from_double(w[3 * i]), y = df_from_double(w[3 * i + 1]), z = df_from_double(w[3 * i + 2]);
        d.swh[i] = make_float4(x.hi, y.hi, z.hi, 0.f);
        d.swl[i] = make_float4(x.lo, y.lo, z.lo, 0.f);
    }
}

__global__ void kSetClumpVelocity(DeviceState d, int c, double vx, double vy, double vz)
{
    const dfl x = df_from_double(vx), y = df_from_double(vy), z = df_from_double(vz);
    d.cvH[c] = make_float4(x.hi, y.hi, z.hi, 0.f);
    d.cvL[c] = make_float4(x.lo, y.lo, z.lo, 0.f);
}

// Clump state as planar FP64: centroid, velocity, acceleration, spin, torque
// (3n each) and orientation (4n).
__global__ void kClumpOut(DeviceState d, double* out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= d.nc) return;
    const size_t n3 = 3 * (size_t)d.nc;
    const float4 pH = d.cpH[c], pL = d.cpL[c], vH = d.cvH[c], vL = d.cvL[c], wH = d.cwH[c], wL = d.cwL[c];
    const float4 a = d.cacc[c], t = d.ctorque[c];
    double* o = out + 3 * (size_t)c;
    o[0] = d.minB[0] + ((double)pH.x + pL.x);
    o[1] = d.minB[1] + ((double)pH.y + pL.y);
    o[2] = d.minB[2] + ((double)pH.z + pL.z);
    o[n3 + 0] = (double)vH.x + vL.x;
    o[n3 + 1] = (double)vH.y + vL.y;
    o[n3 + 2] = (double)vH.z + vL.z;
    o[2 * n3 + 0] = a.x;
    o[2 * n3 + 1] = a.y;
    o[2 * n3 + 2] = a.z;
    o[3 * n3 + 0] = (double)wH.x + wL.x;
    o[3 * n3 + 1] = (double)wH.y + wL.y;
    o[3 * n3 + 2] = (double)wH.z + wL.z;
    o[4 * n3 + 0] = t.x;
    o[4 * n3 + 1] = t.y;
    o[4 * n3 + 2] = t.z;
    const double4 q = d.cq[c];
    double* oq = out + 5 * n3 + 4 * (size_t)c;
    oq[0] = q.x;
    oq[1] = q.y;
    oq[2] = q.z;
    oq[3] = q.w;
}

// addExternalForce (core/dataBase.cpp:179-195): a += F * invM.
__global__ void kAddForce(DeviceState d, int i, float fx, float fy, float fz)
{
    const float im = d.sph[i].w;
    float4 a = d.sacc[i];
    a.x += fx * im;
    a.y += fy * im;
    a.z += fz * im;
    d.sacc[i] = a;
}

// addGlobalDamping (core/dataBase.cpp:197-224): F += -C |F| v/|v|, T += -C |T| w/|w|.
__global__ void kAddDamping(DeviceState d, int i, float cd)
{
    const float im = d.sph[i].w;
    if (!(im >= 1.e-10f)) return;
    float3 F = xyz(d.sacc[i]) / im;
    float3 T = xyz(d.storque[i]);
    const float3 v = xyz(d.svh[i]), w = xyz(d.swh[i]);
    if (len3(v) > 1.e-10f) F = F + unit3(v) * (-cd * len3(F));
    if (len3(w) > 1.e-10f) T = T + unit3(w) * (-cd * len3(T));
    d.sacc[i] = f4(F * im);
    d.storque[i] = f4(T);
}

// ---- conservation audit (FP64) ----
// Per block, FP64 sums of: mass, momentum (3), translational and rotational
// kinetic energy, potential energy (-m g . x, x from the grid minimum) and
// the fluid densities.  Fluids, solids with mass outside clumps, and clumps
// as rigid bodies (their pebbles are not counted twice).
constexpr int AUDIT_N = 8;
constexpr int AUDIT_T = 256;

__global__ void __launch_bounds__(AUDIT_T) kAudit(DeviceState d, double* partial)
{
    __shared__ double sh[AUDIT_N][AUDIT_T];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double q[AUDIT_N] = {0, 0, 0, 0, 0, 0, 0, 0};
    auto add = [&](double m, double3 v, double3 x, double rot, double rho) {
        q[0] += m;
        q[1] += m * v.x;
        q[2] += m * v.y;
        q[3] += m * v.z;
        q[4] += 0.5 * m * (v.x * v.x + v.y * v.y + v.z * v.z);
        q[5] += rot;
        q[6] -= m * (d.g64[0] * x.x + d.g64[1] * x.y + d.g64[2] * x.z);
        q[7] += rho;
    };
    auto dfv = [](float4 h, float4 l) {
        return make_double3((double)h.x + l.x, (double)h.y + l.y, (double)h.z + l.z);
    };
    if (k < d.nf) {
        const int4 c = d.fcell[k];
        const float4 h = d.fph[0][k], l = d.fpl[0][k];
        const float4 par = d.fpar[k];
        const double3 x = make_double3(c.x * d.cs[0] + ((double)h.x + l.x), c.y * d.cs[1] + ((double)h.y + l.y),
                                       c.z * d.cs[2] + ((double)h.z + l.z));
        add(par.w, dfv(d.fvh[0][k], d.fvl[0][k]), x, 0.0, (double)par.x + d.fdrho[0][k]);
    } else if (k < d.nf + d.ns) {
        const int i = k - d.nf;
        const int4 f = d.sflags[i];
        const float im = d.sph[i].w;
        if (im > 0.f && f.z < 0) {
            const double m = 1.0 / im;
            const double3 x = solidAbsPos(d, i);
            const double3 xr = make_double3(x.x - d.minB[0], x.y - d.minB[1], x.z - d.minB[2]);
            const double3 w = dfv(d.swh[i], d.swl[i]);
            const double r = d.srad[i].x;
            add(m, dfv(d.svh[i], d.svl[i]), xr, 0.5 * 0.4 * m * r * r * (w.x * w.x + w.y * w.y + w.z * w.z), 0.0);
        }
    } else if (k < d.nf + d.ns + d.nc) {
        const int c = k - d.nf - d.ns;
        const float im = d.cinvm[c];
        if (im > 0.f) add(1.0 / im, dfv(d.cvH[c], d.cvL[c]), dfv(d.cpH[c], d.cpL[c]), 0.0, 0.0);
    }
    for (int a = 0; a < AUDIT_N; ++a) sh[a][threadIdx.x] = q[a];
    __syncthreads();
    for (int o = AUDIT_T / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int a = 0; a < AUDIT_N; ++a) sh[a][threadIdx.x] += sh[a][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int a = 0; a < AUDIT_N; ++a) partial[(size_t)blockIdx.x * AUDIT_N + a] = sh[a][0];
}

template <class T>
void d2h(std::vector<T>& v, const T* src, size_t n)
{
    v.resize(n);
    if (n) CK(cudaMemcpy(v.data(), src, sizeof(T) * n, cudaMemcpyDeviceToHost));
}

}  // namespace

namespace demsph {

// The host transfers of the state, enqueued on the engine's stream (the
// public calls below add the synchronisation; demsph_update_io enqueues them
// around its steps and synchronises once).
void enqueueDownloadFluids(demsph_engine* e, double* pos, double* vel, double* acc, double* drho, cudaStream_t s,
                           int slot)
{
    DeviceState& d = e->d;
    if (d.nf == 0) return;
    if (!s) s = e->stream;
    const size_t n = d.nf;
    double* buf = scratchDoubles(e, 10 * n, slot);
    ++t_kernelLaunches, kFluidOut<<<blocksFor(d.nf, 256), 256, 0, s>>>(d, buf);
    double* outs[3] = {pos, vel, acc};
    for (int k = 0; k < 3; ++k)
        if (outs[k]) CK(cudaMemcpyAsync(outs[k], buf + 3 * n * k, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    if (drho) CK(cudaMemcpyAsync(drho, buf + 9 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
}

void enqueueDownloadSolids(demsph_engine* e, double* pos, double* vel, double* acc, double* normal, double* torque,
                           double* angvel, cudaStream_t s, int slot)
{
    DeviceState& d = e->d;
    if (d.ns == 0) return;
    if (!s) s = e->stream;
    const size_t n3 = 3 * (size_t)d.ns;
    double* buf = scratchDoubles(e, 6 * n3, slot);
    double* outs[6] = {pos, vel, acc, normal, torque, angvel};
    unsigned want = 0;
    for (int k = 0; k < 6; ++k)
        if (outs[k]) want |= 1u << k;
    ++t_kernelLaunches, kSolidOut<<<blocksFor(d.ns, 256), 256, 0, s>>>(d, buf, want);
    for (int k = 0; k < 6; ++k)
        if (outs[k]) CK(cudaMemcpyAsync(outs[k], buf + n3 * k, sizeof(double) * n3, cudaMemcpyDeviceToHost, s));
}

void enqueueUploadFluids(demsph_engine* e, const double* pos, const double* vel, const double* drho, cudaStream_t s,
                         int slot)
{
    DeviceState& d = e->d;
    if (d.nf == 0) return;
    if (!s) s = e->stream;
    double* buf = scratchDoubles(e, 7 * (size_t)d.nf, slot);
    double* dp = pos ? buf : nullptr;
    double* dv = vel ? buf + 3 * (size_t)d.nf : nullptr;
    double* dr = drho ? buf + 6 * (size_t)d.nf : nullptr;
    if (dp) CK(cudaMemcpyAsync(dp, pos, sizeof(double) * 3 * d.nf, cudaMemcpyHostToDevice, s));
    if (dv) CK(cudaMemcpyAsync(dv, vel, sizeof(double) * 3 * d.nf, cudaMemcpyHostToDevice, s));
    if (dr) CK(cudaMemcpyAsync(dr, drho, sizeof(double) * d.nf, cudaMemcpyHostToDevice, s));
    ++t_kernelLaunches, kFluidIn<<<blocksFor(d.nf, 256), 256, 0, s>>>(d, dp, dv, dr);
}

// The move list after an upload of solid velocities `vel` in which a dummy
// particle started or stopped moving (the device found it); the moving flags
// go back to the device.
void rebuildMoves(demsph_engine* e, const double* vel)
{
    DeviceState& d = e->d;
    bool moveChanged = false;
    for (size_t q = 0; q < e->dummyIdx.size(); ++q) {
        const size_t i = (size_t)e->dummyIdx[q];
        const unsigned char m = (vel[3 * i] != 0.0 || vel[3 * i + 1] != 0.0 || vel[3 * i + 2] != 0.0) ? 1 : 0;
        if (m != e->dummyMoving[q]) {
            e->dummyMoving[q] = m;
            moveChanged = true;
        }
    }
    if (moveChanged) {
        std::vector<int> move;
        move.reserve(e->moveHost.size());
        for (int i = 0; i < d.ns; ++i) {
            const unsigned char k = e->moveKind[i];
            if (k == 1 || (k == 2 && (vel[3 * i] != 0.0 || vel[3 * i + 1] != 0.0 || vel[3 * i + 2] != 0.0)))
                move.push_back(i);
        }
        if (move != e->moveHost) {
            const int first = consecutiveFirst(move.data(), move.size());
            if (move.size() != e->moveHost.size()) {
                void* p = d.moveList;
                freeOne(e, p);
                d.moveList = dalloc<int>(move.size(), e->owned, e->stream);
                d.nmove = (int)move.size();
                dropGraph(e);  // the list is a kernel argument baked into captured graphs
            }
            if (first != d.moveFirst) {
                d.moveFirst = first;
                dropGraph(e);
            }
            if (!move.empty()) {
                // the host vector must outlive the asynchronous copy: keep it as the engine's copy
                e->moveHost.swap(move);
                CK(cudaMemcpyAsync(d.moveList, e->moveHost.data(), sizeof(int) * e->moveHost.size(),
                                   cudaMemcpyHostToDevice, e->stream));
            } else {
                e->moveHost.swap(move);
            }
        }
    }
    e->movingDummies = (int)std::count(e->dummyMoving.begin(), e->dummyMoving.end(), (unsigned char)1);
    if (d.ndummy > 0)
        CK(cudaMemcpyAsync(d.dummyMoving, e->dummyMoving.data(), d.ndummy, cudaMemcpyHostToDevice, e->stream));
}

// Raises moveChanged when an uploaded velocity starts or stops a dummy
// particle's motion.
__global__ void kDummyMoves(DeviceState d, const double* __restrict__ vel)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.ndummy) return;
    const size_t i = (size_t)d.dummyIdx[q];
    const unsigned char m = (vel[3 * i] != 0.0 || vel[3 * i + 1] != 0.0 || vel[3 * i + 2] != 0.0) ? 1 : 0;
    if (m != d.dummyMoving[q]) *(volatile int*)d.moveChanged = 1;
}

void enqueueUploadSolids(demsph_engine* e, const double* pos, const double* vel, const double* angvel, cudaStream_t s,
                         int slot)
{
    DeviceState& d = e->d;
    if (d.ns == 0) return;
    if (!s) s = e->stream;
    double* buf = scratchDoubles(e, 9 * (size_t)d.ns, slot);
    double* dp = pos ? buf : nullptr;
    double* dv = vel ? buf + 3 * (size_t)d.ns : nullptr;
    double* dw = angvel ? buf + 6 * (size_t)d.ns : nullptr;
    if (dp) CK(cudaMemcpyAsync(dp, pos, sizeof(double) * 3 * d.ns, cudaMemcpyHostToDevice, s));
    if (dv) CK(cudaMemcpyAsync(dv, vel, sizeof(double) * 3 * d.ns, cudaMemcpyHostToDevice, s));
    if (dw) CK(cudaMemcpyAsync(dw, angvel, sizeof(double) * 3 * d.ns, cudaMemcpyHostToDevice, s));
    // dummy particles given a velocity join the integration: the move list
    // changes only when one starts or stops moving, which the device finds
    // (one word read back); the host then rebuilds the list
    if (dv && d.ndummy > 0) {
        CK(cudaMemsetAsync(d.moveChanged, 0, sizeof(int), s));
        ++t_kernelLaunches, kDummyMoves<<<blocksFor(d.ndummy, 256), 256, 0, s>>>(d, dv);
        int changed = 0;
        CK(cudaMemcpyAsync(&changed, d.moveChanged, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (changed) {
            // the move list goes up on the engine's stream: the solids' stream joins it before the steps
            rebuildMoves(e, vel);
        }
    }
    // the flag of the step that follows (its list takes the other parity)
    ++t_kernelLaunches, kSolidIn<<<blocksFor(d.ns, 256), 256, 0, s>>>(d, dp, dv, dw, d.rebuild + (e->par ^ 1));
    // solids that never move are otherwise sorted only once
    if (dp && e->nMassive == 0) e->solidSortStale = true;
}

}  // namespace demsph

extern "C" {


int demsph_download_fluids(demsph_engine* e, double* pos, double* vel, double* acc, double* drho)
{
    ENGINE_GUARD(e)
    enqueueDownloadFluids(e, pos, vel, acc, drho);
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_download_solids(demsph_engine* e, double* pos, double* vel, double* acc, double* normal, double* torque,
                           double* angvel)
{
    ENGINE_GUARD(e)
    enqueueDownloadSolids(e, pos, vel, acc, normal, torque, angvel);
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_download_clumps(demsph_engine* e, double* centroid, double* vel, double* acc, double* angvel,
                           double* torque, double* orientation)
{
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    const size_t n = d.nc;
    if (n == 0) return DEMSPH_OK;
    double* buf = scratchDoubles(e, 19 * n);
    ++t_kernelLaunches, kClumpOut<<<blocksFor((long long)n, 128), 128, 0, e->stream>>>(d, buf);
    double* outs[5] = {centroid, vel, acc, angvel, torque};
    for (int k = 0; k < 5; ++k)
        if (outs[k]) CK(cudaMemcpyAsync(outs[k], buf + 3 * n * k, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->stream));
    if (orientation) CK(cudaMemcpyAsync(orientation, buf + 15 * n, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_upload_fluids(demsph_engine* e, const double* pos, const double* vel, const double* drho)
{
    ENGINE_GUARD(e)
    enqueueUploadFluids(e, pos, vel, drho);
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_upload_solids(demsph_engine* e, const double* pos, const double* vel, const double* angvel)
{
    ENGINE_GUARD(e)
    enqueueUploadSolids(e, pos, vel, angvel);
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_set_gravity(demsph_engine* e, const double g[3])
{
    if (!g) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    for (int a = 0; a < 3; ++a) e->d.g64[a] = g[a];
    e->d.g = make_float3((float)g[0], (float)g[1], (float)g[2]);
    dropGraph(e);  // gravity is a kernel argument baked into captured graphs
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_set_contact_models(demsph_engine* e, const demsph_scene* t)
{
    if (!t || !t->hertzian || !t->linear || !t->bonded || t->n_material != e->d.tab.nMat) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    const int nslot = t->n_material * (t->n_material + 1) / 2;
    std::vector<float> all(26 * (size_t)nslot);
    for (int k = 0; k < 8 * nslot; ++k) all[k] = (float)t->hertzian[k];
    for (int k = 0; k < 11 * nslot; ++k) all[8 * nslot + k] = (float)t->linear[k];
    for (int k = 0; k < 6 * nslot; ++k) all[19 * nslot + k] = (float)t->bonded[k];
    for (int k = 0; k < nslot; ++k) {
        const double lr = std::log(t->hertzian[8 * k + 2]);
        all[25 * nslot + k] = (float)(-lr / std::sqrt(lr * lr + 3.1415926535897931 * 3.1415926535897931));
    }
    CK(cudaMemcpyAsync(const_cast<float*>(e->d.tab.hz), all.data(), sizeof(float) * all.size(), cudaMemcpyHostToDevice,
                       e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_set_clump_velocity(demsph_engine* e, int c, const double v[3])
{
    if (!v) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    if (c < 0 || c >= e->d.nc) return DEMSPH_OK;  // the reference ignores out-of-range clumps (dataBase.h:171)
    ++t_kernelLaunches, kSetClumpVelocity<<<1, 1, 0, e->stream>>>(e->d, c, v[0], v[1], v[2]);
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_add_external_force(demsph_engine* e, int i, const double f[3])
{
    if (!f) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    if (i < 0 || i >= e->d.ns) return fail(e, DEMSPH_ERR_ARGUMENT, "solid index out of range");
    ++t_kernelLaunches, kAddForce<<<1, 1, 0, e->stream>>>(e->d, i, (float)f[0], (float)f[1], (float)f[2]);
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_add_global_damping(demsph_engine* e, int i, double cd)
{
    ENGINE_GUARD(e)
    if (i < 0 || i >= e->d.ns) return fail(e, DEMSPH_ERR_ARGUMENT, "solid index out of range");
    ++t_kernelLaunches, kAddDamping<<<1, 1, 0, e->stream>>>(e->d, i, (float)cd);
    CK(cudaStreamSynchronize(e->stream));
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_get_counts(demsph_engine* e, demsph_counts* out)
{
    if (!out) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    *out = demsph_counts{};
    std::vector<int> ffc, fsc;
    d2h(ffc, d.ffc, d.nf);
    d2h(fsc, d.fsc, d.nf);
    long long ff = 0, fs = 0;
    for (int i = 0; i < d.nf; ++i) {
        ff += std::min(ffc[i], d.kff);
        fs += std::min(fsc[i], d.kfs);
    }
    out->fluid_pairs = ff / 2;
    out->fluid_solid_pairs = fs;
    std::vector<int> fc;
    d2h(fc, d.fcnt[e->par], d.nrow);
    long long np = 0;
    for (int r = 0; r < d.nrow; ++r) np += std::min(fc[r], d.scap);
    out->solid_pairs = np;
    out->bonds = d.nb;
    std::vector<int> on;
    d2h(on, d.bon, d.nb);
    for (int b = 0; b < d.nb; ++b) out->bonds_intact += on[b] != 0;
    out->grid_cells = d.grid.num;
    out->grid_size[0] = d.grid.gx;
    out->grid_size[1] = d.grid.gy;
    out->grid_size[2] = d.grid.gz;
    for (int a = 0; a < 3; ++a) out->cell_size[a] = d.cs[a];
    return DEMSPH_OK;
    ENGINE_END(e)
}

// objectHash + cell spans (core/neighborSearch.cu:71-113).  For fluids these
// are the structures of the last fluid list rebuild.
int demsph_export_cell_hash(demsph_engine* e, int which, int* value, int* index, int* start, int* end)
{
    if (which != 0 && which != 1) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    const int n = which == 0 ? d.nf : d.ns;
    std::vector<int> cs;
    if (which == 0) {
        // fluids are reordered by cell only when their list candidates are
        // rebuilt: the (key, index) order of this step is restored here
        std::vector<int4> cell;
        std::vector<int> id;
        d2h(cell, d.fcell, n);
        d2h(id, d.fid, n);
        std::vector<std::pair<int, int>> kv(n);
        for (int s = 0; s < n; ++s) kv[s] = {cell[s].w, id[s]};
        std::sort(kv.begin(), kv.end());
        cs.assign((size_t)d.grid.num + 1, 0);
        for (int s = 0; s < n; ++s) cs[kv[s].first + 1]++;
        for (int k = 0; k < d.grid.num; ++k) cs[k + 1] += cs[k];
        for (int s = 0; s < n; ++s) {
            if (value) value[s] = kv[s].first;
            if (index) index[s] = kv[s].second;
        }
    } else {
        // the solids' keys are computed every step, their device-side sort only
        // when a list needs it: the (key, index) order is restored here, from
        // the keys the last neighbour search used
        std::vector<int> key, order(n);
        d2h(key, e->keysAdvanced ? d.skeySearch : d.skey, n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return key[x] < key[y]; });
        cs.assign((size_t)d.grid.num + 1, 0);
        for (int i = 0; i < n; ++i) cs[key[i] + 1]++;
        for (int k = 0; k < d.grid.num; ++k) cs[k + 1] += cs[k];
        for (int p = 0; p < n; ++p) {
            if (value) value[p] = key[order[p]];
            if (index) index[p] = order[p];
        }
    }
    for (int k = 0; k < d.grid.num; ++k) {
        const bool empty = cs[k] == cs[k + 1];
        if (start) start[k] = empty ? -1 : cs[k];
        if (end) end[k] = empty ? -1 : cs[k + 1];
    }
    return DEMSPH_OK;
    ENGINE_END(e)
}

// fluid2Fluid half list (core/neighborSearch.cu:115-220): for each fluid i in
// original order, its partners j > i in walk order.  Returns the pair count
// through prefix[n-1]; pairs beyond capacity are not written.
int demsph_export_fluid_pairs(demsph_engine* e, int* prefix, int* pointed, int* pointing, long long cap)
{
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    const int n = d.nf;
    std::vector<unsigned> ff;
    std::vector<int> ffc, id, slot;
    if (d.fluidTiles && n > 0) {
        // tile mode keeps the lists as membership bits: write them out as list
        // entries (in a buffer made for exports) first
        d2h(ffc, d.ffc, n);
        const int most = *std::max_element(ffc.begin(), ffc.end());
        if (!d.ff || most > d.kff) {
            void* p = d.ff;
            freeOne(e, p);
            d.kff = std::max(d.kff, most);
            d.ff = dalloc<unsigned>((size_t)d.kff * n, e->owned, e->stream, false);
        }
        launchBitsToLists(d, e->stream);
        CK(cudaStreamSynchronize(e->stream));
    }
    d2h(ff, d.ff, (size_t)d.kff * n);
    d2h(ffc, d.ffc, n);
    d2h(id, d.fid, n);
    slot.resize(n);
    for (int s = 0; s < n; ++s) slot[id[s]] = s;
    // the reference's order: by walk position, then by index (its stable
    // (cell, index) sort)
    long long w = 0;
    std::vector<std::pair<long long, int>> order;
    for (int i = 0; i < n; ++i) {
        const int s = slot[i];
        const int m = std::min(ffc[s], d.kff);
        order.clear();
        for (int k = 0; k < m; ++k) {
            const unsigned v = ff[(size_t)k * n + s];
            order.push_back({(long long)entryWalk(v) * n + id[ffPartner(v)], ffPartner(v)});
        }
        std::sort(order.begin(), order.end());
        for (const auto& o : order) {
            const int j = id[o.second];
            if (j <= i) continue;
            if (w < cap) {
                if (pointed) pointed[w] = i;
                if (pointing) pointing[w] = j;
            }
            ++w;
        }
        if (prefix) prefix[i] = (int)w;
    }
    return DEMSPH_OK;
    ENGINE_END(e)
}

// fluid2Solid list (core/neighborSearch.cu:115-220) with the coupling force of
// each pair (core/integrate.cu:282-330) as of the last step (debug bit 0) or
// zeros otherwise.
int demsph_export_fluid_solid_pairs(demsph_engine* e, int* prefix, int* pointed, int* pointing, double* force,
                                    long long cap)
{
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    const int n = d.nf;
    std::vector<int> fs, fsc, id, slot;
    std::vector<float4> pf;
    d2h(fs, d.fs, (size_t)d.kfs * n);
    d2h(fsc, d.fsc, n);
    d2h(id, d.fid, n);
    if (d.fsPairForce) d2h(pf, d.fsPairForce, (size_t)d.kfs * n);
    slot.resize(n);
    for (int s = 0; s < n; ++s) slot[id[s]] = s;
    long long w = 0;
    std::vector<std::pair<long long, int>> order;
    for (int i = 0; i < n; ++i) {
        const int s = slot[i];
        const int m = std::min(fsc[s], d.kfs);
        order.clear();
        for (int k = 0; k < m; ++k) {
            const int v = fs[(size_t)k * n + s];
            order.push_back({(long long)entryWalk((unsigned)v) * d.ns + fsPartner(v), k});
        }
        std::sort(order.begin(), order.end());  // walk position, then index
        for (const auto& o : order) {
            const int k = o.second;
            if (w < cap) {
                if (pointed) pointed[w] = i;
                if (pointing) pointing[w] = fsPartner(fs[(size_t)k * n + s]);
                if (force) {
                    const float4 f = pf.empty() ? make_float4(0, 0, 0, 0) : pf[(size_t)k * n + s];
                    force[3 * w] = f.x;
                    force[3 * w + 1] = f.y;
                    force[3 * w + 2] = f.z;
                }
            }
            ++w;
        }
        if (prefix) prefix[i] = (int)w;
    }
    return DEMSPH_OK;
    ENGINE_END(e)
}

// solid2Solid list (core/neighborSearch.cu:222-312) with the contact forces,
// torques and springs of the last contact phase (core/integrate.cu:423-512).
int demsph_export_solid_pairs(demsph_engine* e, int* prefix, int* pointed, int* pointing, double* force,
                              double* torque, double* sliding, double* rolling, double* torsion, long long cap)
{
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    const int ns = d.ns, nr = d.nrow, C = d.scap;
    const int par = e->par;
    std::vector<int> fc, fw, rs, key;
    std::vector<int4> centre;
    d2h(fc, d.fcnt[par], nr);
    d2h(fw, d.fwd[par], (size_t)C * nr);
    d2h(rs, d.rowSolid, nr);
    const bool walkOrder = e->walkOrder[par];
    if (!walkOrder) {
        d2h(key, e->keysAdvanced ? d.skeySearch : d.skey, ns);
        d2h(centre, e->keysAdvanced ? d.scentreSearch : d.scentre, nr);
    }
    std::vector<float4> F, T, S0, S1, S2;
    const size_t all = (size_t)C * nr;
    if (force) d2h(F, d.pF, all);
    if (torque) d2h(T, d.pT, all);
    if (sliding) d2h(S0, d.springOut[par][0], all);
    if (rolling) d2h(S1, d.springOut[par][1], all);
    if (torsion) d2h(S2, d.springOut[par][2], all);
    // the reference adds each bond's force and torque onto its pair's
    // (integrate.cu:802-803); the engine keeps them per bond
    if ((force || torque) && d.nb > 0) {
        std::vector<int2> ab;
        std::vector<float4> FnTt, FsH, FsL, TbH, TbL, N;
        d2h(ab, d.bab, d.nb);
        d2h(FnTt, d.bFnTt, d.nb);
        d2h(FsH, d.bFsH, d.nb);
        d2h(FsL, d.bFsL, d.nb);
        d2h(TbH, d.bTbH, d.nb);
        d2h(TbL, d.bTbL, d.nb);
        d2h(N, d.bN, d.nb);
        std::vector<int> rowOf(ns, -1);
        for (int r = 0; r < nr; ++r) rowOf[rs[r]] = r;
        for (int b = 0; b < d.nb; ++b) {
            const int r = rowOf[ab[b].x];
            if (r < 0) continue;
            for (int q = 0; q < std::min(fc[r], C); ++q) {
                const size_t k = (size_t)q * nr + r;
                if (fw[k] != ab[b].y) continue;
                const float fn = FnTt[b].x + FnTt[b].y, tt = FnTt[b].z + FnTt[b].w;
                if (force) {
                    F[k].x += N[b].x * fn + (FsH[b].x + FsL[b].x);
                    F[k].y += N[b].y * fn + (FsH[b].y + FsL[b].y);
                    F[k].z += N[b].z * fn + (FsH[b].z + FsL[b].z);
                }
                if (torque) {
                    T[k].x += N[b].x * tt + (TbH[b].x + TbL[b].x);
                    T[k].y += N[b].y * tt + (TbH[b].y + TbL[b].y);
                    T[k].z += N[b].z * tt + (TbH[b].z + TbL[b].z);
                }
                break;
            }
        }
    }
    auto put = [&](double* out, const std::vector<float4>& v, long long w, size_t k) {
        if (!out) return;
        out[3 * w] = v[k].x;
        out[3 * w + 1] = v[k].y;
        out[3 * w + 2] = v[k].z;
    };
    // Rows ascend with the solid index, as the reference's CSR does.  A list
    // kept in index order is put back in the reference's walk order: the
    // partners of A by the position, in A's 27-cell walk ((z, y, x) loops
    // around its centre cell, core/neighborSearch.cu:236-245), of the first
    // visited cell whose key is the partner's key - the k-th copy of a partner
    // listed twice (a key visited twice) at the k-th such cell - then by index
    // (the stable (cell, index) sort).
    const int gx = d.grid.gx, gy = d.grid.gy, num = d.grid.num;
    std::vector<std::pair<long long, size_t>> order;
    std::vector<int> walk;
    long long w = 0;
    int row = 0;
    for (int i = 0; i < ns; ++i) {
        if (row < nr && rs[row] == i) {
            const int n = std::min(fc[row], C);
            order.clear();
            if (!walkOrder) {
                walk.clear();
                const int4 c = centre[row];
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const long long h = (long long)(c.z + dz) * gy * gx + (long long)(c.y + dy) * gx + (c.x + dx);
                            walk.push_back(h >= 0 && h < num ? (int)h : -1);
                        }
            }
            for (int q = 0; q < n; ++q) {
                const size_t k = (size_t)q * nr + row;
                const int b = fw[k];
                long long rank = q;
                if (!walkOrder) {
                    int copy = 0;  // earlier copies of b in this (index-ordered) row
                    for (int p = q - 1; p >= 0 && fw[(size_t)p * nr + row] == b; --p) ++copy;
                    int t = 27;
                    for (int u = 0; u < 27; ++u)
                        if (walk[u] == key[b] && copy-- == 0) {
                            t = u;
                            break;
                        }
                    rank = (long long)t * ns + b;
                }
                order.push_back({rank, k});
            }
            std::sort(order.begin(), order.end());
            for (const auto& o : order) {
                if (w < cap) {
                    if (pointed) pointed[w] = i;
                    if (pointing) pointing[w] = fw[o.second];
                    put(force, F, w, o.second);
                    put(torque, T, w, o.second);
                    put(sliding, S0, w, o.second);
                    put(rolling, S1, w, o.second);
                    put(torsion, S2, w, o.second);
                }
                ++w;
            }
            ++row;
        }
        if (prefix) prefix[i] = (int)w;
    }
    return DEMSPH_OK;
    ENGINE_END(e)
}

// interactionBonded (core/deviceStructs.h:714-789).  The contact point is the
// bond's stored lever added to the current position of its first sphere.
int demsph_export_bonds(demsph_engine* e, int* pointed, int* pointing, int* isb, double* fn, double* tt, double* fs,
                        double* tb, double* normal, double* point, long long cap)
{
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    const int nb = d.nb;
    std::vector<int2> ab;
    std::vector<int> on;
    std::vector<float4> FnTt, FsH, FsL, TbH, TbL, N, L;
    d2h(ab, d.bab, nb);
    d2h(on, d.bon, nb);
    d2h(FnTt, d.bFnTt, nb);
    d2h(FsH, d.bFsH, nb);
    d2h(FsL, d.bFsL, nb);
    d2h(TbH, d.bTbH, nb);
    d2h(TbL, d.bTbL, nb);
    d2h(N, d.bN, nb);
    d2h(L, d.bLever, nb);
    std::vector<double> pos;
    if (point && d.ns > 0) {
        pos.resize(3 * (size_t)d.ns);
        const int rc = demsph_download_solids(e, pos.data(), nullptr, nullptr, nullptr, nullptr, nullptr);
        if (rc != DEMSPH_OK) return rc;
    }
    for (int b = 0; b < nb && b < cap; ++b) {
        if (pointed) pointed[b] = ab[b].x;
        if (pointing) pointing[b] = ab[b].y;
        if (isb) isb[b] = on[b];
        if (fn) fn[b] = (double)FnTt[b].x + FnTt[b].y;
        if (tt) tt[b] = (double)FnTt[b].z + FnTt[b].w;
        for (int a = 0; a < 3; ++a) {
            const float* sh = &FsH[b].x; const float* sl = &FsL[b].x;
            const float* th = &TbH[b].x; const float* tl = &TbL[b].x;
            if (fs) fs[3 * b + a] = (double)sh[a] + sl[a];
            if (tb) tb[3 * b + a] = (double)th[a] + tl[a];
            if (normal) normal[3 * b + a] = (&N[b].x)[a];
            if (point) point[3 * b + a] = pos[3 * (size_t)ab[b].x + a] + (&L[b].x)[a];
        }
    }
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_audit(demsph_engine* e, demsph_audit_values* out)
{
    if (!out) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    const long long n = (long long)d.nf + d.ns + d.nc;
    const int blocks = blocksFor(std::max(1LL, n), AUDIT_T);
    double* buf = scratchDoubles(e, (size_t)blocks * AUDIT_N);
    ++t_kernelLaunches, kAudit<<<blocks, AUDIT_T, 0, e->stream>>>(d, buf);
    std::vector<double> h((size_t)blocks * AUDIT_N);
    CK(cudaMemcpyAsync(h.data(), buf, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    double q[AUDIT_N] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < blocks; ++b)
        for (int a = 0; a < AUDIT_N; ++a) q[a] += h[(size_t)b * AUDIT_N + a];
    out->mass = q[0];
    for (int a = 0; a < 3; ++a) out->momentum[a] = q[1 + a];
    out->kinetic_energy = q[4];
    out->rotational_energy = q[5];
    out->potential_energy = q[6];
    out->fluid_density_sum = q[7];
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_export_fluid_sumw0(demsph_engine* e, double* out)
{
    if (!out) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    DeviceState& d = e->d;
    CK(cudaStreamSynchronize(e->stream));
    // sumW0 = sigma(h) * S0 with sigma = 21 / (16 pi h^3) (core/SPHKernelDEMContactModel.h:5-13)
    std::vector<float2> w;
    std::vector<float4> ph, pl;
    std::vector<int> id;
    d2h(w, d.fsumW0, d.nf);
    d2h(ph, d.fph[0], d.nf);
    d2h(pl, d.fpl[0], d.nf);
    d2h(id, d.fid, d.nf);
    for (int s = 0; s < d.nf; ++s) {
        const double h = (double)ph[s].w + (double)pl[s].w;
        out[id[s]] = 21.0 / (16.0 * 3.1415926535897931 * h * h * h) * ((double)w[s].x + (double)w[s].y);
    }
    return DEMSPH_OK;
    ENGINE_END(e)
}

}  // extern "C"
