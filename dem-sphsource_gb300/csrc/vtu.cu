// Frame files of class solverBase (core/solverBase.cpp:69-333 in the
// reference: <dir>/fluid_NNNN.vtu, solid_NNNN.vtu and fluid2Solid_NNNN.vtu,
// VTK unstructured grids of vertices with the same arrays, names and order)
// written as binary VTU ("appended", raw, UInt64 block headers) by a
// background thread.
//
// The reference downloads the state and formats every value as ASCII text on
// the simulation thread; a frame of a million particles then holds the run
// for seconds.  Here a frame is one pack kernel on the engine's stream (the
// file's FP32 arrays, in the original particle order, into a device slot)
// and an event; the writer thread waits for the event, copies the slot into
// pinned memory on its own stream and writes the file while the next steps
// run.  Each kind has two slots: a third frame of a kind waits, on the host,
// until the writer has finished the first one's file.
//
// The values are those of the reference's files read back by a VTU reader:
// the reference prints FP64 values with ten decimals into arrays declared
// Float32, which a reader rounds to FP32; here the FP64 value (positions
// rebuilt as cell origin + double-float offset, as the state downloads do)
// is rounded to FP32 once.
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <filesystem>
#include <mutex>
#include <sstream>
#include <iomanip>
#include <string>
#include <thread>
#include <vector>

#include "engine_impl.cuh"

using namespace demsph;

namespace {

constexpr int KINDS = 3;  // fluid, solid, fluid2Solid
constexpr int SLOTS = 2;

__device__ __forceinline__ double originOf(const DeviceState& d, int a, int c) { return d.minB[a] + (double)c * d.cs[a]; }

__device__ __forceinline__ double3 fluidPosition(const DeviceState& d, int s)
{
    const int4 c = d.fcell[s];
    const float4 h = d.fph[0][s], l = d.fpl[0][s];
    return make_double3(originOf(d, 0, c.x) + ((double)h.x + (double)l.x),
                        originOf(d, 1, c.y) + ((double)h.y + (double)l.y),
                        originOf(d, 2, c.z) + ((double)h.z + (double)l.z));
}

__device__ __forceinline__ double3 solidPosition(const DeviceState& d, int a)
{
    const int4 c = d.scell[a];
    const float4 h = d.sph[a], l = d.spl[a];
    return make_double3(originOf(d, 0, c.x) + ((double)h.x + (double)l.x),
                        originOf(d, 1, c.y) + ((double)h.y + (double)l.y),
                        originOf(d, 2, c.z) + ((double)h.z + (double)l.z));
}

__device__ __forceinline__ void put3(float* o, double x, double y, double z)
{
    o[0] = (float)x;
    o[1] = (float)y;
    o[2] = (float)z;
}

// Fluid slot, n = nf: position[3n] velocity[3n] density[n] pressure[n]
// (density rho0 + dRho, pressure dRho c^2: core/solverBase.cpp:151-161).
__global__ void kFluidFrame(DeviceState d, float* out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.nf) return;
    const size_t n = d.nf, id = d.fid[s];
    const double3 p = fluidPosition(d, s);
    put3(out + 3 * id, p.x, p.y, p.z);
    const float4 vh = d.fvh[0][s], vl = d.fvl[0][s];
    put3(out + 3 * n + 3 * id, (double)vh.x + vl.x, (double)vh.y + vl.y, (double)vh.z + vl.z);
    const float4 par = d.fpar[s];
    const double dr = d.fdrho[0][s];
    out[6 * n + id] = (float)((double)par.x + dr);
    out[7 * n + id] = (float)(dr * ((double)par.y * (double)par.y));
}

// Solid slot, n = ns: position[3n] velocity[3n] angularVelocity[3n] normal[3n].
__global__ void kSolidFrame(DeviceState d, float* out)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= d.ns) return;
    const size_t n = d.ns;
    const double3 p = solidPosition(d, a);
    put3(out + 3 * (size_t)a, p.x, p.y, p.z);
    const float4 vh = d.svh[a], vl = d.svl[a];
    put3(out + 3 * n + 3 * (size_t)a, (double)vh.x + vl.x, (double)vh.y + vl.y, (double)vh.z + vl.z);
    const float4 wh = d.swh[a], wl = d.swl[a];
    put3(out + 6 * n + 3 * (size_t)a, (double)wh.x + wl.x, (double)wh.y + wl.y, (double)wh.z + wl.z);
    const float4 nr = d.snormal[a];
    put3(out + 9 * n + 3 * (size_t)a, nr.x, nr.y, nr.z);
}

// fluid2Solid, step 1: each fluid's pair count, in original order.
__global__ void kPairCounts(DeviceState d, int* count)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.nf) return;
    count[d.fid[s]] = min(d.fsc[s], d.kfs);
}

// fluid2Solid, step 2: the pairs in the reference's order (fluids in original
// order, each fluid's partners by walk position, then by index - the order of
// demsph_export_fluid_solid_pairs): midpoint[3N] then force[3N] at
// out + 3 cap.  A fluid's rank of a pair is the number of its pairs with a
// smaller key (keys differ: a solid appears once in a fluid's list).  The
// count of all pairs goes to *total.
__global__ void kPairFrame(DeviceState d, const int* count, const int* offset, float* out, long long cap,
                           long long* total)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.nf) return;
    const size_t n = d.nf;
    const int id = d.fid[s];
    const int m = count[id];
    const long long first = offset[id];
    if (id == d.nf - 1) *total = first + m;
    if (m == 0) return;
    const double3 pf = fluidPosition(d, s);
    for (int k = 0; k < m; ++k) {
        const int v = d.fs[(size_t)k * n + s];
        const long long key = (long long)entryWalk((unsigned)v) * d.ns + fsPartner(v);
        int rank = 0;
        for (int q = 0; q < m; ++q) {
            const int u = d.fs[(size_t)q * n + s];
            rank += (long long)entryWalk((unsigned)u) * d.ns + fsPartner(u) < key ? 1 : 0;
        }
        const long long w = first + rank;
        if (w >= cap) continue;
        const double3 ps = solidPosition(d, fsPartner(v));
        put3(out + 3 * w, 0.5 * (pf.x + ps.x), 0.5 * (pf.y + ps.y), 0.5 * (pf.z + ps.z));
        const float4 f = d.fsPairForce ? d.fsPairForce[(size_t)k * n + s] : make_float4(0.f, 0.f, 0.f, 0.f);
        put3(out + 3 * cap + 3 * w, f.x, f.y, f.z);
    }
}

// One array of a file: type, name, components, bytes.
struct Block {
    const char* type;
    const char* name;
    int comps;
    const void* data;
    size_t bytes;
};

// Writes one VTU file: the XML header with every array "appended", then the
// raw blocks, each after its UInt64 byte count.  Returns "" or the error.
std::string writeVtu(const std::string& path, double time, int step, long long npts, const Block& points,
                     const std::vector<Block>& cells, const char* scalars, const std::vector<Block>& pointData)
{
    std::ostringstream x;
    size_t off = 0;
    auto arr = [&](const Block& b, const char* indent) {
        x << indent << "<DataArray type=\"" << b.type << "\"";
        if (b.name) x << " Name=\"" << b.name << "\"";
        if (b.comps > 1) x << " NumberOfComponents=\"" << b.comps << "\"";
        x << " format=\"appended\" offset=\"" << off << "\"/>\n";
        off += sizeof(unsigned long long) + b.bytes;
    };
    x << "<?xml version=\"1.0\"?>\n"
      << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
      << "  <UnstructuredGrid>\n"
      << "    <FieldData>\n"
      << "      <DataArray type=\"Float32\" Name=\"TIME\"  NumberOfTuples=\"1\" format=\"ascii\"> " << std::fixed
      << std::setprecision(10) << time << " </DataArray>\n"
      << "      <DataArray type=\"Int32\"   Name=\"STEP\"  NumberOfTuples=\"1\" format=\"ascii\"> " << step
      << " </DataArray>\n"
      << "    </FieldData>\n"
      << "    <Piece NumberOfPoints=\"" << npts << "\" NumberOfCells=\"" << npts << "\">\n"
      << "      <Points>\n";
    arr(points, "        ");
    x << "      </Points>\n      <Cells>\n";
    for (const auto& b : cells) arr(b, "        ");
    x << "      </Cells>\n      <PointData Scalars=\"" << scalars << "\">\n";
    for (const auto& b : pointData) arr(b, "        ");
    x << "      </PointData>\n    </Piece>\n  </UnstructuredGrid>\n  <AppendedData encoding=\"raw\">\n_";
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return "cannot open " + path;
    const std::string head = x.str();
    bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
    auto raw = [&](const Block& b) {
        const unsigned long long nb = b.bytes;
        ok = ok && std::fwrite(&nb, sizeof(nb), 1, f) == 1;
        if (b.bytes) ok = ok && std::fwrite(b.data, 1, b.bytes, f) == b.bytes;
    };
    raw(points);
    for (const auto& b : cells) raw(b);
    for (const auto& b : pointData) raw(b);
    const char tail[] = "\n  </AppendedData>\n</VTKFile>\n";
    ok = ok && std::fwrite(tail, 1, sizeof(tail) - 1, f) == sizeof(tail) - 1;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? std::string() : "cannot write " + path;
}

std::string frameName(const std::string& dir, const char* stem, int frame)
{
    std::ostringstream s;
    s << dir << "/" << stem << "_" << std::setw(4) << std::setfill('0') << frame << ".vtu";
    return s.str();
}

}  // namespace

struct demsph_frame_writer {
    demsph_engine* e = nullptr;
    std::string dir;
    int nf = 0, ns = 0;
    // static arrays from the scene (original order)
    std::vector<float> smoothing, radius;
    std::vector<int> cluster, clump;
    // per kind and slot: device staging, pinned copy, the event of its pack
    struct Slot {
        float* dev = nullptr;
        size_t devFloats = 0;
        float* host = nullptr;
        size_t hostFloats = 0;
        long long cap = 0;     // fluid2Solid: pairs the slot holds
        long long* devTotal = nullptr;
        long long* hostTotal = nullptr;
        cudaEvent_t packed = nullptr;
        bool busy = false;
    };
    Slot slot[KINDS][SLOTS];
    int next[KINDS] = {0, 0, 0};
    int* pairCount = nullptr;  // fluid2Solid scratch: counts, offsets, scan workspace
    int* pairOffset = nullptr;
    int* scanWork = nullptr;
    // connectivity, offsets and types of the largest frame so far
    std::vector<int> conn, offs;
    std::vector<unsigned char> types;
    cudaStream_t copyStream = nullptr;

    struct Job {
        int kind, s, frame, step;
        double time;
    };
    std::mutex m;
    std::condition_variable cv;
    std::deque<Job> jobs;
    bool stop = false;
    int inFlight = 0;
    std::string error;  // the first error of the writer thread
    std::thread thread;

    void run();
    std::string writeJob(const Job& j);
    void cells(long long n)
    {
        if ((long long)conn.size() >= n) return;
        const size_t old = conn.size();
        conn.resize(n);
        offs.resize(n);
        types.resize(n, 1);  // VTK_VERTEX
        for (size_t i = old; i < (size_t)n; ++i) {
            conn[i] = (int)i;
            offs[i] = (int)i + 1;
        }
    }
};

void demsph_frame_writer::run()
{
    cudaSetDevice(e->device);
    for (;;) {
        Job j;
        {
            std::unique_lock<std::mutex> lk(m);
            cv.wait(lk, [&] { return stop || !jobs.empty(); });
            if (jobs.empty()) return;
            j = jobs.front();
            jobs.pop_front();
        }
        std::string err = writeJob(j);
        {
            std::lock_guard<std::mutex> lk(m);
            if (!err.empty() && error.empty()) error = err;
            slot[j.kind][j.s].busy = false;
            --inFlight;
        }
        cv.notify_all();
    }
}

std::string demsph_frame_writer::writeJob(const Job& j)
{
    Slot& sl = slot[j.kind][j.s];
    cudaError_t c = cudaEventSynchronize(sl.packed);
    if (c != cudaSuccess) return std::string("frame pack: ") + cudaGetErrorString(c);
    long long n = j.kind == 0 ? nf : j.kind == 1 ? ns : 0;
    size_t floats = j.kind == 0 ? 8 * (size_t)nf : 12 * (size_t)ns;
    if (j.kind == 2) {
        c = cudaMemcpyAsync(sl.hostTotal, sl.devTotal, sizeof(long long), cudaMemcpyDeviceToHost, copyStream);
        if (c == cudaSuccess) c = cudaStreamSynchronize(copyStream);
        if (c != cudaSuccess) return std::string("frame copy: ") + cudaGetErrorString(c);
        n = nf > 0 ? std::min(*sl.hostTotal, sl.cap) : 0;
        floats = 6 * (size_t)n;
    }
    if (floats > sl.hostFloats) {
        if (sl.host) cudaFreeHost(sl.host);
        sl.host = nullptr;
        sl.hostFloats = 0;
        c = cudaHostAlloc(reinterpret_cast<void**>(&sl.host), sizeof(float) * floats * 5 / 4 + 16, cudaHostAllocDefault);
        if (c != cudaSuccess) return std::string("frame buffer: ") + cudaGetErrorString(c);
        sl.hostFloats = floats * 5 / 4 + 4;
    }
    if (floats) {
        if (j.kind == 2) {  // midpoints at 0, forces at 3 cap on the device
            c = cudaMemcpyAsync(sl.host, sl.dev, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, copyStream);
            if (c == cudaSuccess)
                c = cudaMemcpyAsync(sl.host + 3 * n, sl.dev + 3 * sl.cap, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost,
                                    copyStream);
        } else {
            c = cudaMemcpyAsync(sl.host, sl.dev, sizeof(float) * floats, cudaMemcpyDeviceToHost, copyStream);
        }
        if (c == cudaSuccess) c = cudaStreamSynchronize(copyStream);
        if (c != cudaSuccess) return std::string("frame copy: ") + cudaGetErrorString(c);
    }
    cells(n);
    const float* h = sl.host;
    const size_t un = (size_t)n;
    const std::vector<Block> cellBlocks = {{"Int32", "connectivity", 1, conn.data(), 4 * un},
                                           {"Int32", "offsets", 1, offs.data(), 4 * un},
                                           {"UInt8", "types", 1, types.data(), un}};
    if (j.kind == 0)  // core/solverBase.cpp:69-170
        return writeVtu(frameName(dir, "fluid", j.frame), j.time, j.step, n, {"Float32", nullptr, 3, h, 12 * un},
                        cellBlocks, "smooth length",
                        {{"Float32", "smooth length", 1, smoothing.data(), 4 * un},
                         {"Float32", "velocity", 3, h + 3 * un, 12 * un},
                         {"Float32", "density", 1, h + 6 * un, 4 * un},
                         {"Float32", "pressure", 1, h + 7 * un, 4 * un}});
    if (j.kind == 1)  // core/solverBase.cpp:172-257
        return writeVtu(frameName(dir, "solid", j.frame), j.time, j.step, n, {"Float32", nullptr, 3, h, 12 * un},
                        cellBlocks, "radius",
                        {{"Float32", "radius", 1, radius.data(), 4 * un},
                         {"Int32", "clusterID", 1, cluster.data(), 4 * un},
                         {"Int32", "clumpID", 1, clump.data(), 4 * un},
                         {"Float32", "velocity", 3, h + 3 * un, 12 * un},
                         {"Float32", "angularVelocity", 3, h + 6 * un, 12 * un},
                         {"Float32", "normal", 3, h + 9 * un, 12 * un}});
    // core/solverBase.cpp:259-333
    return writeVtu(frameName(dir, "fluid2Solid", j.frame), j.time, j.step, n, {"Float32", nullptr, 3, h, 12 * un},
                    cellBlocks, "force", {{"Float32", "force", 3, h + 3 * un, 12 * un}});
}

namespace {

void freeWriter(demsph_frame_writer* w)
{
    {
        std::lock_guard<std::mutex> lk(w->m);
        w->stop = true;
    }
    w->cv.notify_all();
    if (w->thread.joinable()) w->thread.join();
    cudaSetDevice(w->e->device);
    for (auto& kind : w->slot)
        for (auto& s : kind) {
            if (s.dev) cudaFree(s.dev);
            if (s.host) cudaFreeHost(s.host);
            if (s.devTotal) cudaFree(s.devTotal);
            if (s.hostTotal) cudaFreeHost(s.hostTotal);
            if (s.packed) cudaEventDestroy(s.packed);
        }
    if (w->pairCount) cudaFree(w->pairCount);
    if (w->pairOffset) cudaFree(w->pairOffset);
    if (w->scanWork) cudaFree(w->scanWork);
    if (w->copyStream) cudaStreamDestroy(w->copyStream);
    delete w;
}

template <class T>
void devAlloc(T*& p, size_t n)
{
    if (p) CK(cudaFree(p));
    p = nullptr;
    CK(cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * std::max<size_t>(n, 1)));
}

}  // namespace

extern "C" {

int demsph_frame_writer_open(demsph_engine* e, const demsph_scene* scene, const char* dir, demsph_frame_writer** out)
{
    if (!out) return DEMSPH_ERR_ARGUMENT;
    *out = nullptr;
    if (!scene || !dir || !*dir) return DEMSPH_ERR_ARGUMENT;
    ENGINE_GUARD(e)
    if (scene->n_fluid != e->d.nf || scene->n_solid != e->d.ns)
        return fail(e, DEMSPH_ERR_ARGUMENT, "frame writer: the scene's particle counts differ from the engine's");
    std::error_code ec;
    std::filesystem::create_directories(dir, ec);
    if (ec) return fail(e, DEMSPH_ERR_IO, std::string("frame writer: cannot create ") + dir + ": " + ec.message());
    auto* w = new demsph_frame_writer;
    w->e = e;
    w->dir = dir;
    w->nf = e->d.nf;
    w->ns = e->d.ns;
    try {
        w->smoothing.resize(w->nf);
        for (int i = 0; i < w->nf; ++i) w->smoothing[i] = (float)scene->fluid_smoothing_length[i];
        w->radius.resize(w->ns);
        w->cluster.resize(w->ns);
        w->clump.resize(w->ns);
        for (int i = 0; i < w->ns; ++i) {
            w->radius[i] = (float)scene->solid_radius[i];
            w->cluster[i] = scene->solid_cluster ? scene->solid_cluster[i] : -1;
            w->clump[i] = scene->solid_clump ? scene->solid_clump[i] : -1;
        }
        CK(cudaStreamCreateWithFlags(&w->copyStream, cudaStreamNonBlocking));
        for (int k = 0; k < KINDS; ++k)
            for (auto& s : w->slot[k]) {
                CK(cudaEventCreateWithFlags(&s.packed, cudaEventDisableTiming));
                if (k == 0) devAlloc(s.dev, (s.devFloats = 8 * (size_t)w->nf));
                if (k == 1) devAlloc(s.dev, (s.devFloats = 12 * (size_t)w->ns));
                if (k == 2) {
                    devAlloc(s.devTotal, 1);
                    CK(cudaHostAlloc(reinterpret_cast<void**>(&s.hostTotal), sizeof(long long), cudaHostAllocDefault));
                }
            }
        if (w->nf > 0) {
            devAlloc(w->pairCount, w->nf);
            devAlloc(w->pairOffset, w->nf);
            devAlloc(w->scanWork, scanWorkspaceInts(w->nf));
        }
    } catch (const CudaError& c) {
        freeWriter(w);
        return cudaFail(e, c);
    }
    w->thread = std::thread([w] { w->run(); });
    *out = w;
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_frame_writer_write(demsph_frame_writer* w, int what, int frame, int step, double time)
{
    if (!w) return DEMSPH_ERR_ARGUMENT;
    demsph_engine* e = w->e;
    if (what & ~DEMSPH_FRAME_ALL) return fail(e, DEMSPH_ERR_ARGUMENT, "frame writer: unknown frame kinds");
    if (frame < 0) return fail(e, DEMSPH_ERR_ARGUMENT, "frame writer: negative frame number");
    ENGINE_GUARD(e)
    {
        std::lock_guard<std::mutex> lk(w->m);
        if (!w->error.empty()) return fail(e, DEMSPH_ERR_IO, "frame writer: " + w->error);
    }
    DeviceState& d = e->d;
    // the slots and static arrays are sized for the counts at open
    // (demsph_append changes them: open a writer for the new counts)
    if (d.nf != w->nf || d.ns != w->ns)
        return fail(e, DEMSPH_ERR_STATE, "frame writer: the engine's particle counts changed since it was opened");
    for (int k = 0; k < KINDS; ++k) {
        if (!(what & (1 << k))) continue;
        const int si = w->next[k];
        w->next[k] ^= 1;
        auto& sl = w->slot[k][si];
        {
            // the slot's previous frame must be on disk before it is packed again
            std::unique_lock<std::mutex> lk(w->m);
            w->cv.wait(lk, [&] { return !sl.busy; });
        }
        if (k == 0 && d.nf > 0) {
            ++t_kernelLaunches, kFluidFrame<<<blocksFor(d.nf, 256), 256, 0, e->stream>>>(d, sl.dev);
        } else if (k == 1 && d.ns > 0) {
            ++t_kernelLaunches, kSolidFrame<<<blocksFor(d.ns, 256), 256, 0, e->stream>>>(d, sl.dev);
        } else if (k == 2) {
            if (d.nf > 0 && d.ns > 0) {
                const long long cap = (long long)d.kfs * d.nf;
                if (cap > sl.cap) {
                    devAlloc(sl.dev, (sl.devFloats = 6 * (size_t)cap));
                    sl.cap = cap;
                }
                ++t_kernelLaunches, kPairCounts<<<blocksFor(d.nf, 256), 256, 0, e->stream>>>(d, w->pairCount);
                scanExclusive(w->pairCount, w->pairOffset, d.nf, w->scanWork, e->stream);
                ++t_kernelLaunches, kPairFrame<<<blocksFor(d.nf, 128), 128, 0, e->stream>>>(
                    d, w->pairCount, w->pairOffset, sl.dev, sl.cap, sl.devTotal);
            } else {
                CK(cudaMemsetAsync(sl.devTotal, 0, sizeof(long long), e->stream));
            }
        }
        CK(cudaGetLastError());
        CK(cudaEventRecord(sl.packed, e->stream));
        {
            std::lock_guard<std::mutex> lk(w->m);
            sl.busy = true;
            ++w->inFlight;
            w->jobs.push_back({k, si, frame, step, time});
        }
        w->cv.notify_all();
    }
    return DEMSPH_OK;
    ENGINE_END(e)
}

int demsph_frame_writer_flush(demsph_frame_writer* w)
{
    if (!w) return DEMSPH_ERR_ARGUMENT;
    std::unique_lock<std::mutex> lk(w->m);
    w->cv.wait(lk, [&] { return w->inFlight == 0; });
    if (!w->error.empty()) return fail(w->e, DEMSPH_ERR_IO, "frame writer: " + w->error);
    return DEMSPH_OK;
}

int demsph_frame_writer_close(demsph_frame_writer* w)
{
    if (!w) return DEMSPH_ERR_ARGUMENT;
    const int st = demsph_frame_writer_flush(w);
    freeWriter(w);
    return st;
}

}  // extern "C"
