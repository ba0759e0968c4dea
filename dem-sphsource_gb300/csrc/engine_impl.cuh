// Host-side engine object shared by engine.cu (life cycle, step schedule,
// batching) and engine_io.cu (state transfer, setters, artefact export).
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "../../include/demsph_gb300.h"

namespace demsph {

enum SolidFlagBits { F_DUMMY = 1, F_FIXED = 2, F_MASSIVE = 4, F_HASMASS = 8 };

struct CudaError {
    cudaError_t e;
    const char* what;
};

#define CK(call)                                           \
    do {                                                   \
        cudaError_t _e = (call);                           \
        if (_e != cudaSuccess) throw demsph::CudaError{_e, #call}; \
    } while (0)

template <class T>
inline T* dalloc(size_t n, std::vector<void*>& owned, bool zero = true)
{
    T* p = nullptr;
    if (n == 0) n = 1;
    CK(cudaMalloc(&p, sizeof(T) * n));
    if (zero) CK(cudaMemset(p, 0, sizeof(T) * n));
    owned.push_back(p);
    return p;
}

}  // namespace demsph

struct demsph_engine {
    demsph::DeviceState d{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> owned;     // every cudaMalloc'd buffer
    std::string err;
    int par = 1;                  // parity of the last successful solid list build
    bool forceWalk = false;       // next contact list from the reference's 27-cell walk
    bool walkOrder[2] = {true, true};  // list of each parity is in the reference's walk order
    bool initialized = false;
    int debug = 0;
    double hmax = 0;              // largest fluid smoothing length
    int nMassive = 0;
    // CUDA graph of one period of steps
    cudaGraphExec_t graph = nullptr;
    int graphPeriod = 0, graphGap = 0, graphParity = -1;
    double graphDt = 0;
    // contact tables as uploaded (FP32)
    std::vector<float> hzF, lnF, bdF, dampF;
    // kernel launch accounting (demsph_kernel_launches)
    long long launchBase = 0;        // t_kernelLaunches when the engine was created
    long long capturedLaunches = 0;  // launch calls recorded into graphs (not executed then)
    long long replayedKernels = 0;   // kernels executed by graph replays
    long long graphKernels = 0;      // kernels in the current graph
    // stage timing (demsph_set_profiling)
    bool profiling = false;
    struct Timed {
        const char* tag;
        cudaEvent_t a, b;
    };
    std::vector<Timed> timed;
    // scratch for downloads (device, grown on demand)
    double* dscratch = nullptr;
    size_t dscratchN = 0;

    ~demsph_engine()
    {
        for (auto& t : timed) {
            cudaEventDestroy(t.a);
            cudaEventDestroy(t.b);
        }
        if (graph) cudaGraphExecDestroy(graph);
        for (void* p : owned) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace demsph {

inline int fail(demsph_engine* e, int code, const std::string& msg)
{
    if (e) e->err = msg;
    return code;
}

inline int cudaFail(demsph_engine* e, const CudaError& c)
{
    return fail(e, c.e == cudaErrorMemoryAllocation ? DEMSPH_ERR_OUT_OF_MEMORY : DEMSPH_ERR_CUDA,
                std::string(c.what) + ": " + cudaGetErrorString(c.e));
}

void freeOne(demsph_engine* e, void*& p);
void dropGraph(demsph_engine* e);
int readStatus(demsph_engine* e, int* stepsDone = nullptr);
double* scratchDoubles(demsph_engine* e, size_t n);
void splitPosition(const DeviceState& d, double3 p, int4& c, float4& h, float4& l);

}  // namespace demsph

#define ENGINE_GUARD(e)                                   \
    if (!(e) || !(e)->stream) return DEMSPH_ERR_ARGUMENT; \
    try {                                                 \
        CK(cudaSetDevice((e)->device));

#define ENGINE_END(e)                   \
    }                                   \
    catch (const demsph::CudaError& c)  \
    {                                   \
        return demsph::cudaFail((e), c); \
    }
