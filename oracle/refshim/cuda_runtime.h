// CPU launch shim: the subset of the CUDA runtime the reference's code calls,
// implemented on host memory, plus a sequential kernel-launch emulator.
//
// Purpose: compile the reference's own kernels (core/neighborSearch.cu,
// core/integrate.cu) and host classes (core/dataBase.cpp, core/solverBase.cpp)
// as ordinary C++ so that the reference itself can be run on a machine without
// a GPU, to pin the project's FP64 oracle.  This is test infrastructure: it is
// compiled only by oracle/build_ref.sh into oracle/_ref/ and is never part of
// the product.
#pragma once
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <utility>
#include "vector_types.h"
#include "vector_functions.h"

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};

// "Device" memory is plain host memory; every allocation is a malloc.
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t bytes)
{
    *p = static_cast<T*>(std::malloc(bytes ? bytes : 1));
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t bytes, cudaMemcpyKind)
{
    if (bytes) std::memmove(d, s, bytes);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void* p, int v, size_t bytes)
{
    if (bytes) std::memset(p, v, bytes);
    return cudaSuccess;
}
inline const char* cudaGetErrorString(cudaError_t) { return "cpu launch shim error"; }
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

// Built-in index variables: the emulator sets them before running each thread.
inline uint3 threadIdx;
inline uint3 blockIdx;
inline dim3 blockDim;
inline dim3 gridDim;

template <class T>
inline T atomicAdd(T* a, T v)
{
    T old = *a;
    *a = old + v;
    return old;
}

namespace refshim {

// A hook sees a launch's argument tuple before the first thread (phase 0),
// after every thread (phase 1, with that thread's global index) and after the
// last thread (phase 2).  It is keyed by the kernel's address.
using Hook = void (*)(void* argTuple, int phase, long long globalThread);

inline std::map<const void*, Hook>& hooks()
{
    static std::map<const void*, Hook> m;
    return m;
}

// Runs every thread of a 1-D launch in order: block 0 thread 0, thread 1, ...
template <class... P>
struct Launch {
    void (*kernel)(P...);
    unsigned grid, block;

    template <class... A>
    void operator()(A&&... a) const
    {
        std::tuple<P...> args(std::forward<A>(a)...);
        auto it = hooks().find(reinterpret_cast<const void*>(kernel));
        Hook h = it == hooks().end() ? nullptr : it->second;
        if (h) h(&args, 0, -1);
        gridDim = dim3(grid);
        blockDim = dim3(block);
        for (unsigned b = 0; b < grid; ++b) {
            for (unsigned t = 0; t < block; ++t) {
                blockIdx.x = b; blockIdx.y = 0; blockIdx.z = 0;
                threadIdx.x = t; threadIdx.y = 0; threadIdx.z = 0;
                std::apply(kernel, args);
                if (h) h(&args, 1, (long long)b * block + t);
            }
        }
        if (h) h(&args, 2, -1);
    }
};

template <class... P>
inline Launch<P...> launch(int grid, int block, void (*k)(P...))
{
    return Launch<P...>{k, (unsigned)grid, (unsigned)block};
}

}  // namespace refshim
