/*
 * Host stand-in for <cuda_runtime.h>, used ONLY by oracle/ref_harness.cpp to
 * compile the reference's kernel templates as ordinary host C++ (test
 * infrastructure; never part of the product).  Device memory is host memory,
 * a "launch" is a loop over (block, thread) with the built-in indices set,
 * and atomics are plain read-modify-writes (the harness is single-threaded).
 */
#ifndef PCS_REF_SHIM_CUDA_RUNTIME_H
#define PCS_REF_SHIM_CUDA_RUNTIME_H

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
typedef struct pcs_shim_stream* cudaStream_t;
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};

struct uint3 { unsigned x, y, z; };
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

template <typename T>
inline cudaError_t cudaMalloc(T** p, std::size_t n)
{
    *p = static_cast<T*>(std::calloc(n ? n : 1, 1));
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, std::size_t n, cudaMemcpyKind)
{
    std::memcpy(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, std::size_t n, cudaMemcpyKind k,
                                   cudaStream_t = nullptr)
{
    return cudaMemcpy(d, s, n, k);
}
inline cudaError_t cudaMemset(void* d, int v, std::size_t n) { std::memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaMemsetAsync(void* d, int v, std::size_t n, cudaStream_t = nullptr)
{
    return cudaMemset(d, v, n);
}
inline const char* cudaGetErrorString(cudaError_t) { return "host shim error"; }
inline const char* cudaGetErrorName(cudaError_t) { return "cudaErrorHostShim"; }

inline unsigned atomicInc(unsigned* a, unsigned limit)
{
    unsigned old = *a;
    *a = (old >= limit) ? 0u : old + 1u;
    return old;
}

/* Only referenced by the unrolled kernel, which the harness never runs. */
inline float __logf(float x) { return std::log(x); }
inline float __sinf(float x) { return std::sin(x); }
inline void __sincosf(float x, float* s, float* c) { *s = std::sin(x); *c = std::cos(x); }
inline void sincos(double x, double* s, double* c) { *s = std::sin(x); *c = std::cos(x); }

#endif
