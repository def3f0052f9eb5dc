// af_emu.h -- host execution of CUDA kernel sources for the oracle pins (test build only).
//
// Compiles the reference's .cu kernels as plain C++: kernel qualifiers become nothing,
// threadIdx/blockIdx/blockDim/gridDim are per-emulated-thread globals, "device" memory is host
// memory, atomics are plain read-modify-writes (emulated threads never run concurrently), and
// a launch runs every thread of every block in order.  Kernels that call __syncthreads run each
// block's threads as cooperative fibers (ucontext) that switch at every barrier.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__
#define __shared__
#define __restrict__

struct uint3 {
    unsigned x, y, z;
};
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

enum cudaError_t { cudaSuccess = 0, cudaErrorUnknown = 999 };
typedef cudaError_t cudaError;
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};

inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t) { return "emulated"; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t n) {
    *p = static_cast<T*>(std::malloc(n ? n : 1));
    return cudaSuccess;
}
inline cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    std::memmove(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void* d, int v, size_t n) {
    std::memset(d, v, n);
    return cudaSuccess;
}
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n, size_t off = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice) {
    std::memcpy(reinterpret_cast<char*>(&sym) + off, src, n);
    return cudaSuccess;
}

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

template <class T>
inline T atomicAdd(T* p, T v) {
    T old = *p;
    *p = old + v;
    return old;
}
inline unsigned atomicAdd(unsigned* p, int v) { return atomicAdd<unsigned>(p, (unsigned)v); }

void __syncthreads();

namespace af_emu {
void launch(dim3 grid, dim3 block, size_t smem, const std::function<void()>& body);
void launch_sync(dim3 grid, dim3 block, size_t smem, const std::function<void()>& body);
void* dynamic_smem();
}  // namespace af_emu

// the reference's device code calls these unqualified, as CUDA's headers allow
using std::abs;
using std::isinf;
using std::isnan;
using std::pow;
