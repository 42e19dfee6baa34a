/* CUDA stand-in for compiling the reference's kernel sources as host C++.
 * Test infrastructure only (oracle/_ref).  Kernels become plain functions;
 * launches are replayed block by block, thread by thread, by ref_harness.cpp.
 * Exact for the reference's kernels: none uses __syncthreads, atomics or
 * another thread's shared-memory slots. */
#ifndef REF_EMUL_CUDA_RUNTIME_H
#define REF_EMUL_CUDA_RUNTIME_H
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
#define __forceinline__ inline

struct uint3 { unsigned int x, y, z; };
struct dim3 {
    unsigned int x, y, z;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

typedef int cudaError_t;
static const cudaError_t cudaSuccess = 0;
typedef void* cudaStream_t;
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& symbol, const void* src, size_t n) {
    std::memcpy((void*)&symbol, src, n);
    return cudaSuccess;
}
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
#endif
