/* Stand-in for the reference's lib/utils/helper_cuda.h in the device-code
 * build of its kernels (oracle/_ref/ref_kernels_bg1.cubin) -- TEST
 * INFRASTRUCTURE ONLY.  The original's host-side device-query helpers use
 * cudaDeviceProp fields CUDA 13 removed; the kernels use none of it, and the
 * host functions compiled beside them need only checkCudaErrors. */
#ifndef REF_GPU_HELPER_CUDA_H
#define REF_GPU_HELPER_CUDA_H
#include <cstdio>
#include <cstdlib>
#define checkCudaErrors(val) (val)
#define getLastCudaError(msg) ((void)0)
#endif
