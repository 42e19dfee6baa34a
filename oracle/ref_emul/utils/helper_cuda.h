/* Stand-in for the reference's lib/utils/helper_cuda.h (CUDA sample header). */
#ifndef REF_EMUL_HELPER_CUDA_H
#define REF_EMUL_HELPER_CUDA_H
#include <cstdio>
#include <cstdlib>
#define checkCudaErrors(val) do { if ((val) != 0) { std::fprintf(stderr, "emulated CUDA call failed\n"); std::abort(); } } while (0)
#endif
