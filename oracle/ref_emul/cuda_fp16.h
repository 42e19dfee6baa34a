/* fp16 stand-in: the reference's float build never converts through these. */
#ifndef REF_EMUL_CUDA_FP16_H
#define REF_EMUL_CUDA_FP16_H
struct half { unsigned short bits; };
inline half __float2half_rn(float) { std::abort(); }
inline half __float2half(float) { std::abort(); }
inline float __half2float(half) { std::abort(); }
#endif
