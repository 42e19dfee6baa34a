// Device pieces shared by the channel generators (channel.cu, batch.cu):
// Philox4x32-10 (Salmon et al., SC'11), log / sin / cos from +, -, *, / and
// sqrt only (bit-identical to the CPU oracle), and the staircase encoder.
#pragma once
#include <cuda_runtime.h>

#include "nrldpc_internal.h"

namespace nrldpc {
namespace dev {

__device__ __forceinline__ void philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                           uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int round = 0; round < 10; round++) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c1 = lo1;
        c3 = lo0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// ln(x), x in (0, 1]: x = m 2^e, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(f),
// f = (m-1)/(m+1), odd series to f^11.
__device__ __forceinline__ float log_det(float x) {
    uint32_t u = __float_as_uint(x);
    int e = static_cast<int>((u >> 23) & 0xffu) - 127;
    u = (u & 0x007fffffu) | 0x3f800000u;
    float m = __uint_as_float(u);
    if (m > 1.41421356f) {
        m = __fmul_rn(m, 0.5f);
        e = e + 1;
    }
    const float f = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float f2 = __fmul_rn(f, f);
    float p = __fmul_rn(f2, 1.0f / 11.0f);
    p = __fadd_rn(p, 1.0f / 9.0f);
    p = __fmul_rn(p, f2);
    p = __fadd_rn(p, 1.0f / 7.0f);
    p = __fmul_rn(p, f2);
    p = __fadd_rn(p, 1.0f / 5.0f);
    p = __fmul_rn(p, f2);
    p = __fadd_rn(p, 1.0f / 3.0f);
    p = __fmul_rn(p, f2);
    float lnm = __fmul_rn(p, f);
    lnm = __fadd_rn(lnm, f);
    lnm = __fmul_rn(lnm, 2.0f);
    const float fe = static_cast<float>(e);
    const float hi = __fmul_rn(fe, 0.693145752f);
    const float lo = __fmul_rn(fe, 1.42860677e-06f);
    float r = __fadd_rn(lo, lnm);
    r = __fadd_rn(r, hi);
    return r;
}

// sin, cos of 2 pi u for u in [0, 1): exact quadrant/octant reduction on u,
// Taylor series on |x| <= pi/4.
__device__ __forceinline__ void sincos2pi_det(float u, float* s_out, float* c_out) {
    const int q = static_cast<int>(__fmul_rn(u, 4.0f));
    float r = __fsub_rn(u, __fmul_rn(static_cast<float>(q), 0.25f));
    bool flip = false;
    if (r > 0.125f) {
        r = __fsub_rn(0.25f, r);
        flip = true;
    }
    const float x = __fmul_rn(r, 6.28318548f);
    const float x2 = __fmul_rn(x, x);
    float sp = __fmul_rn(x2, -1.0f / 362880.0f);
    sp = __fadd_rn(sp, 1.0f / 5040.0f);
    sp = __fmul_rn(sp, x2);
    sp = __fsub_rn(sp, 1.0f / 120.0f);
    sp = __fmul_rn(sp, x2);
    sp = __fadd_rn(sp, 1.0f / 6.0f);
    sp = __fmul_rn(sp, x2);
    float sn = __fmul_rn(sp, x);
    sn = __fsub_rn(x, sn);
    float cp = __fmul_rn(x2, 1.0f / 40320.0f);
    cp = __fsub_rn(cp, 1.0f / 720.0f);
    cp = __fmul_rn(cp, x2);
    cp = __fadd_rn(cp, 1.0f / 24.0f);
    cp = __fmul_rn(cp, x2);
    cp = __fsub_rn(cp, 0.5f);
    cp = __fmul_rn(cp, x2);
    const float cs = __fadd_rn(cp, 1.0f);
    const float s0 = flip ? cs : sn, c0 = flip ? sn : cs;
    float s, c;
    switch (q) {
        case 0: s = s0; c = c0; break;
        case 1: s = c0; c = -s0; break;
        case 2: s = -s0; c = -c0; break;
        default: s = -c0; c = s0; break;
    }
    *s_out = s;
    *c_out = c;
}

// Encode the codeword whose kb*Z systematic bits are already in x[] (one
// byte per bit, shared memory); acc[] is Z bytes of scratch.  Plan: first
// parity column from the staircase sum, staircase rows in order, then every
// extension row at once.  Ends with a barrier.
__device__ __forceinline__ void encode_in_smem(const CodeTable& tab, int n_stair, int p0_col,
                                               int p0_shift, int n_steps, const uint8_t* step_row,
                                               const uint8_t* step_col, uint8_t* x, uint8_t* acc) {
    const int z = tab.z;
    for (int k = threadIdx.x; k < z; k += blockDim.x) {
        uint32_t v = 0;
        for (int r = 0; r < n_stair; r++)
            for (int e = tab.row_ptr[r]; e < tab.row_ptr[r + 1]; e++) {
                const int c = tab.edge_col[e];
                if (c >= tab.kb) continue;
                int t = k + tab.edge_shift[e];
                if (t >= z) t -= z;
                v ^= x[c * z + t];
            }
        acc[k] = static_cast<uint8_t>(v);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < z; k += blockDim.x) {
        int t = k - p0_shift;
        if (t < 0) t += z;
        x[p0_col * z + k] = acc[t];
    }
    __syncthreads();
    for (int st = 0; st < n_steps; st++) {
        const int r = step_row[st], u = step_col[st];
        if (r >= n_stair) {  // every remaining step is independent: all at once
            const int n_rest = n_steps - st;
            for (int w = threadIdx.x; w < n_rest * z; w += blockDim.x) {
                const int sr = st + w / z, k = w % z;
                const int rr = step_row[sr], uu = step_col[sr];
                uint32_t v = 0;
                for (int e = tab.row_ptr[rr]; e < tab.row_ptr[rr + 1]; e++) {
                    const int c = tab.edge_col[e];
                    if (c == uu) continue;
                    int t = k + tab.edge_shift[e];
                    if (t >= z) t -= z;
                    v ^= x[c * z + t];
                }
                x[uu * z + k] = static_cast<uint8_t>(v);
            }
            break;
        }
        for (int k = threadIdx.x; k < z; k += blockDim.x) {
            uint32_t v = 0;
            for (int e = tab.row_ptr[r]; e < tab.row_ptr[r + 1]; e++) {
                const int c = tab.edge_col[e];
                if (c == u) continue;
                int t = k + tab.edge_shift[e];
                if (t >= z) t -= z;
                v ^= x[c * z + t];
            }
            x[u * z + k] = static_cast<uint8_t>(v);
        }
        __syncthreads();
    }
    __syncthreads();
}

// Two Gaussians per (u1, u2) pair of Philox words, Box-Muller.
__device__ __forceinline__ void gauss4(const uint32_t o[4], float g[4]) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const float u1 = __fmul_rn(static_cast<float>((o[2 * h] >> 8) + 1u), 5.9604645e-08f);
        const float u2 = __fmul_rn(static_cast<float>(o[2 * h + 1] >> 8), 5.9604645e-08f);
        float l = log_det(u1);
        l = __fmul_rn(l, -2.0f);
        const float rad = __fsqrt_rn(l);
        float sn, cs;
        sincos2pi_det(u2, &sn, &cs);
        g[2 * h] = __fmul_rn(rad, cs);
        g[2 * h + 1] = __fmul_rn(rad, sn);
    }
}

// LLR of BPSK bit `bit` received with noise g * sigma: (2y)/(sigma^2).
__device__ __forceinline__ float bpsk_llr(int bit, float g, float sg, float s2) {
    const float xv = bit ? -1.0f : 1.0f;
    const float y = __fadd_rn(xv, __fmul_rn(g, sg));
    return __fdiv_rn(__fmul_rn(y, 2.0f), s2);
}

}  // namespace dev
}  // namespace nrldpc
