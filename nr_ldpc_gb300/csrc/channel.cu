// Seeded channel simulation on the GPU: info bits, structural QC encoder,
// BPSK, AWGN and LLRs, plus an info-bit error counter.
//
// No reference counterpart on the GPU: the reference builds its inputs on the
// host (src/encoding_tools.cpp:13-99 with the OAI encoder).  This generator
// keeps the reference's signal model -- BPSK 0 -> +1, y = x + noise*sigma
// (src/encoding_tools.cpp:62), LLR = (2y)/(sigma*sigma) with the first 2Z
// columns punctured to 0 (src/encoding_tools.cpp:85-99) -- and draws its
// randomness from Philox4x32-10 (Salmon et al., SC'11) keyed by
// (seed, codeword id), with Gaussians by Box-Muller using log / sin / cos
// evaluated from +, -, *, / and sqrt only.  Every float operation is an
// explicit round-to-nearest intrinsic in the same order as the CPU oracle's
// C code, so both produce the same bits.
#include <cuda_runtime.h>

#include <vector>

#include "nrldpc_internal.h"

namespace nrldpc {
namespace {

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

struct GenArgs {
    uint64_t seed, cw_base;
    const float* sigma;
    float* llr;
    uint8_t* cw_packed;
    int n_cw, n_punct_cols;
    int n_stair, p0_col, p0_shift, n_core_steps;
    uint8_t step_row[kMaxRows];
    uint8_t step_col[kMaxRows];
};

// One CTA per codeword (grid-stride over codewords).
__global__ void __launch_bounds__(256) gen_llr_kernel(const __grid_constant__ CodeTable tab,
                                                      const __grid_constant__ GenArgs g) {
    extern __shared__ uint8_t x[];  // [n_bp] codeword bits, then [z] scratch
    const int z = tab.z, n = tab.n_bp, K = tab.kb * z;
    uint8_t* acc = x + n;
    const uint32_t k0 = static_cast<uint32_t>(g.seed), k1 = static_cast<uint32_t>(g.seed >> 32);
    for (int i = blockIdx.x; i < g.n_cw; i += gridDim.x) {
        const uint64_t id = g.cw_base + static_cast<uint64_t>(i);
        const uint32_t id0 = static_cast<uint32_t>(id), id1 = static_cast<uint32_t>(id >> 32);
        // info bits: block b holds bits 128b .. 128b+127
        for (int b = threadIdx.x; b * 128 < K; b += blockDim.x) {
            uint32_t o[4];
            philox4x32(static_cast<uint32_t>(b), id0, id1, 1u, k0, k1, o);
            for (int j = 0; j < 128 && b * 128 + j < K; j++) x[b * 128 + j] = (o[j >> 5] >> (j & 31)) & 1u;
        }
        __syncthreads();
        // first parity column: P^{-v} * XOR of the staircase rows' systematic parts
        for (int k = threadIdx.x; k < z; k += blockDim.x) {
            uint32_t v = 0;
            for (int r = 0; r < g.n_stair; r++)
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
            int t = k - g.p0_shift;
            if (t < 0) t += z;
            x[g.p0_col * z + k] = acc[t];
        }
        __syncthreads();
        // remaining parity columns; staircase steps in order, the rest at once
        for (int st = 0; st < g.n_core_steps; st++) {
            const int r = g.step_row[st], u = g.step_col[st];
            if (r >= g.n_stair) {
                // every remaining step is independent: do them all, then leave
                const int n_rest = g.n_core_steps - st;
                for (int w = threadIdx.x; w < n_rest * z; w += blockDim.x) {
                    const int sr = st + w / z, k = w % z;
                    const int rr = g.step_row[sr], uu = g.step_col[sr];
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
        if (g.cw_packed) {
            uint8_t* out = g.cw_packed + static_cast<size_t>(i) * tab.packed_bytes;
            for (int b = threadIdx.x; b < tab.packed_bytes; b += blockDim.x) {
                uint32_t v = 0;
                for (int j = 0; j < 8; j++)
                    if (8 * b + j < n) v |= static_cast<uint32_t>(x[8 * b + j]) << j;
                out[b] = static_cast<uint8_t>(v);
            }
        }
        const float sg = g.sigma[i];
        const float s2 = __fmul_rn(sg, sg);
        const int p0 = g.n_punct_cols * z;
        float* out = g.llr + static_cast<size_t>(i) * n;
        for (int j = threadIdx.x; j < p0; j += blockDim.x) out[j] = 0.0f;
        const int n_blk = (n - p0 + 3) / 4;
        for (int t = threadIdx.x; t < n_blk; t += blockDim.x) {
            uint32_t o[4];
            philox4x32(static_cast<uint32_t>(t), id0, id1, 2u, k0, k1, o);
            float gs[4];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float u1 = __fmul_rn(static_cast<float>((o[2 * h] >> 8) + 1u), 5.9604645e-08f);
                const float u2 = __fmul_rn(static_cast<float>(o[2 * h + 1] >> 8), 5.9604645e-08f);
                float l = log_det(u1);
                l = __fmul_rn(l, -2.0f);
                const float rad = __fsqrt_rn(l);
                float sn, cs;
                sincos2pi_det(u2, &sn, &cs);
                gs[2 * h] = __fmul_rn(rad, cs);
                gs[2 * h + 1] = __fmul_rn(rad, sn);
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int j = p0 + 4 * t + k;
                if (j >= n) break;
                const float xv = x[j] ? -1.0f : 1.0f;
                const float ns = __fmul_rn(gs[k], sg);
                const float y = __fadd_rn(xv, ns);
                const float y2 = __fmul_rn(y, 2.0f);
                out[j] = __fdiv_rn(y2, s2);
            }
        }
        __syncthreads();  // x is rewritten for the next codeword
    }
}

__global__ void __launch_bounds__(256) count_errors_kernel(const uint8_t* __restrict__ packed,
                                                           const uint8_t* __restrict__ cw,
                                                           int n_cw, int packed_bytes, int n_info,
                                                           unsigned long long* counts) {
    __shared__ unsigned int warp_sum[8];
    for (int i = blockIdx.x; i < n_cw; i += gridDim.x) {
        const uint8_t* a = packed + static_cast<size_t>(i) * packed_bytes;
        const uint8_t* b = cw + static_cast<size_t>(i) * packed_bytes;
        unsigned int errs = 0;
        const int full = n_info / 8, rem = n_info % 8;
        for (int k = threadIdx.x; k < full; k += blockDim.x) errs += __popc(a[k] ^ b[k]);
        if (rem && threadIdx.x == 0) errs += __popc((a[full] ^ b[full]) & ((1u << rem) - 1u));
        for (int off = 16; off > 0; off >>= 1) errs += __shfl_down_sync(0xffffffffu, errs, off);
        if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = errs;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int tot = 0;
            for (int w = 0; w < (blockDim.x + 31) / 32; w++) tot += warp_sum[w];
            if (tot) {
                atomicAdd(&counts[0], static_cast<unsigned long long>(tot));
                atomicAdd(&counts[1], 1ull);
            }
        }
        __syncthreads();
    }
}

}  // namespace

// Staircase encoding plan (host): see the oracle's structural encoder.
bool make_encode_plan(const CodeTable& tab, EncodePlan* plan) {
    const int z = tab.z, kb = tab.kb;
    std::vector<int> col_deg(tab.cols, 0);
    for (int e = 0; e < tab.n_edges; e++) col_deg[tab.edge_col[e]]++;
    int m = 0;
    for (int r = 0; r < tab.rows; r++) {
        const int last = tab.edge_col[tab.row_ptr[r + 1] - 1];
        if (col_deg[last] == 1 && r > 0) break;
        m = r + 1;
    }
    std::vector<int> cnt(z, 0);
    for (int r = 0; r < m; r++)
        for (int e = tab.row_ptr[r]; e < tab.row_ptr[r + 1]; e++)
            if (tab.edge_col[e] == kb) cnt[tab.edge_shift[e]]++;
    int v_odd = -1;
    for (int v = 0; v < z; v++)
        if (cnt[v] & 1) {
            if (v_odd >= 0) return false;
            v_odd = v;
        }
    if (v_odd < 0) return false;
    std::vector<int> solved(tab.cols, 0);
    for (int j = 0; j <= kb && j < tab.cols; j++) solved[j] = 1;
    int n = 0;
    for (int r = 0; r < tab.rows; r++) {
        if (r == m - 1) continue;
        int unknown = -1;
        for (int e = tab.row_ptr[r]; e < tab.row_ptr[r + 1]; e++) {
            const int j = tab.edge_col[e];
            if (solved[j]) continue;
            if (unknown < 0 && tab.edge_shift[e] == 0) unknown = j;
            else return false;
        }
        if (unknown < 0) continue;
        solved[unknown] = 1;
        plan->core_row[n] = r;
        plan->core_col[n] = unknown;
        n++;
    }
    for (int j = 0; j < tab.cols; j++)
        if (!solved[j]) return false;
    plan->n_core_steps = n;
    plan->p0_col = kb;
    plan->p0_shift = v_odd;
    plan->n_stair = m;
    return true;
}

cudaError_t launch_gen_llr(const CodeTable& tab, const EncodePlan& plan, uint64_t seed,
                           uint64_t cw_base, int n_cw, const float* sigma, int n_punct_cols,
                           float* llr, uint8_t* cw_packed, cudaStream_t stream) {
    GenArgs g{};
    g.seed = seed;
    g.cw_base = cw_base;
    g.sigma = sigma;
    g.llr = llr;
    g.cw_packed = cw_packed;
    g.n_cw = n_cw;
    g.n_punct_cols = n_punct_cols;
    g.n_stair = plan.n_stair;
    g.p0_col = plan.p0_col;
    g.p0_shift = plan.p0_shift;
    g.n_core_steps = plan.n_core_steps;
    for (int k = 0; k < plan.n_core_steps; k++) {
        g.step_row[k] = static_cast<uint8_t>(plan.core_row[k]);
        g.step_col[k] = static_cast<uint8_t>(plan.core_col[k]);
    }
    const int grid = n_cw < 4096 ? n_cw : 4096;
    const size_t smem = static_cast<size_t>(tab.n_bp) + tab.z;
    gen_llr_kernel<<<grid, 256, smem, stream>>>(tab, g);
    return cudaGetLastError();
}

cudaError_t launch_count_errors(const uint8_t* packed, const uint8_t* cw_packed, int n_cw,
                                int packed_bytes, int n_info, unsigned long long* counts,
                                cudaStream_t stream) {
    const int grid = n_cw < 4096 ? n_cw : 4096;
    count_errors_kernel<<<grid, 256, 0, stream>>>(packed, cw_packed, n_cw, packed_bytes, n_info,
                                                  counts);
    return cudaGetLastError();
}

}  // namespace nrldpc
