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
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <vector>

#include "channel_dev.cuh"
#include "nrldpc_internal.h"

namespace nrldpc {
namespace {
using namespace dev;

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
        encode_in_smem(tab, g.n_stair, g.p0_col, g.p0_shift, g.n_core_steps, g.step_row, g.step_col, x,
                       acc);
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
            gauss4(o, gs);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int j = p0 + 4 * t + k;
                if (j >= n) break;
                out[j] = bpsk_llr(x[j], gs[k], sg, s2);
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

// CRC of the first n_bits of each packed codeword, MSB-first long division
// (bit i of the packed bytes = coefficient of D^(n-1-i)), byte-wise with a
// 256-entry table built per CTA in shared memory.  One thread per codeword.
__global__ void __launch_bounds__(256) crc_kernel(const uint8_t* __restrict__ packed, int n_cw,
                                                  int stride, int n_bits, uint32_t poly, int len,
                                                  uint32_t* __restrict__ rem) {
    __shared__ uint32_t table[256];
    const uint32_t mask = (len >= 32) ? 0xffffffffu : ((1u << len) - 1u), top = 1u << (len - 1);
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        uint32_t r = static_cast<uint32_t>(i) << (len - 8);
        for (int k = 0; k < 8; k++) r = ((r & top) ? ((r << 1) ^ poly) : (r << 1)) & mask;
        table[i] = r;
    }
    __syncthreads();
    const int cw = blockIdx.x * blockDim.x + threadIdx.x;
    if (cw >= n_cw) return;
    const uint8_t* p = packed + static_cast<size_t>(cw) * stride;
    uint32_t r = 0;
    const int nb = n_bits / 8;
    for (int b = 0; b < nb; b++) {
        const uint32_t v = __brev(static_cast<uint32_t>(p[b])) >> 24;  // first bit -> MSB
        r = ((r << 8) ^ table[((r >> (len - 8)) ^ v) & 0xffu]) & mask;
    }
    for (int i = nb * 8; i < n_bits; i++) {
        const uint32_t fb = ((r & top) != 0) ^ ((p[i >> 3] >> (i & 7)) & 1u);
        r = (r << 1) & mask;
        if (fb) r ^= poly;
    }
    rem[cw] = r;
}

// Widen transferred LLRs to fp32: qtype 1 = IEEE half (exact), 2 = int8
// times `scale` (one rounding, the product).
__global__ void __launch_bounds__(256) dequant_kernel(const void* __restrict__ in, int qtype,
                                                      float scale, size_t n, float* __restrict__ out) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        if (qtype == 1)
            out[i] = __half2float(__ushort_as_half(static_cast<const unsigned short*>(in)[i]));
        else
            out[i] = __fmul_rn(static_cast<float>(static_cast<const int8_t*>(in)[i]), scale);
    }
}

}  // namespace

cudaError_t launch_dequant(const void* in, int qtype, float scale, size_t n, float* out,
                           cudaStream_t stream) {
    const size_t blocks = (n + 255) / 256;
    dequant_kernel<<<static_cast<unsigned>(blocks < 4096 ? blocks : 4096), 256, 0, stream>>>(in, qtype, scale,
                                                                                             n, out);
    return cudaGetLastError();
}

// ---- code-block segmentation (TS 38.212 5.2.2) ------------------------------------
// One thread per output byte: block r's byte j holds bits 8j..8j+7 of its
// data, which are transport-block bits r*data_bits + 8j + i (bits at or past
// data_bits are left zero for the CRC and the padding).
__global__ void __launch_bounds__(256) cb_gather_blocks_kernel(const uint8_t* __restrict__ tb, int C,
                                                               int data_bits, int k_prime,
                                                               uint8_t* __restrict__ blocks, int stride) {
    const int nbytes = (k_prime + 7) / 8;
    const long idx = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
    if (idx >= static_cast<long>(C) * nbytes) return;
    const int r = static_cast<int>(idx / nbytes), j = static_cast<int>(idx - static_cast<long>(r) * nbytes);
    uint32_t v = 0;
    for (int i = 0; i < 8; i++) {
        const int k = 8 * j + i;
        if (k < data_bits) {
            const long t = static_cast<long>(r) * data_bits + k;
            v |= ((tb[t >> 3] >> (t & 7)) & 1u) << i;
        }
    }
    blocks[static_cast<size_t>(r) * stride + j] = static_cast<uint8_t>(v);
}

// One thread per block: CRC of the data bits, appended MSB first (parity bit
// p_0 = remainder bit len-1), so the block's remainder over all its bits is 0.
__global__ void __launch_bounds__(128) cb_attach_crc_kernel(uint8_t* __restrict__ blocks, int C, int data_bits,
                                                            int stride, uint32_t poly, int len) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= C) return;
    uint8_t* p = blocks + static_cast<size_t>(r) * stride;
    const uint32_t mask = (len >= 32) ? 0xffffffffu : ((1u << len) - 1u), top = 1u << (len - 1);
    uint32_t rem = 0;
    for (int i = 0; i < data_bits; i++) {
        const uint32_t fb = ((rem & top) != 0) ^ ((p[i >> 3] >> (i & 7)) & 1u);
        rem = (rem << 1) & mask;
        if (fb) rem ^= poly;
    }
    for (int i = 0; i < len; i++) {
        const int k = data_bits + i;
        const uint32_t bit = (rem >> (len - 1 - i)) & 1u;
        p[k >> 3] = static_cast<uint8_t>((p[k >> 3] & ~(1u << (k & 7))) | (bit << (k & 7)));
    }
}

// One thread per transport-block byte: bit t comes from block t / data_bits.
__global__ void __launch_bounds__(256) cb_gather_tb_kernel(const uint8_t* __restrict__ blocks, int stride, int C,
                                                           int data_bits, uint8_t* __restrict__ tb) {
    const long total = static_cast<long>(C) * data_bits;
    const long j = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
    if (j >= (total + 7) / 8) return;
    uint32_t v = 0;
    for (int i = 0; i < 8; i++) {
        const long t = 8 * j + i;
        if (t < total) {
            const int r = static_cast<int>(t / data_bits), k = static_cast<int>(t - static_cast<long>(r) * data_bits);
            v |= ((blocks[static_cast<size_t>(r) * stride + (k >> 3)] >> (k & 7)) & 1u) << i;
        }
    }
    tb[j] = static_cast<uint8_t>(v);
}

cudaError_t launch_crc(const uint8_t* packed, int n_cw, int stride, int n_bits, uint32_t poly, int len,
                       uint32_t* rem, cudaStream_t stream) {
    crc_kernel<<<(n_cw + 255) / 256, 256, 0, stream>>>(packed, n_cw, stride, n_bits, poly, len, rem);
    return cudaGetLastError();
}

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

namespace nrldpc {
cudaError_t launch_cb_gather_blocks(const uint8_t* tb, int C, int data_bits, int k_prime, uint8_t* blocks,
                                    int stride, cudaStream_t stream) {
    const long n = static_cast<long>(C) * ((k_prime + 7) / 8);
    cb_gather_blocks_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(tb, C, data_bits, k_prime,
                                                                                         blocks, stride);
    return cudaGetLastError();
}
cudaError_t launch_cb_attach_crc(uint8_t* blocks, int C, int data_bits, int stride, uint32_t poly, int len,
                                 cudaStream_t stream) {
    cb_attach_crc_kernel<<<(C + 127) / 128, 128, 0, stream>>>(blocks, C, data_bits, stride, poly, len);
    return cudaGetLastError();
}
cudaError_t launch_cb_gather_tb(const uint8_t* blocks, int stride, int C, int data_bits, uint8_t* tb,
                                cudaStream_t stream) {
    const long n = (static_cast<long>(C) * data_bits + 7) / 8;
    cb_gather_tb_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(blocks, stride, C, data_bits, tb);
    return cudaGetLastError();
}
}  // namespace nrldpc
