// Internal types shared by the CUDA sources and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/nr_gpu_ldpc_gb300.h"

namespace nrldpc {

constexpr int kMaxRows = 46;    // BG1
constexpr int kMaxCols = 68;    // BG1
constexpr int kMaxEdges = 320;  // BG1 has 316
constexpr int kMaxDeg = 19;     // BG1 rows 0..3
constexpr int kMaxZ = 384;
constexpr int kMaxThreads = 384;  // decode CTA size bound (cw_per_cta * Z)

// Lifted-code description passed to kernels by value (__grid_constant__).
struct alignas(16) CodeTable {
    int rows, cols, z, n_edges, n_bp, packed_bytes;
    int kb;                        // systematic base columns (encoder)
    // Base columns [n_core, cols) are suffix columns: each has degree 1 and is
    // the last edge of its row, and no row has two.  (5G NR: the extension
    // parity columns, 42 of 68 in BG1, 38 of 52 in BG2.)  The decoder keeps
    // their posteriors in the owning row's check-node state instead of in
    // shared memory.
    int n_core;
    int core_floats;               // n_core * Z rounded up to a multiple of 4
    uint16_t row_ptr[kMaxRows + 1];
    uint8_t row_deg[kMaxRows];
    uint8_t sync_after[kMaxRows];  // 1: CTA barrier after this row (row groups
                                   // between barriers share no base column)
    uint8_t row_sfx[kMaxRows];     // 1: the row's last edge is a suffix column
    uint8_t sfx_row[kMaxCols];     // suffix column -> its row
    // per edge, row-major ascending (row, then column) = the reference's
    // h_compact1 order: low 16 bits blk_col*Z + V, high 16 bits Z - V
    uint32_t edge[kMaxEdges];
    // the same edge as byte offset (blk_col*Z + V)*4 into a posterior buffer
    // and wrap threshold Z - V: the sub-row s column is at s*4 + ebase4,
    // minus 4Z when s >= ethr
    uint32_t ebase4[kMaxEdges];
    uint16_t ethr[kMaxEdges];
    uint8_t edge_col[kMaxEdges];
    uint16_t edge_shift[kMaxEdges];  // V mod Z
    // {ebase4, ethr} of each edge in one 64-bit word: one read per edge for
    // the layered decoder and for the mixed-batch kernel, which copies the
    // whole table into shared memory
    uint2 eaddr[kMaxEdges];
};

// Check-node state of one lifted row, kept between iterations (16 B, one
// uint4 per (row, sub-row), [slot][rows][Z]): min1 (raw |Q|), min2,
// info = idx (bits 0..4) | R sign of edge i at bit 8+i, and the posterior of
// the row's suffix column at this sub-row (unused in rows without one).
constexpr size_t kStateBytesPerRow = 16;
// Learned weights of the weighted decoder, passed by value as a kernel
// parameter (constant bank: every lane of a warp reads the same edge's
// weight).  Rows t < n_w_iters hold w[t][e]; row kMaxWIters stays zero (no
// previous message in the first iteration).
constexpr int kMaxWIters = 16;
struct alignas(16) WeightTable {
    float w[kMaxWIters + 1][kMaxEdges];
};
struct NoWeights {
    int unused;
};
struct DecodeArgs {
    const float* llr;
    uint8_t* packed;
    float* app;
    int32_t* iters;
    uint32_t* state;        // [grid * cpb][rows * Z][4]
    int* work_counter;      // dynamic codeword-group scheduler, zeroed per launch
    int* error_flag;        // bounded-wait failures
    int n_cw, n_iter, cpb, n_groups, n_w_iters, early_stop;
    int llr_from_host;      // 1: llr is pinned host memory read over the host link
    float alpha;
    // bounded-wait self-test only (0 in every decode): iterations of the LLR
    // copy wait (0: the default limit), and bytes the copy barrier expects
    // beyond what the copies deliver, so that wait runs out
    int wait_limit;
    uint32_t extra_tx;
};

enum DeviceError : int { kErrNone = 0, kErrLlrLoadTimeout = 1 };

// Mixed-code batches (batch.cu): a work item is up to `count` codewords of
// one code, listed at order[start .. start+count).
struct WorkItem {
    int32_t code;   // index into the table array
    int32_t start;
    int32_t count;
    int32_t spt;    // sub-rows per thread: Z / spt threads per codeword (1 or 2)
};
constexpr size_t kHeaderBytesBatch = 1024;  // mbarrier, item id, per-slot flags
constexpr size_t kBatchTableCopy = (sizeof(CodeTable) + 15) / 16 * 16;
constexpr size_t kBatchTableBytes = (kBatchTableCopy + 127) / 128 * 128;
struct BatchDecodeArgs {
    const CodeTable* tables;
    const WorkItem* items;
    const int32_t* order;       // job indices sorted by code
    const nrldpc_job* jobs;
    const float* llr;
    uint8_t* packed;
    int32_t* iters;
    uint32_t* state;            // [grid][slot_words]
    int* work_counter;
    int* error_flag;
    size_t slot_words;          // state words per CTA (largest cpb * 4 * rows * Z)
    int n_items, n_iter, early_stop;
    float alpha;
};
// Shared memory of one decode group of cpb codewords: Lold and Lnew over the
// core columns, plus one hard-decision byte per lifted row for the suffix
// columns.
inline size_t group_smem_bytes(const CodeTable& t, int cpb) {
    const size_t hd = (static_cast<size_t>(cpb) * t.rows * t.z + 15) / 16 * 16;
    return 2 * static_cast<size_t>(cpb) * t.core_floats * sizeof(float) + hd;
}
cudaError_t launch_batch_decode(const BatchDecodeArgs& args, int grid, int threads, size_t smem,
                                cudaStream_t stream);
const void* batch_decode_kernel_ptr();

// Host-side launchers (decode.cu / channel.cu).
// minb: CTAs per SM the kernel's register budget assumes (1 or 2).
// weights: null for the plain decoder; layered: row-sequential schedule (no
// reference counterpart) instead of flooding.
cudaError_t launch_decode(const CodeTable& tab, const DecodeArgs& args, const WeightTable* weights, int grid,
                          int threads, size_t smem, bool layered, int minb, cudaStream_t stream);
size_t decode_smem_bytes(const CodeTable& tab, int cpb);
cudaError_t decode_kernel_attributes(size_t smem);
int decode_max_ctas_per_sm(bool weighted, int minb, int threads, size_t smem);

// Learned weighted min-sum training kernels (wms.cu).
size_t wms_smem_bytes(const CodeTable& tab, int cpb);
cudaError_t wms_kernel_attributes(size_t smem);
int wms_ctas_per_sm(const CodeTable& tab, int threads, size_t smem);
cudaError_t launch_wms(bool backward, bool layered, const CodeTable& tab, const float* llr, const uint8_t* cw,
                       const float* weights, uint4* states, float* gseed, uint4* gq, float* gh, double* loss,
                       double* grad, float* app, int* counters, int n_cw, int T, int cpb, int grid,
                       int threads, size_t smem, float scale, cudaStream_t stream);
cudaError_t launch_adam(int n, float* w, const double* grad, float* m, float* v, int step, float lr,
                        float b1, float b2, float eps, float w_min, cudaStream_t stream);

// 5G NR (bg, z) code table, built on the caller's storage (no allocation).
bool make_nr_table(int bg, int z, CodeTable* t);

struct EncodePlan {
    int n_core_steps;              // rows solved one parity column at a time
    int core_row[kMaxRows];
    int core_col[kMaxRows];
    int p0_col, p0_shift;          // first parity column = P^{-v} * sum(lambda)
    int n_stair;                   // staircase rows summed for p0
};
bool make_encode_plan(const CodeTable& tab, EncodePlan* plan);
cudaError_t launch_gen_llr(const CodeTable& tab, const EncodePlan& plan, uint64_t seed,
                           uint64_t cw_base, int n_cw, const float* sigma, int n_punct_cols,
                           float* llr, uint8_t* cw_packed, cudaStream_t stream);
cudaError_t launch_dequant(const void* in, int qtype, float scale, size_t n, float* out,
                           cudaStream_t stream);
cudaError_t launch_crc(const uint8_t* packed, int n_cw, int stride, int n_bits, uint32_t poly, int len,
                       uint32_t* rem, cudaStream_t stream);
// Code-block segmentation (channel.cu): bit gathers between a transport
// block and C code blocks of k_prime bits (data_bits = k_prime - L each), and
// CRC attachment of the last L bits of each block.
cudaError_t launch_cb_gather_blocks(const uint8_t* tb, int C, int data_bits, int k_prime, uint8_t* blocks,
                                    int stride, cudaStream_t stream);
cudaError_t launch_cb_attach_crc(uint8_t* blocks, int C, int data_bits, int stride, uint32_t poly, int len,
                                 cudaStream_t stream);
cudaError_t launch_cb_gather_tb(const uint8_t* blocks, int stride, int C, int data_bits, uint8_t* tb,
                                cudaStream_t stream);
cudaError_t launch_count_errors(const uint8_t* packed, const uint8_t* cw_packed, int n_cw,
                                int packed_bytes, int n_info, unsigned long long* counts,
                                cudaStream_t stream);

}  // namespace nrldpc
