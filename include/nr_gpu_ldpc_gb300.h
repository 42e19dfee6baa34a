/*
 * nr_gpu_ldpc_gb300 -- GB300 (sm_103a) 5G NR / QC-LDPC normalized min-sum decoder.
 *
 * C ABI: plain pointers and sizes, no C++ or framework types.  Every entry
 * point returns an nrldpc_status (0 = OK, negative = error) and never exits
 * the process.  Calls taking a cudaStream_t are stream-ordered and
 * asynchronous unless documented otherwise; the caller synchronizes.
 *
 * Reference interfaces replaced (ctarver/NR_GPU_LDPC):
 *   nrldpc_setup_ldpc      <- ldpc_params setup_ldpc(int, float, int)       src/nr_ldpc.h:14,
 *                                                                           src/nr_ldpc.cpp:31-230
 *   nrldpc_init            <- setup_dev_memory + setup_gpu_grid +
 *                             put_h_compact_and_params_in_constant_memory   src/setup_exp.h:16-30,
 *                                                                           src/setup_exp.cu:102-166,286-313
 *   nrldpc_destroy         <- (none: the reference never frees its device memory)
 *   nrldpc_decode          <- perform_gpu_ldpc_decoding<T>, decode part     src/gpu_decoder_top.h:13-18,
 *                             (device LLR in, device packed bits out)       src/gpu_decoder_top.cu:25-49
 *   nrldpc_decode_host_async <- perform_gpu_ldpc_decoding<T>, whole call:   src/gpu_decoder_top.cu:16-52
 *                             H2D of the LLR batch, decode, D2H of packed
 *                             hard decisions, all queued on one stream
 *                             (src/cuda_gpu_wrapper/gpu_setup.cu:75-97)
 *
 * Data formats (identical to the reference where it defines them):
 *   LLR      fp32 [n_cw][cols*Z], codeword-bit order, positive = bit 0; the
 *            punctured first 2Z columns carry LLR 0 (src/encoding_tools.cpp:85-99).
 *   packed   uint8 [n_cw][ceil(cols*Z/8)]: bit i of byte b is the hard
 *            decision of column 8b+i (1 when the posterior is not > 0),
 *            src/ldpc_kernels.cu:463-467,482-500, src/host_helpers.cpp:60-64.
 *            For Z % 8 == 0 this is byte-identical to the reference stream.
 */
#ifndef NR_GPU_LDPC_GB300_H
#define NR_GPU_LDPC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* nrldpc_stream_t; /* same object as cudaStream_t */
typedef struct nrldpc_handle nrldpc_handle;

typedef enum {
    NRLDPC_OK = 0,
    NRLDPC_ERR_INVALID_ARG = -1,   /* null pointer, negative count, bad option */
    NRLDPC_ERR_BAD_CONFIG = -2,    /* unsupported base graph / lifting size */
    NRLDPC_ERR_CUDA = -3,          /* a CUDA runtime call or launch failed */
    NRLDPC_ERR_ALIGNMENT = -4,     /* device LLR pointer not 16-byte aligned */
    NRLDPC_ERR_TOO_LARGE = -5,     /* batch beyond the handle's max_batch */
    NRLDPC_ERR_TIMEOUT = -6,       /* a bounded device-side wait expired */
    NRLDPC_ERR_NO_MEMORY = -7,     /* host or device allocation failed */
    NRLDPC_ERR_NO_DEVICE = -8,     /* no CUDA device / wrong architecture */
    NRLDPC_ERR_SCRATCH_TOO_SMALL = -9 /* code needs more scratch than the fixed array holds */
} nrldpc_status;

/* Code parameters as the reference computes them (mirror of ldpc_params,
 * src/types.h:38-55; pointer members replaced by the iLS index). */
typedef struct {
    int A, bg_index, Z, K, N, H_rows, H_cols, n_nz_in_row, n_nz_in_col;
    int n_iterations, N_before_puncture, i_ls, C, K_b;
    float rate;
} nrldpc_ldpc_params;

/* Host-only; no GPU needed.  Same selection rules (and quirks) as the
 * reference's setup_ldpc.  Returns NRLDPC_ERR_BAD_CONFIG where the
 * reference would read an uninitialized set index. */
int nrldpc_setup_ldpc(int A, float rate, int n_iterations, nrldpc_ldpc_params* out);

/* Lifting-size set index of Z (TS 38.212 Table 5.3.2-1), or -1. */
int nrldpc_set_index(int z);

/* Dense base matrix of (bg, iLS) into out[rows*cols] (-1 = zero block,
 * unreduced shifts).  Host-only.  rows/cols may be NULL. */
int nrldpc_base_matrix(int bg, int ils, int* out, int* rows, int* cols);

typedef struct {
    int bg;          /* 1 or 2; 0 = custom base matrix (nrldpc_init_custom) */
    int z;           /* lifting size */
    int max_batch;   /* largest n_cw of one decode call */
    float alpha;     /* normalization; the reference hard-codes 0.75 */
    int device;      /* CUDA device ordinal */
    int cw_per_cta;  /* codewords per CTA; 0 = tuned default */
} nrldpc_config;

int nrldpc_init(const nrldpc_config* cfg, nrldpc_handle** out);
/* Custom QC base matrix (rows <= 46, cols <= 68, row degree <= 19), e.g.
 * the 802.11n 12x24 matrix.  Shifts are reduced mod z. */
int nrldpc_init_custom(const int* base, int rows, int cols, const nrldpc_config* cfg,
                       nrldpc_handle** out);
int nrldpc_destroy(nrldpc_handle* h);

/* Code geometry of a handle (any pointer may be NULL). */
int nrldpc_geometry(const nrldpc_handle* h, int* rows, int* cols, int* z, int* n_edges,
                    int* n_bp, int* packed_bytes);

/* Decode n_cw codewords for n_iter iterations (device pointers).
 *   d_llr     [n_cw][n_bp] fp32, 16-byte aligned
 *   d_packed  [n_cw][packed_bytes]
 *   d_app     NULL or [n_cw][n_bp] fp32: posterior of the iteration decided on
 *   d_iters   NULL or [n_cw] int32: iterations after which the decision was taken
 *   early_stop  0: fixed n_iter (reference behaviour); 1: stop a codeword once
 *               its hard decisions satisfy every parity check. */
int nrldpc_decode(nrldpc_handle* h, const float* d_llr, uint8_t* d_packed, int n_cw, int n_iter,
                  int early_stop, float* d_app, int32_t* d_iters, nrldpc_stream_t stream);

/* Host buffers (pinned for overlap, pageable works): H2D into the handle's
 * staging, decode, D2H -- queued on `stream`, returns without waiting.  The
 * batch moves in chunks: the host->device copy of chunk k+1 runs on the
 * handle's own copy stream while chunk k decodes, even chunks on `stream`
 * and odd ones on a second stream the handle owns (with its own check-node
 * scratch); all of it is ordered after earlier work on `stream` and done
 * when `stream` is.  Pinned
 * buffers may instead be read and written by the decoder itself over the
 * host link (nrldpc_set_host_transfer, below). */
int nrldpc_decode_host_async(nrldpc_handle* h, const float* h_llr, uint8_t* h_packed, int n_cw,
                             int n_iter, int early_stop, nrldpc_stream_t stream);

/* As nrldpc_decode_host_async with narrow LLRs over the host link (the
 * reference's CHAR_PRC / HALF_PRC transfer idea, src/setup_exp.cu:26-46,
 * README TODO "make the memory transfer take place in fp16"): qtype 1 =
 * IEEE fp16, 2 = int8 with LLR = q * scale.  Widened to fp32 on the GPU and
 * decoded in fp32 (results = fp32 decode of the widened values). */
int nrldpc_decode_host_async_q(nrldpc_handle* h, const void* h_llr_q, int qtype, float scale,
                               uint8_t* h_packed, int n_cw, int n_iter, int early_stop,
                               nrldpc_stream_t stream);

/* How nrldpc_decode_host_async moves fp32 LLRs and packed bits (no reference
 * counterpart; results are the same either way).
 *   HOST_COPY    staged copies in chunks (the pipeline described above).
 *   HOST_DIRECT  one launch whose threads read the LLRs from host memory and
 *                write the packed bits back over the host link; both buffers
 *                must be pinned (cudaHostAlloc / cudaHostRegister), else the
 *                call returns NRLDPC_ERR_INVALID_ARG.
 *   HOST_AUTO    (default) DIRECT when both buffers are pinned, the GPU
 *                reaches host memory over a coherent link (Grace CPU with
 *                NVLink-C2C: cudaDevAttrPageableMemoryAccessUsesHostPageTables)
 *                and the batch is at most 4 rounds of the decoder's resident
 *                CTAs (1216 BG1 Z=384 codewords on a GB300); otherwise COPY. */
enum { NRLDPC_HOST_AUTO = 0, NRLDPC_HOST_COPY = 1, NRLDPC_HOST_DIRECT = 2 };
int nrldpc_set_host_transfer(nrldpc_handle* h, int mode);

/* Learned weighted min-sum: per (iteration, base edge) scale factors
 * w[n_w_iters][n_edges] replacing alpha (iterations past n_w_iters reuse the
 * last row; n_w_iters <= 16, else NRLDPC_ERR_TOO_LARGE).  Host pointer; copied
 * into the handle.  n_w_iters = 0 clears. */
int nrldpc_set_weights(nrldpc_handle* h, const float* w, int n_w_iters);
/* As nrldpc_decode, with the weights set on the handle. */
int nrldpc_decode_weighted(nrldpc_handle* h, const float* d_llr, uint8_t* d_packed, int n_cw,
                           int n_iter, int early_stop, float* d_app, int32_t* d_iters,
                           nrldpc_stream_t stream);

/* Message-passing schedule of a handle's decodes (nrldpc_decode,
 * nrldpc_decode_weighted, the host-buffer calls).  FLOODING (default) is the
 * reference's: every check row reads the previous iteration's posterior
 * (src/gpu_decoder_top.cu:25-49).  LAYERED has no reference counterpart:
 * base rows run in ascending order and each updates the posterior in place
 * (Q = A - R_old, A = Q + R_new), so later rows of an iteration see earlier
 * rows' messages; it converges in about 0.6x the iterations.  With early stop
 * a layered decode checks the syndrome after each iteration and reports
 * d_iters = iterations run. */
enum { NRLDPC_SCHEDULE_FLOODING = 0, NRLDPC_SCHEDULE_LAYERED = 1 };
int nrldpc_set_schedule(nrldpc_handle* h, int schedule);

/* ---- learned weighted min-sum training (no reference counterpart) ----------
 * Model: R^t_e = w[t][e] * sign * min (weights per iteration t < n_iter and
 * base edge e, shared by all lifted copies); posterior as the decoder;
 * loss = loss_scale * sum over t = 1..n_iter, codewords, columns of
 * softplus(-y * L^t), y = +1 for bit 0 (BCE on the posterior LLRs).
 * The caller allocates d_workspace of nrldpc_wms_workspace_bytes (per-iteration
 * compressed check-node states + loss gradient seeds + adjoint scratch). */
int nrldpc_wms_workspace_bytes(nrldpc_handle* h, int n_cw, int n_iter, size_t* bytes);
/* Unrolled forward: *d_loss += loss; d_app (may be NULL) gets L^{n_iter}. */
int nrldpc_wms_forward(nrldpc_handle* h, const float* d_llr, const uint8_t* d_cw_packed, int n_cw,
                       int n_iter, const float* d_weights, void* d_workspace, float loss_scale,
                       double* d_loss, float* d_app, nrldpc_stream_t stream);
/* Adjoint of the last forward on this workspace: d_grad[n_iter][n_edges] += dloss/dw.
 * Check-node messages are rebuilt from the stored two-min states, not stored. */
int nrldpc_wms_backward(nrldpc_handle* h, int n_cw, int n_iter, const float* d_weights,
                        void* d_workspace, double* d_grad, nrldpc_stream_t stream);
/* Adam on n parameters (bias-corrected, step >= 1), weights clamped >= w_min. */
int nrldpc_adam_step(int n, float* d_w, const double* d_grad, float* d_m, float* d_v, int step,
                     float lr, float beta1, float beta2, float eps, float w_min,
                     nrldpc_stream_t stream);

/* Seeded channel generator on the GPU (bit-identical to the CPU oracle's):
 * info bits (Philox4x32-10), encode, BPSK, AWGN sigma[i], LLR = 2y/sigma^2;
 * first n_punct_cols columns get LLR 0.  d_cw_packed may be NULL. */
int nrldpc_gen_llr(nrldpc_handle* h, uint64_t seed, uint64_t cw_base, int n_cw,
                   const float* d_sigma, int n_punct_cols, float* d_llr, uint8_t* d_cw_packed,
                   nrldpc_stream_t stream);

/* Count info-bit errors of decoded vs transmitted packed words over the
 * first n_info bits: d_counts[2] += {bit errors, frame errors}. */
int nrldpc_count_errors(nrldpc_handle* h, const uint8_t* d_packed, const uint8_t* d_cw_packed,
                        int n_cw, int n_info, unsigned long long* d_counts,
                        nrldpc_stream_t stream);

/* ---- mixed-code batches (no reference counterpart; the reference compiles
 * in one base graph and one Z per process, src/globals.h:15) ----------------
 * A job is one codeword of any 5G NR (bg, z), optionally rate matched
 * (3GPP TS 38.212 5.4.2.1 bit selection from a full circular buffer, then the
 * 5.4.2.2 bit interleaver for modulation order qm) with filler bits.  The
 * rate-matched LLRs are in transmission order.  All offsets index caller
 * buffers. */
typedef struct {
    int32_t bg, z;        /* base graph 1|2 and lifting size */
    int32_t k_prime;      /* information bits before filler; 0 = kb*Z (no filler) */
    int32_t e;            /* rate-matched length (a multiple of qm); 0 = one pass over the buffer */
    int32_t rv;           /* redundancy version 0..3 */
    float sigma;          /* noise std-dev (channel generator only) */
    int32_t qm;           /* modulation order 1, 2, 4, 6, 8 or 10 (bit interleaver); 0 = 1 */
    int32_t reserved;     /* 0 */
    int64_t llr_offset;   /* float offset of the mother-code LLRs [cols*Z], multiple of 4 */
    int64_t e_offset;     /* float offset of the rate-matched LLRs [e] */
    int64_t out_offset;   /* byte offset of the packed hard decisions / codeword */
} nrldpc_job;

typedef struct nrldpc_batch nrldpc_batch;

/* Tables of every (bg, z) on `device`, scratch for up to max_jobs jobs. */
int nrldpc_batch_create(int device, int max_jobs, float alpha, nrldpc_batch** out);
int nrldpc_batch_destroy(nrldpc_batch* b);
/* Launch geometry per code, the autotuner's two knobs (the reference fixes
 * it: one thread per sub-row, roundup32(Z) x codewords per block,
 * src/setup_exp.cu:131-166).  Codewords per CTA: 0 restores the largest that
 * the CTA's 384 threads and shared memory admit.  Sub-rows per thread 1 or 2
 * (0 = 1): threads per codeword = Z / spt, thread t owning sub-rows t and
 * t + Z/2 (Z even); changing it clamps codewords per CTA to what fits.  The
 * batch's CTA has the threads of its widest work item.  Results do not
 * depend on either knob.  Apply before nrldpc_batch_set_jobs. */
int nrldpc_batch_set_cw_per_cta(nrldpc_batch* b, int bg, int z, int cw_per_cta);
int nrldpc_batch_get_cw_per_cta(nrldpc_batch* b, int bg, int z, int* cw_per_cta);
int nrldpc_batch_set_sub_rows_per_thread(nrldpc_batch* b, int bg, int z, int sub_rows_per_thread);
int nrldpc_batch_get_sub_rows_per_thread(nrldpc_batch* b, int bg, int z, int* sub_rows_per_thread);
/* Load a job list (host array): validated, grouped by code into the device
 * work queue (largest work first).  Synchronous. */
int nrldpc_batch_set_jobs(nrldpc_batch* b, const nrldpc_job* jobs, int n_jobs);
/* Seeded rate-matched transmissions of the loaded jobs (bit-identical to the
 * oracle): every bit on the wire (after the bit interleaver) through BPSK and
 * AWGN, d_llr_e at e_offset in transmission order, transmitted codewords at
 * out_offset of d_cw. */
int nrldpc_batch_gen(nrldpc_batch* b, uint64_t seed, uint64_t cw_base, float* d_llr_e,
                     uint8_t* d_cw, nrldpc_stream_t stream);
/* De-rate-matching: rate-matched LLRs in transmission order -> de-interleaved
 * -> mother-code LLRs at llr_offset (punctured/unsent 0, filler +inf,
 * repetitions added in rate-matching order). */
int nrldpc_batch_derate(nrldpc_batch* b, const float* d_llr_e, float* d_llr, nrldpc_stream_t stream);
/* Decode all loaded jobs in one persistent launch (device work queue),
 * replayed from a CUDA graph; d_iters (may be NULL) indexed by job. */
int nrldpc_batch_decode(nrldpc_batch* b, const float* d_llr, uint8_t* d_packed, int n_iter,
                        int early_stop, int32_t* d_iters, nrldpc_stream_t stream);
/* d_counts[2] += {bit errors, frame errors} over each job's k_prime info bits. */
int nrldpc_batch_count_errors(nrldpc_batch* b, const uint8_t* d_packed, const uint8_t* d_cw,
                              unsigned long long* d_counts, nrldpc_stream_t stream);
/* Host helper: k0 of redundancy version rv (TS 38.212 Table 5.4.2.1-2, full buffer). */
int nrldpc_rm_k0(int bg, int z, int rv);

/* Decode without allocating anything (no reference counterpart).  For
 * callers that cannot call cudaMalloc at decode time -- a physical-layer
 * pipeline that reserves all device memory at start-up and must not allocate
 * (allocation can block the device) while it processes slots, or code inside
 * another runtime's memory manager -- and so cannot hold an nrldpc_handle.
 * Same results as nrldpc_decode for 5G NR (bg, z) with alpha (device
 * pointers, 16-byte aligned d_llr; packed output as nrldpc_decode).  Scratch
 * is one static 96 MiB device array in the library; a code whose per-CTA
 * check-node state does not fit returns NRLDPC_ERR_SCRATCH_TOO_SMALL.  A GPU
 * reserves the array when the runtime loads the library module that holds
 * it, and keeps it until the process exits: under lazy module loading (the
 * default) at the first call on that GPU that touches it (this entry point
 * or nrldpc_noalloc_device_error), under CUDA_MODULE_LOADING=EAGER at
 * context creation on every GPU the process uses -- whether or not this
 * entry point is ever called.  The first
 * successful call on a device (the current one) sets it up: make it before
 * any stream capture; a failed set-up is retried by the next call.  Calls
 * share the array: calls that overlap on the GPU race; serialise them.
 * A bounded device-side wait that ran out is reported by
 * nrldpc_noalloc_device_error, not by this call's return value. */
int nrldpc_decode_noalloc(int bg, int z, float alpha, const float* d_llr, uint8_t* d_packed,
                          int n_cw, int n_iter, int early_stop, nrldpc_stream_t stream);

/* Device-side error of nrldpc_decode_noalloc calls on the current device
 * since the last query (NRLDPC_ERR_TIMEOUT when a bounded wait ran out, the
 * call's output then unwritten; NRLDPC_OK otherwise), and clears it.  A
 * synchronous symbol copy, no allocation: synchronise the decode's stream
 * first.  No reference counterpart (the reference checks no kernel error). */
int nrldpc_noalloc_device_error(void);

/* Self-test of nrldpc_decode_noalloc's bounded wait (no reference
 * counterpart), as nrldpc_selftest_wait_timeout for a handle: one iteration
 * whose copy barrier expects 16 bytes that no copy delivers (no copy is
 * issued), with a short wait limit; nrldpc_noalloc_device_error then returns
 * NRLDPC_ERR_TIMEOUT.  Nothing faults or spins without end. */
int nrldpc_selftest_noalloc_wait_timeout(int bg, int z, const float* d_llr, uint8_t* d_packed, int n_cw,
                                         nrldpc_stream_t stream);

/* CRC (3GPP TS 38.212 5.1) of the first n_bits of each of n_cw packed
 * words (stride_bytes apart); bit i of the packed bytes is the i-th bit of
 * the sequence.  crc_type 0 = CRC24A, 1 = CRC24B, 2 = CRC16.  d_rem[i] = 0
 * when the sequence ends in its own valid CRC.  No reference counterpart
 * (the reference computes the CRC length only, src/nr_ldpc.cpp:37). */
int nrldpc_crc(const uint8_t* d_packed, int n_cw, int stride_bytes, int n_bits, int crc_type,
               uint32_t* d_rem, nrldpc_stream_t stream);

/* Code-block segmentation (3GPP TS 38.212 5.2.2) of a transport block of B
 * bits (TB CRC included) for base graph bg: C blocks of k_prime bits each
 * (CRC24B of L = 24 bits per block when C > 1), lifting size zc, K = kb_max*zc
 * decoder info bits of which filler = K - k_prime are <NULL>.  B' = B + C*L
 * must divide by C (TS 38.214's TB sizes do).  No reference counterpart: the
 * reference computes C (src/nr_ldpc.cpp:64-81) but supports C = 1 only. */
typedef struct {
    int B, C, L, k_prime, k, zc, kb, filler, bg;
} nrldpc_segment_info;
int nrldpc_segment(int B, int bg, nrldpc_segment_info* out);

/* Device side of the segmentation.  d_tb: B bits packed LSB-first.
 * nrldpc_cb_segment writes C blocks of k_prime bits (data, then CRC24B when
 * C > 1; bits past k_prime zero) at d_blocks + r * block_stride.
 * nrldpc_cb_desegment is its inverse on decoded blocks: the data bits go back
 * to d_tb, and d_crc_rem[r] (C entries, may be NULL when C = 1) is the CRC24B
 * remainder of block r (0 = block CRC passes). */
int nrldpc_cb_segment(const uint8_t* d_tb, const nrldpc_segment_info* info, uint8_t* d_blocks,
                      int block_stride, nrldpc_stream_t stream);
int nrldpc_cb_desegment(const uint8_t* d_blocks, int block_stride, const nrldpc_segment_info* info,
                        uint8_t* d_tb, uint32_t* d_crc_rem, nrldpc_stream_t stream);

/* Last device-side error recorded by a bounded wait (0 if none); clears it. */
int nrldpc_device_error(nrldpc_handle* h);

/* Self-test of the bounded device-side wait (no reference counterpart): one
 * device-resident decode of n_cw codewords whose copy barrier is told to
 * expect 16 bytes more than the LLR copies deliver, with a short wait limit;
 * no copy is issued, so nothing is in flight when the wait runs out.  Every
 * CTA's wait for its first codeword runs out, the kernel records the timeout
 * (nrldpc_device_error then returns NRLDPC_ERR_TIMEOUT) and its CTAs return
 * without writing d_packed.  Nothing faults or spins without end.  The
 * handle stays usable. */
int nrldpc_selftest_wait_timeout(nrldpc_handle* h, const float* d_llr, uint8_t* d_packed, int n_cw,
                                 nrldpc_stream_t stream);

const char* nrldpc_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif
