/*
 * CPU oracle for the QC-LDPC min-sum decode path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the checker (or the timed CPU baseline).
 * The decoder product never links or calls it.
 *
 * What it restates (reference = ctarver/NR_GPU_LDPC):
 *   - compact row/column edge orders: src/setup_exp.cu:221-271
 *   - first-iteration check-node pass:  src/ldpc_kernels.cu:73-181
 *   - check-node pass, iterations >= 2: src/ldpc_kernels.cu:199-314
 *   - variable-node pass (incremental posterior, ascending base rows):
 *                                       src/ldpc_kernels.cu:330-395, 411-468
 *   - hard-decision packing (LSB first): src/ldpc_kernels.cu:482-500
 *   - iteration orchestration:          src/gpu_decoder_top.cu:25-49
 * Float semantics are the reference's float branch on a signed-char
 * platform with every C statement rounded on its own (built with
 * -ffp-contract=off).  Pinned against the reference's own kernel source run
 * on the CPU (oracle/_ref) through the committed fixtures in tests/golden.
 *
 * Additions with no reference counterpart (their own oracles): syndrome early
 * stop, FP64 twin, learned weighted min-sum forward/adjoint, a structural
 * encoder, and a Philox4x32-10 + Box-Muller channel generator whose float
 * arithmetic is written so the GPU generator reproduces it bit for bit.
 */
#ifndef NR_LDPC_ORACLE_H
#define NR_LDPC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_code orc_code;

/* Build a lifted code from a dense base matrix (rows x cols, -1 = zero block,
 * otherwise the table shift V; V is reduced mod Z).  Returns NULL on error. */
orc_code* orc_code_new(const int* base, int rows, int cols, int z);
void orc_code_free(orc_code* c);
int orc_code_edges(const orc_code* c);

/* Flooding normalized min-sum, fp32, reference semantics.
 *   llr     [n_cw][cols*Z]         channel LLRs (punctured columns = 0)
 *   packed  [n_cw][ceil(cols*Z/8)]       hard decisions, bit i of byte b = bit 8b+i
 *   app     [n_cw][cols*Z] or NULL final posterior (APP of the last iteration)
 *   iters   [n_cw] or NULL         iterations after which HD was taken
 * early_stop != 0: stop after iteration t when the syndrome of HD_t is zero.
 * n_threads > 1 decodes codewords on that many POSIX threads. */
/* Process-wide switch of orc_minsum_f32: compute dt = R_new - R_old as one
 * fused multiply-add (what a contracting compiler makes of the reference's
 * dt line) instead of two roundings.  Off by default. */
void orc_set_fma_dt(int on);
int orc_minsum_f32(const orc_code* c, const float* llr, int n_cw, int n_iter, float alpha,
                   int early_stop, uint8_t* packed, float* app, int32_t* iters, int n_threads);

/* The same algorithm carried out in double precision (alpha exact). */
int orc_minsum_f64(const orc_code* c, const double* llr, int n_cw, int n_iter, double alpha,
                   int early_stop, uint8_t* packed, double* app, int32_t* iters);

/* Syndrome weight (number of unsatisfied lifted checks) of packed bits. */
int orc_syndrome_weight(const orc_code* c, const uint8_t* packed);

/* Structural encoder.  kb systematic base columns, info = kb*Z bits (one per
 * byte, 0/1), cw_packed = ceil(cols*Z/8) bytes.  Returns 0 or a negative error. */
int orc_encode(const orc_code* c, int kb, const uint8_t* info, uint8_t* cw_packed);

/* Channel generator: for codeword id (cw_base + i), draw kb*Z info bits,
 * encode, BPSK (0 -> +1), add Gaussian noise sigma[i], LLR = (2y)/(sigma^2);
 * the first n_punct columns' LLRs are 0 (punctured), as are LLRs of columns
 * beyond n_tx transmitted bits.  Outputs: llr [n_cw][cols*Z],
 * cw_packed [n_cw][ceil(cols*Z/8)] (may be NULL). */
int orc_gen_llr(const orc_code* c, int kb, uint64_t seed, uint64_t cw_base, int n_cw,
                const float* sigma, int n_punct_cols, float* llr, uint8_t* cw_packed);

/* ---- rate matching (no reference counterpart; 3GPP TS 38.212 5.4.2.1) ------
 * Mother codeword x[cols*Z]; circular buffer d[j] = x[2Z + j], Ncb = cols*Z - 2Z
 * (full buffer); filler bits x[k_prime .. kb*Z) are NULL (never sent, known 0).
 * k0 from rv as the standard's table; E bits e_k = d[(k0 + j) mod Ncb] taken in
 * order skipping NULLs; then the bit interleaver of 5.4.2.2 for modulation
 * order Qm (E a multiple of Qm): f[i + j*Qm] = e[i*E/Qm + j], i < Qm,
 * j < E/Qm.  Qm = 1 (or 0) leaves the order as it is.  Every transmitted bit
 * goes through BPSK + AWGN here, so Qm only fixes the bit order on the wire. */
int orc_rm_k0(int bg, int z, int rv);
/* e index of the bit sent at position p (f_p = e_k) for length e, order qm. */
int orc_interleave_src(int e, int qm, int p);
/* d index (0 .. Ncb-1) of rate-matched bit k. */
int orc_rm_index(int z, int ncb, int kb_z, int k_prime, int k0, int k);
/* Seeded rate-matched transmission: info bits (k_prime random, filler 0),
 * encode, select e bits, interleave for qm[i] (NULL: 1), BPSK + AWGN sigma[i]
 * per transmitted position; llr_e [n_cw][e_stride] in transmission order. */
int orc_gen_rm_llr(const orc_code* c, int kb, int bg, uint64_t seed, uint64_t cw_base, int n_cw,
                   const float* sigma, const int* k_prime, const int* e, const int* rv, const int* qm,
                   int e_stride, float* llr_e, uint8_t* cw_packed);
/* Receiver: rate-matched LLRs -> mother-code LLRs [n_cw][cols*Z]: punctured
 * and unsent columns 0, filler +inf, repeated bits added in rate-matching
 * order (first copy taken as is); llr_e in transmission order for qm[i]
 * (NULL: 1), de-interleaved first. */
int orc_derate_match(const orc_code* c, int kb, int bg, int n_cw, const float* llr_e, int e_stride,
                     const int* k_prime, const int* e, const int* rv, const int* qm, float* llr);

/* ---- CRC (3GPP TS 38.212 5.1), bitwise long division ------------------------
 * poly: generator without the leading term (CRC24A 0x864CFB, CRC24B 0x800063,
 * CRC16 0x1021), len = 24 or 16.  Bits a_0 .. a_{n-1} are bit i of the packed
 * bytes (LSB first); a_0 is the highest-order coefficient.  Returns the
 * remainder of a(D) * D^len; appending its bits p_0..p_{len-1} (p_0 = MSB)
 * gives a sequence whose remainder over n+len bits is 0. */
uint32_t orc_crc(const uint8_t* packed, int n_bits, uint32_t poly, int len);

/* Philox4x32-10 block (Salmon et al., SC'11) and the float helpers used by the
 * generator, exposed for the generator's own tests. */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float orc_logf(float x);
void orc_sincos2pi(float u, float* s, float* c);

/* ---- learned weighted min-sum (per iteration t, per base edge e weights) ----
 * Forward (double): R^t_e = w[t][e] * sign * min (extrinsic), posterior
 * L^{t+1} = llr + sum_e R^t_e, loss = mean over t=1..T, codewords and columns
 * of softplus(-y*L^t), y = +1 for bit 0 and -1 for bit 1.
 * grad (may be NULL) receives dloss/dw [T][edges] by the adjoint recursion.
 * app (may be NULL) receives L^T. Returns the loss. */
double orc_wms_loss_grad_f64(const orc_code* c, const float* llr, const uint8_t* cw_packed,
                             int n_cw, int n_iter, const double* w, double* grad, double* app);

/* fp32 forward of the weighted decoder as an inference decoder (weights
 * replace alpha; t >= n_weight_iters reuse the last row).  Same outputs as
 * orc_minsum_f32. */
int orc_wms_decode_f32(const orc_code* c, const float* llr, int n_cw, int n_iter,
                       const float* w, int n_weight_iters, int early_stop, uint8_t* packed,
                       float* app, int32_t* iters);

/* Layered (row-sequential) normalized or weighted min-sum, fp32.  No
 * reference counterpart (the reference's schedule is flooding).  Rows in
 * ascending order update the posterior in place: Q = A - R_old,
 * A = Q + R_new; check-node rules as orc_minsum_f32.  w == NULL -> alpha,
 * else weights [n_weight_iters][E] (t >= n_weight_iters reuse the last row).
 * early_stop: stop after iteration t when the syndrome of HD_t is zero
 * (iters = t + 1). */
int orc_layered_f32(const orc_code* c, const float* llr, int n_cw, int n_iter, float alpha,
                    const float* w, int n_weight_iters, int early_stop, uint8_t* packed, float* app,
                    int32_t* iters, int n_threads);

/* Loss and gradient of the layered weighted min-sum (double precision; same
 * loss as orc_wms_loss_grad_f64, posterior updated row by row in place). */
double orc_wms_layered_loss_grad_f64(const orc_code* c, const float* llr, const uint8_t* cw_packed,
                                     int n_cw, int n_iter, const double* w, double* grad, double* app);
/* As above; f32_forward != 0 runs the forward in fp32 with the decoder's
 * rounding (the GPU forward's argmins and signs), loss and adjoint in double. */
double orc_wms_layered_loss_grad(const orc_code* c, const float* llr, const uint8_t* cw_packed, int n_cw,
                                 int n_iter, const double* w, double* grad, double* app, int f32_forward);

#ifdef __cplusplus
}
#endif
#endif
