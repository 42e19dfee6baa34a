/*
 * CPU oracle for the QC-LDPC min-sum decode path -- TEST INFRASTRUCTURE ONLY.
 * See ldpc_oracle.h for what is restated from which reference file:line.
 * Build with -ffp-contract=off: every float statement below is meant to be
 * rounded on its own, as the reference's C source reads.
 */
#include "ldpc_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

struct orc_code {
    int rows, cols, z, n_edges;
    int* row_ptr;  /* [rows+1]; edges of a row in ascending column order (setup_exp.cu:241-250) */
    int* e_row;    /* [n_edges] base row of edge */
    int* e_col;    /* [n_edges] base column of edge */
    int* e_shift;  /* [n_edges] V mod Z */
    int* col_ptr;  /* [cols+1] */
    int* col_edge; /* edges of a column in ascending row order (setup_exp.cu:261-270) */
};

orc_code* orc_code_new(const int* base, int rows, int cols, int z) {
    if (!base || rows <= 0 || cols <= 0 || z <= 0) return NULL;
    orc_code* c = (orc_code*)calloc(1, sizeof(orc_code));
    int n = 0;
    for (int i = 0; i < rows * cols; i++) n += base[i] != -1;
    c->rows = rows; c->cols = cols; c->z = z; c->n_edges = n;
    c->row_ptr = (int*)malloc(sizeof(int) * (rows + 1));
    c->e_row = (int*)malloc(sizeof(int) * n);
    c->e_col = (int*)malloc(sizeof(int) * n);
    c->e_shift = (int*)malloc(sizeof(int) * n);
    c->col_ptr = (int*)calloc(cols + 1, sizeof(int));
    c->col_edge = (int*)malloc(sizeof(int) * n);
    int e = 0;
    for (int r = 0; r < rows; r++) {
        c->row_ptr[r] = e;
        for (int j = 0; j < cols; j++) {
            int v = base[r * cols + j];
            if (v == -1) continue;
            if (v < 0) { orc_code_free(c); return NULL; }
            c->e_row[e] = r; c->e_col[e] = j; c->e_shift[e] = v % z;
            c->col_ptr[j + 1]++;
            e++;
        }
    }
    c->row_ptr[rows] = e;
    for (int j = 0; j < cols; j++) c->col_ptr[j + 1] += c->col_ptr[j];
    int* fill = (int*)calloc(cols, sizeof(int));
    for (int k = 0; k < n; k++) { /* edges visited row-major => rows ascend per column */
        int j = c->e_col[k];
        c->col_edge[c->col_ptr[j] + fill[j]++] = k;
    }
    free(fill);
    return c;
}

void orc_code_free(orc_code* c) {
    if (!c) return;
    free(c->row_ptr); free(c->e_row); free(c->e_col); free(c->e_shift);
    free(c->col_ptr); free(c->col_edge); free(c);
}

int orc_code_edges(const orc_code* c) { return c ? c->n_edges : 0; }

/* Column of sub-row s in the block of edge e: (s + V) mod Z, with V < Z
 * (ldpc_kernels.cu:126-132). */
static inline int edge_col(const orc_code* c, int e, int s) {
    int t = s + c->e_shift[e];
    if (t >= c->z) t -= c->z;
    return c->e_col[e] * c->z + t;
}
/* Sub-row of the block of edge e that hits sub-column s (ldpc_kernels.cu:370-373). */
static inline int edge_subrow(const orc_code* c, int e, int s) {
    int t = s - c->e_shift[e];
    if (t < 0) t += c->z;
    return t;
}

/* Packed bits: ceil(n/8) bytes, byte b = sum_i hd[8b+i] << i
 * (ldpc_kernels.cu:495-499), bits past n zero. */
#define PACKED_BYTES(n) (((n) + 7) / 8)
static void pack_hd(const uint8_t* hd, int n, uint8_t* packed) {
    for (int b = 0; b < PACKED_BYTES(n); b++) {
        unsigned v = 0;
        for (int i = 0; i < 8 && 8 * b + i < n; i++) v |= (unsigned)hd[8 * b + i] << i;
        packed[b] = (uint8_t)v;
    }
}

static int syndrome_weight_hd(const orc_code* c, const uint8_t* hd) {
    int w = 0, z = c->z;
    for (int r = 0; r < c->rows; r++)
        for (int s = 0; s < z; s++) {
            int p = 0;
            for (int e = c->row_ptr[r]; e < c->row_ptr[r + 1]; e++) p ^= hd[edge_col(c, e, s)];
            w += p;
        }
    return w;
}

int orc_syndrome_weight(const orc_code* c, const uint8_t* packed) {
    int n = c->cols * c->z;
    uint8_t* hd = (uint8_t*)malloc(n);
    for (int i = 0; i < n; i++) hd[i] = (packed[i >> 3] >> (i & 7)) & 1;
    int w = syndrome_weight_hd(c, hd);
    free(hd);
    return w;
}

/* ------------------------------------------------------------------------- */
/* fp32 decode of one codeword.  weights == NULL -> alpha for every edge.     */
typedef struct {
    float* L;   /* [N] posterior */
    float* R;   /* [E*Z] check-to-variable messages, edge-major */
    float* dt;  /* [E*Z] R_new - R_old */
    uint8_t* hd;
} ws_f32;

/* dt = R_new - R_old computed as the fused fmaf(+-a, min, -R_old) -- one
 * rounding -- instead of two roundings; what a compiler that contracts
 * ldpc_kernels.cu:308-310 (dt = R_temp - RCache, R_temp ending in a product)
 * into a fused multiply-add would compute.  Off by default (the source's
 * semantics, each statement rounded). */
static int g_fma_dt = 0;
void orc_set_fma_dt(int on) { g_fma_dt = on != 0; }

static void decode_one_f32(const orc_code* c, const float* llr, int n_iter, float alpha,
                           const float* w, int n_w_iters, int early, ws_f32* ws,
                           uint8_t* packed, float* app, int32_t* iters) {
    const int z = c->z, N = c->cols * z;
    float* L = ws->L; float* R = ws->R; float* dt = ws->dt; uint8_t* hd = ws->hd;
    memcpy(L, llr, sizeof(float) * N);
    int t_done = n_iter;
    for (int t = 0; t < n_iter; t++) {
        /* check-node pass: ldpc_kernels.cu:73-181 (t == 0), :199-314 (t > 0) */
        for (int r = 0; r < c->rows; r++) {
            const int e0 = c->row_ptr[r], deg = c->row_ptr[r + 1] - e0;
            for (int s = 0; s < z; s++) {
                int q_sign = 0, idx_min = 0;
                float sign = 1.0f, rmin1 = 1000.0f, rmin2 = 1000.0f;
                for (int i = 0; i < deg; i++) {
                    const int e = e0 + i;
                    float q;
                    if (t == 0) {
                        q = L[edge_col(c, e, s)];
                    } else {
                        const float r_old = R[e * z + s];
                        q = L[edge_col(c, e, s)] - r_old;
                    }
                    const float q_abs = fabsf(q);
                    const int sq = q < 0.0f;
                    sign = sign * (float)(1 - sq * 2);
                    q_sign |= sq << i;
                    if (q_abs < rmin1) {
                        rmin2 = rmin1; rmin1 = q_abs; idx_min = i;
                    } else if (q_abs < rmin2) {
                        rmin2 = q_abs;
                    }
                }
                for (int i = 0; i < deg; i++) {
                    const int e = e0 + i;
                    const float sq = (float)(1 - 2 * ((q_sign >> i) & 1));
                    const float a = w ? w[(t < n_w_iters ? t : n_w_iters - 1) * c->n_edges + e] : alpha;
                    float r_new = a * sign;
                    r_new = r_new * sq;
                    const float m = i != idx_min ? rmin1 : rmin2;
                    const float sa = r_new;  /* +-a, exact */
                    r_new = r_new * m;
                    if (t == 0) {
                        dt[e * z + s] = r_new;
                    } else {
                        const float d = g_fma_dt ? fmaf(sa, m, -R[e * z + s]) : r_new - R[e * z + s];
                        dt[e * z + s] = d;
                    }
                    R[e * z + s] = r_new;
                }
            }
        }
        /* variable-node pass: ldpc_kernels.cu:330-395 / 411-468 */
        for (int j = 0; j < c->cols; j++) {
            for (int s = 0; s < z; s++) {
                float a = L[j * z + s];
                for (int k = c->col_ptr[j]; k < c->col_ptr[j + 1]; k++) {
                    const int e = c->col_edge[k];
                    a = a + dt[e * z + edge_subrow(c, e, s)];
                }
                L[j * z + s] = a; /* last iteration: only feeds HD and the app output */
                hd[j * z + s] = (a > 0.0f) ? 0 : 1;
            }
        }
        if (early && t < n_iter - 1 && syndrome_weight_hd(c, hd) == 0) { t_done = t + 1; break; }
    }
    pack_hd(hd, N, packed);
    if (app) memcpy(app, L, sizeof(float) * N);
    if (iters) *iters = t_done;
}

typedef struct {
    const orc_code* c; const float* llr; int n_iter; float alpha; const float* w; int n_w;
    int early; uint8_t* packed; float* app; int32_t* iters;
    int cw_begin, cw_end, layered;
} job_f32;

static void decode_one_layered_f32(const orc_code* c, const float* llr, int n_iter, float alpha,
                                   const float* w, int n_w_iters, int early, ws_f32* ws,
                                   uint8_t* packed, float* app, int32_t* iters);

static void* run_job_f32(void* arg) {
    job_f32* j = (job_f32*)arg;
    const orc_code* c = j->c;
    const int N = c->cols * c->z, EZ = c->n_edges * c->z;
    ws_f32 ws;
    ws.L = (float*)malloc(sizeof(float) * N);
    ws.R = (float*)malloc(sizeof(float) * EZ);
    ws.dt = (float*)malloc(sizeof(float) * EZ);
    ws.hd = (uint8_t*)malloc(N);
    for (int i = j->cw_begin; i < j->cw_end; i++)
        (j->layered ? decode_one_layered_f32 : decode_one_f32)(
            c, j->llr + (size_t)i * N, j->n_iter, j->alpha, j->w, j->n_w, j->early, &ws,
            j->packed + (size_t)i * PACKED_BYTES(N), j->app ? j->app + (size_t)i * N : NULL,
            j->iters ? j->iters + i : NULL);
    free(ws.L); free(ws.R); free(ws.dt); free(ws.hd);
    return NULL;
}

static int decode_f32_common(const orc_code* c, const float* llr, int n_cw, int n_iter,
                             float alpha, const float* w, int n_w, int early, uint8_t* packed,
                             float* app, int32_t* iters, int n_threads, int layered) {
    if (!c || !llr || !packed || n_cw < 0 || n_iter < 1) return -1;
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n_cw) n_threads = n_cw > 0 ? n_cw : 1;
    pthread_t th[256];
    job_f32 jobs[256];
    if (n_threads > 256) n_threads = 256;
    for (int k = 0; k < n_threads; k++) {
        jobs[k] = (job_f32){c, llr, n_iter, alpha, w, n_w, early, packed, app, iters,
                            (int)((long)n_cw * k / n_threads), (int)((long)n_cw * (k + 1) / n_threads),
                            layered};
    }
    if (n_threads == 1) { run_job_f32(&jobs[0]); return 0; }
    for (int k = 0; k < n_threads; k++) pthread_create(&th[k], NULL, run_job_f32, &jobs[k]);
    for (int k = 0; k < n_threads; k++) pthread_join(th[k], NULL);
    return 0;
}

int orc_minsum_f32(const orc_code* c, const float* llr, int n_cw, int n_iter, float alpha,
                   int early_stop, uint8_t* packed, float* app, int32_t* iters, int n_threads) {
    return decode_f32_common(c, llr, n_cw, n_iter, alpha, NULL, 0, early_stop, packed, app, iters,
                             n_threads, 0);
}

int orc_wms_decode_f32(const orc_code* c, const float* llr, int n_cw, int n_iter, const float* w,
                       int n_weight_iters, int early_stop, uint8_t* packed, float* app,
                       int32_t* iters) {
    if (!w || n_weight_iters < 1) return -1;
    return decode_f32_common(c, llr, n_cw, n_iter, 0.0f, w, n_weight_iters, early_stop, packed, app,
                             iters, 1, 0);
}

int orc_layered_f32(const orc_code* c, const float* llr, int n_cw, int n_iter, float alpha,
                    const float* w, int n_weight_iters, int early_stop, uint8_t* packed, float* app,
                    int32_t* iters, int n_threads) {
    if (w && n_weight_iters < 1) return -1;
    return decode_f32_common(c, llr, n_cw, n_iter, alpha, w, w ? n_weight_iters : 0, early_stop, packed,
                             app, iters, n_threads, 1);
}

/* ------------------------------------------------------------------------- */
/* Layered (row-sequential) schedule, fp32.  No reference counterpart: the
 * reference decodes with the flooding schedule only.  Same check-node rules
 * as decode_one_f32 (strict '<' from 1000.0f, first argmin, R = +-fl(a*min));
 * rows run in ascending order and each updates the posterior in place:
 *   Q_e = A[col] - R_old_e;  A[col] = Q_e + R_new_e.
 * early: after iteration t < n_iter - 1, stop when the syndrome of HD(A) is
 * zero (iters = t + 1). */
static void decode_one_layered_f32(const orc_code* c, const float* llr, int n_iter, float alpha,
                                   const float* w, int n_w_iters, int early, ws_f32* ws,
                                   uint8_t* packed, float* app, int32_t* iters) {
    const int z = c->z, N = c->cols * z;
    float* A = ws->L; float* R = ws->R; float* Q = ws->dt; uint8_t* hd = ws->hd;
    memcpy(A, llr, sizeof(float) * N);
    memset(R, 0, sizeof(float) * (size_t)c->n_edges * z);
    int t_done = n_iter;
    for (int t = 0; t < n_iter; t++) {
        for (int r = 0; r < c->rows; r++) {
            const int e0 = c->row_ptr[r], deg = c->row_ptr[r + 1] - e0;
            for (int s = 0; s < z; s++) {
                int q_sign = 0, idx_min = 0;
                float sign = 1.0f, rmin1 = 1000.0f, rmin2 = 1000.0f;
                for (int i = 0; i < deg; i++) {
                    const int e = e0 + i;
                    const float q = A[edge_col(c, e, s)] - R[e * z + s];
                    Q[e * z + s] = q;
                    const float q_abs = fabsf(q);
                    const int sq = q < 0.0f;
                    sign = sign * (float)(1 - sq * 2);
                    q_sign |= sq << i;
                    if (q_abs < rmin1) {
                        rmin2 = rmin1; rmin1 = q_abs; idx_min = i;
                    } else if (q_abs < rmin2) {
                        rmin2 = q_abs;
                    }
                }
                for (int i = 0; i < deg; i++) {
                    const int e = e0 + i;
                    const float sq = (float)(1 - 2 * ((q_sign >> i) & 1));
                    const float a = w ? w[(t < n_w_iters ? t : n_w_iters - 1) * c->n_edges + e] : alpha;
                    float r_new = a * sign;
                    r_new = r_new * sq;
                    r_new = r_new * (i != idx_min ? rmin1 : rmin2);
                    R[e * z + s] = r_new;
                    A[edge_col(c, e, s)] = Q[e * z + s] + r_new;
                }
            }
        }
        for (int i = 0; i < N; i++) hd[i] = (A[i] > 0.0f) ? 0 : 1;
        if (early && t < n_iter - 1 && syndrome_weight_hd(c, hd) == 0) { t_done = t + 1; break; }
    }
    pack_hd(hd, N, packed);
    if (app) memcpy(app, A, sizeof(float) * N);
    if (iters) *iters = t_done;
}

/* ------------------------------------------------------------------------- */
int orc_minsum_f64(const orc_code* c, const double* llr, int n_cw, int n_iter, double alpha,
                   int early_stop, uint8_t* packed, double* app, int32_t* iters) {
    if (!c || !llr || !packed || n_iter < 1) return -1;
    const int z = c->z, N = c->cols * z, EZ = c->n_edges * z;
    double* L = (double*)malloc(sizeof(double) * N);
    double* R = (double*)malloc(sizeof(double) * EZ);
    double* dt = (double*)malloc(sizeof(double) * EZ);
    uint8_t* hd = (uint8_t*)malloc(N);
    for (int cw = 0; cw < n_cw; cw++) {
        memcpy(L, llr + (size_t)cw * N, sizeof(double) * N);
        int t_done = n_iter;
        for (int t = 0; t < n_iter; t++) {
            for (int r = 0; r < c->rows; r++) {
                const int e0 = c->row_ptr[r], deg = c->row_ptr[r + 1] - e0;
                for (int s = 0; s < z; s++) {
                    int q_sign = 0, idx_min = 0;
                    double sign = 1.0, rmin1 = 1000.0, rmin2 = 1000.0;
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        const double q = t == 0 ? L[edge_col(c, e, s)] : L[edge_col(c, e, s)] - R[e * z + s];
                        const double q_abs = fabs(q);
                        const int sq = q < 0.0;
                        sign = sign * (double)(1 - sq * 2);
                        q_sign |= sq << i;
                        if (q_abs < rmin1) { rmin2 = rmin1; rmin1 = q_abs; idx_min = i; }
                        else if (q_abs < rmin2) rmin2 = q_abs;
                    }
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        const double sq = (double)(1 - 2 * ((q_sign >> i) & 1));
                        const double r_new = alpha * sign * sq * (i != idx_min ? rmin1 : rmin2);
                        dt[e * z + s] = t == 0 ? r_new : r_new - R[e * z + s];
                        R[e * z + s] = r_new;
                    }
                }
            }
            for (int j = 0; j < c->cols; j++)
                for (int s = 0; s < z; s++) {
                    double a = L[j * z + s];
                    for (int k = c->col_ptr[j]; k < c->col_ptr[j + 1]; k++) {
                        const int e = c->col_edge[k];
                        a += dt[e * z + edge_subrow(c, e, s)];
                    }
                    L[j * z + s] = a;
                    hd[j * z + s] = a > 0.0 ? 0 : 1;
                }
            if (early_stop && t < n_iter - 1 && syndrome_weight_hd(c, hd) == 0) { t_done = t + 1; break; }
        }
        pack_hd(hd, N, packed + (size_t)cw * PACKED_BYTES(N));
        if (app) memcpy(app + (size_t)cw * N, L, sizeof(double) * N);
        if (iters) iters[cw] = t_done;
    }
    free(L); free(R); free(dt); free(hd);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Structural encoder (no reference counterpart; the reference vendors OAI's).
 * Lifted block semantics: (P^V x)[k] = x[(k + V) mod Z].
 * Staircase rows 0..m-1 (m = 4 for NR, all rows for the 12x24 matrix): the
 * sum of all staircase rows leaves only parity column kb with one odd shift v,
 * so p0 = P^{-v} * sum(lambda).  Each later staircase row adds exactly one new
 * parity column with shift 0.  Rows past the staircase end in their own
 * degree-1 column (shift 0). */
static void acc_shift(uint8_t* dst, const uint8_t* x, int v, int z) {
    for (int k = 0; k < z; k++) dst[k] ^= x[(k + v) % z];
}

int orc_encode(const orc_code* c, int kb, const uint8_t* info, uint8_t* cw_packed) {
    const int z = c->z, N = c->cols * z, rows = c->rows;
    uint8_t* x = (uint8_t*)calloc(N, 1);
    uint8_t* acc = (uint8_t*)malloc(z);
    int* solved = (int*)calloc(c->cols, sizeof(int));
    int rc = 0;
    for (int i = 0; i < kb * z; i++) x[i] = info[i] & 1;
    for (int j = 0; j < kb; j++) solved[j] = 1;
    /* staircase size: rows whose last parity column lies before the first degree-1 column */
    int m = 0;
    for (int r = 0; r < rows; r++) {
        int last = c->e_col[c->row_ptr[r + 1] - 1];
        int deg1 = (c->col_ptr[last + 1] - c->col_ptr[last]) == 1;
        if (deg1 && r > 0) break;
        m = r + 1;
    }
    /* p0 */
    {
        int cnt[1024] = {0};
        int v_odd = -1;
        memset(acc, 0, z);
        for (int r = 0; r < m; r++)
            for (int e = c->row_ptr[r]; e < c->row_ptr[r + 1]; e++) {
                if (c->e_col[e] < kb) acc_shift(acc, x + c->e_col[e] * z, c->e_shift[e], z);
                if (c->e_col[e] == kb) cnt[c->e_shift[e]]++;
            }
        for (int v = 0; v < z; v++) if (cnt[v] & 1) { if (v_odd >= 0) { rc = -2; goto done; } v_odd = v; }
        if (v_odd < 0) { rc = -2; goto done; }
        for (int k = 0; k < z; k++) x[kb * z + k] = acc[((k - v_odd) % z + z) % z];
        solved[kb] = 1;
    }
    for (int r = 0; r < rows; r++) {
        if (r == m - 1) continue; /* implied by the sum */
        int unknown = -1;
        memset(acc, 0, z);
        for (int e = c->row_ptr[r]; e < c->row_ptr[r + 1]; e++) {
            int j = c->e_col[e];
            if (solved[j]) acc_shift(acc, x + j * z, c->e_shift[e], z);
            else if (unknown < 0 && c->e_shift[e] == 0) unknown = j;
            else { rc = -3; goto done; }
        }
        if (unknown < 0) continue;
        memcpy(x + unknown * z, acc, z);
        solved[unknown] = 1;
    }
    for (int j = 0; j < c->cols; j++) if (!solved[j]) { rc = -4; goto done; }
    pack_hd(x, N, cw_packed);
done:
    free(x); free(acc); free(solved);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* Philox4x32-10: J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11. */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; round++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1; c3 = (uint32_t)p0; c0 = n0; c2 = n2;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Natural log for x in (0, 1] from +,-,*,/ only, so any IEEE binary32
 * machine without contraction gets the same bits.  x = m * 2^e with
 * m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(f), f = (m-1)/(m+1), by the
 * odd series f + f^3/3 + ... + f^11/11 (|f| <= 0.1716). */
float orc_logf(float x) {
    union { float f; uint32_t u; } v = {x};
    int e = (int)((v.u >> 23) & 0xff) - 127;
    v.u = (v.u & 0x007fffffu) | 0x3f800000u; /* m in [1, 2) */
    float m = v.f;
    if (m > 1.41421356f) { m = m * 0.5f; e = e + 1; }
    const float f = (m - 1.0f) / (m + 1.0f);
    const float f2 = f * f;
    float p = f2 * (1.0f / 11.0f);
    p = p + (1.0f / 9.0f); p = p * f2;
    p = p + (1.0f / 7.0f); p = p * f2;
    p = p + (1.0f / 5.0f); p = p * f2;
    p = p + (1.0f / 3.0f); p = p * f2;
    float lnm = p * f;
    lnm = lnm + f;
    lnm = lnm * 2.0f;
    const float fe = (float)e;
    const float hi = fe * 0.693145752f;          /* ln 2 split: exact product for |e| < 2^9 */
    const float lo = fe * 1.42860677e-06f;
    float r = lo + lnm;
    r = r + hi;
    return r;
}

/* sin/cos of 2*pi*u for u in [0, 1): quadrant and octant reduction on u (exact
 * for u with <= 24 significant bits), then Taylor series to x^9 / x^8 on
 * |x| <= pi/4. */
void orc_sincos2pi(float u, float* s_out, float* c_out) {
    const int q = (int)(u * 4.0f);            /* 0..3 */
    float r = u - (float)q * 0.25f;           /* [0, 0.25) exact */
    int flip = 0;
    if (r > 0.125f) { r = 0.25f - r; flip = 1; } /* exact */
    const float x = r * 6.28318548f;
    const float x2 = x * x;
    float sp = x2 * (-1.0f / 362880.0f);
    sp = sp + (1.0f / 5040.0f); sp = sp * x2;
    sp = sp - (1.0f / 120.0f);  sp = sp * x2;
    sp = sp + (1.0f / 6.0f);    sp = sp * x2;
    float sn = sp * x;
    sn = x - sn;
    float cp = x2 * (1.0f / 40320.0f);
    cp = cp - (1.0f / 720.0f); cp = cp * x2;
    cp = cp + (1.0f / 24.0f);  cp = cp * x2;
    cp = cp - 0.5f;            cp = cp * x2;
    const float cs = cp + 1.0f;
    float s0 = flip ? cs : sn, c0 = flip ? sn : cs;
    float s, c;
    switch (q) {
        case 0: s = s0; c = c0; break;
        case 1: s = c0; c = -s0; break;
        case 2: s = -s0; c = -c0; break;
        default: s = -c0; c = s0; break;
    }
    *s_out = s; *c_out = c;
}

/* Generator stream layout (shared with the GPU generator):
 *   key = (seed_lo, seed_hi); counter = (block, cw_lo, cw_hi, tag)
 *   tag 1: info bits, 128 per block, word w bit b -> info bit 128*block+32*w+b
 *   tag 2: noise, 4 Gaussians per block for transmitted bits 4*block..+3:
 *          (u1, u2) from words 0,1 and 2,3; u1 = ((w>>8)+1)*2^-24 in (0,1],
 *          u2 = (w>>8)*2^-24 in [0,1); rad = sqrt(-2 ln u1);
 *          g0 = rad*cos(2 pi u2), g1 = rad*sin(2 pi u2). */
static inline float u01_open0(uint32_t w) { return (float)((w >> 8) + 1u) * 5.9604645e-08f; }
static inline float u01_open1(uint32_t w) { return (float)(w >> 8) * 5.9604645e-08f; }

int orc_gen_llr(const orc_code* c, int kb, uint64_t seed, uint64_t cw_base, int n_cw,
                const float* sigma, int n_punct_cols, float* llr, uint8_t* cw_packed) {
    const int z = c->z, N = c->cols * z, K = kb * z;
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint8_t* info = (uint8_t*)malloc(K);
    uint8_t* cwp = (uint8_t*)malloc(PACKED_BYTES(N));
    int rc = 0;
    for (int i = 0; i < n_cw; i++) {
        const uint64_t id = cw_base + (uint64_t)i;
        for (int blk = 0; blk * 128 < K; blk++) {
            uint32_t ctr[4] = {(uint32_t)blk, (uint32_t)id, (uint32_t)(id >> 32), 1u}, o[4];
            orc_philox4x32(ctr, key, o);
            for (int b = 0; b < 128 && blk * 128 + b < K; b++) info[blk * 128 + b] = (o[b >> 5] >> (b & 31)) & 1;
        }
        rc = orc_encode(c, kb, info, cwp);
        if (rc) break;
        if (cw_packed) memcpy(cw_packed + (size_t)i * PACKED_BYTES(N), cwp, PACKED_BYTES(N));
        const float sg = sigma[i];
        const float s2 = sg * sg;
        const int p0 = n_punct_cols * z;
        float* out = llr + (size_t)i * N;
        for (int j = 0; j < p0; j++) out[j] = 0.0f;
        for (int t = 0; t * 4 < N - p0; t++) {
            uint32_t ctr[4] = {(uint32_t)t, (uint32_t)id, (uint32_t)(id >> 32), 2u}, o[4];
            orc_philox4x32(ctr, key, o);
            float g[4];
            for (int h = 0; h < 2; h++) {
                const float u1 = u01_open0(o[2 * h]), u2 = u01_open1(o[2 * h + 1]);
                float l = orc_logf(u1);
                l = l * -2.0f;
                const float rad = sqrtf(l);
                float sn, cs;
                orc_sincos2pi(u2, &sn, &cs);
                g[2 * h] = rad * cs;
                g[2 * h + 1] = rad * sn;
            }
            for (int k = 0; k < 4; k++) {
                const int j = p0 + 4 * t + k;
                if (j >= N) break;
                const int bit = (cwp[j >> 3] >> (j & 7)) & 1;
                const float x = bit ? -1.0f : 1.0f;
                const float ns = g[k] * sg;          /* encoding_tools.cpp:62 */
                const float y = x + ns;
                const float y2 = y * 2.0f;           /* encoding_tools.cpp:95 */
                out[j] = y2 / s2;
            }
        }
    }
    free(info); free(cwp);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* Rate matching, TS 38.212 5.4.2.1 (full circular buffer, BPSK).            */
int orc_rm_k0(int bg, int z, int rv) {
    /* k0 = floor(a * Ncb / (n * Z)) * Z with Ncb = n * Z: a per BG and rv */
    static const int a1[4] = {0, 17, 33, 56}, a2[4] = {0, 13, 25, 43};
    if (rv < 0 || rv > 3 || (bg != 1 && bg != 2)) return -1;
    const int n = bg == 1 ? 66 : 50;
    const long ncb = (long)n * z;
    return (int)(((bg == 1 ? a1[rv] : a2[rv]) * ncb) / ((long)n * z)) * z;
}

/* Non-NULL positions form a compressed buffer of Ncb - F entries; bit k is
 * compressed entry (c0 + k) mod (Ncb - F), c0 = k0 with the filler run
 * [f0, f1) of d removed (a k0 inside the run starts right after it). */
int orc_rm_index(int z, int ncb, int kb_z, int k_prime, int k0, int k) {
    const int f0 = k_prime - 2 * z, f1 = kb_z - 2 * z, nf = f1 - f0, nc = ncb - nf;
    const int c0 = k0 < f0 ? k0 : (k0 < f1 ? f0 : k0 - nf);
    const int c = (int)(((long)c0 + k) % nc);
    return c < f0 ? c : c + nf;
}

/* TS 38.212 5.4.2.2: f_{i + j*Qm} = e_{i*E/Qm + j}.  Inverse of position p:
 * i = p mod Qm, j = p div Qm. */
int orc_interleave_src(int e, int qm, int p) {
    if (qm <= 1) return p;
    return (p % qm) * (e / qm) + p / qm;
}

static int valid_qm(int q) { return q == 1 || q == 2 || q == 4 || q == 6 || q == 8 || q == 10; }

int orc_gen_rm_llr(const orc_code* c, int kb, int bg, uint64_t seed, uint64_t cw_base, int n_cw,
                   const float* sigma, const int* k_prime, const int* e, const int* rv, const int* qm,
                   int e_stride, float* llr_e, uint8_t* cw_packed) {
    const int z = c->z, N = c->cols * z, K = kb * z, ncb = N - 2 * z;
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint8_t* info = (uint8_t*)malloc(K);
    uint8_t* cwp = (uint8_t*)malloc(PACKED_BYTES(N));
    int rc = 0;
    for (int i = 0; i < n_cw && !rc; i++) {
        const uint64_t id = cw_base + (uint64_t)i;
        const int kp = k_prime[i] > 0 ? k_prime[i] : K;
        const int q = qm && qm[i] > 0 ? qm[i] : 1;
        if (kp > K || kp < 2 * z || e[i] > e_stride || e[i] < 1 || !valid_qm(q) || e[i] % q) { rc = -1; break; }
        for (int blk = 0; blk * 128 < K; blk++) {
            uint32_t ctr[4] = {(uint32_t)blk, (uint32_t)id, (uint32_t)(id >> 32), 1u}, o[4];
            orc_philox4x32(ctr, key, o);
            for (int b = 0; b < 128 && blk * 128 + b < K; b++) {
                const int pos = blk * 128 + b;
                info[pos] = pos < kp ? (o[b >> 5] >> (b & 31)) & 1 : 0;
            }
        }
        rc = orc_encode(c, kb, info, cwp);
        if (rc) break;
        if (cw_packed) memcpy(cw_packed + (size_t)i * PACKED_BYTES(N), cwp, PACKED_BYTES(N));
        const int k0 = orc_rm_k0(bg, z, rv[i]);
        const float sg = sigma[i], s2 = sg * sg;
        float* out = llr_e + (size_t)i * e_stride;
        for (int t = 0; t * 4 < e[i]; t++) {
            uint32_t ctr[4] = {(uint32_t)t, (uint32_t)id, (uint32_t)(id >> 32), 3u}, o[4];
            orc_philox4x32(ctr, key, o);
            float g[4];
            for (int h = 0; h < 2; h++) {
                const float u1 = u01_open0(o[2 * h]), u2 = u01_open1(o[2 * h + 1]);
                float l = orc_logf(u1);
                l = l * -2.0f;
                const float rad = sqrtf(l);
                float sn, cs;
                orc_sincos2pi(u2, &sn, &cs);
                g[2 * h] = rad * cs;
                g[2 * h + 1] = rad * sn;
            }
            for (int h = 0; h < 4 && 4 * t + h < e[i]; h++) {
                const int p = 4 * t + h; /* transmitted position */
                const int k = orc_interleave_src(e[i], q, p);
                const int j = 2 * z + orc_rm_index(z, ncb, K, kp, k0, k);
                const int bit = (cwp[j >> 3] >> (j & 7)) & 1;
                const float x = bit ? -1.0f : 1.0f;
                const float ns = g[h] * sg;
                const float y = x + ns;
                const float y2 = y * 2.0f;
                out[p] = y2 / s2;
            }
        }
    }
    free(info); free(cwp);
    return rc;
}

int orc_derate_match(const orc_code* c, int kb, int bg, int n_cw, const float* llr_e, int e_stride,
                     const int* k_prime, const int* e, const int* rv, const int* qm, float* llr) {
    const int z = c->z, N = c->cols * z, K = kb * z, ncb = N - 2 * z;
    uint8_t* seen = (uint8_t*)malloc(N);
    for (int i = 0; i < n_cw; i++) {
        const int kp = k_prime[i] > 0 ? k_prime[i] : K;
        const int q = qm && qm[i] > 0 ? qm[i] : 1;
        if (kp > K || kp < 2 * z || e[i] > e_stride || e[i] < 1 || !valid_qm(q) || e[i] % q) {
            free(seen);
            return -1;
        }
        const int k0 = orc_rm_k0(bg, z, rv[i]);
        float* out = llr + (size_t)i * N;
        for (int j = 0; j < N; j++) out[j] = 0.0f;
        for (int j = kp; j < K; j++) out[j] = INFINITY; /* filler: known 0 */
        memset(seen, 0, N);
        for (int k = 0; k < e[i]; k++) {
            const int j = 2 * z + orc_rm_index(z, ncb, K, kp, k0, k);
            /* position of e_k on the wire: k = i*E/Qm + jj -> p = i + jj*Qm */
            const int p = q == 1 ? k : (k / (e[i] / q)) + (k % (e[i] / q)) * q;
            const float v = llr_e[(size_t)i * e_stride + p];
            if (seen[j]) out[j] = out[j] + v;
            else { out[j] = v; seen[j] = 1; }
        }
    }
    free(seen);
    return 0;
}

/* ------------------------------------------------------------------------- */
uint32_t orc_crc(const uint8_t* packed, int n_bits, uint32_t poly, int len) {
    const uint32_t top = 1u << (len - 1), mask = (len == 32) ? 0xffffffffu : ((1u << len) - 1u);
    uint32_t r = 0;
    for (int i = 0; i < n_bits; i++) {
        const uint32_t bit = (packed[i >> 3] >> (i & 7)) & 1u;
        const uint32_t fb = ((r & top) != 0) ^ bit;
        r = (r << 1) & mask;
        if (fb) r ^= poly;
    }
    return r;
}

/* ------------------------------------------------------------------------- */
/* Learned weighted min-sum: forward + adjoint in double precision.          */
static inline double softplus(double x) { return x > 0 ? x + log1p(exp(-x)) : log1p(exp(x)); }
static inline double sigm(double x) { return x >= 0 ? 1.0 / (1.0 + exp(-x)) : exp(x) / (1.0 + exp(x)); }

double orc_wms_loss_grad_f64(const orc_code* c, const float* llr, const uint8_t* cw_packed,
                             int n_cw, int n_iter, const double* w, double* grad, double* app) {
    const int z = c->z, N = c->cols * z, E = c->n_edges, EZ = E * z, T = n_iter;
    double* Q = (double*)malloc(sizeof(double) * (size_t)T * EZ);     /* Q^t */
    double* Lh = (double*)malloc(sizeof(double) * (size_t)(T + 1) * N); /* L^0..L^T */
    double* R = (double*)malloc(sizeof(double) * EZ);
    double* Rn = (double*)malloc(sizeof(double) * EZ);
    double* gL = (double*)malloc(sizeof(double) * N);
    double* gQn = (double*)malloc(sizeof(double) * EZ); /* gQ^{t+1} */
    double* gQ = (double*)malloc(sizeof(double) * EZ);
    const double scale = 1.0 / ((double)T * n_cw * N);
    double loss = 0.0;
    if (grad) memset(grad, 0, sizeof(double) * T * E);
    for (int cw = 0; cw < n_cw; cw++) {
        const uint8_t* bits = cw_packed + (size_t)cw * PACKED_BYTES(N);
        double* L0 = Lh;
        for (int i = 0; i < N; i++) L0[i] = llr[(size_t)cw * N + i];
        memset(R, 0, sizeof(double) * EZ);
        for (int t = 0; t < T; t++) {
            const double* L = Lh + (size_t)t * N;
            double* Lnext = Lh + (size_t)(t + 1) * N;
            double* Qt = Q + (size_t)t * EZ;
            for (int r = 0; r < c->rows; r++) {
                const int e0 = c->row_ptr[r], deg = c->row_ptr[r + 1] - e0;
                for (int s = 0; s < z; s++) {
                    int q_sign = 0, i1 = 0;
                    double m1 = 1000.0, m2 = 1000.0;
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        const double q = L[edge_col(c, e, s)] - R[e * z + s];
                        Qt[e * z + s] = q;
                        const double qa = fabs(q);
                        q_sign ^= (q < 0) << i;
                        if (qa < m1) { m2 = m1; m1 = qa; i1 = i; } else if (qa < m2) m2 = qa;
                    }
                    const int par = __builtin_popcount(q_sign) & 1;
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        const int sb = par ^ ((q_sign >> i) & 1);
                        const double mag = i != i1 ? m1 : m2;
                        Rn[e * z + s] = w[t * E + e] * (sb ? -mag : mag);
                    }
                }
            }
            memcpy(Lnext, L, sizeof(double) * N);
            for (int e = 0; e < E; e++)
                for (int s = 0; s < z; s++) {
                    const int col = edge_col(c, e, s);
                    Lnext[col] += Rn[e * z + s] - R[e * z + s];
                }
            double* tmp = R; R = Rn; Rn = tmp;
            for (int i = 0; i < N; i++) {
                const double y = ((bits[i >> 3] >> (i & 7)) & 1) ? -1.0 : 1.0;
                loss += scale * softplus(-y * Lnext[i]);
            }
        }
        if (app) memcpy(app + (size_t)cw * N, Lh + (size_t)T * N, sizeof(double) * N);
        if (!grad) continue;
        /* adjoint: L^{t+1} = llr + sum_e R^t_e ; Q^t_e = L^t[col] - R^{t-1}_e */
        memset(gQn, 0, sizeof(double) * EZ);
        memset(gL, 0, sizeof(double) * N); /* accumulates dloss/dL^{t+1} from Q^{t+1} */
        for (int t = T - 1; t >= 0; t--) {
            const double* Ln = Lh + (size_t)(t + 1) * N;
            for (int i = 0; i < N; i++) {
                const double y = ((bits[i >> 3] >> (i & 7)) & 1) ? -1.0 : 1.0;
                gL[i] += scale * (-y) * sigm(-y * Ln[i]);
            }
            const double* Qt = Q + (size_t)t * EZ;
            memset(gQ, 0, sizeof(double) * EZ);
            for (int r = 0; r < c->rows; r++) {
                const int e0 = c->row_ptr[r], deg = c->row_ptr[r + 1] - e0;
                for (int s = 0; s < z; s++) {
                    int q_sign = 0, i1 = -1, i2 = -1;
                    double m1 = 1000.0, m2 = 1000.0;
                    for (int i = 0; i < deg; i++) {
                        const double q = Qt[(e0 + i) * z + s];
                        const double qa = fabs(q);
                        q_sign ^= (q < 0) << i;
                        if (qa < m1) { m2 = m1; i2 = i1; m1 = qa; i1 = i; }
                        else if (qa < m2) { m2 = qa; i2 = i; }
                    }
                    const int par = __builtin_popcount(q_sign) & 1;
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        const double gR = gL[edge_col(c, e, s)] - gQn[e * z + s];
                        const int sb = par ^ ((q_sign >> i) & 1);
                        const double sgn = sb ? -1.0 : 1.0;
                        const double mag = i != i1 ? m1 : m2;
                        const int k = i != i1 ? i1 : i2;
                        grad[t * E + e] += gR * sgn * mag;
                        if (k >= 0) {
                            const double qk = Qt[(e0 + k) * z + s];
                            gQ[(e0 + k) * z + s] += gR * w[t * E + e] * sgn * (qk < 0 ? -1.0 : 1.0);
                        }
                    }
                }
            }
            /* Q^t -> L^t (gL for the next step down) and R^{t-1} (via gQn) */
            memset(gL, 0, sizeof(double) * N);
            for (int e = 0; e < E; e++)
                for (int s = 0; s < z; s++) gL[edge_col(c, e, s)] += gQ[e * z + s];
            double* tmp = gQn; gQn = gQ; gQ = tmp;
        }
    }
    free(Q); free(Lh); free(R); free(Rn); free(gL); free(gQn); free(gQ);
    return loss;
}

double orc_wms_layered_loss_grad(const orc_code* c, const float* llr, const uint8_t* cw_packed, int n_cw,
                                 int n_iter, const double* w, double* grad, double* app, int f32_forward);

/* Layered weighted min-sum: forward + adjoint in double precision.  No
 * reference counterpart.  Forward per iteration t, rows ascending:
 *   Q^t_e = A[col] - R^{t-1}_e;  R^t_e = w[t][e] * sign_e * min_e;
 *   A[col] = Q^t_e + R^t_e;  loss += scale * sum_c softplus(-y_c A_c) after t.
 * Adjoint, t = T-1 .. 0, rows descending, with g = dloss/dA and
 * h_e = dloss/dR^t_e from iteration t+1 (Q^{t+1}_e = A - R^t_e):
 *   dR_e = g[col] + h_e;  dQ_e = g[col] + (argmin terms);  g[col] = dQ_e;
 *   h_e <- -dQ_e for iteration t-1. */
double orc_wms_layered_loss_grad_f64(const orc_code* c, const float* llr, const uint8_t* cw_packed,
                                     int n_cw, int n_iter, const double* w, double* grad, double* app) {
    return orc_wms_layered_loss_grad(c, llr, cw_packed, n_cw, n_iter, w, grad, app, 0);
}

/* f32_forward != 0: the forward runs in fp32 with the decoder's rounding
 * (Q = fl(A - R_old), R = +-fl(w * min), A = fl(Q + R)), so its argmins and
 * signs are the GPU forward's exactly; the loss and adjoint stay in double. */
double orc_wms_layered_loss_grad(const orc_code* c, const float* llr, const uint8_t* cw_packed, int n_cw,
                                 int n_iter, const double* w, double* grad, double* app, int f32_forward) {
    const int z = c->z, N = c->cols * z, E = c->n_edges, EZ = E * z, T = n_iter;
    double* Qs = (double*)malloc(sizeof(double) * (size_t)T * EZ); /* Q^t per edge */
    double* Ah = (double*)malloc(sizeof(double) * (size_t)T * N);  /* A after iteration t */
    double* A = (double*)malloc(sizeof(double) * N);
    double* R = (double*)malloc(sizeof(double) * EZ);
    double* g = (double*)malloc(sizeof(double) * N);
    double* h = (double*)malloc(sizeof(double) * EZ);
    double* dR = (double*)malloc(sizeof(double) * 32);
    const double scale = 1.0 / ((double)T * n_cw * N);
    double loss = 0.0;
    if (grad) memset(grad, 0, sizeof(double) * T * E);
    for (int cw = 0; cw < n_cw; cw++) {
        const uint8_t* bits = cw_packed + (size_t)cw * PACKED_BYTES(N);
        for (int i = 0; i < N; i++) A[i] = llr[(size_t)cw * N + i];
        memset(R, 0, sizeof(double) * EZ);
        for (int t = 0; t < T; t++) {
            double* Qt = Qs + (size_t)t * EZ;
            for (int r = 0; r < c->rows; r++) {
                const int e0 = c->row_ptr[r], deg = c->row_ptr[r + 1] - e0;
                for (int s = 0; s < z; s++) {
                    int q_sign = 0, i1 = 0;
                    double m1 = 1000.0, m2 = 1000.0;
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        const double q = f32_forward ? (double)((float)A[edge_col(c, e, s)] - (float)R[e * z + s])
                                                     : A[edge_col(c, e, s)] - R[e * z + s];
                        Qt[e * z + s] = q;
                        const double qa = fabs(q);
                        q_sign ^= (q < 0) << i;
                        if (qa < m1) { m2 = m1; m1 = qa; i1 = i; } else if (qa < m2) m2 = qa;
                    }
                    const int par = __builtin_popcount(q_sign) & 1;
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        const int sb = par ^ ((q_sign >> i) & 1);
                        const double mag = i != i1 ? m1 : m2;
                        if (f32_forward) {
                            const float rm = (float)w[t * E + e] * (float)mag;
                            R[e * z + s] = sb ? -rm : rm;
                            A[edge_col(c, e, s)] = (double)((float)Qt[e * z + s] + (float)R[e * z + s]);
                        } else {
                            R[e * z + s] = w[t * E + e] * (sb ? -mag : mag);
                            A[edge_col(c, e, s)] = Qt[e * z + s] + R[e * z + s];
                        }
                    }
                }
            }
            memcpy(Ah + (size_t)t * N, A, sizeof(double) * N);
            for (int i = 0; i < N; i++) {
                const double y = ((bits[i >> 3] >> (i & 7)) & 1) ? -1.0 : 1.0;
                loss += scale * softplus(-y * A[i]);
            }
        }
        if (app) memcpy(app + (size_t)cw * N, A, sizeof(double) * N);
        if (!grad) continue;
        memset(g, 0, sizeof(double) * N);
        memset(h, 0, sizeof(double) * EZ);
        for (int t = T - 1; t >= 0; t--) {
            const double* At = Ah + (size_t)t * N;
            for (int i = 0; i < N; i++) {
                const double y = ((bits[i >> 3] >> (i & 7)) & 1) ? -1.0 : 1.0;
                g[i] += scale * (-y) * sigm(-y * At[i]);
            }
            const double* Qt = Qs + (size_t)t * EZ;
            for (int r = c->rows - 1; r >= 0; r--) {
                const int e0 = c->row_ptr[r], deg = c->row_ptr[r + 1] - e0;
                for (int s = 0; s < z; s++) {
                    int q_sign = 0, i1 = -1, i2 = -1;
                    double m1 = 1000.0, m2 = 1000.0;
                    for (int i = 0; i < deg; i++) {
                        const double qa = fabs(Qt[(e0 + i) * z + s]);
                        q_sign ^= (Qt[(e0 + i) * z + s] < 0) << i;
                        if (qa < m1) { m2 = m1; i2 = i1; m1 = qa; i1 = i; }
                        else if (qa < m2) { m2 = qa; i2 = i; }
                    }
                    const int par = __builtin_popcount(q_sign) & 1;
                    double to1 = 0.0, to2 = 0.0; /* dloss/dQ at the argmin edges via R */
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        dR[i] = g[edge_col(c, e, s)] + h[e * z + s];
                        const double sgn = (par ^ ((q_sign >> i) & 1)) ? -1.0 : 1.0;
                        grad[t * E + e] += dR[i] * sgn * (i != i1 ? m1 : m2);
                        const double term = dR[i] * w[t * E + e] * sgn;
                        if (i != i1) to1 += term; else to2 += term;
                    }
                    for (int i = 0; i < deg; i++) {
                        const int e = e0 + i;
                        const int col = edge_col(c, e, s);
                        double dq = g[col];
                        const double sq = Qt[e * z + s] < 0 ? -1.0 : 1.0;
                        if (i == i1 && i1 >= 0) dq += to1 * sq;
                        if (i == i2 && i2 >= 0) dq += to2 * sq;
                        g[col] = dq;
                        h[e * z + s] = -dq;
                    }
                }
            }
        }
    }
    free(Qs); free(Ah); free(A); free(R); free(g); free(h); free(dR);
    return loss;
}
