// Learned weighted min-sum: training forward, adjoint and Adam (sm_103a).
//
// No reference counterpart: the reference hard-codes alpha = 0.75
// (src/ldpc_kernels.cu:164,295).  Here R^t_e = w[t][e] * sign_e * min_e with a
// weight per iteration t and base edge e (shared by all Z lifted copies and
// all lifting sizes), the rest of the decoder unchanged: same two-min rules,
// same incremental posterior L^{t+1} = L^t + sum_e (R^t_e - R^{t-1}_e), which
// equals llr + sum_e R^t_e.  Loss (multi-iteration BCE on the posteriors):
//   loss = scale * sum_{t, cw, c} softplus(-y_c * L^{t+1}_c),  y = +1 for bit 0.
//
// Forward: one CTA per codeword group, like the decoder; per iteration it
// stores each lifted row's compressed state (min1, min2, argmin, second
// argmin, Q sign bits: 16 B) and the loss gradient seed dloss/dL^{t+1}.
// Adjoint: walks t = T-1 .. 0 and rebuilds every message from the stored
// state (no per-edge message is kept).  Through R = w * s * min, only the two
// argmin edges of a row receive gradient (min1 feeds every other edge, min2
// feeds the argmin edge), so dloss/dQ of a row is two numbers; they are kept
// per row between steps.  Gradients w.r.t. L are scattered with shared-memory
// atomics (the order of these adds does not matter for a gradient).
//
// Layered schedule (no reference counterpart): rows in ascending order update
// one posterior A in place, Q^t_e = A[col] - R^{t-1}_e, A[col] = Q^t_e + R^t_e.
// Its adjoint walks iterations and rows in reverse with g = dloss/dA in
// shared memory: dloss/dR^t_e = g[col] + h_e, dloss/dQ^t_e = g[col] + (argmin
// terms), g[col] = dloss/dQ^t_e, and h_e = -dloss/dQ^t_e is carried to
// iteration t-1 as the gradient of R^{t-1}_e (per lifted edge, in global
// memory: it does not compress to two numbers per row).
#include <cuda_runtime.h>

#include "nrldpc_internal.h"

namespace nrldpc {
namespace {

constexpr int kHdr = 1024;

__device__ __forceinline__ float max_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}


__device__ __forceinline__ int cw_bit(const uint8_t* cw, int c) { return (cw[c >> 3] >> (c & 7)) & 1; }

// ---- forward ------------------------------------------------------------------------
template <int D, bool LAYERED>
__device__ __forceinline__ void fwd_row(const CodeTable& tab, int e0, uint32_t s, const float* lold,
                                        float* lnew, const float* w_prev, const float* w_cur,
                                        uint4 st, uint4* st_out) {
    const uint32_t z = static_cast<uint32_t>(tab.z);
    uint32_t addr[D];
    float lv[D], rold[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
        const uint32_t ed = tab.edge[e0 + i];
        uint32_t a = s + (ed & 0xffffu);
        if (s >= (ed >> 16)) a -= z;
        addr[i] = a;
        lv[i] = lold[a];
    }
    const float om1 = __uint_as_float(st.x), om2 = __uint_as_float(st.y);
    const uint32_t oq = st.z >> 8;
    const int oidx = static_cast<int>(st.z & 31u);
    const uint32_t opar = static_cast<uint32_t>(__popc(oq) & 1);
    float m1 = 1000.0f, m2 = 1000.0f;
    int i1 = 0, i2 = 31;
    uint32_t qmask = 0;
#pragma unroll
    for (int i = 0; i < D; i++) {
        const float mag = __fmul_rn(w_prev[e0 + i], i == oidx ? om2 : om1);
        const uint32_t sb = (opar ^ (oq >> i)) & 1u;
        rold[i] = __uint_as_float(__float_as_uint(mag) ^ (sb << 31));
        const float q = __fsub_rn(lv[i], rold[i]);
        if (LAYERED) rold[i] = q;  // the layered update needs Q, not R_old
        const float qa = fabsf(q);
        if (q < 0.0f) qmask |= 1u << i;
        const bool p1 = qa < m1, p2 = qa < m2;
        i2 = p1 ? i1 : (p2 ? i : i2);
        i1 = p1 ? i : i1;
        const float mx = max_nan(m1, qa);
        m1 = fminf(m1, qa);
        m2 = fminf(m2, mx);
    }
    const uint32_t par = static_cast<uint32_t>(__popc(qmask) & 1);
    float nv[D];
#pragma unroll
    for (int i = 0; i < D; i++) nv[i] = LAYERED ? 0.0f : lnew[addr[i]];
#pragma unroll
    for (int i = 0; i < D; i++) {
        const float mag = __fmul_rn(w_cur[e0 + i], i == i1 ? m2 : m1);
        const uint32_t sb = (par ^ (qmask >> i)) & 1u;
        const float rn = __uint_as_float(__float_as_uint(mag) ^ (sb << 31));
        if (LAYERED)
            lnew[addr[i]] = __fadd_rn(rold[i], rn);  // A = Q + R_new
        else
            lnew[addr[i]] = __fadd_rn(nv[i], __fsub_rn(rn, rold[i]));
    }
    *st_out = make_uint4(__float_as_uint(m1), __float_as_uint(m2),
                         static_cast<uint32_t>(i1) | (qmask << 8), static_cast<uint32_t>(i2));
}

template <bool LAYERED>
__device__ __forceinline__ void fwd_dispatch(int deg, const CodeTable& tab, int e0, uint32_t s,
                                             const float* lold, float* lnew, const float* wp,
                                             const float* wc, uint4 st, uint4* st_out) {
    switch (deg) {
#define NRLDPC_FWD_CASE(D) \
    case D: fwd_row<D, LAYERED>(tab, e0, s, lold, lnew, wp, wc, st, st_out); break;
        NRLDPC_FWD_CASE(1) NRLDPC_FWD_CASE(2) NRLDPC_FWD_CASE(3) NRLDPC_FWD_CASE(4)
        NRLDPC_FWD_CASE(5) NRLDPC_FWD_CASE(6) NRLDPC_FWD_CASE(7) NRLDPC_FWD_CASE(8)
        NRLDPC_FWD_CASE(9) NRLDPC_FWD_CASE(10) NRLDPC_FWD_CASE(11) NRLDPC_FWD_CASE(12)
        NRLDPC_FWD_CASE(13) NRLDPC_FWD_CASE(14) NRLDPC_FWD_CASE(15) NRLDPC_FWD_CASE(16)
        NRLDPC_FWD_CASE(17) NRLDPC_FWD_CASE(18) NRLDPC_FWD_CASE(19)
#undef NRLDPC_FWD_CASE
        default: break;
    }
}

struct WmsArgs {
    const float* llr;
    const uint8_t* cw;       // transmitted codewords (packed), the training targets
    const float* weights;    // [T][E]
    uint4* states;           // [T][n_cw][rows*Z]
    float* gseed;            // [T][n_cw][n_bp]
    uint4* gq;               // [grid*cpb][rows*Z] adjoint per-row dloss/dQ (flooding backward)
    float* gh;               // [grid*cpb][E*Z] adjoint per-edge dloss/dR (layered backward)
    double* loss;            // forward: += loss
    double* grad;            // backward: += dloss/dw [T][E]
    float* app;              // optional L^T
    int* work_counter;
    int* error_flag;
    int n_cw, T, cpb, n_groups;
    float scale;
};

template <bool LAYERED>
__global__ void __launch_bounds__(kMaxThreads, 1)
    wms_forward_kernel(const __grid_constant__ CodeTable tab, const __grid_constant__ WmsArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_group = reinterpret_cast<int*>(smem);
    float* s_red = reinterpret_cast<float*>(smem + 64);  // warp partial losses
    float* wbuf = reinterpret_cast<float*>(smem + kHdr);  // [2][E] previous / current weights
    float* bufs = wbuf + 2 * kMaxEdges;
    const int z = tab.z, n = tab.n_bp, cpb = a.cpb, rows = tab.rows, E = tab.n_edges;
    const int tid = threadIdx.x, slot = tid / z;
    const uint32_t s = static_cast<uint32_t>(tid - slot * z);
    const bool valid = slot < cpb;
    for (;;) {
        if (tid == 0) *s_group = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int g = *s_group;
        if (g >= a.n_groups) break;
        const int cw = g * cpb + slot;
        const bool act = valid && cw < a.n_cw;
        float* lold = bufs + static_cast<size_t>(slot) * n;
        float* lnew = LAYERED ? lold : bufs + static_cast<size_t>(cpb + slot) * n;
        // this thread's codeword bits at positions s, s + Z, s + 2Z, ... (at
        // most kMaxCols of them) as a 128-bit mask, read once per group
        uint64_t ybits0 = 0, ybits1 = 0;
        if (act) {
            const float4* src = reinterpret_cast<const float4*>(a.llr + static_cast<size_t>(cw) * n);
#pragma unroll 4
            for (int k = static_cast<int>(s); k < n / 4; k += z) reinterpret_cast<float4*>(lold)[k] = src[k];
            const uint8_t* bits = a.cw + static_cast<size_t>(cw) * tab.packed_bytes;
#pragma unroll 4
            for (int k = 0; k < tab.cols; k++) {
                const uint64_t b = static_cast<uint64_t>(cw_bit(bits, static_cast<int>(s) + k * z));
                if (k < 64)
                    ybits0 |= b << k;
                else
                    ybits1 |= b << (k - 64);
            }
        }
        float loss_part = 0.0f;
        for (int t = 0; t < a.T; t++) {
            for (int e = tid; e < E; e += blockDim.x) {
                wbuf[e] = t == 0 ? 0.0f : a.weights[(t - 1) * E + e];
                wbuf[kMaxEdges + e] = a.weights[t * E + e];
            }
            __syncthreads();
            if (act && !LAYERED)
                for (int k = static_cast<int>(s); k < n / 4; k += z)
                    reinterpret_cast<float4*>(lnew)[k] = reinterpret_cast<const float4*>(lold)[k];
            __syncthreads();
            const size_t cw_off = static_cast<size_t>(act ? cw : 0) * rows * z;
            const uint4* st_prev =
                a.states + static_cast<size_t>(t > 0 ? t - 1 : 0) * a.n_cw * rows * z + cw_off;
            uint4* st_cur = a.states + static_cast<size_t>(t) * a.n_cw * rows * z + cw_off;
            // previous iteration's state of row r+2 requested while row r runs
            auto fetch = [&](int r) -> uint4 {
                return (act && t > 0 && r < rows) ? __ldcg(st_prev + r * z + s) : make_uint4(0u, 0u, 0u, 0u);
            };
            uint4 p0 = fetch(0), p1 = fetch(1);
            for (int r = 0; r < rows; r++) {
                const uint4 p2 = fetch(r + 2);
                if (act)
                    fwd_dispatch<LAYERED>(tab.row_deg[r], tab, tab.row_ptr[r], s, lold, lnew, wbuf,
                                          wbuf + kMaxEdges, p0, st_cur + r * z + s);
                p0 = p1;
                p1 = p2;
                if (tab.sync_after[r]) __syncthreads();
            }
            // loss term and its gradient seed at L^{t+1}
            if (act) {
                float* seed = a.gseed + (static_cast<size_t>(t) * a.n_cw + cw) * n;
                uint64_t y0 = ybits0, y1 = ybits1;
                // softplus(zz) = max(zz, 0) + log1p(e) and sigmoid(zz) =
                // 1/(1 + e) (zz >= 0) or e/(1 + e) (zz < 0), e = exp(-|zz|):
                // one exponential per position
#pragma unroll 4
                for (int c = static_cast<int>(s); c < n; c += z) {
                    const float y = (y0 & 1u) ? -1.0f : 1.0f;
                    y0 = (y0 >> 1) | (y1 << 63);
                    y1 >>= 1;
                    const float zz = -y * lnew[c];
                    const float e = expf(-fabsf(zz));
                    loss_part += fmaxf(zz, 0.0f) + log1pf(e);
                    const float r = __frcp_rn(1.0f + e);
                    seed[c] = a.scale * (-y) * (zz >= 0.0f ? r : e * r);
                }
            }
            float* tmp = lold;
            lold = lnew;
            lnew = tmp;
        }
        if (act && a.app)
            for (int c = static_cast<int>(s); c < n; c += z) a.app[static_cast<size_t>(cw) * n + c] = lold[c];
        // block reduction of the loss
        for (int off = 16; off > 0; off >>= 1) loss_part += __shfl_xor_sync(0xffffffffu, loss_part, off);
        if ((tid & 31) == 0) s_red[tid >> 5] = loss_part;
        __syncthreads();
        if (tid == 0) {
            double tot = 0.0;
            for (int w = 0; w < (blockDim.x + 31) / 32; w++) tot += s_red[w];
            atomicAdd(a.loss, tot * static_cast<double>(a.scale));
        }
        __syncthreads();
    }
}

// Sums v[i] over the 32 lanes of the warp for every i < D and adds the sums
// to acc[i] (shared memory), one atomic per edge: a transposing butterfly
// (at each level a lane keeps one half of its values and trades the other
// half with its partner, P - 1 shuffles for P = D rounded up to a power of
// two) followed by a plain reduction over the remaining lane bits, instead of
// a 5-shuffle reduction per value.
template <int D>
__device__ __forceinline__ void warp_sum_to(float (&v)[D], float* acc) {
    constexpr int P = D <= 1 ? 1 : D <= 2 ? 2 : D <= 4 ? 4 : D <= 8 ? 8 : D <= 16 ? 16 : 32;
    constexpr int LOGP = P == 1 ? 0 : P == 2 ? 1 : P == 4 ? 2 : P == 8 ? 3 : P == 16 ? 4 : 5;
    const int lane = static_cast<int>(threadIdx.x & 31u);
    float w[P];
#pragma unroll
    for (int j = 0; j < P; j++) w[j] = j < D ? v[j] : 0.0f;
#pragma unroll
    for (int lvl = 0; lvl < LOGP; lvl++) {
        const int k = P >> (lvl + 1);  // values kept after this level
        const int o = 16 >> lvl;       // partner lane distance
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < k; j++) {
            const float send = up ? w[j] : w[j + k];
            const float keep = up ? w[j + k] : w[j];
            w[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
#pragma unroll
    for (int o = 16 >> LOGP; o > 0; o >>= 1) w[0] += __shfl_xor_sync(0xffffffffu, w[0], o);
    // lane L now holds the sum for value L >> (5 - LOGP)
    if ((lane & ((32 >> LOGP) - 1)) == 0) {
        const int i = lane >> (5 - LOGP);
        if (i < D) atomicAdd(&acc[i], w[0]);
    }
}

// ---- adjoint ------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void bwd_row(const CodeTable& tab, int e0, uint32_t s, bool act,
                                        const float* gl, float* gl_next, const float* w_cur,
                                        float* gw_acc, uint4 st, uint4 gin, uint4* gq_io, bool scatter) {
    const uint32_t z = static_cast<uint32_t>(tab.z);
    const float m1 = __uint_as_float(st.x), m2 = __uint_as_float(st.y);
    const int i1 = static_cast<int>(st.z & 31u), i2 = static_cast<int>(st.w);
    const uint32_t q = st.z >> 8;
    const uint32_t par = static_cast<uint32_t>(__popc(q) & 1);
    const float g1n = __uint_as_float(gin.x), g2n = __uint_as_float(gin.y);
    const int j1 = static_cast<int>(gin.z), j2 = static_cast<int>(gin.w);
    uint32_t ad1 = 0, ad2 = 0;  // columns of the two argmin edges
    float acc1 = 0.0f, acc2 = 0.0f;
    float gwv[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
        const uint32_t ed = tab.edge[e0 + i];
        uint32_t a = s + (ed & 0xffffu);
        if (s >= (ed >> 16)) a -= z;
        ad1 = i == i1 ? a : ad1;
        ad2 = i == i2 ? a : ad2;
        float gr = 0.0f;
        if (act) gr = gl[a] - (i == j1 ? g1n : (i == j2 ? g2n : 0.0f));
        const float sg = ((par ^ (q >> i)) & 1u) ? -1.0f : 1.0f;
        const float mag = i == i1 ? m2 : m1;
        gwv[i] = act ? gr * sg * mag : 0.0f;
        const float t = gr * w_cur[e0 + i] * sg;
        if (i == i1) acc2 = t;
        else acc1 += t;
    }
    warp_sum_to<D>(gwv, gw_acc + e0);
    float g1 = 0.0f, g2 = 0.0f;
    if (act) {
        if (m1 < 1000.0f) g1 = acc1 * (((q >> i1) & 1u) ? -1.0f : 1.0f);
        if (i2 < D && m2 < 1000.0f) g2 = acc2 * (((q >> i2) & 1u) ? -1.0f : 1.0f);
        if (scatter) {
            if (m1 < 1000.0f) atomicAdd(&gl_next[ad1], g1);
            if (i2 < D && m2 < 1000.0f) atomicAdd(&gl_next[ad2], g2);
        }
        *gq_io = make_uint4(__float_as_uint(g1), __float_as_uint(g2), static_cast<uint32_t>(i1),
                            static_cast<uint32_t>(i2 < D ? i2 : 31));
    }
}

__device__ __forceinline__ void bwd_dispatch(int deg, const CodeTable& tab, int e0, uint32_t s,
                                             bool act, const float* gl, float* gln, const float* wc,
                                             float* gw_acc, uint4 st, uint4 gin, uint4* gq, bool scatter) {
    switch (deg) {
#define NRLDPC_BWD_CASE(D) \
    case D: bwd_row<D>(tab, e0, s, act, gl, gln, wc, gw_acc, st, gin, gq, scatter); break;
        NRLDPC_BWD_CASE(1) NRLDPC_BWD_CASE(2) NRLDPC_BWD_CASE(3) NRLDPC_BWD_CASE(4)
        NRLDPC_BWD_CASE(5) NRLDPC_BWD_CASE(6) NRLDPC_BWD_CASE(7) NRLDPC_BWD_CASE(8)
        NRLDPC_BWD_CASE(9) NRLDPC_BWD_CASE(10) NRLDPC_BWD_CASE(11) NRLDPC_BWD_CASE(12)
        NRLDPC_BWD_CASE(13) NRLDPC_BWD_CASE(14) NRLDPC_BWD_CASE(15) NRLDPC_BWD_CASE(16)
        NRLDPC_BWD_CASE(17) NRLDPC_BWD_CASE(18) NRLDPC_BWD_CASE(19)
#undef NRLDPC_BWD_CASE
        default: break;
    }
}

__global__ void __launch_bounds__(kMaxThreads, 1)
    wms_backward_kernel(const __grid_constant__ CodeTable tab, const __grid_constant__ WmsArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_group = reinterpret_cast<int*>(smem);
    float* wcur = reinterpret_cast<float*>(smem + kHdr);  // [E]
    float* gw_acc = wcur + kMaxEdges;                     // [E]
    float* bufs = gw_acc + kMaxEdges;
    const int z = tab.z, n = tab.n_bp, cpb = a.cpb, rows = tab.rows, E = tab.n_edges;
    const int tid = threadIdx.x, slot = tid / z;
    const uint32_t s = static_cast<uint32_t>(tid - slot * z);
    const bool valid = slot < cpb;
    uint4* gq = a.gq + (static_cast<size_t>(blockIdx.x) * cpb + (valid ? slot : 0)) * rows * z;
    for (;;) {
        if (tid == 0) *s_group = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int g = *s_group;
        if (g >= a.n_groups) break;
        const int cw = g * cpb + slot;
        const bool act = valid && cw < a.n_cw;
        float* gl = bufs + static_cast<size_t>(slot) * n;           // dloss/dL^{t+1}
        float* gln = bufs + static_cast<size_t>(cpb + slot) * n;    // dloss/dL^t
        if (act) {
            const float* seed = a.gseed + (static_cast<size_t>(a.T - 1) * a.n_cw + cw) * n;
#pragma unroll 4
            for (int c = static_cast<int>(s); c < n; c += z) gl[c] = seed[c];
            for (int k = 0; k < rows; k++) gq[k * z + s] = make_uint4(0u, 0u, 31u, 31u);
        }
        for (int t = a.T - 1; t >= 0; t--) {
            for (int e = tid; e < E; e += blockDim.x) {
                wcur[e] = a.weights[t * E + e];
                gw_acc[e] = 0.0f;
            }
            if (act) {
                if (t > 0) {
                    const float* seed = a.gseed + (static_cast<size_t>(t - 1) * a.n_cw + cw) * n;
#pragma unroll 4
                    for (int c = static_cast<int>(s); c < n; c += z) gln[c] = seed[c];
                }
            }
            __syncthreads();
            const uint4* st = a.states + (static_cast<size_t>(t) * a.n_cw + (act ? cw : 0)) * rows * z;
            // state and per-row dloss/dQ of row r+2 requested while row r runs
            auto fetch = [&](int r, uint4& sv, uint4& gv) {
                sv = make_uint4(0u, 0u, 0u, 31u);
                gv = make_uint4(0u, 0u, 31u, 31u);
                if (act && r < rows) {
                    sv = __ldcg(st + r * z + s);
                    gv = __ldcg(gq + r * z + s);
                }
            };
            uint4 s0, g0, s1, g1;
            fetch(0, s0, g0);
            fetch(1, s1, g1);
            for (int r = 0; r < rows; r++) {
                uint4 s2, g2;
                fetch(r + 2, s2, g2);
                bwd_dispatch(tab.row_deg[r], tab, tab.row_ptr[r], s, act, gl, gln, wcur, gw_acc, s0, g0,
                             gq + r * z + s, t > 0);
                s0 = s1;
                g0 = g1;
                s1 = s2;
                g1 = g2;
            }
            __syncthreads();
            for (int e = tid; e < E; e += blockDim.x)
                if (gw_acc[e] != 0.0f) atomicAdd(&a.grad[t * E + e], static_cast<double>(gw_acc[e]));
            float* tmp = gl;
            gl = gln;
            gln = tmp;
            __syncthreads();
        }
    }
}

template <int D>
__device__ __forceinline__ void bwd_layered_row(const CodeTable& tab, int e0, uint32_t s, bool act, float* g,
                                                const float* w_cur, float* gw_acc, uint4 st, float* gh_row,
                                                bool has_h, bool write_h) {
    const uint32_t z = static_cast<uint32_t>(tab.z);
    const float m1 = __uint_as_float(st.x), m2 = __uint_as_float(st.y);
    const int i1 = static_cast<int>(st.z & 31u), i2 = static_cast<int>(st.w);
    const uint32_t q = st.z >> 8;
    const uint32_t par = static_cast<uint32_t>(__popc(q) & 1);
    uint32_t ad[D];
    float ga[D];
    float gwv[D];
    float to1 = 0.0f, to2 = 0.0f;  // dloss/dQ at the argmin edges through R
#pragma unroll
    for (int i = 0; i < D; i++) {
        const uint32_t ed = tab.edge[e0 + i];
        uint32_t a = s + (ed & 0xffffu);
        if (s >= (ed >> 16)) a -= z;
        ad[i] = a;
        float dr = 0.0f;
        ga[i] = 0.0f;
        if (act) {
            ga[i] = g[a];
            dr = ga[i] + (has_h ? gh_row[i * z] : 0.0f);
        }
        const float sg = ((par ^ (q >> i)) & 1u) ? -1.0f : 1.0f;
        const float mag = i == i1 ? m2 : m1;
        gwv[i] = act ? dr * sg * mag : 0.0f;
        const float t = dr * w_cur[e0 + i] * sg;
        if (i == i1) to2 = t;
        else to1 += t;
    }
    warp_sum_to<D>(gwv, gw_acc + e0);
    if (!act) return;
    const float g1 = m1 < 1000.0f ? to1 * (((q >> i1) & 1u) ? -1.0f : 1.0f) : 0.0f;
    const float g2 = (i2 < D && m2 < 1000.0f) ? to2 * (((q >> i2) & 1u) ? -1.0f : 1.0f) : 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        float dq = ga[i];
        if (i == i1) dq += g1;
        if (i == i2) dq += g2;
        if (i == i1 || i == i2) g[ad[i]] = dq;  // dloss/dA before this row
        if (write_h) gh_row[i * z] = -dq;      // dloss/dR^{t-1}
    }
}

__device__ __forceinline__ void bwd_layered_dispatch(int deg, const CodeTable& tab, int e0, uint32_t s, bool act,
                                                     float* g, const float* wc, float* gw_acc, uint4 st,
                                                     float* gh_row, bool has_h, bool write_h) {
    switch (deg) {
#define NRLDPC_BWDL_CASE(D) \
    case D: bwd_layered_row<D>(tab, e0, s, act, g, wc, gw_acc, st, gh_row, has_h, write_h); break;
        NRLDPC_BWDL_CASE(1) NRLDPC_BWDL_CASE(2) NRLDPC_BWDL_CASE(3) NRLDPC_BWDL_CASE(4)
        NRLDPC_BWDL_CASE(5) NRLDPC_BWDL_CASE(6) NRLDPC_BWDL_CASE(7) NRLDPC_BWDL_CASE(8)
        NRLDPC_BWDL_CASE(9) NRLDPC_BWDL_CASE(10) NRLDPC_BWDL_CASE(11) NRLDPC_BWDL_CASE(12)
        NRLDPC_BWDL_CASE(13) NRLDPC_BWDL_CASE(14) NRLDPC_BWDL_CASE(15) NRLDPC_BWDL_CASE(16)
        NRLDPC_BWDL_CASE(17) NRLDPC_BWDL_CASE(18) NRLDPC_BWDL_CASE(19)
#undef NRLDPC_BWDL_CASE
        default: break;
    }
}

__global__ void __launch_bounds__(kMaxThreads, 1)
    wms_backward_layered_kernel(const __grid_constant__ CodeTable tab, const __grid_constant__ WmsArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_group = reinterpret_cast<int*>(smem);
    float* wcur = reinterpret_cast<float*>(smem + kHdr);  // [E]
    float* gw_acc = wcur + kMaxEdges;                     // [E]
    float* bufs = gw_acc + kMaxEdges;
    const int z = tab.z, n = tab.n_bp, cpb = a.cpb, rows = tab.rows, E = tab.n_edges;
    const int tid = threadIdx.x, slot = tid / z;
    const uint32_t s = static_cast<uint32_t>(tid - slot * z);
    const bool valid = slot < cpb;
    float* gh = a.gh + (static_cast<size_t>(blockIdx.x) * cpb + (valid ? slot : 0)) * E * z;
    for (;;) {
        if (tid == 0) *s_group = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int grp = *s_group;
        if (grp >= a.n_groups) break;
        const int cw = grp * cpb + slot;
        const bool act = valid && cw < a.n_cw;
        float* g = bufs + static_cast<size_t>(valid ? slot : 0) * n;  // dloss/dA
        if (act)
            for (int c = static_cast<int>(s); c < n; c += z) g[c] = 0.0f;
        for (int t = a.T - 1; t >= 0; t--) {
            for (int e = tid; e < E; e += blockDim.x) {
                wcur[e] = a.weights[t * E + e];
                gw_acc[e] = 0.0f;
            }
            if (act) {
                const float* seed = a.gseed + (static_cast<size_t>(t) * a.n_cw + cw) * n;
#pragma unroll 4
                for (int c = static_cast<int>(s); c < n; c += z) g[c] += seed[c];
            }
            __syncthreads();
            const uint4* st = a.states + (static_cast<size_t>(t) * a.n_cw + (act ? cw : 0)) * rows * z;
            auto fetch = [&](int r) -> uint4 {  // state of row r-2 requested while row r runs
                return (act && r >= 0) ? __ldcg(st + r * z + s) : make_uint4(0u, 0u, 0u, 31u);
            };
            uint4 s0 = fetch(rows - 1), s1 = fetch(rows - 2);
            for (int r = rows - 1; r >= 0; r--) {
                const uint4 s2 = fetch(r - 2);
                bwd_layered_dispatch(tab.row_deg[r], tab, tab.row_ptr[r], s, act, g, wcur, gw_acc, s0,
                                     gh + static_cast<size_t>(tab.row_ptr[r]) * z + s, t < a.T - 1, t > 0);
                s0 = s1;
                s1 = s2;
                if (r > 0 && tab.sync_after[r - 1]) __syncthreads();
            }
            __syncthreads();
            for (int e = tid; e < E; e += blockDim.x)
                if (gw_acc[e] != 0.0f) atomicAdd(&a.grad[t * E + e], static_cast<double>(gw_acc[e]));
            __syncthreads();
        }
    }
}

__global__ void adam_kernel(int n, float* w, const double* grad, float* m, float* v, float lr,
                            float b1, float b2, float eps, float c1, float c2, float w_min) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = static_cast<float>(grad[i]);
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float upd = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = fmaxf(w[i] - upd, w_min);
}

}  // namespace

size_t wms_smem_bytes(const CodeTable& tab, int cpb) {
    return kHdr + 2 * kMaxEdges * sizeof(float) + 2 * static_cast<size_t>(cpb) * tab.n_bp * sizeof(float);
}

cudaError_t wms_kernel_attributes(size_t smem) {
    const void* ks[4] = {reinterpret_cast<const void*>(&wms_forward_kernel<false>),
                         reinterpret_cast<const void*>(&wms_forward_kernel<true>),
                         reinterpret_cast<const void*>(&wms_backward_kernel),
                         reinterpret_cast<const void*>(&wms_backward_layered_kernel)};
    for (const void* k : ks) {
        cudaError_t e =
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_wms(bool backward, bool layered, const CodeTable& tab, const float* llr, const uint8_t* cw,
                       const float* weights, uint4* states, float* gseed, uint4* gq, float* gh, double* loss,
                       double* grad, float* app, int* counters, int n_cw, int T, int cpb, int grid,
                       int threads, size_t smem, float scale, cudaStream_t stream) {
    WmsArgs a{};
    a.llr = llr;
    a.cw = cw;
    a.weights = weights;
    a.states = states;
    a.gseed = gseed;
    a.gq = gq;
    a.gh = gh;
    a.loss = loss;
    a.grad = grad;
    a.app = app;
    a.work_counter = counters;
    a.error_flag = counters + 1;
    a.n_cw = n_cw;
    a.T = T;
    a.cpb = cpb;
    a.n_groups = (n_cw + cpb - 1) / cpb;
    a.scale = scale;
    grid = grid < a.n_groups ? grid : a.n_groups;
    if (backward && layered)
        wms_backward_layered_kernel<<<grid, threads, smem, stream>>>(tab, a);
    else if (backward)
        wms_backward_kernel<<<grid, threads, smem, stream>>>(tab, a);
    else if (layered)
        wms_forward_kernel<true><<<grid, threads, smem, stream>>>(tab, a);
    else
        wms_forward_kernel<false><<<grid, threads, smem, stream>>>(tab, a);
    return cudaGetLastError();
}

cudaError_t launch_adam(int n, float* w, const double* grad, float* m, float* v, int step, float lr,
                        float b1, float b2, float eps, float w_min, cudaStream_t stream) {
    const float c1 = 1.0f - powf(b1, static_cast<float>(step));
    const float c2 = 1.0f - powf(b2, static_cast<float>(step));
    adam_kernel<<<(n + 255) / 256, 256, 0, stream>>>(n, w, grad, m, v, lr, b1, b2, eps, c1, c2, w_min);
    return cudaGetLastError();
}

}  // namespace nrldpc
