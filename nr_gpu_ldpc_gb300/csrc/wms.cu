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

// Per-thread asynchronous copies global -> shared (each thread waits only
// for its own groups; the sources are in-bounds device memory, so every
// copy completes).
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The BG2 flooding adjoint stages each row's state, per-row dloss/dQ and
// suffix seed through a per-thread ring of kRing rows in shared memory
// (kRing - 1 rows requested ahead: the rows come from DRAM, where two rows
// of look-ahead in registers left the kernel waiting on loads).
constexpr int kRing = 4;
constexpr size_t kRingBytes = static_cast<size_t>(kRing) * kMaxThreads * (16 + 16 + 4);

// Stored state of one lifted row after iteration t (16 B): min1, min2,
// info = i1 | i2 << 5 | Q sign bits << 10 (i2 = 31: no second argmin), and
// the posterior of the row's suffix column at this sub-row after the
// iteration (unused in rows without one).  Suffix columns (degree 1, the last
// edge of their row: 5G NR's extension parity) are touched by one row only,
// so their posteriors and loss terms stay with that row's thread and only the
// core columns live in shared memory.
__device__ __forceinline__ uint32_t pack_info(int i1, int i2, uint32_t qmask) {
    return static_cast<uint32_t>(i1) | (static_cast<uint32_t>(i2) << 5) | (qmask << 10);
}

// Position (c*Z + (s + V) mod Z) of sub-row s on edge word ed.
__device__ __forceinline__ uint32_t edge_at(uint32_t ed, uint32_t s, uint32_t z) {
    uint32_t a = s + (ed & 0xffffu);
    if (s >= (ed >> 16)) a -= z;
    return a;
}

// softplus(zz) = max(zz, 0) + log1p(e) and sigmoid(zz) = 1/(1 + e) (zz >= 0)
// or e/(1 + e) (zz < 0), e = exp(-|zz|): one exponential per position, with
// the fast hardware exponential, logarithm and division (relative errors of
// about 1e-6, far below what the loss and its gradient are used for);
// log1p(e) = log(u) * e / (u - 1) with u = 1 + e (Goldberg's correction:
// u - 1 is exact, the ratio restores what rounding u lost; e itself when u
// rounds to 1).  Adds the position's loss to *loss and returns its seed.
__device__ __forceinline__ float loss_term(float L, bool bit1, float scale, float* loss) {
    const float y = bit1 ? -1.0f : 1.0f;
    const float zz = -y * L;
    const float e = __expf(-fabsf(zz));
    const float u = 1.0f + e;
    const float l1p = u == 1.0f ? e : __logf(u) * __fdividef(e, u - 1.0f);
    *loss += fmaxf(zz, 0.0f) + l1p;
    const float r = __fdividef(1.0f, u);
    return scale * (-y) * (zz >= 0.0f ? r : e * r);
}

// ---- forward ------------------------------------------------------------------------
// Forward weights of the iteration in shared memory, one padded row of kWPad
// floats per base row (previous iteration's rows, then the current ones), so
// a row's weights come in as 128-bit loads: [2][kMaxRows][kWPad].
constexpr int kWPad = 20;
constexpr int kFwdWeightFloats = 2 * kMaxRows * kWPad;

// Weight i of a padded row held as float4s (i is constant after unrolling).
__device__ __forceinline__ float wsel(const float4* w, int i) {
    const float4 v = w[i >> 2];
    const int c = i & 3;
    return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}

// sfx: the row's last edge is a suffix column, its posterior is st.w (read)
// and the stored state's w (written); its loss term and seed are taken here.
// Signs: R_old_i's is bit i of the previous Q signs XOR their parity; Q_i's
// is the sign bit of Q_i + 0 ((Q < 0): -0 gives +0, a NaN result is the
// canonical positive NaN), collected by a funnel shift (edge i at bit
// D-1-i) and bit-reversed into the stored order (edge i at bit i).
template <int D, bool LAYERED>
__device__ __forceinline__ void fwd_row(const CodeTable& tab, int e0, uint32_t s, const float* lold,
                                        float* lnew, const float4* w_prev, const float4* w_cur,
                                        uint4 st, uint4* st_out, bool sfx, bool ybit, float* seed_t,
                                        float scale, float* loss) {
    constexpr int LAST = D - 1;
    const uint32_t z = static_cast<uint32_t>(tab.z);
    uint32_t addr[D];
    float lv[D], rold[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
        addr[i] = edge_at(tab.edge[e0 + i], s, z);
        lv[i] = (i == LAST && sfx) ? __uint_as_float(st.w) : lold[addr[i]];
    }
    const float om1 = __uint_as_float(st.x), om2 = __uint_as_float(st.y);
    const uint32_t oq = st.z >> 10;
    const int oidx = static_cast<int>(st.z & 31u);
    const uint32_t orsign = oq ^ (0u - (static_cast<uint32_t>(__popc(oq)) & 1u));  // R_old_i's sign at bit i
    float m1 = 1000.0f, m2 = 1000.0f;
    int i1 = 0, i2 = 31;
    uint32_t qrev = 0;
#pragma unroll
    for (int i = 0; i < D; i++) {
        const float mag = __fmul_rn(wsel(w_prev, i), i == oidx ? om2 : om1);
        rold[i] = __uint_as_float(__float_as_uint(mag) ^ ((orsign << (31 - i)) & 0x80000000u));
        const float q = __fsub_rn(lv[i], rold[i]);
        if (LAYERED) rold[i] = q;  // the layered update needs Q, not R_old
        const float qa = fabsf(q);
        qrev = __funnelshift_l(__float_as_uint(__fadd_rn(q, 0.0f)), qrev, 1);
        const bool p1 = qa < m1, p2 = qa < m2;
        i2 = p1 ? i1 : (p2 ? i : i2);
        i1 = p1 ? i : i1;
        const float mx = max_nan(m1, qa);
        m1 = fminf(m1, qa);
        m2 = fminf(m2, mx);
    }
    const uint32_t qmask = __brev(qrev) >> (32 - D);  // Q_i's sign at bit i
    const uint32_t rsign = qmask ^ (0u - (static_cast<uint32_t>(__popc(qmask)) & 1u));  // R_new_i's
    float nv[D];
#pragma unroll
    for (int i = 0; i < D; i++) nv[i] = (LAYERED || (i == LAST && sfx)) ? lv[i] : lnew[addr[i]];
    float sfx_new = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
        const float mag = __fmul_rn(wsel(w_cur, i), i == i1 ? m2 : m1);
        const float rn = __uint_as_float(__float_as_uint(mag) ^ ((rsign << (31 - i)) & 0x80000000u));
        // layered: A = Q + R_new; flooding: Lnew += R_new - R_old
        const float v = LAYERED ? __fadd_rn(rold[i], rn) : __fadd_rn(nv[i], __fsub_rn(rn, rold[i]));
        if (i == LAST && sfx)
            sfx_new = v;
        else
            lnew[addr[i]] = v;
    }
    *st_out = make_uint4(__float_as_uint(m1), __float_as_uint(m2), pack_info(i1, i2, qmask),
                         __float_as_uint(sfx_new));
    if (sfx) seed_t[addr[LAST]] = loss_term(sfx_new, ybit, scale, loss);
}

// Degree switch up to MAXD (the code's largest row degree class: 10 covers
// BG2, 19 BG1), so a BG2 kernel holds no registers for BG1's long rows.
#define NRLDPC_DEG_SWITCH(CASE)                                                                  \
    switch (deg) {                                                                               \
        CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9) CASE(10)        \
        CASE(11) CASE(12) CASE(13) CASE(14) CASE(15) CASE(16) CASE(17) CASE(18) CASE(19)        \
        default: break;                                                                          \
    }

template <int MAXD, bool LAYERED>
__device__ __forceinline__ void fwd_dispatch(int deg, const CodeTable& tab, int e0, uint32_t s,
                                             const float* lold, float* lnew, const float4* wp,
                                             const float4* wc, uint4 st, uint4* st_out, bool sfx, bool ybit,
                                             float* seed_t, float scale, float* loss) {
#define NRLDPC_FWD_CASE(D)                                                                         \
    case D:                                                                                        \
        if constexpr (D <= MAXD)                                                                   \
            fwd_row<D, LAYERED>(tab, e0, s, lold, lnew, wp, wc, st, st_out, sfx, ybit, seed_t, scale, loss); \
        break;
    NRLDPC_DEG_SWITCH(NRLDPC_FWD_CASE)
#undef NRLDPC_FWD_CASE
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

// Two CTAs per SM: registers are capped for it (the BG1 kernels spill a
// little at degree 19, the BG2 ones do not).
constexpr int kWmsMinBlocks = 2;

template <int MAXD, bool LAYERED>
__global__ void __launch_bounds__(kMaxThreads, kWmsMinBlocks)
    wms_forward_kernel(const __grid_constant__ CodeTable tab, const __grid_constant__ WmsArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_group = reinterpret_cast<int*>(smem);
    float* s_red = reinterpret_cast<float*>(smem + 64);  // warp partial losses
    float* wbuf = reinterpret_cast<float*>(smem + kHdr);  // [2][kMaxRows][kWPad] previous / current
    const float4* wrow = reinterpret_cast<const float4*>(wbuf);
    float* bufs = wbuf + kFwdWeightFloats;
    const int z = tab.z, n = tab.n_bp, cpb = a.cpb, rows = tab.rows, E = tab.n_edges;
    const int cf = tab.core_floats, ncz = tab.n_core * z;
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
        float* lold = bufs + static_cast<size_t>(valid ? slot : 0) * cf;
        float* lnew = LAYERED ? lold : bufs + static_cast<size_t>(cpb + (valid ? slot : 0)) * cf;
        const float* gllr = a.llr + static_cast<size_t>(act ? cw : 0) * n;
        // this thread's codeword bits: core positions s, s + Z, ... (at most
        // kMaxCols) as a 128-bit mask, and bit r = the bit at row r's suffix
        // position of sub-row s; read once per group
        uint64_t ybits0 = 0, ybits1 = 0, ysfx = 0;
        if (act) {
#pragma unroll 4
            for (int k = static_cast<int>(s); k < cf / 4; k += z)
                reinterpret_cast<float4*>(lold)[k] = reinterpret_cast<const float4*>(gllr)[k];
            const uint8_t* bits = a.cw + static_cast<size_t>(cw) * tab.packed_bytes;
            for (int k = 0; k < tab.n_core; k++) {
                const uint64_t b = static_cast<uint64_t>(cw_bit(bits, static_cast<int>(s) + k * z));
                if (k < 64)
                    ybits0 |= b << k;
                else
                    ybits1 |= b << (k - 64);
            }
            for (int r = 0; r < rows; r++)
                if (tab.row_sfx[r])
                    ysfx |= static_cast<uint64_t>(
                                cw_bit(bits, static_cast<int>(edge_at(tab.edge[tab.row_ptr[r + 1] - 1], s, z))))
                            << r;
        }
        float loss_part = 0.0f;
        for (int t = 0; t < a.T; t++) {
            for (int k = tid; k < kFwdWeightFloats; k += blockDim.x) {  // padded rows, zero previous at t = 0
                const int half = k >= kMaxRows * kWPad ? 1 : 0;
                const int rem = k - half * kMaxRows * kWPad;
                const int r = rem / kWPad, j = rem - r * kWPad;
                float v = 0.0f;
                if (r < rows && j < tab.row_deg[r] && (half || t > 0))
                    v = a.weights[(t - 1 + half) * E + tab.row_ptr[r] + j];
                wbuf[k] = v;
            }
            __syncthreads();
            if (act && !LAYERED)
                for (int k = static_cast<int>(s); k < cf / 4; k += z)
                    reinterpret_cast<float4*>(lnew)[k] = reinterpret_cast<const float4*>(lold)[k];
            __syncthreads();
            const size_t cw_off = static_cast<size_t>(act ? cw : 0) * rows * z;
            const uint4* st_prev =
                a.states + static_cast<size_t>(t > 0 ? t - 1 : 0) * a.n_cw * rows * z + cw_off;
            uint4* st_cur = a.states + static_cast<size_t>(t) * a.n_cw * rows * z + cw_off;
            float* seed_t = a.gseed + (static_cast<size_t>(t) * a.n_cw + (act ? cw : 0)) * n;
            // previous iteration's state of row r+2 requested while row r
            // runs; in the first iteration only the suffix LLR, from global
            auto fetch = [&](int r) -> uint4 {
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (!act || r >= rows) return v;
                if (t > 0) return __ldcg(st_prev + r * z + s);
                if (tab.row_sfx[r])
                    v.w = __float_as_uint(__ldcs(gllr + edge_at(tab.edge[tab.row_ptr[r + 1] - 1], s, z)));
                return v;
            };
            uint4 p0 = fetch(0), p1 = fetch(1);
            for (int r = 0; r < rows; r++) {
                const uint4 p2 = fetch(r + 2);
                if (act)
                    fwd_dispatch<MAXD, LAYERED>(tab.row_deg[r], tab, tab.row_ptr[r], s, lold, lnew,
                                                wrow + r * (kWPad / 4), wrow + (kMaxRows + r) * (kWPad / 4), p0,
                                                st_cur + r * z + s, tab.row_sfx[r] != 0,
                                                (ysfx >> r) & 1u, seed_t, a.scale, &loss_part);
                p0 = p1;
                p1 = p2;
                if (tab.sync_after[r]) __syncthreads();
            }
            // loss terms and gradient seeds of the core columns at L^{t+1}
            if (act) {
                uint64_t y0 = ybits0, y1 = ybits1;
#pragma unroll 4
                for (int c = static_cast<int>(s); c < ncz; c += z) {
                    seed_t[c] = loss_term(lnew[c], y0 & 1u, a.scale, &loss_part);
                    y0 = (y0 >> 1) | (y1 << 63);
                    y1 >>= 1;
                }
            }
            float* tmp = lold;
            lold = lnew;
            lnew = tmp;
        }
        if (act && a.app) {
            float* app = a.app + static_cast<size_t>(cw) * n;
            for (int c = static_cast<int>(s); c < ncz; c += z) app[c] = lold[c];
            const uint4* st_last = a.states + (static_cast<size_t>(a.T - 1) * a.n_cw + cw) * rows * z;
            for (int r = 0; r < rows; r++)
                if (tab.row_sfx[r])
                    app[edge_at(tab.edge[tab.row_ptr[r + 1] - 1], s, z)] =
                        __uint_as_float(__ldcg(&st_last[r * z + s].w));
        }
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
// gl = dloss/dL^{t+1} and gl_next = dloss/dL^t over the core columns.  The
// suffix edge's dloss/dL^{t+1} is its loss seed plus what the next
// iteration's row sent back through Q (only this row touches the column).
template <int D>
__device__ __forceinline__ void bwd_row(const CodeTable& tab, int e0, uint32_t s, bool act,
                                        const float* gl, float* gl_next, const float* w_cur,
                                        float* gw_acc, uint4 st, uint4 gin, uint4* gq_io, bool scatter,
                                        bool sfx, float sfx_seed) {
    constexpr int LAST = D - 1;
    const uint32_t z = static_cast<uint32_t>(tab.z);
    const float m1 = __uint_as_float(st.x), m2 = __uint_as_float(st.y);
    const int i1 = static_cast<int>(st.z & 31u), i2 = static_cast<int>((st.z >> 5) & 31u);
    const uint32_t q = st.z >> 10;
    const uint32_t par = static_cast<uint32_t>(__popc(q) & 1);
    const float g1n = __uint_as_float(gin.x), g2n = __uint_as_float(gin.y);
    const int j1 = static_cast<int>(gin.z), j2 = static_cast<int>(gin.w);
    uint32_t ad1 = 0, ad2 = 0;  // columns of the two argmin edges
    float acc1 = 0.0f, acc2 = 0.0f;
    float gwv[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
        const uint32_t a = edge_at(tab.edge[e0 + i], s, z);
        ad1 = i == i1 ? a : ad1;
        ad2 = i == i2 ? a : ad2;
        float gr = 0.0f;
        if (act) {
            const float back = i == j1 ? g1n : (i == j2 ? g2n : 0.0f);
            const float glv = (i == LAST && sfx) ? __fadd_rn(sfx_seed, back) : gl[a];
            gr = glv - back;
        }
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
        if (scatter) {  // the suffix column's share comes back through gq instead
            if (m1 < 1000.0f && !(sfx && i1 == LAST)) atomicAdd(&gl_next[ad1], g1);
            if (i2 < D && m2 < 1000.0f && !(sfx && i2 == LAST)) atomicAdd(&gl_next[ad2], g2);
        }
        *gq_io = make_uint4(__float_as_uint(g1), __float_as_uint(g2), static_cast<uint32_t>(i1),
                            static_cast<uint32_t>(i2 < D ? i2 : 31));
    }
}

template <int MAXD>
__device__ __forceinline__ void bwd_dispatch(int deg, const CodeTable& tab, int e0, uint32_t s,
                                             bool act, const float* gl, float* gln, const float* wc,
                                             float* gw_acc, uint4 st, uint4 gin, uint4* gq, bool scatter,
                                             bool sfx, float sfx_seed) {
#define NRLDPC_BWD_CASE(D)                                                                           \
    case D:                                                                                          \
        if constexpr (D <= MAXD) bwd_row<D>(tab, e0, s, act, gl, gln, wc, gw_acc, st, gin, gq, scatter, sfx, sfx_seed); \
        break;
    NRLDPC_DEG_SWITCH(NRLDPC_BWD_CASE)
#undef NRLDPC_BWD_CASE
}

template <int MAXD>
__global__ void __launch_bounds__(kMaxThreads, kWmsMinBlocks)
    wms_backward_kernel(const __grid_constant__ CodeTable tab, const __grid_constant__ WmsArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_group = reinterpret_cast<int*>(smem);
    float* wcur = reinterpret_cast<float*>(smem + kHdr);  // [E]
    float* gw_acc = wcur + kMaxEdges;                     // [E]
    float* bufs = gw_acc + kMaxEdges;
    const int z = tab.z, n = tab.n_bp, cpb = a.cpb, rows = tab.rows, E = tab.n_edges;
    const int cf = tab.core_floats, ncz = tab.n_core * z;
    const int tid = threadIdx.x, slot = tid / z;
    const uint32_t s = static_cast<uint32_t>(tid - slot * z);
    const bool valid = slot < cpb;
    // row ring (BG2 kernels): [kRing][blockDim] states, dloss/dQ, seeds
    uint4* ring_st = reinterpret_cast<uint4*>(bufs + 2 * static_cast<size_t>(cpb) * cf);
    uint4* ring_gq = ring_st + kRing * blockDim.x;
    float* ring_sd = reinterpret_cast<float*>(ring_gq + kRing * blockDim.x);
    uint4* gq = a.gq + (static_cast<size_t>(blockIdx.x) * cpb + (valid ? slot : 0)) * rows * z;
    for (;;) {
        if (tid == 0) *s_group = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int g = *s_group;
        if (g >= a.n_groups) break;
        const int cw = g * cpb + slot;
        const bool act = valid && cw < a.n_cw;
        float* gl = bufs + static_cast<size_t>(valid ? slot : 0) * cf;          // dloss/dL^{t+1}
        float* gln = bufs + static_cast<size_t>(cpb + (valid ? slot : 0)) * cf;  // dloss/dL^t
        if (act) {
            const float* seed = a.gseed + (static_cast<size_t>(a.T - 1) * a.n_cw + cw) * n;
#pragma unroll 4
            for (int c = static_cast<int>(s); c < ncz; c += z) gl[c] = seed[c];
            for (int k = 0; k < rows; k++) gq[k * z + s] = make_uint4(0u, 0u, 31u, 31u);
        }
        for (int t = a.T - 1; t >= 0; t--) {
            for (int e = tid; e < E; e += blockDim.x) {
                wcur[e] = a.weights[t * E + e];
                gw_acc[e] = 0.0f;
            }
            if (act && t > 0) {
                const float* seed = a.gseed + (static_cast<size_t>(t - 1) * a.n_cw + cw) * n;
#pragma unroll 4
                for (int c = static_cast<int>(s); c < ncz; c += z) gln[c] = seed[c];
            }
            __syncthreads();
            const uint4* st = a.states + (static_cast<size_t>(t) * a.n_cw + (act ? cw : 0)) * rows * z;
            const float* seed_t = a.gseed + (static_cast<size_t>(t) * a.n_cw + (act ? cw : 0)) * n;
            if constexpr (MAXD <= 10) {
                // rows r .. r + kRing - 2 in flight in the shared-memory ring
                const int nt = blockDim.x;
                auto issue = [&](int r) {
                    if (act && r < rows) {
                        const int k = (r % kRing) * nt + tid;
                        cp_async16(&ring_st[k], st + r * z + s);
                        cp_async16(&ring_gq[k], gq + r * z + s);
                        if (tab.row_sfx[r])
                            cp_async4(&ring_sd[k], seed_t + edge_at(tab.edge[tab.row_ptr[r + 1] - 1], s, z));
                    }
                    cp_async_commit();
                };
                for (int r = 0; r < kRing - 1; r++) issue(r);
                for (int r = 0; r < rows; r++) {
                    issue(r + kRing - 1);
                    cp_async_wait<kRing - 1>();  // this thread's copies of row r have landed
                    const int k = (r % kRing) * nt + tid;
                    const uint4 sv = act ? ring_st[k] : make_uint4(0u, 0u, 31u << 5, 0u);
                    const uint4 gv = act ? ring_gq[k] : make_uint4(0u, 0u, 31u, 31u);
                    const float sd = (act && tab.row_sfx[r]) ? ring_sd[k] : 0.0f;
                    bwd_dispatch<MAXD>(tab.row_deg[r], tab, tab.row_ptr[r], s, act, gl, gln, wcur, gw_acc, sv, gv,
                                       gq + r * z + s, t > 0, tab.row_sfx[r] != 0, sd);
                }
                cp_async_wait<0>();
            } else {
                // state, per-row dloss/dQ and the suffix edge's loss seed of
                // row r+2 requested while row r runs
                auto fetch = [&](int r, uint4& sv, uint4& gv, float& sd) {
                    sv = make_uint4(0u, 0u, 31u << 5, 0u);
                    gv = make_uint4(0u, 0u, 31u, 31u);
                    sd = 0.0f;
                    if (act && r < rows) {
                        sv = __ldcg(st + r * z + s);
                        gv = __ldcg(gq + r * z + s);
                        if (tab.row_sfx[r]) sd = __ldcs(seed_t + edge_at(tab.edge[tab.row_ptr[r + 1] - 1], s, z));
                    }
                };
                uint4 s0, g0, s1, g1;
                float d0, d1;
                fetch(0, s0, g0, d0);
                fetch(1, s1, g1, d1);
                for (int r = 0; r < rows; r++) {
                    uint4 s2, g2;
                    float d2;
                    fetch(r + 2, s2, g2, d2);
                    bwd_dispatch<MAXD>(tab.row_deg[r], tab, tab.row_ptr[r], s, act, gl, gln, wcur, gw_acc, s0, g0,
                                       gq + r * z + s, t > 0, tab.row_sfx[r] != 0, d0);
                    s0 = s1;
                    g0 = g1;
                    d0 = d1;
                    s1 = s2;
                    g1 = g2;
                    d1 = d2;
                }
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

// g = dloss/dA over the core columns.  The suffix column's dloss/dA before
// its row is its loss seed minus the dloss/dR carried from the next
// iteration (h = -dloss/dQ there), the value the in-place A had.
template <int D, bool SEED_IN_ROW>
__device__ __forceinline__ void bwd_layered_row(const CodeTable& tab, int e0, uint32_t s, bool act, float* g,
                                                const float* w_cur, float* gw_acc, uint4 st, float* gh_row,
                                                bool has_h, bool write_h, bool sfx, float sfx_seed,
                                                const float* seed_t) {
    constexpr int LAST = D - 1;
    const uint32_t z = static_cast<uint32_t>(tab.z);
    const float m1 = __uint_as_float(st.x), m2 = __uint_as_float(st.y);
    const int i1 = static_cast<int>(st.z & 31u), i2 = static_cast<int>((st.z >> 5) & 31u);
    const uint32_t q = st.z >> 10;
    const uint32_t par = static_cast<uint32_t>(__popc(q) & 1);
    uint32_t ad[D];
    float ga[D];
    float gwv[D];
    float to1 = 0.0f, to2 = 0.0f;  // dloss/dQ at the argmin edges through R
#pragma unroll
    for (int i = 0; i < D; i++) {
        const uint32_t a = edge_at(tab.edge[e0 + i], s, z);
        ad[i] = a;
        float dr = 0.0f;
        ga[i] = 0.0f;
        if (act) {
            const float h = has_h ? gh_row[i * z] : 0.0f;
            ga[i] = (i == LAST && sfx) ? __fsub_rn(SEED_IN_ROW ? __ldcs(seed_t + a) : sfx_seed, h) : g[a];
            dr = ga[i] + h;
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
        if ((i == i1 || i == i2) && !(i == LAST && sfx)) g[ad[i]] = dq;  // dloss/dA before this row
        if (write_h) gh_row[i * z] = -dq;                                // dloss/dR^{t-1}
    }
}

template <int MAXD>
__device__ __forceinline__ void bwd_layered_dispatch(int deg, const CodeTable& tab, int e0, uint32_t s, bool act,
                                                     float* g, const float* wc, float* gw_acc, uint4 st,
                                                     float* gh_row, bool has_h, bool write_h, bool sfx,
                                                     float sfx_seed, const float* seed_t) {
#define NRLDPC_BWDL_CASE(D)                                                                                 \
    case D:                                                                                                 \
        if constexpr (D <= MAXD)                                                                            \
            bwd_layered_row<D, (MAXD > 10)>(tab, e0, s, act, g, wc, gw_acc, st, gh_row, has_h, write_h, sfx,      \
                                            sfx_seed, seed_t);                                                    \
        break;
    NRLDPC_DEG_SWITCH(NRLDPC_BWDL_CASE)
#undef NRLDPC_BWDL_CASE
}

template <int MAXD>
__global__ void __launch_bounds__(kMaxThreads, kWmsMinBlocks)
    wms_backward_layered_kernel(const __grid_constant__ CodeTable tab, const __grid_constant__ WmsArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    int* s_group = reinterpret_cast<int*>(smem);
    float* wcur = reinterpret_cast<float*>(smem + kHdr);  // [E]
    float* gw_acc = wcur + kMaxEdges;                     // [E]
    float* bufs = gw_acc + kMaxEdges;
    const int z = tab.z, n = tab.n_bp, cpb = a.cpb, rows = tab.rows, E = tab.n_edges;
    const int cf = tab.core_floats, ncz = tab.n_core * z;
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
        float* g = bufs + static_cast<size_t>(valid ? slot : 0) * cf;  // dloss/dA
        if (act)
            for (int c = static_cast<int>(s); c < ncz; c += z) g[c] = 0.0f;
        for (int t = a.T - 1; t >= 0; t--) {
            for (int e = tid; e < E; e += blockDim.x) {
                wcur[e] = a.weights[t * E + e];
                gw_acc[e] = 0.0f;
            }
            const float* seed_t = a.gseed + (static_cast<size_t>(t) * a.n_cw + (act ? cw : 0)) * n;
            if (act) {
#pragma unroll 4
                for (int c = static_cast<int>(s); c < ncz; c += z) g[c] += seed_t[c];
            }
            __syncthreads();
            const uint4* st = a.states + (static_cast<size_t>(t) * a.n_cw + (act ? cw : 0)) * rows * z;
            // state of row r-2 requested while row r runs, with its suffix
            // loss seed in the degree-10 kernels (at degree 19 the extra
            // registers of the seed ring cost more in spills than it saves)
            auto fetch = [&](int r, float& sd) -> uint4 {
                sd = 0.0f;
                if (!act || r < 0) return make_uint4(0u, 0u, 31u << 5, 0u);
                if (MAXD <= 10 && tab.row_sfx[r])
                    sd = __ldcs(seed_t + edge_at(tab.edge[tab.row_ptr[r + 1] - 1], s, z));
                return __ldcg(st + r * z + s);
            };
            float d0, d1;
            uint4 s0 = fetch(rows - 1, d0), s1 = fetch(rows - 2, d1);
            for (int r = rows - 1; r >= 0; r--) {
                float d2;
                const uint4 s2 = fetch(r - 2, d2);
                bwd_layered_dispatch<MAXD>(tab.row_deg[r], tab, tab.row_ptr[r], s, act, g, wcur, gw_acc, s0,
                                           gh + static_cast<size_t>(tab.row_ptr[r]) * z + s, t < a.T - 1, t > 0,
                                           tab.row_sfx[r] != 0, d0, seed_t);
                s0 = s1;
                s1 = s2;
                d0 = d1;
                d1 = d2;
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

namespace {
int max_row_degree(const CodeTable& tab) {
    int maxd = 0;
    for (int r = 0; r < tab.rows; r++) maxd = tab.row_deg[r] > maxd ? tab.row_deg[r] : maxd;
    return maxd;
}
}  // namespace

// Shared memory: header, weight rows (the forward's padded layout, larger than
// the adjoints' two [E] arrays), two core-column buffers per codeword, and
// for codes of row degree <= 10 the flooding adjoint's row ring.
size_t wms_smem_bytes(const CodeTable& tab, int cpb) {
    return kHdr + kFwdWeightFloats * sizeof(float) + 2 * static_cast<size_t>(cpb) * tab.core_floats * sizeof(float) +
           (max_row_degree(tab) <= 10 ? kRingBytes : 0);
}

namespace {
// kernel k of the degree class: 0 forward flooding, 1 forward layered,
// 2 adjoint flooding, 3 adjoint layered
template <int MAXD>
const void* wms_kernel(int k) {
    switch (k) {
        case 0: return reinterpret_cast<const void*>(&wms_forward_kernel<MAXD, false>);
        case 1: return reinterpret_cast<const void*>(&wms_forward_kernel<MAXD, true>);
        case 2: return reinterpret_cast<const void*>(&wms_backward_kernel<MAXD>);
        default: return reinterpret_cast<const void*>(&wms_backward_layered_kernel<MAXD>);
    }
}
const void* wms_kernel_for(const CodeTable& tab, int k) {
    return max_row_degree(tab) <= 10 ? wms_kernel<10>(k) : wms_kernel<19>(k);
}
}  // namespace

cudaError_t wms_kernel_attributes(size_t smem) {
    for (int k = 0; k < 4; k++)
        for (const void* f : {wms_kernel<10>(k), wms_kernel<19>(k)}) {
            cudaError_t e =
                cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

int wms_ctas_per_sm(const CodeTable& tab, int threads, size_t smem) {
    int n = 1 << 30;
    for (int k = 0; k < 4; k++) {
        int c = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, wms_kernel_for(tab, k), threads, smem) !=
            cudaSuccess)
            return 0;
        n = c < n ? c : n;
    }
    return n;
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
    const void* k = wms_kernel_for(tab, (backward ? 2 : 0) + (layered ? 1 : 0));
    void* params[2] = {const_cast<CodeTable*>(&tab), &a};
    return cudaLaunchKernel(k, dim3(grid), dim3(threads), params, smem, stream);
}

cudaError_t launch_adam(int n, float* w, const double* grad, float* m, float* v, int step, float lr,
                        float b1, float b2, float eps, float w_min, cudaStream_t stream) {
    const float c1 = 1.0f - powf(b1, static_cast<float>(step));
    const float c2 = 1.0f - powf(b2, static_cast<float>(step));
    adam_kernel<<<(n + 255) / 256, 256, 0, stream>>>(n, w, grad, m, v, lr, b1, b2, eps, c1, c2, w_min);
    return cudaGetLastError();
}

}  // namespace nrldpc
