// Fused flooding normalized min-sum decoder for sm_103a.
//
// One CTA holds `cpb` whole codewords on chip for all iterations:
//   * two fp32 posterior buffers per codeword in shared memory over the core
//     columns, Lold (read by the check-node pass) and Lnew (accumulates the
//     posterior update);
//   * the check-node state between iterations, compressed to 16 B per lifted
//     row (min1, min2, argmin + R sign bits, and the posterior of the row's
//     degree-1 suffix column) as one uint4 per (row, sub-row), in a per-CTA
//     slot of global memory that stays L2-resident (each CTA reuses its slot
//     for every codeword it takes), requested two rows ahead.  Keeping the
//     suffix columns (5G NR: the extension parity, 42 of 68 BG1 columns) out
//     of shared memory halves it, so two CTAs run per SM.
// The core LLRs come into shared memory with one cp.async.bulk copy per
// codeword (mbarrier completion, bounded wait); the suffix LLRs are read from
// global memory by the first iteration's state fetch.
//
// Bit-exactness with the reference (ctarver/NR_GPU_LDPC):
//   * check-node arithmetic of src/ldpc_kernels.cu:73-181 (first iteration)
//     and :199-314: Q = L - R_old, two-min with strict '<' from 1000.0f,
//     first argmin, R = +-fl(alpha * min) (the reference's
//     0.75f*sign*sq*min is exact up to the final product), dt = R - R_old;
//   * variable-node update of src/ldpc_kernels.cu:330-395, 411-468:
//     APP = L + dt_row0 + dt_row1 + ... in ascending base-row order.  Here
//     each base row adds its dt into Lnew right after its check-node pass;
//     rows run in ascending order and a column receives at most one edge per
//     base row, so every column sees the same fp32 add chain.  Rows between
//     two CTA barriers share no base column, so their adds commute.
//   * all float ops are explicit round-to-nearest intrinsics (no FMA
//     contraction), matching the reference's C semantics.
//   * hard decision APP > 0 ? 0 : 1, packed LSB-first (src/ldpc_kernels.cu:463-500).
#include <cuda_runtime.h>

#include "nrldpc_internal.h"

namespace nrldpc {
namespace {

constexpr int kMaxCpb = 48;
constexpr int kHeaderBytes = 1024;  // mbarrier, group id, per-slot flags
// Weights of the current iteration in shared memory, one padded row of
// kWPad floats per base row (previous-iteration row block, then current), so
// a row's weights come in with 128-bit loads: [2][kMaxRows][kWPad].
constexpr int kWPad = 20;
constexpr int kWeightBytes = 2 * kMaxRows * kWPad * 4;

// Weight i of a padded row held as float4s (i is constant after unrolling).
__device__ __forceinline__ float wsel(const float4* w, int i) {
    const float4 v = w[i >> 2];
    const int c = i & 3;
    return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}
constexpr long kWaitLimit = 1L << 20;
// Early stop: per-slot row of the last failed syndrome check, kFarOffset ints
// after the per-slot fail flags in the header (both kernels: flags at byte
// 16, up to kMaxCpb of each, header 1024 bytes); from row kFarRow on, the next
// check is bit-sliced.
constexpr int kFarOffset = 60;
constexpr int kFarRow = 12;

__device__ __forceinline__ float max_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// x + 0 per lane: -0 becomes +0, everything else is unchanged
__device__ __forceinline__ float4 canon4(float4 v) {
    return make_float4(__fadd_rn(v.x, 0.0f), __fadd_rn(v.y, 0.0f), __fadd_rn(v.z, 0.0f), __fadd_rn(v.w, 0.0f));
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false when the limit ran out (the caller records an error).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long limit = kWaitLimit) {
    for (long i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32-bit shared-memory accesses by byte address.  Volatile keeps them in
// program order; a row touches each of its columns once (the load of a
// position before its store), and rows between barriers touch disjoint
// columns.
__device__ __forceinline__ float lds(uint32_t a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ void sts(uint32_t a, float v) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

__device__ __forceinline__ void sts_u8(uint32_t a, uint32_t v) {
    asm volatile("st.shared.u8 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lds_u8(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared.u8 %0, [%1];" : "=r"(v) : "r"(a));
    return v;
}

// One lifted row (base row with D edges, sub-row s) of one iteration.
// The first iteration passes a zero state (and a zero previous weight), so
// R_old = +0 and Q = L - (+0) = L, dt = R - (+0) = R exactly, as in
// cnp_kernel_1st_iter.
//   s4old: shared byte address of this slot's Lold plus 4*s;
//   dnew:  byte distance from Lold to Lnew; z4 = 4*Z;
//   sfx:   the last edge is a suffix column: its posterior is st.w (read)
//          and goes to the stored state's w (written), not shared memory;
//   st:    this row's state from the previous iteration; st_out: where this
//          iteration's goes (written when store);
//   hd:    shared byte address for the suffix column's hard decision of
//          the posterior written (bit 1; written when sfx and write_hd).
// Unweighted flooding (kPlain, the reference's decoder) reads Q = L - R_old
// from Lold, which holds the posterior with -0 made +0 (run_group's copies),
// so the sign bit of Q is (Q < 0) as it is; Lnew and the suffix posterior in
// the state accumulate the exact sums.  The weighted and layered kernels take
// the sign from Q + 0 and keep null addresses for the stores they skip (each
// form measured fastest for its kernels).
// LAYERED (no reference counterpart): one posterior buffer updated in place,
// A = Q + R_new (dnew = 0), instead of Lnew += R_new - R_old.
template <int D, bool WEIGHTED, bool LAYERED, bool PACKED>
__device__ __forceinline__ void row_update(const CodeTable& tab, int e0, bool sfx, uint32_t s,
                                           uint32_t s4old, uint32_t dnew, uint32_t z4,
                                           const float4* wprev, const float4* wcur, uint4 st, uint4* st_out,
                                           bool store, bool write_hd, uint32_t hd, float alpha) {
    constexpr int LAST = D - 1;
    constexpr bool kPlain = !WEIGHTED && !LAYERED;
    uint32_t addr[D];
    float lv[D];
    const float sraw = __uint_as_float(st.w);  // the suffix posterior as accumulated
#pragma unroll
    for (int i = 0; i < D; i++) {
        if (i == LAST && sfx) {
            addr[i] = 0;
            lv[i] = kPlain ? __fadd_rn(sraw, 0.0f) : __uint_as_float(st.w);  // kPlain: -0 read as +0, like Lold
        } else {
            uint32_t a;
            // one 64-bit table read per edge: faster for the layered kernels and
            // for a table in shared memory (mixed batch); the single-code
            // flooding kernels read the two words from their parameter bank
            if (LAYERED || PACKED) {
                const uint2 ea = tab.eaddr[e0 + i];
                a = s4old + ea.x;
                if (s >= ea.y) a -= z4;  // column (s + V) mod Z of the edge's block
            } else {
                a = s4old + tab.ebase4[e0 + i];
                if (s >= tab.ethr[e0 + i]) a -= z4;
            }
            addr[i] = a;
            lv[i] = lds(a);
        }
    }
    // old messages R_old from the previous iteration's state; kept per edge:
    // R_old (flooding, for dt) or Q (layered, for A = Q + R_new)
    float keep[D];
    const float om1 = __uint_as_float(st.x), om2 = __uint_as_float(st.y);
    const uint32_t oinfo = st.z;
    const int oidx = static_cast<int>(oinfo & 31u);
    float oa1 = 0.0f, oa2 = 0.0f;
    if (!WEIGHTED) {
        oa1 = __fmul_rn(alpha, om1);
        oa2 = __fmul_rn(alpha, om2);
    }
    float m1 = 1000.0f, m2 = 1000.0f;
    int idx = 0;
    uint32_t qmask = 0;
#pragma unroll
    for (int i = 0; i < D; i++) {
        float mag;
        if (WEIGHTED)
            mag = __fmul_rn(wsel(wprev, i), i == oidx ? om2 : om1);
        else
            mag = i == oidx ? oa2 : oa1;
        const float ro = __uint_as_float(__float_as_uint(mag) ^ ((oinfo << (24 - D + i)) & 0x80000000u));
        const float q = __fsub_rn(lv[i], ro);
        keep[i] = LAYERED ? q : ro;
        const float qa = fabsf(q);
        // the sign bit of q is (q < 0) when q is never -0 (kPlain: L is
        // never -0, so neither is L - R_old); the others take it from q + 0,
        // -0 becoming +0; NaN results are canonical (+)
        const float qs = kPlain ? q : __fadd_rn(q, 0.0f);
        qmask = __funnelshift_l(__float_as_uint(qs), qmask, 1);  // edge i at bit D-1-i
        if (i == 0) {  // from m1 = m2 = 1000: min2 stays 1000 whatever |Q_0| is
            m1 = fminf(m1, qa);
            continue;
        }
        if (!LAYERED && qa < m1) idx = i;  // layered: found below from the kept Q
        const float mx = max_nan(m1, qa);  // NaN |Q| leaves min1/min2 untouched
        m1 = fminf(m1, qa);
        m2 = fminf(m2, mx);
    }
    const uint32_t par = static_cast<uint32_t>(__popc(qmask) & 1);
    const uint32_t rsign = qmask ^ (0u - par);  // sign of R_i = product of the other signs
    float a1 = 0.0f, a2 = 0.0f;
    if (!WEIGHTED) {
        a1 = __fmul_rn(alpha, m1);
        a2 = __fmul_rn(alpha, m2);
    }
    float sfx_new = 0.0f;
    if (LAYERED) {
        // The edge that gets min2 is any edge with |Q| == min1: the first
        // argmin when the minimum is unique, and when it is not, min2 ==
        // min1 and every such edge gets the same message.
#pragma unroll
        for (int i = 0; i < D; i++) {
            const bool at_min = fabsf(keep[i]) == m1;
            if (at_min) idx = i;
            float mag;
            if (WEIGHTED)
                mag = __fmul_rn(wsel(wcur, i), at_min ? m2 : m1);
            else
                mag = at_min ? a2 : a1;
            const float rn = __uint_as_float(__float_as_uint(mag) ^ ((rsign << (32 - D + i)) & 0x80000000u));
            const float v = __fadd_rn(keep[i], rn);
            if (i == LAST && sfx)
                sfx_new = v;
            else
                sts(addr[i], v);
        }
    } else {
        // Lnew read-modify-write with the loads kPipe edges ahead of the stores
        // (fewer live registers than loading the whole row first); the
        // suffix edge adds to the exact suffix posterior
        constexpr int kPipe = 4;
        float nv[D];
#pragma unroll
        for (int i = 0; i < kPipe && i < D; i++)
            nv[i] = (i == LAST && sfx) ? (kPlain ? sraw : lv[i]) : lds(addr[i] + dnew);
#pragma unroll
        for (int i = 0; i < D; i++) {
            if (i + kPipe < D)
                nv[i + kPipe] =
                    (i + kPipe == LAST && sfx) ? (kPlain ? sraw : lv[i + kPipe]) : lds(addr[i + kPipe] + dnew);
            float mag;
            if (WEIGHTED)
                mag = __fmul_rn(wsel(wcur, i), i == idx ? m2 : m1);
            else
                mag = i == idx ? a2 : a1;
            const float rn = __uint_as_float(__float_as_uint(mag) ^ ((rsign << (32 - D + i)) & 0x80000000u));
            const float dt = __fsub_rn(rn, keep[i]);
            const float v = __fadd_rn(nv[i], dt);
            if (i == LAST && sfx)
                sfx_new = v;
            else
                sts(addr[i] + dnew, v);
        }
    }
    if (sfx && (kPlain ? write_hd : hd != 0u)) sts_u8(hd, sfx_new > 0.0f ? 0u : 2u);
    if (kPlain ? store : st_out != nullptr) {
        const uint32_t info = static_cast<uint32_t>(idx) | ((rsign & ((1u << D) - 1u)) << 8);
        __stcg(st_out, make_uint4(__float_as_uint(m1), __float_as_uint(m2), info, __float_as_uint(sfx_new)));
    }
}

template <bool WEIGHTED, bool LAYERED, bool PACKED>
__device__ __forceinline__ void row_dispatch(int deg, const CodeTable& tab, int e0, bool sfx, uint32_t s,
                                             uint32_t s4old, uint32_t dnew, uint32_t z4,
                                             const float4* wprev, const float4* wcur, uint4 st, uint4* st_out,
                                             bool store, bool write_hd, uint32_t hd, float alpha) {
    switch (deg) {
#define NRLDPC_ROW_CASE(D)                                                                         \
    case D:                                                                                        \
        row_update<D, WEIGHTED, LAYERED, PACKED>(tab, e0, sfx, s, s4old, dnew, z4, wprev, wcur, st, st_out, store, \
                                         write_hd, hd, alpha);                                    \
        break;
        NRLDPC_ROW_CASE(1) NRLDPC_ROW_CASE(2) NRLDPC_ROW_CASE(3) NRLDPC_ROW_CASE(4)
        NRLDPC_ROW_CASE(5) NRLDPC_ROW_CASE(6) NRLDPC_ROW_CASE(7) NRLDPC_ROW_CASE(8)
        NRLDPC_ROW_CASE(9) NRLDPC_ROW_CASE(10) NRLDPC_ROW_CASE(11) NRLDPC_ROW_CASE(12)
        NRLDPC_ROW_CASE(13) NRLDPC_ROW_CASE(14) NRLDPC_ROW_CASE(15) NRLDPC_ROW_CASE(16)
        NRLDPC_ROW_CASE(17) NRLDPC_ROW_CASE(18) NRLDPC_ROW_CASE(19)
#undef NRLDPC_ROW_CASE
        default:
            break;
    }
}

// Position (c*Z + (s + V) mod Z) of sub-row s on edge e.
__device__ __forceinline__ int edge_pos(const CodeTable& tab, int e, uint32_t s) {
    int p = static_cast<int>(tab.edge[e] & 0xffffu) + static_cast<int>(s);
    if (s >= tab.ethr[e]) p -= tab.z;
    return p;
}

// Hard decisions (and optionally posterior / iteration count) of one codeword
// slot at the bytes / positions of sub-row s (the slot's threads call it once
// per sub-row they own; tpc = threads per codeword).  L: core-column posteriors in shared
// memory; hd: the slot's suffix hard-decision bytes, bit `bit` taken; the
// suffix posteriors come from the state slot when app_from_state (otherwise
// the row pass already wrote them).
__device__ __forceinline__ void write_outputs(const CodeTable& tab, const float* L, const uint8_t* hd,
                                              int bit, const uint4* st_slot, uint32_t s, uint32_t tpc,
                                              uint8_t* packed, float* app, int32_t* iters, int it,
                                              bool app_from_state) {
    const int n = tab.n_bp, z = tab.z, ncz = tab.n_core * z;
    if ((tpc & 31u) == 0) {
        // Warp ballots (the slot is whole warps of tpc threads, each calling
        // for sub-row s): thread s decides positions
        // s + k*Z (column k, sub-position s); one ballot over a warp is the
        // 32 bits of positions 32*w .. 32*w + 31, LSB first = 4 packed bytes.
        const uint32_t lane = s & 31u;
        const bool word_store = (reinterpret_cast<uintptr_t>(packed) & 3u) == 0;
        for (int k = 0, pos = static_cast<int>(s); pos < n; k++, pos += z) {
            uint32_t one;
            if (k < tab.n_core) {
                one = L[pos] > 0.0f ? 0u : 1u;
            } else {
                const int r = tab.sfx_row[k];
                int sr = static_cast<int>(s) - static_cast<int>(tab.edge_shift[tab.row_ptr[r + 1] - 1]);
                if (sr < 0) sr += z;
                one = (hd[r * z + sr] >> bit) & 1u;
            }
            const uint32_t word = __ballot_sync(0xffffffffu, one);
            uint8_t* dst = packed + ((pos - static_cast<int>(lane)) >> 3);
            if (word_store) {
                if (lane == 0) *reinterpret_cast<uint32_t*>(dst) = word;
            } else if (lane < 4) {
                dst[lane] = static_cast<uint8_t>(word >> (8 * lane));
            }
        }
    } else {
    for (int b = static_cast<int>(s); b < tab.packed_bytes; b += z) {
        int pos = 8 * b;
        int c = pos / z, p = pos - c * z;
        uint32_t v = 0;
        for (int i = 0; i < 8 && pos < n; i++, pos++) {
            uint32_t one;
            if (pos < ncz) {
                one = L[pos] > 0.0f ? 0u : 1u;
            } else {
                const int r = tab.sfx_row[c];
                int sr = p - static_cast<int>(tab.edge_shift[tab.row_ptr[r + 1] - 1]);
                if (sr < 0) sr += z;
                one = (hd[r * z + sr] >> bit) & 1u;
            }
            v |= one << i;
            if (++p == z) {
                p = 0;
                c++;
            }
        }
        packed[b] = static_cast<uint8_t>(v);
    }
    }
    if (app) {
        for (int pos = static_cast<int>(s); pos < ncz; pos += z) app[pos] = L[pos];
        if (app_from_state)
            for (int c = tab.n_core; c < tab.cols; c++) {
                const int r = tab.sfx_row[c];
                app[edge_pos(tab, tab.row_ptr[r + 1] - 1, s)] = __uint_as_float(__ldcg(&st_slot[r * z + s].w));
            }
    }
    if (iters && s == 0) *iters = it;
}

// All base rows of one iteration, ascending.  The state of row r+2 is
// requested while row r runs (L2 latency spans more than one row); in the
// first iteration the state is zero and only the suffix posterior is
// fetched, from the codeword's LLRs in global memory.  SPT = 2: the thread
// owns sub-rows s and s + tpc and runs both in each row, the state of the
// next row's two sub-rows requested while this row's run.
//   store: write this iteration's state; write_hd: write the suffix hard
//   decisions.
template <bool WEIGHTED, bool LAYERED, int SPT, bool PACKED>
__device__ __forceinline__ void iterate_rows(const CodeTable& tab, uint32_t s, uint32_t tpc, uint32_t s4old,
                                             uint32_t dnew, const float4* wpad, uint4* st_base,
                                             const float* gllr,
                                             uint32_t hd_base, bool act, bool first, bool store, bool write_hd,
                                             float alpha) {
    const int z = tab.z, rows = tab.rows;
    const uint32_t z4 = 4u * static_cast<uint32_t>(z);
    auto fetch = [&](int r, uint32_t sj) -> uint4 {
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (!act || r >= rows) return v;
        if (!first) return __ldcg(st_base + r * z + sj);
        if (tab.row_sfx[r]) v.w = __float_as_uint(__ldcs(gllr + edge_pos(tab, tab.row_ptr[r + 1] - 1, sj)));
        return v;
    };
    // unweighted flooding: the state and decision addresses are always formed
    // and the stores guarded by the flags (0.8% faster there); the other
    // kernels get null addresses for the stores they skip (faster for them)
    constexpr bool kPlain = !WEIGHTED && !LAYERED;
    auto run = [&](int r, uint32_t j, uint4 st) {
        const uint32_t sj = s + j * tpc;
        const bool sfx = tab.row_sfx[r] != 0;
        row_dispatch<WEIGHTED, LAYERED, PACKED>(
            tab.row_deg[r], tab, tab.row_ptr[r], sfx, sj, s4old + 4u * j * tpc, dnew, z4, wpad + r * (kWPad / 4),
            wpad + (kMaxRows + r) * (kWPad / 4), st, (kPlain || store) ? st_base + r * z + sj : nullptr, store,
            kPlain ? write_hd : (write_hd && sfx),
            (kPlain || (write_hd && sfx)) ? hd_base + j * tpc + static_cast<uint32_t>(r * z) : 0u, alpha);
    };
    if constexpr (SPT == 1) {
        uint4 s0 = fetch(0, s), s1 = fetch(1, s);
        for (int r = 0; r < rows; r++) {
            const uint4 s2 = fetch(r + 2, s);
            if (act) run(r, 0, s0);
            s0 = s1;
            s1 = s2;
            if (tab.sync_after[r]) __syncthreads();
        }
    } else {
        uint4 a0 = fetch(0, s), a1 = fetch(0, s + tpc);
        for (int r = 0; r < rows; r++) {
            const uint4 b0 = fetch(r + 1, s);
            if (act) run(r, 0, a0);
            const uint4 b1 = fetch(r + 1, s + tpc);
            if (act) run(r, 1, a1);
            a0 = b0;
            a1 = b1;
            if (tab.sync_after[r]) __syncthreads();
        }
    }
}

// Syndrome of the slot's hard decisions after an iteration: sets *fail when
// a lifted check is unsatisfied.  Core columns are read from the posterior
// just written (s4a: its shared address plus 4*s), suffix columns from bit 1
// of their hard-decision bytes.  Threads stop at the first failure seen by
// any thread of the slot, so an iteration far from convergence costs a few
// rows; *far gets the row of the failure.
template <bool PACKED>
__device__ __forceinline__ void check_rows(const CodeTable& tab, uint32_t s, uint32_t s4a, uint32_t hd_base,
                                           volatile int* fail, int* far) {
    const int z = tab.z;
    const uint32_t z4 = 4u * static_cast<uint32_t>(z);
    for (int r = 0; r < tab.rows; r++) {
        if (*fail) return;
        const int e0 = tab.row_ptr[r], e1 = tab.row_ptr[r + 1] - (tab.row_sfx[r] ? 1 : 0);
        uint32_t par = tab.row_sfx[r] ? (lds_u8(hd_base + static_cast<uint32_t>(r * z)) >> 1) & 1u : 0u;
        for (int e = e0; e < e1; e++) {
            uint32_t a;
            if (PACKED) {
                const uint2 ea = tab.eaddr[e];
                a = s4a + ea.x;
                if (s >= ea.y) a -= z4;
            } else {
                a = s4a + tab.ebase4[e];
                if (s >= tab.ethr[e]) a -= z4;
            }
            par ^= lds(a) > 0.0f ? 0u : 1u;
        }
        if (par) {
            *fail = 1;
            *far = r;
            return;
        }
    }
}

// Four suffix hard decisions (bit 1 of four consecutive bytes, little-endian)
// moved into the top nibble of acc, which shifts down by four: after eight
// words the nibble of the first word sits at bits 0..3.
__device__ __forceinline__ uint32_t sfx_nibble(uint32_t w, uint32_t acc) {
    // the multiply moves bits 1, 9, 17, 25 to 28, 29, 30, 31 (no carries)
    return (acc >> 4) | (((w & 0x02020202u) * 0x08102040u) & 0xf0000000u);
}

// Syndrome of every slot after an iteration, 32 sub-rows at a time (Z a
// multiple of 32; same hard-decision rule as check_rows).  The core hard
// decisions of the posterior just written (lnew0: slot 0, slots cf floats
// apart) are packed into words, each column block stored twice in a row so
// that a 32-bit window never wraps: word x of block c of slot j
// (bits + (j*n_core + c)*2*nw + x, nw = Z/32) holds the decisions of
// positions c*Z + 32*(x mod nw) + 0..31.  Then, for (slot j, row r, word k),
// the XOR over the row's core edges (column c, shift V) of the window of
// block c that starts at bit (32k + V) mod Z -- the decisions the sub-rows
// 32k..32k+31 see -- and of the suffix decisions of those sub-rows (bit 1 of
// their bytes in hd0, slots rows*Z bytes apart) is nonzero exactly when one
// of these lifted checks fails (a failing slot's s_far is set to rows).  The table entries these tasks need are
// copied next to the packed words first (edge: window word offset
// c*2*nw + V/32 and bit offset V mod 32 in 16 bits; row: first and end core
// edge, suffix flag), so every lane can take a task of its own.  Every
// thread of the CTA calls it (one barrier inside); the scratch is
// cpb*n_core*2*nw words + rows words + n_edges halfwords.
__device__ __forceinline__ void check_bits(const CodeTable& tab, int cpb, const float* lnew0, const uint8_t* hd0,
                                           uint32_t* bits, int* s_fail, int* s_far) {
    const int z = tab.z, nw = z >> 5, rows = tab.rows, nc = tab.n_core;
    const int tid = static_cast<int>(threadIdx.x), nt = static_cast<int>(blockDim.x);
    uint32_t* rinfo = bits + cpb * nc * 2 * nw;               // [rows]
    uint16_t* einfo = reinterpret_cast<uint16_t*>(rinfo + rows);  // [n_edges]
    for (int e = tid; e < tab.n_edges; e += nt) {
        const uint32_t v = tab.edge_shift[e];
        einfo[e] = static_cast<uint16_t>(((tab.edge_col[e] * 2u * nw + (v >> 5)) << 5) | (v & 31u));
    }
    for (int r = tid; r < rows; r += nt) {
        const uint32_t sfx = tab.row_sfx[r] ? 1u : 0u;
        rinfo[r] = tab.row_ptr[r] | ((tab.row_ptr[r + 1] - sfx) << 16) | (sfx << 31);
    }
    {   // pack: thread = word x of blocks bc0, bc0 + step, ... (bc = j*nc + c).
        // The words of a warp's lanes start 128 bytes apart (one bank), so
        // lane t reads its 32 posteriors starting at the t-th (all 32 banks
        // per load) and rotates the collected word back by t.
        const int x = tid % nw, step = nt / nw, rot = tid & 31;
        for (int bc = tid / nw; bc < cpb * nc && tid < step * nw; bc += step) {
            const float* src = lnew0 + static_cast<size_t>(bc) * z + 32 * x;
            uint32_t w = 0;  // bit i: decision of position (i + rot) mod 32
#pragma unroll
            for (int i = 0; i < 32; i++) w |= (src[(i + rot) & 31] > 0.0f ? 0u : 1u) << i;
            w = __funnelshift_l(w, w, static_cast<uint32_t>(rot));
            uint32_t* dst = bits + bc * 2 * nw + x;
            dst[0] = w;
            dst[nw] = w;
        }
    }
    __syncthreads();
    // tasks: thread = (slot, word) pair jk of rows r0, r0 + step, ...
    const int pairs = cpb * nw, step = nt / pairs, jk = tid % pairs;
    if (tid >= step * pairs) return;
    const int j = jk / nw, k = jk - j * nw;
    const uint32_t* wb = bits + j * nc * 2 * nw + k;
    const uint8_t* hj = hd0 + static_cast<size_t>(j) * rows * z + 32 * k;
    uint32_t fail = 0;
    for (int r = tid / pairs; r < rows; r += step) {
        const uint32_t ri = rinfo[r];
        uint32_t acc = 0;
#pragma unroll 4
        for (int e = static_cast<int>(ri & 0xffffu); e < static_cast<int>((ri >> 16) & 0x7fffu); e++) {
            const uint32_t ei = einfo[e];
            const uint32_t* w = wb + (ei >> 5);
            acc ^= __funnelshift_r(w[0], w[1], ei & 31u);
        }
        if (ri >> 31) {
            const uint4* h = reinterpret_cast<const uint4*>(hj + r * z);
            const uint4 h0 = h[0], h1 = h[1];
            uint32_t sb = 0;
            sb = sfx_nibble(h0.x, sb);
            sb = sfx_nibble(h0.y, sb);
            sb = sfx_nibble(h0.z, sb);
            sb = sfx_nibble(h0.w, sb);
            sb = sfx_nibble(h1.x, sb);
            sb = sfx_nibble(h1.y, sb);
            sb = sfx_nibble(h1.z, sb);
            sb = sfx_nibble(h1.w, sb);
            acc ^= sb;
        }
        fail |= acc;
    }
    if (fail) {
        s_fail[j] = 1;
        s_far[j] = rows;  // a failing slot keeps the bit-sliced check
    }
}

// Per-slot destinations of one decoded codeword (null pointers: not wanted).
struct SlotOut {
    uint8_t* packed;
    float* app;
    int32_t* iters;
};

// All iterations of one codeword group whose core LLRs are already in buf0
// (Lold): cpb slots, this thread = sub-row s of slot `slot`; gllr = the
// slot's codeword in global memory (suffix LLRs).  Ends with a barrier.
// Flooding accumulates into Lnew and copies it back to Lold; LAYERED updates
// Lold in place.  Early stop: after iteration t < n_iter - 1, a codeword
// whose hard decisions satisfy every check stops with iters = t + 1 (the
// oracle's rule, ldpc_oracle.c decode_one_f32).
// PACKED: the table is in shared memory (the mixed batch): each edge's
// address words come as one 64-bit read.
template <bool WEIGHTED, bool LAYERED, int SPT = 1, bool PACKED = false>
__device__ __forceinline__ void run_group(const CodeTable& tab, int cpb, int slot, uint32_t s, uint32_t tpc,
                                          bool slot_done, float* buf0, uint8_t* hd0,
                                          int* s_fail, uint4* st_base, const float* gllr, SlotOut out,
                                          int n_iter, int early_stop, float alpha, const float* wtab, float4* wpad,
                                          int n_w_iters) {
    const int z = tab.z, cf = tab.core_floats, tid = threadIdx.x;
    int* s_far = s_fail + kFarOffset;  // per slot: row of the last failed check
    float* lold = buf0 + static_cast<size_t>(slot) * cf;  // read by the check-node pass
    float* lnew = LAYERED ? lold : lold + static_cast<size_t>(cpb) * cf;  // the posterior written
    const uint8_t* hd = hd0 + static_cast<size_t>(slot) * tab.rows * z;
    const uint32_t s4old = smem_addr(lold) + 4u * s;
    const uint32_t dnew = LAYERED ? 0u : static_cast<uint32_t>(cpb) * static_cast<uint32_t>(cf) * 4u;
    const uint32_t hd_base = smem_addr(hd) + s;
    const int nt = static_cast<int>(tpc);  // threads of the slot
    // flooding: Lnew starts as the LLRs; unweighted, Lold as the LLRs with
    // -0 made +0 (the check-node pass then needs no per-edge sign fix-up)
    if (!LAYERED && !slot_done)
        for (int k = static_cast<int>(s); k < cf / 4; k += nt) {
            const float4 v = reinterpret_cast<const float4*>(lold)[k];
            reinterpret_cast<float4*>(lnew)[k] = v;
            if (!WEIGHTED) reinterpret_cast<float4*>(lold)[k] = canon4(v);
        }
    for (int t = 0; t < n_iter; t++) {
        const bool first = t == 0, last = t == n_iter - 1;
        // weight rows in parameter space (uniform constant-cache reads); the
        // zero row at t = 0, where there is no previous R
        if (WEIGHTED) {  // this iteration's weights into shared memory, padded per base row
            const float* wprev = wtab + (first ? kMaxWIters : min(t - 1, n_w_iters - 1)) * kMaxEdges;
            const float* wcur = wtab + min(t, n_w_iters - 1) * kMaxEdges;
            float* wp = reinterpret_cast<float*>(wpad);
            for (int k = tid; k < 2 * kMaxRows * kWPad; k += blockDim.x) {
                const int half = k >= kMaxRows * kWPad ? 1 : 0;
                const int rem = k - half * kMaxRows * kWPad;
                const int r = rem / kWPad, j = rem - r * kWPad;
                float v = 0.0f;
                if (r < tab.rows && j < tab.row_deg[r]) v = (half ? wcur : wprev)[tab.row_ptr[r] + j];
                wp[k] = v;
            }
        }
        if (tid < cpb) s_fail[tid] = 0;
        // the syndrome pass of this iteration: bit-sliced when a codeword of
        // the CTA failed its previous check at row kFarRow or later (near
        // convergence: a row-by-row scan would run through most rows), else
        // row by row with an early exit (s_far was written before the
        // previous iteration's closing barriers)
        const bool far_check = __syncthreads_or(!slot_done && s_far[slot] >= kFarRow);
        const bool act = !slot_done;
        const bool store = !last || out.app != nullptr;
        iterate_rows<WEIGHTED, LAYERED, SPT, PACKED>(tab, s, tpc, s4old, dnew, wpad, st_base, gllr, hd_base, act,
                                                     first, store, early_stop || last, alpha);
        if (early_stop && !last) {  // the rows ended with a barrier
            // bit-sliced scratch: flooding in Lold (read again only after the
            // copy-back below), layered in the weight rows (restaged at the
            // next iteration's start)
            const int scratch = cpb * tab.n_core * (z >> 4) + tab.rows + (tab.n_edges + 1) / 2;
            if (far_check && (z & 31) == 0 && scratch <= (LAYERED ? kWeightBytes / 4 : cpb * cf))
                check_bits(tab, cpb, lnew - static_cast<size_t>(slot) * cf, hd0,
                           LAYERED ? reinterpret_cast<uint32_t*>(wpad) : reinterpret_cast<uint32_t*>(buf0), s_fail,
                           s_far);
            else if (act)
                for (int j = 0; j < SPT; j++)
                    check_rows<PACKED>(tab, s + j * tpc, s4old + 4u * j * tpc + dnew, hd_base + j * tpc,
                                       &s_fail[slot], &s_far[slot]);
            __syncthreads();
            const bool conv = act && s_fail[slot] == 0;
            if (conv)  // HD of this iteration is a codeword
                for (int j = 0; j < SPT; j++)
                    write_outputs(tab, lnew, hd, 1, st_base, s + j * tpc, tpc, out.packed, out.app, out.iters, t + 1,
                                  true);
            slot_done = slot_done || conv;
            if (__syncthreads_and(slot_done)) break;
        }
        if (last) {
            if (!slot_done)
                for (int j = 0; j < SPT; j++)
                    write_outputs(tab, lnew, hd, 1, st_base, s + j * tpc, tpc, out.packed, out.app, out.iters, n_iter,
                                  true);
            break;
        }
        if (!LAYERED && !slot_done)  // the posterior just accumulated is the next iteration's input
            for (int k = static_cast<int>(s); k < cf / 4; k += nt)  // unweighted: -0 as +0
                reinterpret_cast<float4*>(lold)[k] = WEIGHTED ? reinterpret_cast<const float4*>(lnew)[k]
                                                              : canon4(reinterpret_cast<const float4*>(lnew)[k]);
    }
    __syncthreads();  // buffers are rewritten by the next group's copy
    if (tid < cpb) s_far[tid] = 0;  // read again only after the next group's barriers
}

// MINB = CTAs per SM the register budget is sized for: 1 when shared memory
// admits a single CTA per SM anyway (BG1 Z=384), 2 otherwise.
template <bool W>
struct WeightParam {
    using type = NoWeights;
};
template <>
struct WeightParam<true> {
    using type = WeightTable;
};

// FROM_HOST: a.llr is pinned host memory (a separate instantiation, so the
// device-resident kernels keep their register allocation).
template <bool WEIGHTED, int MINB, bool LAYERED, bool FROM_HOST>
__global__ void __launch_bounds__(kMaxThreads, MINB)
    decode_kernel(const __grid_constant__ CodeTable tab, const __grid_constant__ DecodeArgs a,
                  const __grid_constant__ typename WeightParam<WEIGHTED>::type wt) {
    extern __shared__ __align__(128) unsigned char smem[];
    const uint32_t bar = smem_addr(smem);
    int* s_group = reinterpret_cast<int*>(smem + 8);
    int* s_fail = reinterpret_cast<int*>(smem + 16);
    float4* wpad = reinterpret_cast<float4*>(smem + kHeaderBytes);
    float* buf0 = reinterpret_cast<float*>(smem + kHeaderBytes + kWeightBytes);
    const float* wtab = nullptr;
    if constexpr (WEIGHTED) wtab = &wt.w[0][0];

    const int z = tab.z, n = tab.n_bp, cpb = a.cpb, rows = tab.rows, cf = tab.core_floats;
    uint8_t* hd0 = reinterpret_cast<uint8_t*>(buf0 + 2 * static_cast<size_t>(cpb) * cf);
    const int tid = threadIdx.x;
    const int slot = tid / z;
    const uint32_t s = static_cast<uint32_t>(tid - slot * z);
    const bool valid_thread = slot < cpb;
    uint4* st_base = reinterpret_cast<uint4*>(a.state) +
                     (static_cast<size_t>(blockIdx.x) * cpb + (valid_thread ? slot : 0)) * rows * z;

    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < kMaxCpb) s_fail[kFarOffset + threadIdx.x] = 0;
    __syncthreads();
    uint32_t phase = 0;

    for (;;) {
        if (tid == 0) *s_group = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int g = *s_group;
        if (g >= a.n_groups) break;
        const int cw0 = g * cpb;
        const int n_valid = min(cpb, a.n_cw - cw0);
        if constexpr (FROM_HOST) {
            // pinned host memory: the CTA's threads read the core columns of
            // each codeword in 16-byte pieces, up to eight in flight per
            // thread (the suffix LLRs come with the first iteration's state
            // fetch, as in the device-resident kernel)
            const int core4 = cf / 4;
            for (int k = 0; k < n_valid; k++) {
                const float4* src = reinterpret_cast<const float4*>(a.llr + static_cast<size_t>(cw0 + k) * n);
                float4* dst = reinterpret_cast<float4*>(buf0 + static_cast<size_t>(k) * cf);
#pragma unroll 8
                for (int m = tid; m < core4; m += blockDim.x) dst[m] = __ldcs(src + m);
            }
            __syncthreads();
        } else {
            if (tid == 0) {  // core-column LLRs of each codeword into its Lold
                fence_proxy_async();
                mbar_arrive_expect_tx(bar, static_cast<uint32_t>(n_valid) * cf * 4u + a.extra_tx);
                // the timeout self-test (extra_tx != 0) expects bytes but
                // issues no copy, so nothing is in flight when its wait runs out
                if (a.extra_tx == 0)
                    for (int k = 0; k < n_valid; k++)
                        bulk_g2s(smem_addr(buf0 + static_cast<size_t>(k) * cf),
                                 a.llr + static_cast<size_t>(cw0 + k) * n, cf * 4u, bar);
            }
            const long limit = a.wait_limit > 0 ? a.wait_limit : kWaitLimit;
            bool ok = mbar_wait_bounded(bar, phase, limit);
            if (!__syncthreads_and(ok)) {
                // In a decode the copies read a valid device buffer and land
                // (the wait only times out when they take longer than the
                // limit); a second bounded wait gives them that time again
                // before the CTA leaves, so no copy into this CTA's shared
                // memory outlives it.  The self-test has none in flight.
                if (tid == 0) atomicExch(a.error_flag, kErrLlrLoadTimeout);
                if (a.extra_tx == 0) mbar_wait_bounded(bar, phase, limit);
                return;
            }
            phase ^= 1u;
        }
        const bool slot_done = !valid_thread || slot >= n_valid;
        const size_t cw = static_cast<size_t>(cw0 + (slot_done ? 0 : slot));
        SlotOut out{a.packed + cw * tab.packed_bytes, a.app ? a.app + cw * n : nullptr,
                    a.iters ? a.iters + cw : nullptr};
        run_group<WEIGHTED, LAYERED>(tab, cpb, slot, s, static_cast<uint32_t>(z), slot_done, buf0, hd0, s_fail,
                                     st_base, a.llr + cw * n, out, a.n_iter, a.early_stop, a.alpha, wtab, wpad,
                                     a.n_w_iters);
    }
}

// Mixed batch: one persistent launch over work items of several (BG, Z)
// codes.  Each item = up to cpb codewords of one code; the item's code table
// is copied into shared memory and every codeword is fetched from its own
// offset with its own bulk copy.
__global__ void __launch_bounds__(kMaxThreads, 2)
    batch_decode_kernel(const __grid_constant__ BatchDecodeArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const uint32_t bar = smem_addr(smem);
    int* s_item = reinterpret_cast<int*>(smem + 8);
    int* s_fail = reinterpret_cast<int*>(smem + 16);
    CodeTable* stab = reinterpret_cast<CodeTable*>(smem + kHeaderBytesBatch);
    float* buf0 = reinterpret_cast<float*>(smem + kHeaderBytesBatch + kBatchTableBytes);
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < kMaxCpb) s_fail[kFarOffset + threadIdx.x] = 0;
    __syncthreads();
    uint32_t phase = 0;
    for (;;) {
        if (tid == 0) *s_item = atomicAdd(a.work_counter, 1);
        __syncthreads();
        const int it = *s_item;
        if (it >= a.n_items) break;
        const WorkItem item = a.items[it];
        {   // code table of this item into shared memory
            const uint4* src = reinterpret_cast<const uint4*>(a.tables + item.code);
            uint4* dst = reinterpret_cast<uint4*>(stab);
            for (int k = tid; k < static_cast<int>(kBatchTableCopy / 16); k += blockDim.x) dst[k] = src[k];
        }
        __syncthreads();
        const CodeTable& tab = *stab;
        const int z = tab.z, cf = tab.core_floats, cpb = item.count;
        const int tpc = z / item.spt;  // threads per codeword: each owns spt sub-rows
        uint8_t* hd0 = reinterpret_cast<uint8_t*>(buf0 + 2 * static_cast<size_t>(cpb) * cf);
        const int slot = tid / tpc;
        const uint32_t s = static_cast<uint32_t>(tid - slot * tpc);
        const bool valid_thread = slot < cpb;
        if (tid == 0) {
            fence_proxy_async();
            mbar_arrive_expect_tx(bar, static_cast<uint32_t>(cpb) * cf * 4u);
            for (int k = 0; k < cpb; k++) {
                const nrldpc_job& j = a.jobs[a.order[item.start + k]];
                bulk_g2s(smem_addr(buf0 + static_cast<size_t>(k) * cf), a.llr + j.llr_offset, cf * 4u, bar);
            }
        }
        bool ok = mbar_wait_bounded(bar, phase);
        if (!__syncthreads_and(ok)) {
            // the copies read valid device buffers and land; a second bounded
            // wait lets them do so before the CTA leaves (as decode_kernel)
            if (tid == 0) atomicExch(a.error_flag, kErrLlrLoadTimeout);
            mbar_wait_bounded(bar, phase);
            return;
        }
        phase ^= 1u;
        const int jidx = valid_thread ? a.order[item.start + slot] : 0;
        const nrldpc_job& job = a.jobs[jidx];
        SlotOut out{a.packed + job.out_offset, nullptr, a.iters ? a.iters + jidx : nullptr};
        uint4* st_base = reinterpret_cast<uint4*>(a.state + static_cast<size_t>(blockIdx.x) * a.slot_words) +
                         static_cast<size_t>(valid_thread ? slot : 0) * tab.rows * z;
        if (item.spt == 2)
            run_group<false, false, 2, true>(tab, cpb, slot, s, static_cast<uint32_t>(tpc), !valid_thread, buf0, hd0,
                                       s_fail, st_base, a.llr + job.llr_offset, out, a.n_iter, a.early_stop, a.alpha,
                                       nullptr, nullptr, 1);
        else
            run_group<false, false, 1, true>(tab, cpb, slot, s, static_cast<uint32_t>(tpc), !valid_thread, buf0, hd0,
                                       s_fail, st_base, a.llr + job.llr_offset, out, a.n_iter, a.early_stop, a.alpha,
                                       nullptr, nullptr, 1);
    }
}

}  // namespace

size_t decode_smem_bytes(const CodeTable& tab, int cpb) {
    return kHeaderBytes + kWeightBytes + group_smem_bytes(tab, cpb);
}

template <bool W, int MINB, bool LAY, bool HOST = false>
const void* kernel_ptr() {
    return reinterpret_cast<const void*>(&decode_kernel<W, MINB, LAY, HOST>);
}

// from_host: the unweighted kernels that read host-resident LLRs.
const void* select_kernel(bool weighted, int minb, bool layered, bool from_host = false) {
    if (from_host && !weighted) {
        if (layered) return minb >= 2 ? kernel_ptr<false, 2, true, true>() : kernel_ptr<false, 1, true, true>();
        return minb >= 2 ? kernel_ptr<false, 2, false, true>() : kernel_ptr<false, 1, false, true>();
    }
    if (layered) {
        if (weighted) return minb >= 2 ? kernel_ptr<true, 2, true>() : kernel_ptr<true, 1, true>();
        return minb >= 2 ? kernel_ptr<false, 2, true>() : kernel_ptr<false, 1, true>();
    }
    if (weighted) return minb >= 2 ? kernel_ptr<true, 2, false>() : kernel_ptr<true, 1, false>();
    return minb >= 2 ? kernel_ptr<false, 2, false>() : kernel_ptr<false, 1, false>();
}

cudaError_t launch_batch_decode(const BatchDecodeArgs& args, int grid, int threads, size_t smem,
                                cudaStream_t stream) {
    batch_decode_kernel<<<grid, threads, smem, stream>>>(args);
    return cudaGetLastError();
}

const void* batch_decode_kernel_ptr() { return reinterpret_cast<const void*>(&batch_decode_kernel); }

cudaError_t decode_kernel_attributes(size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(batch_decode_kernel_ptr(),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    for (int l = 0; l < 2; l++)
        for (int w = 0; w < 3; w++)  // plain, weighted, plain from host
            for (int m = 1; m <= 2; m++) {
                cudaError_t e = cudaFuncSetAttribute(select_kernel(w == 1, m, l != 0, w == 2),
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     static_cast<int>(smem));
                if (e != cudaSuccess) return e;
            }
    return cudaSuccess;
}

int decode_max_ctas_per_sm(bool weighted, int minb, int threads, size_t smem) {
    int n = 1 << 30;
    for (int l = 0; l < 4; l++) {  // both schedules, device- and host-resident LLRs
        int k = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, select_kernel(weighted, minb, l & 1, l >= 2),
                                                          threads, smem) != cudaSuccess)
            return 0;
        n = k < n ? k : n;
    }
    return n;
}

cudaError_t launch_decode(const CodeTable& tab, const DecodeArgs& args, const WeightTable* weights, int grid,
                          int threads, size_t smem, bool layered, int minb, cudaStream_t stream) {
    if (args.cpb < 1 || args.cpb > kMaxCpb) return cudaErrorInvalidValue;
    const bool weighted = weights != nullptr;
    if (weighted && args.llr_from_host) return cudaErrorInvalidValue;
    const void* k = select_kernel(weighted, minb, layered, args.llr_from_host != 0);
    NoWeights none{};
    void* params[3] = {const_cast<CodeTable*>(&tab), const_cast<DecodeArgs*>(&args),
                       weighted ? const_cast<WeightTable*>(weights) : static_cast<void*>(&none)};
    return cudaLaunchKernel(k, dim3(grid), dim3(threads), params, smem, stream);
}

}  // namespace nrldpc
