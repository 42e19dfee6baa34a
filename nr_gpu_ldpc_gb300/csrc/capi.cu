// C-ABI of the decoder (include/nr_gpu_ldpc_gb300.h): code setup, handles,
// device buffers and launches.  Host code only; kernels live in decode.cu
// and channel.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/nr_gpu_ldpc_gb300.h"
#include "nrldpc_internal.h"

using namespace nrldpc;

namespace {
#include "base_graphs.inc"

const int kBaseZ[8] = {2, 3, 5, 7, 9, 11, 13, 15};
constexpr int kHostChunks = 16;  // most chunks of one host-buffer decode
constexpr int kChunkCounter = 4;  // first scratch word of the per-chunk work counters
constexpr size_t kScratchBytes = 128;
// Largest batch, in CTA rounds, that NRLDPC_HOST_AUTO decodes straight from
// host memory (GB300, BG1 Z=384, 10 iterations, against the two-lane staged
// pipeline: direct ahead by 9% at half a round and 10% at 1, 3% at 4; behind
// by 3% at 6, 1% at 8, 5% at 10 and 2% at 13.5).
constexpr size_t kDirectMaxRounds = 4;

struct Handle {
    int device = 0;
    CodeTable tab{};
    EncodePlan plan{};
    bool plan_ok = false;
    float alpha = 0.75f;
    int max_batch = 0;
    int cpb = 1, threads = 32, ctas_per_sm = 1, sm_count = 1, max_grid = 1, minb = 1;
    size_t smem = 0;
    uint32_t* state = nullptr;
    uint32_t* state2 = nullptr;  // the second lane's check-node state (host-buffer pipeline)
    // [0] work counter, [1] error flag, [kChunkCounter + k] work counter of
    // chunk k of a host-buffer decode
    int* scratch = nullptr;
    float* stage_llr = nullptr;
    uint8_t* stage_packed = nullptr;
    void* stage_q = nullptr;  // fp16 / int8 LLR staging (nrldpc_decode_host_async_q)
    WeightTable* weights = nullptr;  // host copy, passed by value to the weighted kernels
    int n_w_iters = 0;
    bool wms_ready = false;
    int wms_ctas = 1;  // training-kernel CTAs per SM (occupancy of the slowest of the four)
    int schedule = NRLDPC_SCHEDULE_FLOODING;
    int host_mode = NRLDPC_HOST_AUTO;
    bool coherent_host = false;  // the GPU reads host memory over a coherent link (Grace C2C)
    // host-buffer pipeline: copies of chunk k+1 overlap the decode of chunk
    // k; chunks alternate between two lanes (the caller's stream and
    // lane_stream, each with its own check-node state), so a chunk's decode
    // starts while the previous one drains
    cudaStream_t copy_stream = nullptr;
    cudaStream_t lane_stream = nullptr;
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_lane = nullptr;
    cudaEvent_t ev_chunk[kHostChunks] = {};
};

int map_cuda(cudaError_t e) { return e == cudaSuccess ? NRLDPC_OK : NRLDPC_ERR_CUDA; }

bool fill_table(const int* base, int rows, int cols, int z, int kb, CodeTable* t) {
    if (rows < 1 || rows > kMaxRows || cols < 1 || cols > kMaxCols || z < 1 || z > kMaxZ) return false;
    // n_bp % 4 == 0: whole float4 / 16-byte bulk copies of a codeword
    if (cols * z > 0xffff || (cols * z) % 4 != 0) return false;
    std::memset(t, 0, sizeof(*t));
    t->rows = rows;
    t->cols = cols;
    t->z = z;
    t->n_bp = cols * z;
    t->packed_bytes = (t->n_bp + 7) / 8;
    t->kb = kb;
    int e = 0;
    for (int r = 0; r < rows; r++) {
        t->row_ptr[r] = static_cast<uint16_t>(e);
        int deg = 0;
        for (int c = 0; c < cols; c++) {
            const int v = base[r * cols + c];
            if (v == -1) continue;
            if (v < 0 || e >= kMaxEdges) return false;
            const int sh = v % z;
            t->edge[e] = static_cast<uint32_t>(c * z + sh) | (static_cast<uint32_t>(z - sh) << 16);
            t->ebase4[e] = static_cast<uint32_t>(c * z + sh) * 4u;
            t->ethr[e] = static_cast<uint16_t>(z - sh);
            t->eaddr[e] = make_uint2(t->ebase4[e], t->ethr[e]);
            t->edge_col[e] = static_cast<uint8_t>(c);
            t->edge_shift[e] = static_cast<uint16_t>(sh);
            e++;
            deg++;
        }
        if (deg < 1 || deg > kMaxDeg) return false;
        t->row_deg[r] = static_cast<uint8_t>(deg);
    }
    t->row_ptr[rows] = static_cast<uint16_t>(e);
    t->n_edges = e;
    // Suffix columns: the longest run of trailing columns that each have one
    // edge, in distinct rows (each is then the last edge of its row).
    int col_deg[kMaxCols] = {0}, col_row[kMaxCols] = {0};
    for (int r = 0; r < rows; r++)
        for (int k = t->row_ptr[r]; k < t->row_ptr[r + 1]; k++) {
            col_deg[t->edge_col[k]]++;
            col_row[t->edge_col[k]] = r;
        }
    int n_core = cols;
    while (n_core > 0 && col_deg[n_core - 1] == 1 && !t->row_sfx[col_row[n_core - 1]]) {
        n_core--;
        t->row_sfx[col_row[n_core]] = 1;
        t->sfx_row[n_core] = static_cast<uint8_t>(col_row[n_core]);
    }
    t->n_core = n_core;
    t->core_floats = (n_core * z + 3) / 4 * 4;
    // Barrier placement: greedy groups of consecutive rows that pairwise share
    // no base column; a barrier closes each group.
    int used[kMaxCols] = {0};
    for (int r = 0; r < rows; r++) {
        bool clash = false;
        for (int k = t->row_ptr[r]; k < t->row_ptr[r + 1]; k++) clash |= used[t->edge_col[k]] != 0;
        if (clash) {
            t->sync_after[r - 1] = 1;
            std::fill(used, used + kMaxCols, 0);
        }
        for (int k = t->row_ptr[r]; k < t->row_ptr[r + 1]; k++) used[t->edge_col[k]] = 1;
    }
    t->sync_after[rows - 1] = 1;
    return true;
}

int base_matrix_impl(int bg, int ils, int* out, int* rows, int* cols) {
    if ((bg != 1 && bg != 2) || ils < 0 || ils > 7) return NRLDPC_ERR_BAD_CONFIG;
    const int R = bg == 1 ? 46 : 42, C = bg == 1 ? 68 : 52;
    if (rows) *rows = R;
    if (cols) *cols = C;
    if (!out) return NRLDPC_OK;
    for (int i = 0; i < R * C; i++) out[i] = -1;
    const int n = bg == 1 ? NRLDPC_BG1_EDGES : NRLDPC_BG2_EDGES;
    for (int k = 0; k < n; k++) {
        if (bg == 1)
            out[kBg1Row[k] * C + kBg1Col[k]] = kBg1Shift[k][ils];
        else
            out[kBg2Row[k] * C + kBg2Col[k]] = kBg2Shift[k][ils];
    }
    return NRLDPC_OK;
}

void free_handle(Handle* h) {
    if (!h) return;
    cudaFree(h->state);
    cudaFree(h->state2);
    cudaFree(h->scratch);
    cudaFree(h->stage_llr);
    cudaFree(h->stage_packed);
    cudaFree(h->stage_q);
    delete h->weights;
    for (cudaEvent_t e : h->ev_chunk)
        if (e) cudaEventDestroy(e);
    if (h->ev_start) cudaEventDestroy(h->ev_start);
    if (h->ev_lane) cudaEventDestroy(h->ev_lane);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->lane_stream) cudaStreamDestroy(h->lane_stream);
    delete h;
}

int init_impl(const int* base, int rows, int cols, int kb, const nrldpc_config* cfg,
              nrldpc_handle** out) {
    if (!cfg || !out || cfg->max_batch < 1 || !(cfg->alpha > 0.0f) || cfg->cw_per_cta < 0)
        return NRLDPC_ERR_INVALID_ARG;
    *out = nullptr;
    Handle* h = new (std::nothrow) Handle();
    if (!h) return NRLDPC_ERR_NO_MEMORY;
    if (!fill_table(base, rows, cols, cfg->z, kb, &h->tab)) {
        delete h;
        return NRLDPC_ERR_BAD_CONFIG;
    }
    h->plan_ok = make_encode_plan(h->tab, &h->plan);
    h->device = cfg->device;
    h->alpha = cfg->alpha;
    h->max_batch = cfg->max_batch;
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || cfg->device < 0 || cfg->device >= n_dev) {
        delete h;
        return NRLDPC_ERR_NO_DEVICE;
    }
    cudaSetDevice(cfg->device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, cfg->device) != cudaSuccess) {
        delete h;
        return NRLDPC_ERR_NO_DEVICE;
    }
    h->sm_count = prop.multiProcessorCount;
    int uses_host_tables = 0;
    if (cudaDeviceGetAttribute(&uses_host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                               cfg->device) == cudaSuccess)
        h->coherent_host = uses_host_tables != 0;
    const size_t smem_limit = prop.sharedMemPerBlockOptin;
    const int z = cfg->z;
    int cpb = cfg->cw_per_cta;
    if (cpb == 0) {
        cpb = std::max(1, kMaxThreads / z);
        while (cpb > 1 && decode_smem_bytes(h->tab, cpb) > smem_limit) cpb--;
        cpb = std::min(cpb, 48);
    }
    if (cpb * z > kMaxThreads || decode_smem_bytes(h->tab, cpb) > smem_limit || cpb > 48) {
        delete h;
        return NRLDPC_ERR_BAD_CONFIG;
    }
    h->cpb = cpb;
    h->threads = (cpb * z + 31) / 32 * 32;
    h->smem = decode_smem_bytes(h->tab, cpb);
    // opt in to the device maximum once, so handles of any size can coexist
    if (map_cuda(decode_kernel_attributes(smem_limit))) {
        delete h;
        return NRLDPC_ERR_CUDA;
    }
    // two CTAs per SM when shared memory allows (the kernel then caps its
    // registers for two); otherwise one CTA with the full register budget
    h->minb = (2 * (h->smem + 1024) <= prop.sharedMemPerMultiprocessor) ? 2 : 1;
    h->ctas_per_sm = std::max(1, std::min(decode_max_ctas_per_sm(false, h->minb, h->threads, h->smem),
                                          decode_max_ctas_per_sm(true, h->minb, h->threads, h->smem)));
    h->max_grid = h->ctas_per_sm * h->sm_count;
    const size_t state_elems =
        static_cast<size_t>(h->max_grid) * cpb * h->tab.rows * static_cast<size_t>(z);
    const size_t n_llr = static_cast<size_t>(cfg->max_batch) * h->tab.n_bp;
    if (cudaMalloc(&h->state, state_elems * kStateBytesPerRow) != cudaSuccess ||
        cudaMalloc(&h->state2, state_elems * kStateBytesPerRow) != cudaSuccess ||
        cudaMalloc(&h->scratch, kScratchBytes) != cudaSuccess ||
        cudaMemset(h->scratch, 0, kScratchBytes) != cudaSuccess ||
        cudaMalloc(&h->stage_llr, n_llr * sizeof(float)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->lane_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_start, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_lane, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&h->stage_packed,
                   static_cast<size_t>(cfg->max_batch) * h->tab.packed_bytes) != cudaSuccess) {
        free_handle(h);
        return NRLDPC_ERR_NO_MEMORY;
    }
    for (cudaEvent_t& e : h->ev_chunk)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            free_handle(h);
            return NRLDPC_ERR_CUDA;
        }
    *out = reinterpret_cast<nrldpc_handle*>(h);
    return NRLDPC_OK;
}

// llr_from_host: llr is the device view of pinned host memory; the kernel
// reads it with ordinary loads instead of bulk copies.  counter / state: a
// work counter that is already zero and a check-node state of the host-buffer
// pipeline's lanes (null: the handle's own, the counter cleared here).
int decode_impl(Handle* h, const float* llr, uint8_t* packed, int n_cw, int n_iter, int early,
                float* app, int32_t* iters, bool weighted, cudaStream_t stream, bool llr_from_host = false,
                int* counter = nullptr, uint32_t* state = nullptr, int wait_limit = 0, uint32_t extra_tx = 0) {
    if (!h || n_cw < 0 || n_iter < 1 || (early != 0 && early != 1)) return NRLDPC_ERR_INVALID_ARG;
    if (n_cw == 0) return NRLDPC_OK;  // empty batch: nothing to read or write
    if (!llr || !packed) return NRLDPC_ERR_INVALID_ARG;
    if (n_cw > h->max_batch) return NRLDPC_ERR_TOO_LARGE;
    if (reinterpret_cast<uintptr_t>(llr) % 16 != 0) return NRLDPC_ERR_ALIGNMENT;
    if (weighted && (!h->weights || h->n_w_iters < 1)) return NRLDPC_ERR_INVALID_ARG;
    DecodeArgs a{};
    a.llr = llr;
    a.packed = packed;
    a.app = app;
    a.iters = iters;
    a.state = state ? state : h->state;
    a.work_counter = counter ? counter : h->scratch;
    a.error_flag = h->scratch + 1;
    a.n_cw = n_cw;
    a.n_iter = n_iter;
    a.cpb = h->cpb;
    a.n_groups = (n_cw + h->cpb - 1) / h->cpb;
    a.n_w_iters = h->n_w_iters;
    a.early_stop = early;
    a.alpha = h->alpha;
    a.llr_from_host = llr_from_host ? 1 : 0;
    a.wait_limit = wait_limit;
    a.extra_tx = extra_tx;
    const int grid = std::min(a.n_groups, h->max_grid);
    if (!counter && cudaMemsetAsync(h->scratch, 0, sizeof(int), stream) != cudaSuccess) return NRLDPC_ERR_CUDA;
    return map_cuda(launch_decode(h->tab, a, weighted ? h->weights : nullptr, grid, h->threads, h->smem,
                                  h->schedule == NRLDPC_SCHEDULE_LAYERED, h->minb, stream));
}

// Host-buffer decode (fp32 LLRs, or narrow ones widened on the GPU: qtype 1
// fp16, 2 int8 * scale).  The batch is cut into chunks of whole CTA rounds
// (1, 2, 4, ... rounds of max_grid * cpb codewords): chunk k+1's host->device
// copy runs on the handle's copy stream while chunk k decodes, and each
// chunk's packed bits go back as soon as it is decoded.  Even chunks decode
// on the caller's stream, odd ones on the handle's lane stream with their own
// check-node state and work counter, so the next chunk's CTAs take over SMs
// as the current chunk's CTAs finish instead of after the whole launch.
// Device view of a pinned (cudaHostAlloc'd or registered) host buffer, or
// null when the GPU cannot address it.
void* pinned_device_view(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // clear the error of an unknown pointer
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    // the view of p itself (the attributes describe p's allocation at p)
    return at.devicePointer;
}

int host_decode(Handle* h, const void* h_llr, int qtype, float scale, uint8_t* h_packed, int n_cw, int n_iter,
                int early, cudaStream_t s) {
    const size_t round = static_cast<size_t>(h->max_grid) * h->cpb;
    // fp32 buffers the GPU can address: DIRECT decodes the batch straight
    // from host memory; AUTO does so on a coherent link up to
    // kDirectMaxRounds CTA rounds (beyond that the per-group wait for host
    // memory costs more than the staged copies do)
    if (qtype == 0 && h->host_mode != NRLDPC_HOST_COPY) {
        const float* d_in = static_cast<const float*>(pinned_device_view(h_llr));
        uint8_t* d_out = static_cast<uint8_t*>(pinned_device_view(h_packed));
        const bool usable = d_in && d_out && reinterpret_cast<uintptr_t>(d_in) % 16 == 0;
        if (h->host_mode == NRLDPC_HOST_DIRECT && !usable) return NRLDPC_ERR_INVALID_ARG;
        if (usable && (h->host_mode == NRLDPC_HOST_DIRECT ||
                       (h->coherent_host && static_cast<size_t>(n_cw) <= kDirectMaxRounds * round)))
            return decode_impl(h, d_in, d_out, n_cw, n_iter, early, nullptr, nullptr, false, s, true);
    }
    const size_t n_bp = static_cast<size_t>(h->tab.n_bp);
    const size_t in_elem = qtype == 0 ? 4 : (qtype == 1 ? 2 : 1);
    void* stage_in = qtype == 0 ? static_cast<void*>(h->stage_llr) : h->stage_q;
    // per-chunk work counters zeroed at once; the copy stream must not
    // overwrite staging a previous call still reads, and the second lane
    // starts after the caller's earlier work
    if (cudaMemsetAsync(h->scratch + kChunkCounter, 0, kHostChunks * sizeof(int), s) != cudaSuccess ||
        cudaEventRecord(h->ev_start, s) != cudaSuccess ||
        cudaStreamWaitEvent(h->copy_stream, h->ev_start, 0) != cudaSuccess ||
        cudaStreamWaitEvent(h->lane_stream, h->ev_start, 0) != cudaSuccess)
        return NRLDPC_ERR_CUDA;
    int rc = NRLDPC_OK;
    size_t begin = 0;
    size_t rounds = 1;
    for (int k = 0; begin < static_cast<size_t>(n_cw); k++) {
        size_t count = std::min(static_cast<size_t>(n_cw) - begin, rounds * round);
        if (k == kHostChunks - 1) count = static_cast<size_t>(n_cw) - begin;  // last event: the rest
        rounds *= 2;  // each copy hides behind the decode of a chunk half its size
        cudaStream_t ls = (k & 1) ? h->lane_stream : s;
        const char* src = static_cast<const char*>(h_llr) + begin * n_bp * in_elem;
        char* dst = static_cast<char*>(stage_in) + begin * n_bp * in_elem;
        if (cudaMemcpyAsync(dst, src, count * n_bp * in_elem, cudaMemcpyHostToDevice, h->copy_stream) !=
                cudaSuccess ||
            cudaEventRecord(h->ev_chunk[k], h->copy_stream) != cudaSuccess ||
            cudaStreamWaitEvent(ls, h->ev_chunk[k], 0) != cudaSuccess) {
            rc = NRLDPC_ERR_CUDA;
            break;
        }
        float* llr = h->stage_llr + begin * n_bp;
        if (qtype != 0 && launch_dequant(dst, qtype, scale, count * n_bp, llr, ls) != cudaSuccess) {
            rc = NRLDPC_ERR_CUDA;
            break;
        }
        uint8_t* out = h->stage_packed + begin * h->tab.packed_bytes;
        rc = decode_impl(h, llr, out, static_cast<int>(count), n_iter, early, nullptr, nullptr, false, ls, false,
                         h->scratch + kChunkCounter + k, (k & 1) ? h->state2 : h->state);
        if (rc) break;
        if (cudaMemcpyAsync(h_packed + begin * h->tab.packed_bytes, out, count * h->tab.packed_bytes,
                            cudaMemcpyDeviceToHost, ls) != cudaSuccess) {
            rc = NRLDPC_ERR_CUDA;
            break;
        }
        begin += count;
    }
    // the caller's stream covers the second lane's work too
    if (cudaEventRecord(h->ev_lane, h->lane_stream) != cudaSuccess ||
        cudaStreamWaitEvent(s, h->ev_lane, 0) != cudaSuccess)
        return NRLDPC_ERR_CUDA;
    return rc;
}

}  // namespace

namespace nrldpc {
// Lifted-code table of 5G NR (bg, z) without any heap allocation.
bool make_nr_table(int bg, int z, CodeTable* t) {
    const int ils = nrldpc_set_index(z);
    if ((bg != 1 && bg != 2) || ils < 0) return false;
    int H[kMaxRows * kMaxCols];
    int rows = 0, cols = 0;
    if (base_matrix_impl(bg, ils, H, &rows, &cols) != NRLDPC_OK) return false;
    return fill_table(H, rows, cols, z, bg == 1 ? 22 : 10, t);
}
}  // namespace nrldpc

extern "C" {

int nrldpc_set_index(int z) {
    for (int i = 0; i < 8; i++)
        for (int v = kBaseZ[i]; v <= 384; v *= 2)
            if (v == z) return i;
    return -1;
}

int nrldpc_base_matrix(int bg, int ils, int* out, int* rows, int* cols) {
    return base_matrix_impl(bg, ils, out, rows, cols);
}

// Mirror of setup_ldpc (src/nr_ldpc.cpp:31-230), quirks included.
int nrldpc_setup_ldpc(int A, float rate, int n_iterations, nrldpc_ldpc_params* o) {
    if (!o) return NRLDPC_ERR_INVALID_ARG;
    const int l = (A > 3824) ? 24 : 16;
    const int B = A + l;
    int bg, k_cb, k_b;
    if ((A <= 292) || (A < 3824 && rate <= 0.67) || (rate <= 0.25)) {
        bg = 2;
        k_cb = 3840;
        k_b = B > 640 ? 10 : B > 560 ? 9 : B > 192 ? 8 : 6;
    } else {
        bg = 1;
        k_cb = 8448;
        k_b = 22;
    }
    int C, b_prime;
    if (B <= k_cb) {
        C = 1;
        b_prime = B;
    } else {
        C = B / (k_cb - 24);  // ceil() of an integer quotient, as the reference
        b_prime = B + C * 24;
    }
    const int k_prime = b_prime / C;
    const int z_min = k_prime / k_b;
    int z_c = 1000, i_ls = -1;
    for (int i = 0; i < 8; i++) {
        int t = kBaseZ[i];
        for (int k = 0; k < 8; k++) {
            const int v = t < 385 ? t : 0;
            t *= 2;
            if (v >= z_min && v < z_c) {
                z_c = v;
                i_ls = i;
            }
        }
    }
    if (i_ls < 0) return NRLDPC_ERR_BAD_CONFIG;
    std::memset(o, 0, sizeof(*o));
    o->A = A;
    o->rate = rate;
    o->bg_index = bg;
    o->Z = z_c;
    o->K = bg == 1 ? 22 * z_c : 10 * z_c;
    o->N = bg == 1 ? 66 * z_c : 50 * z_c;
    o->H_rows = bg == 1 ? 46 : 42;
    o->H_cols = bg == 1 ? 68 : 52;
    std::vector<int> H(o->H_rows * o->H_cols);
    base_matrix_impl(bg, i_ls, H.data(), nullptr, nullptr);
    int mr = 0, mc = 0;
    for (int r = 0; r < o->H_rows; r++) {
        int c = 0;
        for (int j = 0; j < o->H_cols; j++) c += H[r * o->H_cols + j] != -1;
        mr = std::max(mr, c);
    }
    for (int j = 0; j < o->H_cols; j++) {
        int c = 0;
        for (int r = 0; r < o->H_rows; r++) c += H[r * o->H_cols + j] != -1;
        mc = std::max(mc, c);
    }
    o->n_nz_in_row = mr;
    o->n_nz_in_col = mc;
    o->n_iterations = n_iterations;
    o->N_before_puncture = o->N + 2 * z_c;
    o->i_ls = i_ls;
    o->C = C;
    o->K_b = k_b;
    return NRLDPC_OK;
}

int nrldpc_init(const nrldpc_config* cfg, nrldpc_handle** out) {
    if (!cfg || !out) return NRLDPC_ERR_INVALID_ARG;
    const int ils = nrldpc_set_index(cfg->z);
    if ((cfg->bg != 1 && cfg->bg != 2) || ils < 0) return NRLDPC_ERR_BAD_CONFIG;
    int rows = 0, cols = 0;
    std::vector<int> H(46 * 68);
    base_matrix_impl(cfg->bg, ils, H.data(), &rows, &cols);
    return init_impl(H.data(), rows, cols, cfg->bg == 1 ? 22 : 10, cfg, out);
}

int nrldpc_init_custom(const int* base, int rows, int cols, const nrldpc_config* cfg,
                       nrldpc_handle** out) {
    if (!base || !cfg || !out) return NRLDPC_ERR_INVALID_ARG;
    // systematic columns: everything before the first column of the parity staircase
    return init_impl(base, rows, cols, cols - rows, cfg, out);
}

int nrldpc_destroy(nrldpc_handle* handle) {
    free_handle(reinterpret_cast<Handle*>(handle));
    return NRLDPC_OK;
}

int nrldpc_geometry(const nrldpc_handle* handle, int* rows, int* cols, int* z, int* n_edges,
                    int* n_bp, int* packed_bytes) {
    const Handle* h = reinterpret_cast<const Handle*>(handle);
    if (!h) return NRLDPC_ERR_INVALID_ARG;
    if (rows) *rows = h->tab.rows;
    if (cols) *cols = h->tab.cols;
    if (z) *z = h->tab.z;
    if (n_edges) *n_edges = h->tab.n_edges;
    if (n_bp) *n_bp = h->tab.n_bp;
    if (packed_bytes) *packed_bytes = h->tab.packed_bytes;
    return NRLDPC_OK;
}

int nrldpc_decode(nrldpc_handle* handle, const float* d_llr, uint8_t* d_packed, int n_cw,
                  int n_iter, int early_stop, float* d_app, int32_t* d_iters,
                  nrldpc_stream_t stream) {
    return decode_impl(reinterpret_cast<Handle*>(handle), d_llr, d_packed, n_cw, n_iter, early_stop,
                       d_app, d_iters, false, reinterpret_cast<cudaStream_t>(stream));
}

int nrldpc_selftest_wait_timeout(nrldpc_handle* handle, const float* d_llr, uint8_t* d_packed, int n_cw,
                                 nrldpc_stream_t stream) {
    // 16 bytes more than the copies deliver, 1024 wait iterations
    return decode_impl(reinterpret_cast<Handle*>(handle), d_llr, d_packed, n_cw, 1, 0, nullptr, nullptr, false,
                       reinterpret_cast<cudaStream_t>(stream), false, nullptr, nullptr, 1024, 16);
}

int nrldpc_decode_weighted(nrldpc_handle* handle, const float* d_llr, uint8_t* d_packed, int n_cw,
                           int n_iter, int early_stop, float* d_app, int32_t* d_iters,
                           nrldpc_stream_t stream) {
    return decode_impl(reinterpret_cast<Handle*>(handle), d_llr, d_packed, n_cw, n_iter, early_stop,
                       d_app, d_iters, true, reinterpret_cast<cudaStream_t>(stream));
}

int nrldpc_decode_host_async(nrldpc_handle* handle, const float* h_llr, uint8_t* h_packed,
                             int n_cw, int n_iter, int early_stop, nrldpc_stream_t stream) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h || !h_llr || !h_packed || n_cw < 0) return NRLDPC_ERR_INVALID_ARG;
    if (n_cw > h->max_batch) return NRLDPC_ERR_TOO_LARGE;
    if (n_cw == 0) return NRLDPC_OK;
    if (n_iter < 1 || (early_stop != 0 && early_stop != 1)) return NRLDPC_ERR_INVALID_ARG;
    return host_decode(h, h_llr, 0, 1.0f, h_packed, n_cw, n_iter, early_stop,
                       reinterpret_cast<cudaStream_t>(stream));
}

int nrldpc_decode_host_async_q(nrldpc_handle* handle, const void* h_llr_q, int qtype, float scale,
                               uint8_t* h_packed, int n_cw, int n_iter, int early_stop,
                               nrldpc_stream_t stream) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h || n_cw < 0 || (qtype != 1 && qtype != 2) || (qtype == 2 && !(scale > 0.0f)))
        return NRLDPC_ERR_INVALID_ARG;
    if (n_cw > h->max_batch) return NRLDPC_ERR_TOO_LARGE;
    if (n_cw == 0) return NRLDPC_OK;
    if (!h_llr_q || !h_packed) return NRLDPC_ERR_INVALID_ARG;
    if (n_iter < 1 || (early_stop != 0 && early_stop != 1)) return NRLDPC_ERR_INVALID_ARG;
    if (!h->stage_q) {  // narrow staging, allocated on the first call of this entry point
        const size_t cap = static_cast<size_t>(h->max_batch) * h->tab.n_bp * 2;
        if (cudaMalloc(&h->stage_q, cap) != cudaSuccess) {
            h->stage_q = nullptr;
            return NRLDPC_ERR_NO_MEMORY;
        }
    }
    return host_decode(h, h_llr_q, qtype, scale, h_packed, n_cw, n_iter, early_stop,
                       reinterpret_cast<cudaStream_t>(stream));
}

int nrldpc_set_host_transfer(nrldpc_handle* handle, int mode) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h || (mode != NRLDPC_HOST_AUTO && mode != NRLDPC_HOST_COPY && mode != NRLDPC_HOST_DIRECT))
        return NRLDPC_ERR_INVALID_ARG;
    h->host_mode = mode;
    return NRLDPC_OK;
}

int nrldpc_set_schedule(nrldpc_handle* handle, int schedule) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h || (schedule != NRLDPC_SCHEDULE_FLOODING && schedule != NRLDPC_SCHEDULE_LAYERED))
        return NRLDPC_ERR_INVALID_ARG;
    h->schedule = schedule;
    return NRLDPC_OK;
}

int nrldpc_set_weights(nrldpc_handle* handle, const float* w, int n_w_iters) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h || n_w_iters < 0 || (n_w_iters > 0 && !w)) return NRLDPC_ERR_INVALID_ARG;
    if (n_w_iters > kMaxWIters) return NRLDPC_ERR_TOO_LARGE;
    delete h->weights;
    h->weights = nullptr;
    h->n_w_iters = 0;
    if (n_w_iters == 0) return NRLDPC_OK;
    h->weights = new (std::nothrow) WeightTable();  // zero-initialised, incl. the zero row
    if (!h->weights) return NRLDPC_ERR_NO_MEMORY;
    for (int t = 0; t < n_w_iters; t++)
        std::memcpy(h->weights->w[t], w + static_cast<size_t>(t) * h->tab.n_edges,
                    sizeof(float) * h->tab.n_edges);
    h->n_w_iters = n_w_iters;
    return NRLDPC_OK;
}

// ---- learned weighted min-sum training --------------------------------------------------
namespace {
struct WmsLayout {
    size_t states, gseed, gq, gh, total;
};
// Kernel attributes and CTAs per SM of the training kernels, once per handle.
int wms_prepare(Handle* h) {
    if (h->wms_ready) return NRLDPC_OK;
    const size_t smem = wms_smem_bytes(h->tab, h->cpb);
    if (cudaSetDevice(h->device) != cudaSuccess || wms_kernel_attributes(smem) != cudaSuccess)
        return NRLDPC_ERR_CUDA;
    h->wms_ctas = std::max(1, wms_ctas_per_sm(h->tab, h->threads, smem));
    h->wms_ready = true;
    return NRLDPC_OK;
}
// Workspace: per-iteration states and loss seeds, the flooding adjoint's
// per-row dloss/dQ, and (layered schedule) the per-edge dloss/dR, the last
// two per resident CTA slot.
WmsLayout wms_layout(const Handle* h, int n_cw, int n_iter) {
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    WmsLayout l;
    const size_t rz = static_cast<size_t>(h->tab.rows) * h->tab.z;
    const size_t slots = static_cast<size_t>(h->sm_count) * h->wms_ctas * h->cpb;
    l.states = up(static_cast<size_t>(n_iter) * n_cw * rz * sizeof(uint4));
    l.gseed = up(static_cast<size_t>(n_iter) * n_cw * h->tab.n_bp * sizeof(float));
    l.gq = up(slots * rz * sizeof(uint4));
    l.gh = h->schedule == NRLDPC_SCHEDULE_LAYERED
               ? up(slots * static_cast<size_t>(h->tab.n_edges) * h->tab.z * sizeof(float))
               : 0;
    l.total = l.states + l.gseed + l.gq + l.gh;
    return l;
}
int wms_check(Handle* h, int n_cw, int n_iter) {
    if (!h || n_cw < 1 || n_iter < 1) return NRLDPC_ERR_INVALID_ARG;
    if (n_cw > h->max_batch) return NRLDPC_ERR_TOO_LARGE;
    return wms_prepare(h);
}
}  // namespace

int nrldpc_wms_workspace_bytes(nrldpc_handle* handle, int n_cw, int n_iter, size_t* bytes) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h || !bytes || n_cw < 1 || n_iter < 1) return NRLDPC_ERR_INVALID_ARG;
    const int rc = wms_prepare(h);
    if (rc) return rc;
    *bytes = wms_layout(h, n_cw, n_iter).total;
    return NRLDPC_OK;
}

int nrldpc_wms_forward(nrldpc_handle* handle, const float* d_llr, const uint8_t* d_cw_packed, int n_cw,
                       int n_iter, const float* d_weights, void* d_workspace, float loss_scale,
                       double* d_loss, float* d_app, nrldpc_stream_t stream) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    int rc = wms_check(h, n_cw, n_iter);
    if (rc) return rc;
    if (!d_llr || !d_cw_packed || !d_weights || !d_workspace || !d_loss) return NRLDPC_ERR_INVALID_ARG;
    if (reinterpret_cast<uintptr_t>(d_llr) % 16 != 0) return NRLDPC_ERR_ALIGNMENT;
    const WmsLayout l = wms_layout(h, n_cw, n_iter);
    char* ws = static_cast<char*>(d_workspace);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(h->scratch, 0, sizeof(int), st) != cudaSuccess) return NRLDPC_ERR_CUDA;
    const bool lay = h->schedule == NRLDPC_SCHEDULE_LAYERED;
    return map_cuda(launch_wms(false, lay, h->tab, d_llr, d_cw_packed, d_weights,
                               reinterpret_cast<uint4*>(ws), reinterpret_cast<float*>(ws + l.states),
                               reinterpret_cast<uint4*>(ws + l.states + l.gseed),
                               lay ? reinterpret_cast<float*>(ws + l.states + l.gseed + l.gq) : nullptr,
                               d_loss, nullptr,
                               d_app, h->scratch, n_cw, n_iter, h->cpb, h->sm_count * h->wms_ctas, h->threads,
                               wms_smem_bytes(h->tab, h->cpb), loss_scale, st));
}

int nrldpc_wms_backward(nrldpc_handle* handle, int n_cw, int n_iter, const float* d_weights,
                        void* d_workspace, double* d_grad, nrldpc_stream_t stream) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    int rc = wms_check(h, n_cw, n_iter);
    if (rc) return rc;
    if (!d_weights || !d_workspace || !d_grad) return NRLDPC_ERR_INVALID_ARG;
    const WmsLayout l = wms_layout(h, n_cw, n_iter);
    char* ws = static_cast<char*>(d_workspace);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(h->scratch, 0, sizeof(int), st) != cudaSuccess) return NRLDPC_ERR_CUDA;
    const bool lay = h->schedule == NRLDPC_SCHEDULE_LAYERED;
    return map_cuda(launch_wms(true, lay, h->tab, nullptr, nullptr, d_weights, reinterpret_cast<uint4*>(ws),
                               reinterpret_cast<float*>(ws + l.states),
                               reinterpret_cast<uint4*>(ws + l.states + l.gseed),
                               lay ? reinterpret_cast<float*>(ws + l.states + l.gseed + l.gq) : nullptr,
                               nullptr, d_grad,
                               nullptr, h->scratch, n_cw, n_iter, h->cpb, h->sm_count * h->wms_ctas, h->threads,
                               wms_smem_bytes(h->tab, h->cpb), 0.0f, st));
}

int nrldpc_adam_step(int n, float* d_w, const double* d_grad, float* d_m, float* d_v, int step,
                     float lr, float beta1, float beta2, float eps, float w_min,
                     nrldpc_stream_t stream) {
    if (n < 1 || !d_w || !d_grad || !d_m || !d_v || step < 1) return NRLDPC_ERR_INVALID_ARG;
    return map_cuda(launch_adam(n, d_w, d_grad, d_m, d_v, step, lr, beta1, beta2, eps, w_min,
                                reinterpret_cast<cudaStream_t>(stream)));
}

int nrldpc_gen_llr(nrldpc_handle* handle, uint64_t seed, uint64_t cw_base, int n_cw,
                   const float* d_sigma, int n_punct_cols, float* d_llr, uint8_t* d_cw_packed,
                   nrldpc_stream_t stream) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h || !d_sigma || !d_llr || n_cw < 0 || n_punct_cols < 0 || n_punct_cols > h->tab.cols)
        return NRLDPC_ERR_INVALID_ARG;
    if (!h->plan_ok) return NRLDPC_ERR_BAD_CONFIG;
    if (n_cw == 0) return NRLDPC_OK;
    return map_cuda(launch_gen_llr(h->tab, h->plan, seed, cw_base, n_cw, d_sigma, n_punct_cols, d_llr,
                                   d_cw_packed, reinterpret_cast<cudaStream_t>(stream)));
}

int nrldpc_count_errors(nrldpc_handle* handle, const uint8_t* d_packed, const uint8_t* d_cw_packed,
                        int n_cw, int n_info, unsigned long long* d_counts, nrldpc_stream_t stream) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h || !d_packed || !d_cw_packed || !d_counts || n_cw < 0 || n_info < 0 ||
        n_info > h->tab.n_bp)
        return NRLDPC_ERR_INVALID_ARG;
    if (n_cw == 0) return NRLDPC_OK;
    return map_cuda(launch_count_errors(d_packed, d_cw_packed, n_cw, h->tab.packed_bytes, n_info,
                                        d_counts, reinterpret_cast<cudaStream_t>(stream)));
}

int nrldpc_crc(const uint8_t* d_packed, int n_cw, int stride_bytes, int n_bits, int crc_type,
               uint32_t* d_rem, nrldpc_stream_t stream) {
    // generator polynomials of TS 38.212 5.1 without the leading term:
    //   CRC24A: D^24+D^23+D^18+D^17+D^14+D^11+D^10+D^7+D^6+D^5+D^4+D^3+D+1
    //   CRC24B: D^24+D^23+D^6+D^5+D+1          CRC16: D^16+D^12+D^5+1
    static const uint32_t polys[3] = {0x864CFBu, 0x800063u, 0x1021u};
    static const int lens[3] = {24, 24, 16};
    if (crc_type < 0 || crc_type > 2 || n_cw < 0 || n_bits < 0 || stride_bytes * 8 < n_bits)
        return NRLDPC_ERR_INVALID_ARG;
    if (n_cw == 0) return NRLDPC_OK;
    if (!d_packed || !d_rem) return NRLDPC_ERR_INVALID_ARG;
    return map_cuda(launch_crc(d_packed, n_cw, stride_bytes, n_bits, polys[crc_type], lens[crc_type],
                               d_rem, reinterpret_cast<cudaStream_t>(stream)));
}

int nrldpc_segment(int B, int bg, nrldpc_segment_info* out) {
    if (!out || B < 1 || (bg != 1 && bg != 2)) return NRLDPC_ERR_INVALID_ARG;
    const int kcb = bg == 1 ? 8448 : 3840;  // maximum code block size
    nrldpc_segment_info g{};
    g.B = B;
    g.bg = bg;
    if (B <= kcb) {
        g.L = 0;
        g.C = 1;
    } else {
        g.L = 24;
        g.C = (B + (kcb - g.L) - 1) / (kcb - g.L);
    }
    const long bp = static_cast<long>(B) + static_cast<long>(g.C) * g.L;
    if (bp % g.C != 0) return NRLDPC_ERR_BAD_CONFIG;  // not a TS 38.214 transport block size
    g.k_prime = static_cast<int>(bp / g.C);
    if (bg == 1)
        g.kb = 22;
    else
        g.kb = B > 640 ? 10 : (B > 560 ? 9 : (B > 192 ? 8 : 6));
    int zc = 0;  // smallest lifting size of any set with kb * Z >= K'
    for (int i = 0; i < 8; i++)
        for (int z = kBaseZ[i]; z <= 384; z *= 2)
            if (g.kb * z >= g.k_prime && (zc == 0 || z < zc)) zc = z;
    if (zc == 0) return NRLDPC_ERR_BAD_CONFIG;
    g.zc = zc;
    g.k = (bg == 1 ? 22 : 10) * zc;
    g.filler = g.k - g.k_prime;
    *out = g;
    return NRLDPC_OK;
}

int nrldpc_cb_segment(const uint8_t* d_tb, const nrldpc_segment_info* info, uint8_t* d_blocks,
                      int block_stride, nrldpc_stream_t stream) {
    if (!info || !d_tb || !d_blocks || info->C < 1 || info->k_prime < 1 || info->L < 0 ||
        info->k_prime <= info->L || block_stride * 8 < info->k_prime)
        return NRLDPC_ERR_INVALID_ARG;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int data_bits = info->k_prime - info->L;
    if (launch_cb_gather_blocks(d_tb, info->C, data_bits, info->k_prime, d_blocks, block_stride, st) !=
        cudaSuccess)
        return NRLDPC_ERR_CUDA;
    if (info->L == 0) return NRLDPC_OK;
    return map_cuda(launch_cb_attach_crc(d_blocks, info->C, data_bits, block_stride, 0x800063u, 24, st));
}

int nrldpc_cb_desegment(const uint8_t* d_blocks, int block_stride, const nrldpc_segment_info* info,
                        uint8_t* d_tb, uint32_t* d_crc_rem, nrldpc_stream_t stream) {
    if (!info || !d_tb || !d_blocks || info->C < 1 || info->k_prime < 1 || info->L < 0 ||
        info->k_prime <= info->L || block_stride * 8 < info->k_prime || (info->L > 0 && !d_crc_rem))
        return NRLDPC_ERR_INVALID_ARG;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (info->L > 0 &&
        launch_crc(d_blocks, info->C, block_stride, info->k_prime, 0x800063u, 24, d_crc_rem, st) != cudaSuccess)
        return NRLDPC_ERR_CUDA;
    return map_cuda(launch_cb_gather_tb(d_blocks, block_stride, info->C, info->k_prime - info->L, d_tb, st));
}

int nrldpc_device_error(nrldpc_handle* handle) {
    Handle* h = reinterpret_cast<Handle*>(handle);
    if (!h) return NRLDPC_ERR_INVALID_ARG;
    int v = 0;
    if (cudaMemcpy(&v, h->scratch + 1, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return NRLDPC_ERR_CUDA;
    if (v) cudaMemset(h->scratch + 1, 0, sizeof(int));
    return v ? NRLDPC_ERR_TIMEOUT : NRLDPC_OK;
}

const char* nrldpc_status_string(int status) {
    switch (status) {
        case NRLDPC_OK: return "ok";
        case NRLDPC_ERR_INVALID_ARG: return "invalid argument";
        case NRLDPC_ERR_BAD_CONFIG: return "unsupported code configuration";
        case NRLDPC_ERR_CUDA: return "CUDA error";
        case NRLDPC_ERR_ALIGNMENT: return "device LLR pointer not 16-byte aligned";
        case NRLDPC_ERR_TOO_LARGE: return "batch larger than max_batch";
        case NRLDPC_ERR_TIMEOUT: return "device-side wait timed out";
        case NRLDPC_ERR_NO_MEMORY: return "allocation failed";
        case NRLDPC_ERR_NO_DEVICE: return "no usable CUDA device";
        case NRLDPC_ERR_SCRATCH_TOO_SMALL:
            return "code needs more check-node scratch than the fixed no-alloc array holds";
        default: return "unknown status";
    }
}

}  // extern "C"
