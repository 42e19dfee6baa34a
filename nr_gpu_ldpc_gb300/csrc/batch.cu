// Mixed-code batches: every 5G NR (BG, Z) in one handle, a device work queue
// of codeword groups, one persistent decode launch replayed from a CUDA graph,
// and job-based rate matching (3GPP TS 38.212 5.4.2.1 bit selection with
// filler bits, full circular buffer, BPSK so no interleaver) on the GPU.
// No reference counterpart: the reference compiles in one base graph and one
// Z per process (src/globals.h:15, constant memory in src/ldpc_kernels.cu:18-27)
// and has no rate matching (src/main.cpp:64-65).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/nr_gpu_ldpc_gb300.h"
#include "channel_dev.cuh"
#include "nrldpc_internal.h"

namespace nrldpc {
bool make_nr_table(int bg, int z, CodeTable* t);
}

using namespace nrldpc;

namespace {

constexpr int kNumZ = 51;
constexpr int kNumCodes = 2 * kNumZ;
constexpr int kBaseZ[8] = {2, 3, 5, 7, 9, 11, 13, 15};

struct PlanDev {
    int32_t n_stair, p0_col, p0_shift, n_steps;
    uint8_t step_row[kMaxRows];
    uint8_t step_col[kMaxRows];
};

static_assert(sizeof(nrldpc_job) == 56, "nrldpc_job layout (mirrored by the Python binding)");

// Rate-matching geometry of one job, resolved on the host.
struct JobDev {
    int32_t code;
    int32_t k_prime;   // info bits (filler from k_prime to kb*Z)
    int32_t e;         // transmitted bits
    int32_t k0;        // start in the circular buffer
    float sigma;
    int32_t qm;        // modulation order of the bit interleaver (1: none)
    int64_t llr_offset, e_offset, out_offset;
};

int z_list[kNumZ];
int z_index(int z) {
    for (int i = 0; i < kNumZ; i++)
        if (z_list[i] == z) return i;
    return -1;
}
void init_z_list() {
    if (z_list[0]) return;
    int n = 0;
    for (int zz = 2; zz <= 384; zz++)
        for (int i = 0; i < 8; i++) {
            bool hit = false;
            for (int v = kBaseZ[i]; v <= 384; v *= 2) hit |= v == zz;
            if (hit) {
                z_list[n++] = zz;
                break;
            }
        }
}

int rm_k0(int bg, int z, int rv) {
    static const int a1[4] = {0, 17, 33, 56}, a2[4] = {0, 13, 25, 43};
    if (rv < 0 || rv > 3 || (bg != 1 && bg != 2)) return -1;
    const long n = bg == 1 ? 66 : 50, ncb = n * z;  // full buffer
    return static_cast<int>(((bg == 1 ? a1[rv] : a2[rv]) * ncb) / (n * z)) * z;
}

// d index of transmitted bit k (filler run [f0, f1) of d removed, wrap at Ncb).
__device__ __forceinline__ int rm_index(int z, int ncb, int kbz, int kp, int k0, int k) {
    const int f0 = kp - 2 * z, f1 = kbz - 2 * z, nf = f1 - f0, nc = ncb - nf;
    const int c0 = k0 < f0 ? k0 : (k0 < f1 ? f0 : k0 - nf);
    const int c = static_cast<int>((static_cast<long long>(c0) + k) % nc);
    return c < f0 ? c : c + nf;
}

struct GenBatchArgs {
    const CodeTable* tables;
    const PlanDev* plans;
    const JobDev* jobs;
    float* llr_e;
    uint8_t* cw;
    uint64_t seed, cw_base;
    int n_jobs;
};

// Bit interleaver of TS 38.212 5.4.2.2, f[i + j*Qm] = e[i*E/Qm + j]: the e
// index of the bit sent at position p, and the position of e index k.
__device__ __forceinline__ int il_src(int e, int qm, int p) {
    return qm == 1 ? p : (p % qm) * (e / qm) + p / qm;
}
__device__ __forceinline__ int il_pos(int e, int qm, int k) {
    if (qm == 1) return k;
    const int rows = e / qm;
    return k / rows + (k % rows) * qm;
}

// One CTA per job: info bits, encode, select e bits from k0, interleave,
// BPSK + AWGN per transmitted position.
__global__ void __launch_bounds__(256) batch_gen_kernel(const __grid_constant__ GenBatchArgs g) {
    extern __shared__ uint8_t x[];  // [n_bp] codeword bits, then [z] scratch
    const uint32_t k0s = static_cast<uint32_t>(g.seed), k1s = static_cast<uint32_t>(g.seed >> 32);
    for (int i = blockIdx.x; i < g.n_jobs; i += gridDim.x) {
        const JobDev jb = g.jobs[i];
        const CodeTable& tab = g.tables[jb.code];
        const PlanDev& pl = g.plans[jb.code];
        const int z = tab.z, n = tab.n_bp, K = tab.kb * z, ncb = n - 2 * z;
        uint8_t* acc = x + n;
        const uint64_t id = g.cw_base + static_cast<uint64_t>(i);
        const uint32_t id0 = static_cast<uint32_t>(id), id1 = static_cast<uint32_t>(id >> 32);
        for (int b = threadIdx.x; b * 128 < K; b += blockDim.x) {
            uint32_t o[4];
            dev::philox4x32(static_cast<uint32_t>(b), id0, id1, 1u, k0s, k1s, o);
            for (int j = 0; j < 128 && b * 128 + j < K; j++) {
                const int pos = b * 128 + j;
                x[pos] = pos < jb.k_prime ? (o[j >> 5] >> (j & 31)) & 1u : 0u;
            }
        }
        __syncthreads();
        dev::encode_in_smem(tab, pl.n_stair, pl.p0_col, pl.p0_shift, pl.n_steps, pl.step_row,
                            pl.step_col, x, acc);
        if (g.cw) {
            uint8_t* out = g.cw + jb.out_offset;
            for (int b = threadIdx.x; b < tab.packed_bytes; b += blockDim.x) {
                uint32_t v = 0;
                for (int j = 0; j < 8; j++)
                    if (8 * b + j < n) v |= static_cast<uint32_t>(x[8 * b + j]) << j;
                out[b] = static_cast<uint8_t>(v);
            }
        }
        const float sg = jb.sigma, s2 = __fmul_rn(sg, sg);
        float* out = g.llr_e + jb.e_offset;
        for (int t = threadIdx.x; t * 4 < jb.e; t += blockDim.x) {
            uint32_t o[4];
            dev::philox4x32(static_cast<uint32_t>(t), id0, id1, 3u, k0s, k1s, o);
            float gs[4];
            dev::gauss4(o, gs);
            for (int q = 0; q < 4 && 4 * t + q < jb.e; q++) {
                const int p = 4 * t + q;
                const int j = 2 * z + rm_index(z, ncb, K, jb.k_prime, jb.k0, il_src(jb.e, jb.qm, p));
                out[p] = dev::bpsk_llr(x[j], gs[q], sg, s2);
            }
        }
        __syncthreads();
    }
}

struct DerateArgs {
    const CodeTable* tables;
    const JobDev* jobs;
    const float* llr_e;
    float* llr;
    int n_jobs;
};

// One CTA per job.  Each non-filler position c of the compressed buffer
// collects bits k = k_first, k_first + Nc, ... (< e) in order, each read from
// its interleaved position; the first copy is taken as is, later copies added.
__global__ void __launch_bounds__(256) batch_derate_kernel(const __grid_constant__ DerateArgs a) {
    for (int i = blockIdx.x; i < a.n_jobs; i += gridDim.x) {
        const JobDev jb = a.jobs[i];
        const CodeTable& tab = a.tables[jb.code];
        const int z = tab.z, n = tab.n_bp, K = tab.kb * z, ncb = n - 2 * z;
        const int f0 = jb.k_prime - 2 * z, nf = K - jb.k_prime, nc = ncb - nf;
        const int c0 = jb.k0 < f0 ? jb.k0 : (jb.k0 < f0 + nf ? f0 : jb.k0 - nf);
        float* out = a.llr + jb.llr_offset;
        const float* in = a.llr_e + jb.e_offset;
        for (int j = threadIdx.x; j < 2 * z; j += blockDim.x) out[j] = 0.0f;
        for (int j = jb.k_prime + threadIdx.x; j < K; j += blockDim.x) out[j] = __int_as_float(0x7f800000);
        for (int c = threadIdx.x; c < nc; c += blockDim.x) {
            const int kf = (c - c0 + nc) % nc;
            float v = 0.0f;
            if (kf < jb.e) {
                v = in[il_pos(jb.e, jb.qm, kf)];
                for (int k = kf + nc; k < jb.e; k += nc) v = __fadd_rn(v, in[il_pos(jb.e, jb.qm, k)]);
            }
            out[2 * z + (c < f0 ? c : c + nf)] = v;
        }
        __syncthreads();
    }
}

struct CountArgs {
    const CodeTable* tables;
    const JobDev* jobs;
    const uint8_t* packed;
    const uint8_t* cw;
    unsigned long long* counts;
    int n_jobs;
};

__global__ void __launch_bounds__(256) batch_count_kernel(const __grid_constant__ CountArgs a) {
    __shared__ unsigned int warp_sum[8];
    for (int i = blockIdx.x; i < a.n_jobs; i += gridDim.x) {
        const JobDev jb = a.jobs[i];
        const uint8_t* p = a.packed + jb.out_offset;
        const uint8_t* q = a.cw + jb.out_offset;
        const int full = jb.k_prime / 8, rem = jb.k_prime % 8;
        unsigned int errs = 0;
        for (int k = threadIdx.x; k < full; k += blockDim.x) errs += __popc(p[k] ^ q[k]);
        if (rem && threadIdx.x == 0) errs += __popc((p[full] ^ q[full]) & ((1u << rem) - 1u));
        for (int off = 16; off > 0; off >>= 1) errs += __shfl_down_sync(0xffffffffu, errs, off);
        if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = errs;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned int tot = 0;
            for (int w = 0; w < (blockDim.x + 31) / 32; w++) tot += warp_sum[w];
            if (tot) {
                atomicAdd(&a.counts[0], static_cast<unsigned long long>(tot));
                atomicAdd(&a.counts[1], 1ull);
            }
        }
        __syncthreads();
    }
}

struct Batch {
    int device = 0;
    float alpha = 0.75f;
    int max_jobs = 0;
    int sm_count = 1;
    size_t smem_optin = 0;
    CodeTable h_tables[kNumCodes];
    bool code_ok[kNumCodes];
    int cpb[kNumCodes];
    int spt[kNumCodes];  // sub-rows per thread (threads per codeword = Z / spt)
    CodeTable* d_tables = nullptr;
    PlanDev* d_plans = nullptr;
    // job list
    int n_jobs = 0, n_items = 0;
    std::vector<JobDev> h_jobs;
    JobDev* d_jobs_rm = nullptr;
    nrldpc_job* d_jobs = nullptr;
    int32_t* d_order = nullptr;
    WorkItem* d_items = nullptr;
    size_t slot_words = 0, smem = 0;
    int grid = 0, threads = kMaxThreads;
    uint32_t* d_state = nullptr;
    size_t state_words = 0;
    int* d_scratch = nullptr;
    // decode graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t knode = nullptr;
    BatchDecodeArgs kargs{};
};

int map_cuda(cudaError_t e) { return e == cudaSuccess ? NRLDPC_OK : NRLDPC_ERR_CUDA; }

// Most codewords per CTA of code id with spt sub-rows per thread: Z / spt
// threads each within kMaxThreads, and their shared memory within the
// device's opt-in limit.
int max_cpb(const Batch* b, int id, int spt) {
    const CodeTable& t = b->h_tables[id];
    const int tpc = t.z / spt;
    const size_t room = b->smem_optin - kHeaderBytesBatch - kBatchTableBytes;
    int c = std::max(1, kMaxThreads / tpc);
    while (c > 1 && group_smem_bytes(t, c) > room) c--;
    return std::min(c, 48);
}

int code_id(int bg, int z) {
    const int zi = z_index(z);
    if ((bg != 1 && bg != 2) || zi < 0) return -1;
    return (bg - 1) * kNumZ + zi;
}

void drop_graph(Batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->knode = nullptr;
}

void free_batch(Batch* b) {
    if (!b) return;
    drop_graph(b);
    cudaFree(b->d_tables);
    cudaFree(b->d_plans);
    cudaFree(b->d_jobs_rm);
    cudaFree(b->d_jobs);
    cudaFree(b->d_order);
    cudaFree(b->d_items);
    cudaFree(b->d_state);
    cudaFree(b->d_scratch);
    delete b;
}

}  // namespace

extern "C" {

int nrldpc_rm_k0(int bg, int z, int rv) {
    init_z_list();
    if (z_index(z) < 0) return NRLDPC_ERR_BAD_CONFIG;
    const int k = rm_k0(bg, z, rv);
    return k < 0 ? NRLDPC_ERR_INVALID_ARG : k;
}

int nrldpc_batch_create(int device, int max_jobs, float alpha, nrldpc_batch** out) {
    if (!out || max_jobs < 1 || !(alpha > 0.0f)) return NRLDPC_ERR_INVALID_ARG;
    *out = nullptr;
    init_z_list();
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || device < 0 || device >= n_dev) return NRLDPC_ERR_NO_DEVICE;
    cudaSetDevice(device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return NRLDPC_ERR_NO_DEVICE;
    Batch* b = new (std::nothrow) Batch();
    if (!b) return NRLDPC_ERR_NO_MEMORY;
    b->device = device;
    b->alpha = alpha;
    b->max_jobs = max_jobs;
    b->sm_count = prop.multiProcessorCount;
    b->smem_optin = prop.sharedMemPerBlockOptin;
    std::vector<PlanDev> plans(kNumCodes);
    for (int bg = 1; bg <= 2; bg++)
        for (int zi = 0; zi < kNumZ; zi++) {
            const int id = (bg - 1) * kNumZ + zi, z = z_list[zi];
            CodeTable& t = b->h_tables[id];
            EncodePlan ep{};
            b->code_ok[id] = make_nr_table(bg, z, &t) && make_encode_plan(t, &ep);
            PlanDev& pd = plans[id];
            std::memset(&pd, 0, sizeof(pd));
            if (b->code_ok[id]) {
                pd.n_stair = ep.n_stair;
                pd.p0_col = ep.p0_col;
                pd.p0_shift = ep.p0_shift;
                pd.n_steps = ep.n_core_steps;
                for (int k = 0; k < ep.n_core_steps; k++) {
                    pd.step_row[k] = static_cast<uint8_t>(ep.core_row[k]);
                    pd.step_col[k] = static_cast<uint8_t>(ep.core_col[k]);
                }
            }
            // default: one sub-row per thread, as many codewords as 384
            // threads and shared memory allow
            b->spt[id] = 1;
            b->cpb[id] = max_cpb(b, id, 1);
        }
    if (cudaMalloc(&b->d_tables, sizeof(CodeTable) * kNumCodes) != cudaSuccess ||
        cudaMalloc(&b->d_plans, sizeof(PlanDev) * kNumCodes) != cudaSuccess ||
        cudaMalloc(&b->d_jobs_rm, sizeof(JobDev) * max_jobs) != cudaSuccess ||
        cudaMalloc(&b->d_jobs, sizeof(nrldpc_job) * max_jobs) != cudaSuccess ||
        cudaMalloc(&b->d_order, sizeof(int32_t) * max_jobs) != cudaSuccess ||
        cudaMalloc(&b->d_items, sizeof(WorkItem) * max_jobs) != cudaSuccess ||
        cudaMalloc(&b->d_scratch, 256) != cudaSuccess) {
        free_batch(b);
        return NRLDPC_ERR_NO_MEMORY;
    }
    if (cudaMemcpy(b->d_tables, b->h_tables, sizeof(CodeTable) * kNumCodes, cudaMemcpyHostToDevice) ||
        cudaMemcpy(b->d_plans, plans.data(), sizeof(PlanDev) * kNumCodes, cudaMemcpyHostToDevice) ||
        cudaMemset(b->d_scratch, 0, 256) ||
        cudaFuncSetAttribute(batch_decode_kernel_ptr(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(b->smem_optin))) {
        free_batch(b);
        return NRLDPC_ERR_CUDA;
    }
    *out = reinterpret_cast<nrldpc_batch*>(b);
    return NRLDPC_OK;
}

int nrldpc_batch_destroy(nrldpc_batch* batch) {
    free_batch(reinterpret_cast<Batch*>(batch));
    return NRLDPC_OK;
}

int nrldpc_batch_set_cw_per_cta(nrldpc_batch* batch, int bg, int z, int cpb) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    const int id = b ? code_id(bg, z) : -1;
    if (!b || id < 0 || cpb < 0) return NRLDPC_ERR_INVALID_ARG;
    const int most = max_cpb(b, id, b->spt[id]);
    if (cpb == 0) cpb = most;
    if (cpb > most) return NRLDPC_ERR_BAD_CONFIG;  // threads or shared memory
    b->cpb[id] = cpb;
    return NRLDPC_OK;
}

int nrldpc_batch_set_sub_rows_per_thread(nrldpc_batch* batch, int bg, int z, int spt) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    const int id = b ? code_id(bg, z) : -1;
    if (!b || id < 0 || spt < 0 || spt > 2) return NRLDPC_ERR_INVALID_ARG;
    if (spt == 0) spt = 1;
    if (z % spt != 0) return NRLDPC_ERR_BAD_CONFIG;  // sub-rows s and s + Z/2
    b->spt[id] = spt;
    b->cpb[id] = std::min(b->cpb[id], max_cpb(b, id, spt));
    return NRLDPC_OK;
}

int nrldpc_batch_get_sub_rows_per_thread(nrldpc_batch* batch, int bg, int z, int* spt) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    const int id = b ? code_id(bg, z) : -1;
    if (!b || id < 0 || !spt) return NRLDPC_ERR_INVALID_ARG;
    *spt = b->spt[id];
    return NRLDPC_OK;
}

int nrldpc_batch_get_cw_per_cta(nrldpc_batch* batch, int bg, int z, int* cpb) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    const int id = b ? code_id(bg, z) : -1;
    if (!b || id < 0 || !cpb) return NRLDPC_ERR_INVALID_ARG;
    *cpb = b->cpb[id];
    return NRLDPC_OK;
}

int nrldpc_batch_set_jobs(nrldpc_batch* batch, const nrldpc_job* jobs, int n_jobs) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b || (n_jobs > 0 && !jobs) || n_jobs < 0) return NRLDPC_ERR_INVALID_ARG;
    if (n_jobs > b->max_jobs) return NRLDPC_ERR_TOO_LARGE;
    cudaSetDevice(b->device);
    b->h_jobs.assign(n_jobs, JobDev{});
    std::vector<int32_t> order(n_jobs);
    for (int i = 0; i < n_jobs; i++) {
        const nrldpc_job& j = jobs[i];
        const int id = code_id(j.bg, j.z);
        if (id < 0 || !b->code_ok[id]) return NRLDPC_ERR_BAD_CONFIG;
        const CodeTable& t = b->h_tables[id];
        const int K = t.kb * t.z, ncb = t.n_bp - 2 * t.z;
        const int kp = j.k_prime ? j.k_prime : K;
        const int qm = j.qm ? j.qm : 1;
        const int e = j.e ? j.e : ncb - (K - kp);
        if (kp <= 2 * t.z || kp > K || j.e < 0 || j.rv < 0 || j.rv > 3 || j.llr_offset < 0 ||
            j.llr_offset % 4 != 0 || j.e_offset < 0 || j.out_offset < 0 ||
            (qm != 1 && qm != 2 && qm != 4 && qm != 6 && qm != 8 && qm != 10) || e % qm != 0)
            return NRLDPC_ERR_INVALID_ARG;
        JobDev& d = b->h_jobs[i];
        d.code = id;
        d.k_prime = kp;
        d.e = e;
        d.qm = qm;
        d.k0 = rm_k0(j.bg, t.z, j.rv);
        d.sigma = j.sigma;
        d.llr_offset = j.llr_offset;
        d.e_offset = j.e_offset;
        d.out_offset = j.out_offset;
        order[i] = i;
    }
    // group by code; largest codes first so the tail of the queue is short work
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const CodeTable& a = b->h_tables[b->h_jobs[x].code];
        const CodeTable& c = b->h_tables[b->h_jobs[y].code];
        const long wa = static_cast<long>(a.n_edges) * a.z, wc = static_cast<long>(c.n_edges) * c.z;
        if (wa != wc) return wa > wc;
        return b->h_jobs[x].code < b->h_jobs[y].code;
    });
    std::vector<WorkItem> items;
    size_t slot_words = 0, bufs = 0;
    int threads = 32;
    for (int i = 0; i < n_jobs;) {
        const int id = b->h_jobs[order[i]].code;
        int k = i;
        while (k < n_jobs && b->h_jobs[order[k]].code == id) k++;
        const int cpb = b->cpb[id], spt = b->spt[id];
        const CodeTable& t = b->h_tables[id];
        for (int s = i; s < k; s += cpb) {
            const int cnt = std::min(cpb, k - s);
            items.push_back(WorkItem{id, s, cnt, spt});
            threads = std::max(threads, (cnt * (t.z / spt) + 31) / 32 * 32);
            slot_words = std::max(slot_words, static_cast<size_t>(cnt) * 4 * t.rows * t.z);
            bufs = std::max(bufs, group_smem_bytes(t, cnt));
        }
        i = k;
    }
    b->n_jobs = n_jobs;
    b->n_items = static_cast<int>(items.size());
    b->slot_words = slot_words;
    b->smem = kHeaderBytesBatch + kBatchTableBytes + bufs;
    b->threads = threads;  // the widest work item's threads
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_decode_kernel_ptr(), b->threads, b->smem);
    b->grid = std::max(1, std::min(b->n_items, std::max(per_sm, 1) * b->sm_count));
    const size_t need = static_cast<size_t>(b->grid) * std::max<size_t>(slot_words, 1);
    if (need > b->state_words) {
        cudaFree(b->d_state);
        b->d_state = nullptr;
        b->state_words = 0;
        if (cudaMalloc(&b->d_state, need * sizeof(uint32_t)) != cudaSuccess) return NRLDPC_ERR_NO_MEMORY;
        b->state_words = need;
    }
    if (n_jobs) {
        if (cudaMemcpy(b->d_jobs_rm, b->h_jobs.data(), sizeof(JobDev) * n_jobs, cudaMemcpyHostToDevice) ||
            cudaMemcpy(b->d_jobs, jobs, sizeof(nrldpc_job) * n_jobs, cudaMemcpyHostToDevice) ||
            cudaMemcpy(b->d_order, order.data(), sizeof(int32_t) * n_jobs, cudaMemcpyHostToDevice) ||
            cudaMemcpy(b->d_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice))
            return NRLDPC_ERR_CUDA;
    }
    drop_graph(b);  // launch geometry changed
    return NRLDPC_OK;
}

int nrldpc_batch_gen(nrldpc_batch* batch, uint64_t seed, uint64_t cw_base, float* d_llr_e, uint8_t* d_cw,
                     nrldpc_stream_t stream) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b || !d_llr_e) return NRLDPC_ERR_INVALID_ARG;
    if (b->n_jobs == 0) return NRLDPC_OK;
    GenBatchArgs g{b->d_tables, b->d_plans, b->d_jobs_rm, d_llr_e, d_cw, seed, cw_base, b->n_jobs};
    const int grid = std::min(b->n_jobs, 8 * b->sm_count);
    batch_gen_kernel<<<grid, 256, kMaxCols * kMaxZ + kMaxZ, reinterpret_cast<cudaStream_t>(stream)>>>(g);
    return map_cuda(cudaGetLastError());
}

int nrldpc_batch_derate(nrldpc_batch* batch, const float* d_llr_e, float* d_llr, nrldpc_stream_t stream) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b || !d_llr_e || !d_llr) return NRLDPC_ERR_INVALID_ARG;
    if (b->n_jobs == 0) return NRLDPC_OK;
    DerateArgs a{b->d_tables, b->d_jobs_rm, d_llr_e, d_llr, b->n_jobs};
    const int grid = std::min(b->n_jobs, 8 * b->sm_count);
    batch_derate_kernel<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(a);
    return map_cuda(cudaGetLastError());
}

int nrldpc_batch_count_errors(nrldpc_batch* batch, const uint8_t* d_packed, const uint8_t* d_cw,
                              unsigned long long* d_counts, nrldpc_stream_t stream) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b || !d_packed || !d_cw || !d_counts) return NRLDPC_ERR_INVALID_ARG;
    if (b->n_jobs == 0) return NRLDPC_OK;
    CountArgs a{b->d_tables, b->d_jobs_rm, d_packed, d_cw, d_counts, b->n_jobs};
    const int grid = std::min(b->n_jobs, 8 * b->sm_count);
    batch_count_kernel<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(a);
    return map_cuda(cudaGetLastError());
}

int nrldpc_batch_decode(nrldpc_batch* batch, const float* d_llr, uint8_t* d_packed, int n_iter,
                        int early_stop, int32_t* d_iters, nrldpc_stream_t stream) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b || n_iter < 1 || (early_stop != 0 && early_stop != 1)) return NRLDPC_ERR_INVALID_ARG;
    if (b->n_jobs == 0) return NRLDPC_OK;
    if (!d_llr || !d_packed) return NRLDPC_ERR_INVALID_ARG;
    if (reinterpret_cast<uintptr_t>(d_llr) % 16 != 0) return NRLDPC_ERR_ALIGNMENT;
    BatchDecodeArgs& k = b->kargs;
    k.tables = b->d_tables;
    k.items = b->d_items;
    k.order = b->d_order;
    k.jobs = b->d_jobs;
    k.llr = d_llr;
    k.packed = d_packed;
    k.iters = d_iters;
    k.state = b->d_state;
    k.work_counter = b->d_scratch;
    k.error_flag = b->d_scratch + 1;
    k.slot_words = b->slot_words;
    k.n_items = b->n_items;
    k.n_iter = n_iter;
    k.early_stop = early_stop;
    k.alpha = b->alpha;
    void* params[1] = {&k};
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(batch_decode_kernel_ptr());
    kp.gridDim = dim3(b->grid);
    kp.blockDim = dim3(b->threads);
    kp.sharedMemBytes = static_cast<unsigned int>(b->smem);
    kp.kernelParams = params;
    if (!b->exec) {  // memset of the queue head, then the persistent kernel
        cudaMemsetParams mp{};
        mp.dst = b->d_scratch;
        mp.value = 0;
        mp.elementSize = 4;
        mp.width = 1;
        mp.height = 1;
        cudaGraphNode_t mnode;
        if (cudaGraphCreate(&b->graph, 0) || cudaGraphAddMemsetNode(&mnode, b->graph, nullptr, 0, &mp) ||
            cudaGraphAddKernelNode(&b->knode, b->graph, &mnode, 1, &kp) ||
            cudaGraphInstantiate(&b->exec, b->graph, 0)) {
            drop_graph(b);
            return NRLDPC_ERR_CUDA;
        }
    } else if (cudaGraphExecKernelNodeSetParams(b->exec, b->knode, &kp) != cudaSuccess) {
        return NRLDPC_ERR_CUDA;
    }
    return map_cuda(cudaGraphLaunch(b->exec, reinterpret_cast<cudaStream_t>(stream)));
}

}  // extern "C"
