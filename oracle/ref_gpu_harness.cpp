/*
 * Runs the reference's own CUDA kernels on the GPU -- TEST INFRASTRUCTURE ONLY.
 *
 * oracle/Makefile compiles the reference's src/ldpc_kernels.cu, unmodified,
 * for sm_103a into oracle/_ref/ref_kernels_bg1.cubin with nvcc's default
 * flags (the reference's CMakeLists.txt sets none), so the floating-point
 * code is what the reference's own build produces, contraction included.
 * This driver (CUDA driver API only, no runtime) loads that image, fills its
 * constant memory from oracle/_ref/ref_const_bg1.bin -- the bytes the
 * reference's own put_h_compact_and_params_in_constant_memory wrote
 * (src/setup_exp.cu:286-313, dumped through oracle/ref_harness.cpp) -- and
 * replays perform_gpu_ldpc_decoding (src/gpu_decoder_top.cu:25-49): the first
 * or regular check-node kernel, the normal or last variable-node kernel, then
 * the pack kernel, on the grid setup_gpu_grid builds (src/setup_exp.cu:131-166)
 * for one codeword per block column: check nodes (rows, n_cw) x
 * (roundup32(Z), 1) with rows-degree floats of dynamic shared memory per
 * thread, variable nodes (cols, n_cw) x (roundup32(Z), 1), packing
 * (cols, n_cw) x (roundup32(Z) / 8, 1).  Buffers as setup_dev_memory
 * allocates them: LLR/posterior [n_cw][cols*Z], R and dt dense
 * [n_cw][cols][rows*Z], hard decisions [n_cw][cols*Z] bytes, packed bits.
 */
#include <cuda.h>

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Ctx {
    CUdevice dev = 0;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    std::vector<CUdeviceptr> bufs;
    ~Ctx() {
        for (CUdeviceptr b : bufs)
            if (b) cuMemFree(b);
        if (mod) cuModuleUnload(mod);
        if (ctx) {
            CUcontext popped;
            cuCtxPopCurrent(&popped);
            cuDevicePrimaryCtxRelease(dev);
        }
    }
    CUdeviceptr alloc(size_t bytes) {
        CUdeviceptr p = 0;
        if (cuMemAlloc(&p, bytes) != CUDA_SUCCESS) return 0;
        bufs.push_back(p);
        if (cuMemsetD8(p, 0, bytes) != CUDA_SUCCESS) return 0;
        return p;
    }
};

#define REF_CHECK(x)                      \
    do {                                  \
        if ((x) != CUDA_SUCCESS) return -(__LINE__); \
    } while (0)

}  // namespace

namespace {

struct RefRun {
    CUfunction cnp1, cnp, vnp, vnp_last, pack;
    CUdeviceptr llr, dt, r, hd, packed;
    int rows, cols, z, n_cw;
    unsigned bx, smem;
};

// Module, constant memory, functions and buffers of one run (in c).
int ref_setup(Ctx& c, RefRun& k, const char* cubin, const unsigned char* image, int image_size, int rows, int cols,
              int z, int max_row_deg, int n_cw) {
    REF_CHECK(cuInit(0));
    REF_CHECK(cuDeviceGet(&c.dev, 0));
    REF_CHECK(cuDevicePrimaryCtxRetain(&c.ctx, c.dev));
    if (cuCtxPushCurrent(c.ctx) != CUDA_SUCCESS) {
        cuDevicePrimaryCtxRelease(c.dev);
        c.ctx = nullptr;
        return -(__LINE__);
    }
    REF_CHECK(cuModuleLoad(&c.mod, cubin));
    // constant memory: the parts of the image, in order, must be exactly the
    // module's arrays
    const char* names[5] = {"dev_h_compact1", "dev_h_compact2", "h_element_count_per_row",
                            "h_element_count_per_col", "p"};
    size_t off = 0;
    for (const char* nm : names) {
        CUdeviceptr g = 0;
        size_t bytes = 0;
        REF_CHECK(cuModuleGetGlobal(&g, &bytes, c.mod, nm));
        if (off + bytes > static_cast<size_t>(image_size)) return -(__LINE__);
        REF_CHECK(cuMemcpyHtoD(g, image + off, bytes));
        off += bytes;
    }
    if (off != static_cast<size_t>(image_size)) return -(__LINE__);
    REF_CHECK(cuModuleGetFunction(&k.cnp1, c.mod, "_Z19cnp_kernel_1st_iterIfEvPT_S1_S1_"));
    REF_CHECK(cuModuleGetFunction(&k.cnp, c.mod, "_Z10cnp_kernelIfEvPT_S1_S1_"));
    REF_CHECK(cuModuleGetFunction(&k.vnp, c.mod, "_Z17vnp_kernel_normalIfEvPT_S1_"));
    REF_CHECK(cuModuleGetFunction(&k.vnp_last, c.mod, "_Z20vnp_kernel_last_iterIfEvPT_S1_Pc"));
    REF_CHECK(cuModuleGetFunction(&k.pack, c.mod, "_Z18pack_hard_decisionPcS_"));
    const size_t nbp = static_cast<size_t>(cols) * z;
    const size_t n_llr = static_cast<size_t>(n_cw) * nbp;
    const size_t n_msg = static_cast<size_t>(n_cw) * rows * z * cols;
    k.llr = c.alloc(n_llr * sizeof(float));
    k.dt = c.alloc(n_msg * sizeof(float));
    k.r = c.alloc(n_msg * sizeof(float));
    k.hd = c.alloc(n_llr);
    k.packed = c.alloc(n_llr / 8);
    if (!k.llr || !k.dt || !k.r || !k.hd || !k.packed) return -(__LINE__);
    k.rows = rows;
    k.cols = cols;
    k.z = z;
    k.n_cw = n_cw;
    k.bx = static_cast<unsigned>((z + 31) / 32 * 32);
    k.smem = k.bx * static_cast<unsigned>(max_row_deg) * sizeof(float);  // shared_r_cache_size
    return 0;
}

// The launches of one perform_gpu_ldpc_decoding on the LLRs in k.llr (the
// posterior overwrites them, as in the reference).
int ref_iterate(RefRun& k, int n_iter, CUstream st) {
    for (int it = 0; it < n_iter; it++) {
        void* cnp_args[3] = {&k.llr, &k.dt, &k.r};
        if (it == 0)
            REF_CHECK(cuLaunchKernel(k.cnp1, k.rows, k.n_cw, 1, k.bx, 1, 1, 0, st, cnp_args, nullptr));
        else
            REF_CHECK(cuLaunchKernel(k.cnp, k.rows, k.n_cw, 1, k.bx, 1, 1, k.smem, st, cnp_args, nullptr));
        if (it < n_iter - 1) {
            void* vnp_args[2] = {&k.llr, &k.dt};
            REF_CHECK(cuLaunchKernel(k.vnp, k.cols, k.n_cw, 1, k.bx, 1, 1, 0, st, vnp_args, nullptr));
        } else {
            void* last_args[3] = {&k.llr, &k.dt, &k.hd};
            REF_CHECK(cuLaunchKernel(k.vnp_last, k.cols, k.n_cw, 1, k.bx, 1, 1, 0, st, last_args, nullptr));
            void* pack_args[2] = {&k.hd, &k.packed};
            REF_CHECK(cuLaunchKernel(k.pack, k.cols, k.n_cw, 1, k.bx / 8, 1, 1, 0, st, pack_args, nullptr));
        }
    }
    return 0;
}

}  // namespace

/* Decode n_cw codewords of the code whose tables the image holds (rows x
 * cols base matrix, lifting z, largest row degree max_row_deg) for n_iter
 * iterations with the reference's kernels.  llr: n_cw * cols * z floats;
 * packed: n_cw * cols * z / 8 bytes; app (may be NULL): the posterior the
 * last iteration computed, by one more run of the normal variable-node
 * kernel on a copy of the LLR array with the last dt (the additions of the
 * last-iteration kernel).  Returns 0, or minus the failing source line. */
extern "C" int refgpu_decode(const char* cubin, const unsigned char* image, int image_size, int rows, int cols,
                             int z, int max_row_deg, const float* llr, int n_cw, int n_iter, unsigned char* packed,
                             float* app) {
    if (!cubin || !image || !llr || !packed || n_cw < 1 || n_iter < 1 || z < 8 || z % 8 != 0) return -1;
    Ctx c;
    RefRun k{};
    int rc = ref_setup(c, k, cubin, image, image_size, rows, cols, z, max_row_deg, n_cw);
    if (rc) return rc;
    const size_t n_llr = static_cast<size_t>(n_cw) * cols * z;
    CUdeviceptr d_post = 0;
    if (app && !(d_post = c.alloc(n_llr * sizeof(float)))) return -(__LINE__);
    REF_CHECK(cuMemcpyHtoD(k.llr, llr, n_llr * sizeof(float)));
    rc = ref_iterate(k, n_iter, nullptr);
    if (rc) return rc;
    REF_CHECK(cuCtxSynchronize());
    REF_CHECK(cuMemcpyDtoH(packed, k.packed, n_llr / 8));
    if (app) {
        REF_CHECK(cuMemcpyDtoD(d_post, k.llr, n_llr * sizeof(float)));
        void* vnp_args[2] = {&d_post, &k.dt};
        REF_CHECK(cuLaunchKernel(k.vnp, cols, n_cw, 1, k.bx, 1, 1, 0, nullptr, vnp_args, nullptr));
        REF_CHECK(cuCtxSynchronize());
        REF_CHECK(cuMemcpyDtoH(app, d_post, n_llr * sizeof(float)));
    }
    return 0;
}

/* Device time of the reference's decode: n_cw codewords (at most 446, the
 * reference's own limit for fp32 buffers, whose 32-bit offsets
 * size_R_CW * cw overflow beyond 1787), n_iter iterations, LLRs resident
 * (restored before every decode from a device copy, outside the timed
 * launches: the reference overwrites them with the posterior); `warmup`
 * untimed decodes, then `reps` decodes timed one by one with events, mean
 * milliseconds per decode in *ms. */
extern "C" int refgpu_time(const char* cubin, const unsigned char* image, int image_size, int rows, int cols, int z,
                           int max_row_deg, const float* llr, int n_cw, int n_iter, int warmup, int reps,
                           float* ms) {
    if (!cubin || !image || !llr || !ms || n_cw < 1 || n_cw > 446 || n_iter < 1 || reps < 1 || z % 8 != 0)
        return -1;
    Ctx c;
    RefRun k{};
    int rc = ref_setup(c, k, cubin, image, image_size, rows, cols, z, max_row_deg, n_cw);
    if (rc) return rc;
    const size_t bytes = static_cast<size_t>(n_cw) * cols * z * sizeof(float);
    CUdeviceptr src = c.alloc(bytes);
    if (!src) return -(__LINE__);
    REF_CHECK(cuMemcpyHtoD(src, llr, bytes));
    CUevent e0, e1;
    REF_CHECK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    if (cuEventCreate(&e1, CU_EVENT_DEFAULT) != CUDA_SUCCESS) {
        cuEventDestroy(e0);
        return -(__LINE__);
    }
    float total = 0.0f;
    for (int i = 0; i < warmup + reps && rc == 0; i++) {
        float t = 0.0f;
        if (cuMemcpyDtoD(k.llr, src, bytes) != CUDA_SUCCESS || cuEventRecord(e0, nullptr) != CUDA_SUCCESS) {
            rc = -(__LINE__);
            break;
        }
        rc = ref_iterate(k, n_iter, nullptr);
        if (rc) break;
        if (cuEventRecord(e1, nullptr) != CUDA_SUCCESS || cuEventSynchronize(e1) != CUDA_SUCCESS ||
            cuEventElapsedTime(&t, e0, e1) != CUDA_SUCCESS) {
            rc = -(__LINE__);
            break;
        }
        if (i >= warmup) total += t;
    }
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    if (rc) return rc;
    *ms = total / reps;
    return 0;
}

/* The reference testbench's latency measurement (test_latency,
 * src/main.cpp:147-156) on these kernels: one perform_gpu_ldpc_decoding --
 * H2D of the batch from pinned host memory, the launches, D2H of the packed
 * bits into pinned host memory -- then a context synchronize, timed on the
 * host clock (n_cw at most 446).  `warmup` untimed calls, then `reps` timed
 * ones; the best and the median microseconds in best_us / median_us. */
extern "C" int refgpu_latency(const char* cubin, const unsigned char* image, int image_size, int rows, int cols,
                              int z, int max_row_deg, const float* llr, int n_cw, int n_iter, int warmup, int reps,
                              float* best_us, float* median_us) {
    if (!cubin || !image || !llr || !best_us || !median_us || n_cw < 1 || n_cw > 446 || n_iter < 1 || reps < 1 ||
        z % 8 != 0)
        return -1;
    Ctx c;
    RefRun k{};
    int rc = ref_setup(c, k, cubin, image, image_size, rows, cols, z, max_row_deg, n_cw);
    if (rc) return rc;
    const size_t bytes = static_cast<size_t>(n_cw) * cols * z * sizeof(float);
    const size_t out_bytes = static_cast<size_t>(n_cw) * cols * z / 8;
    void* h_llr = nullptr;
    void* h_out = nullptr;
    if (cuMemAllocHost(&h_llr, bytes) != CUDA_SUCCESS) return -(__LINE__);
    if (cuMemAllocHost(&h_out, out_bytes) != CUDA_SUCCESS) {
        cuMemFreeHost(h_llr);
        return -(__LINE__);
    }
    std::memcpy(h_llr, llr, bytes);
    std::vector<float> us;
    for (int i = 0; i < warmup + reps && rc == 0; i++) {
        const auto t0 = std::chrono::steady_clock::now();
        if (cuMemcpyHtoDAsync(k.llr, h_llr, bytes, nullptr) != CUDA_SUCCESS) {
            rc = -(__LINE__);
            break;
        }
        rc = ref_iterate(k, n_iter, nullptr);
        if (rc) break;
        if (cuMemcpyDtoHAsync(h_out, k.packed, out_bytes, nullptr) != CUDA_SUCCESS ||
            cuCtxSynchronize() != CUDA_SUCCESS) {
            rc = -(__LINE__);
            break;
        }
        const auto t1 = std::chrono::steady_clock::now();
        if (i >= warmup) us.push_back(std::chrono::duration<float, std::micro>(t1 - t0).count());
    }
    cuMemFreeHost(h_llr);
    cuMemFreeHost(h_out);
    if (rc) return rc;
    std::sort(us.begin(), us.end());
    *best_us = us.front();
    *median_us = us[us.size() / 2];
    return 0;
}
