/*
 * Driver for the reference's own decoder source, compiled as host C++ with the
 * stand-in headers in ref_emul/ (TEST INFRASTRUCTURE ONLY; built into
 * oracle/_ref/, never shipped, only where the reference tree is present).
 *
 * It links the reference's unmodified src/ldpc_kernels.cu, src/setup_exp.cu,
 * src/nr_ldpc.cpp, src/encoding_tools.cpp and src/host_helpers.cpp, fills the
 * "constant memory" through the reference's own
 * put_h_compact_and_params_in_constant_memory (src/setup_exp.cu:286-313), and
 * replays the launch sequence of perform_gpu_ldpc_decoding
 * (src/gpu_decoder_top.cu:25-49): CNP first-iteration/regular, VNP
 * normal/last, pack -- each launch as sequential block and thread loops.
 */
#include <cuda_runtime.h>

#include <initializer_list>
#include <memory>
#include <string>
#include <vector>

#include "types.h"
#include "encoding_tools.h"
#include "ldpc_kernels.h"
#include "nr_ldpc.h"
#include "setup_exp.h"
#include "spdlog/sinks/null_sink.h"
#include "spdlog/spdlog.h"

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;
/* extern __shared__ float RCache[] in cnp_kernel resolves to this array. */
float RCache[1 << 16];

/* ---- src/cuda_gpu_wrapper/gpu_setup.cu is not built; setup_exp.cu only
 *      references these through setup_host / setup_dev_memory, never called. */
cudaStream_t* setup_streams(unsigned int) { std::abort(); }
template <typename T> T** allocate_cuda_placeholder(unsigned int, unsigned int) { std::abort(); }
template <typename T> void copy_to_cuda_staged_memory(T*, T**, int, int, int) { std::abort(); }
template <typename T> T** allocate_device_array(unsigned int, unsigned int) { std::abort(); }
template int** allocate_cuda_placeholder<int>(unsigned int, unsigned int);
template char** allocate_cuda_placeholder<char>(unsigned int, unsigned int);
template half** allocate_cuda_placeholder<half>(unsigned int, unsigned int);
template float** allocate_cuda_placeholder<float>(unsigned int, unsigned int);
template void copy_to_cuda_staged_memory<int>(int*, int**, int, int, int);
template void copy_to_cuda_staged_memory<char>(char*, char**, int, int, int);
template void copy_to_cuda_staged_memory<half>(half*, half**, int, int, int);
template void copy_to_cuda_staged_memory<float>(float*, float**, int, int, int);
template char** allocate_device_array<char>(unsigned int, unsigned int);
template half** allocate_device_array<half>(unsigned int, unsigned int);
template float** allocate_device_array<float>(unsigned int, unsigned int);
std::string print_devices() { return "emulated"; }

template <class F>
static void launch(dim3 grid, dim3 block, F kernel) {
    gridDim = grid;
    blockDim = block;
    for (unsigned by = 0; by < grid.y; by++)
        for (unsigned bx = 0; bx < grid.x; bx++) {
            blockIdx = {bx, by, 0};
            for (unsigned ty = 0; ty < block.y; ty++)
                for (unsigned tx = 0; tx < block.x; tx++) {
                    threadIdx = {tx, ty, 0};
                    kernel();
                }
        }
}

static void ensure_loggers() {
    for (const char* name : {"LDPC", "GPU", "RESULTS", "DEBUG"})
        if (!spdlog::get(name))
            spdlog::register_logger(
                std::make_shared<spdlog::logger>(name, std::make_shared<spdlog::sinks::null_sink_st>()));
}

static ldpc_params g_ldpc;
static std::vector<int> g_H;
static std::vector<char> g_row_cnt, g_col_cnt;
static cuda_grid g_grid;
static int g_ready = 0;

/* Reference setup_ldpc, fields flattened:
 * A, bg, Z, K, N, rows, cols, nz_row, nz_col, n_iter, N_bp, H[0] */
extern "C" int ref_setup_ldpc(int A, float rate, int n_iter, int* out) {
    ensure_loggers();
    ldpc_params l = setup_ldpc(A, rate, n_iter);
    out[0] = l.A; out[1] = l.bg_index; out[2] = l.Z; out[3] = l.K; out[4] = l.N;
    out[5] = l.H_rows; out[6] = l.H_cols; out[7] = l.n_nz_in_row; out[8] = l.n_nz_in_col;
    out[9] = l.n_iterations; out[10] = l.N_before_puncture; out[11] = l.H ? l.H[0] : -9999;
    return 0;
}

/* Load a code: dense base matrix (shifts already reduced mod Z by the caller,
 * as the reference itself only runs Z = 384 where V < Z). */
extern "C" int ref_init_code(const int* H, int rows, int cols, int z) {
    ensure_loggers();
    if (rows != BLK_ROW || cols != BLK_COL) return -1;
    g_H.assign(H, H + rows * cols);
    g_row_cnt.assign(rows, 0);
    g_col_cnt.assign(cols, 0);
    int mr = 0, mc = 0;
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++)
            if (H[r * cols + c] != -1) { g_row_cnt[r]++; g_col_cnt[c]++; }
    for (int r = 0; r < rows; r++) mr = g_row_cnt[r] > mr ? g_row_cnt[r] : mr;
    for (int c = 0; c < cols; c++) mc = g_col_cnt[c] > mc ? g_col_cnt[c] : mc;
    if (mr != NON_EMPTY_ROW || mc != NON_EMPTY_COL) return -2;
    g_ldpc = ldpc_params{};
    g_ldpc.Z = z; g_ldpc.H_rows = rows; g_ldpc.H_cols = cols; g_ldpc.H = g_H.data();
    g_ldpc.n_nz_in_row = mr; g_ldpc.n_nz_in_col = mc;
    g_ldpc.h_element_count_per_row = g_row_cnt.data();
    g_ldpc.h_element_count_per_col = g_col_cnt.data();
    g_ldpc.N_before_puncture = cols * z;
    g_ready = 1;
    return 0;
}

/* Decode n_cw codewords (one codeword per "macro-codeword") for n_iter
 * iterations.  packed: n_cw * N_bp / 8 bytes.  app (optional): the posterior
 * the last iteration computed, obtained by running vnp_kernel_normal once
 * more on a copy of the LLR array (same additions as vnp_kernel_last_iter). */
extern "C" int ref_decode(const float* llr, int n_cw, int n_iter, unsigned char* packed, float* app) {
    if (!g_ready || n_iter < 1) return -1;
    const int z = g_ldpc.Z, rows = g_ldpc.H_rows, cols = g_ldpc.H_cols, nbp = cols * z;
    params p{};
    p.n_cw_per_mcw = 1;
    p.n_mcw = n_cw;
    g_grid = setup_gpu_grid(&g_ldpc, 1, n_cw);
    if (g_grid.cnp_threads_per_block * g_ldpc.n_nz_in_row > (int)(sizeof(RCache) / sizeof(float))) return -3;
    put_h_compact_and_params_in_constant_memory(&g_ldpc, &p, &g_grid);
    const size_t n_llr = (size_t)n_cw * nbp, n_msg = (size_t)n_cw * rows * z * cols;
    std::vector<float> d_llr(llr, llr + n_llr), d_dt(n_msg, 0.0f), d_r(n_msg, 0.0f);
    std::vector<char> d_hd(n_llr + 64, 0), d_packed(n_llr / 8 + 64, 0);
    float* L = d_llr.data(); float* dt = d_dt.data(); float* R = d_r.data();
    for (int it = 0; it < n_iter; it++) {
        if (it == 0)
            launch(g_grid.cnp_blocks, g_grid.cnp_threads, [&] { cnp_kernel_1st_iter<float>(L, dt, R); });
        else
            launch(g_grid.cnp_blocks, g_grid.cnp_threads, [&] { cnp_kernel<float>(L, dt, R); });
        if (it < n_iter - 1) {
            launch(g_grid.vnp_blocks, g_grid.vnp_threads, [&] { vnp_kernel_normal<float>(L, dt); });
        } else {
            launch(g_grid.vnp_blocks, g_grid.vnp_threads,
                   [&] { vnp_kernel_last_iter<float>(L, dt, d_hd.data()); });
            launch(g_grid.pack_blocks, g_grid.pack_threads,
                   [&] { pack_hard_decision(d_hd.data(), d_packed.data()); });
        }
    }
    std::memcpy(packed, d_packed.data(), n_llr / 8);
    if (app) {
        std::vector<float> post(d_llr);
        float* P = post.data();
        launch(g_grid.vnp_blocks, g_grid.vnp_threads, [&] { vnp_kernel_normal<float>(P, dt); });
        std::memcpy(app, P, n_llr * sizeof(float));
    }
    return 0;
}

/* The constant memory the reference's own setup writes for a decode with one
 * codeword per block column (put_h_compact_and_params_in_constant_memory,
 * src/setup_exp.cu:286-313, after setup_gpu_grid for n_cw_per_mcw = 1):
 * dev_h_compact1 | dev_h_compact2 | h_element_count_per_row |
 * h_element_count_per_col | p, as bytes, for loading into the reference's
 * kernels built for the GPU (oracle/ref_gpu_harness.cpp).  Returns the size,
 * or -1 before ref_init_code / when out is too small. */
extern h_element dev_h_compact1[H_COMPACT1_COL][H_COMPACT1_ROW];
extern h_element dev_h_compact2[H_COMPACT2_ROW][H_COMPACT2_COL];
extern char h_element_count_per_row[BLK_ROW];
extern char h_element_count_per_col[BLK_COL];
extern kernel_params p[1];
extern "C" int ref_constant_image(unsigned char* out, int cap) {
    if (!g_ready) return -1;
    params pr{};
    pr.n_cw_per_mcw = 1;
    pr.n_mcw = 1;
    g_grid = setup_gpu_grid(&g_ldpc, 1, 1);
    put_h_compact_and_params_in_constant_memory(&g_ldpc, &pr, &g_grid);
    const size_t parts[5] = {sizeof(dev_h_compact1), sizeof(dev_h_compact2), sizeof(h_element_count_per_row),
                             sizeof(h_element_count_per_col), sizeof(p)};
    const void* srcs[5] = {dev_h_compact1, dev_h_compact2, h_element_count_per_row, h_element_count_per_col, p};
    size_t n = 0;
    for (size_t k : parts) n += k;
    if (!out || (size_t)cap < n) return -1;
    for (int i = 0, off = 0; i < 5; off += (int)parts[i], i++) std::memcpy(out + off, srcs[i], parts[i]);
    return (int)n;
}

/* The reference's channel pipeline for BG1 A=8424 (src/setup_exp.cu:177-195):
 * srand(seed) once, then per codeword transmit (rand() info bits, OAI encoder,
 * BPSK, drand48 AWGN) and calculate_llr.  info_out: n_cw * K ints. */
extern "C" int ref_transmit_llr(int A, float rate, int n_cw, float ebn0_db, unsigned seed,
                                float* llr_out, int* info_out) {
    ensure_loggers();
    ldpc_params l = setup_ldpc(A, rate, 1);
    if (!l.H) return -1;
    const float sigma = compute_noise_stddev(ebn0_db, l.rate);
    const int nbp = l.N_before_puncture;
    std::vector<int> info(l.K), cw(nbp);
    std::vector<float> mod(nbp), recv(nbp);
    srand(seed);
    srand48(0x1234ABCDL); /* X = 0x1234ABCD330E: drand48's default state before any seeding */
    for (int i = 0; i < n_cw; i++) {
        transmit(info.data(), cw.data(), mod.data(), nbp * sizeof(int), recv.data(), l.K, nbp, sigma,
                 l.bg_index);
        calculate_llr(llr_out + (size_t)i * nbp, recv.data(), nbp, sigma, l.Z);
        std::memcpy(info_out + (size_t)i * l.K, info.data(), sizeof(int) * l.K);
    }
    return 0;
}
