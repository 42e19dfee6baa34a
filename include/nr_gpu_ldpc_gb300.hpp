// Header-only C++ convenience layer over the C ABI in nr_gpu_ldpc_gb300.h,
// shaped after the reference's host calls (ctarver/NR_GPU_LDPC):
//   setup_ldpc(A, rate, n_iterations)             src/nr_ldpc.h:14
//   perform_gpu_ldpc_decoding<T>(d, h, g, I, s)   src/gpu_decoder_top.h:13-18
// One Decoder stands for the reference's process-global decoder state
// (constant memory + dev_mem), without the globals: several can coexist.
// A Decoder serves one stream at a time; give each concurrent stream its own.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "nr_gpu_ldpc_gb300.h"

namespace nrldpc {

inline void check(int status, const char* what) {
    if (status != NRLDPC_OK)
        throw std::runtime_error(std::string(what) + ": " + nrldpc_status_string(status));
}

// Mirror of setup_ldpc (src/nr_ldpc.cpp:31-230).
inline nrldpc_ldpc_params setup_ldpc(int A, float rate, int n_iterations) {
    nrldpc_ldpc_params p;
    check(nrldpc_setup_ldpc(A, rate, n_iterations, &p), "setup_ldpc");
    return p;
}

class Decoder {
public:
    // Replaces setup_dev_memory + setup_gpu_grid +
    // put_h_compact_and_params_in_constant_memory (src/setup_exp.cu:102-166,286-313).
    Decoder(const nrldpc_ldpc_params& p, int max_batch, float alpha = 0.75f, int device = 0) {
        nrldpc_config cfg{p.bg_index, p.Z, max_batch, alpha, device, 0};
        check(nrldpc_init(&cfg, &h_), "nrldpc_init");
        check(nrldpc_geometry(h_, nullptr, nullptr, nullptr, nullptr, &n_bp_, &packed_bytes_),
              "nrldpc_geometry");
    }
    ~Decoder() { nrldpc_destroy(h_); }
    Decoder(const Decoder&) = delete;
    Decoder& operator=(const Decoder&) = delete;

    int n_bp() const { return n_bp_; }                  // N_before_puncture
    int packed_bytes() const { return packed_bytes_; }  // per codeword
    nrldpc_handle* handle() const { return h_; }

    // perform_gpu_ldpc_decoding (src/gpu_decoder_top.cu:16-52): host LLRs of
    // n_cw codewords in, packed hard decisions out, queued on `stream`
    // (pinned buffers overlap with other streams); the caller synchronizes.
    void perform_gpu_ldpc_decoding(const float* h_llr, uint8_t* h_packed, int n_cw,
                                   int n_iterations, cudaStream_t stream, bool early_stop = false) {
        check(nrldpc_decode_host_async(h_, h_llr, h_packed, n_cw, n_iterations, early_stop ? 1 : 0,
                                       reinterpret_cast<nrldpc_stream_t>(stream)),
              "perform_gpu_ldpc_decoding");
    }

    // The reference's char / half builds (CHAR_PRC / HALF_PRC): narrow LLRs over
    // the host link, qtype 1 = fp16, 2 = int8 with LLR = q * scale.
    void perform_gpu_ldpc_decoding_q(const void* h_llr_q, int qtype, float scale, uint8_t* h_packed,
                                     int n_cw, int n_iterations, cudaStream_t stream, bool early_stop = false) {
        check(nrldpc_decode_host_async_q(h_, h_llr_q, qtype, scale, h_packed, n_cw, n_iterations,
                                         early_stop ? 1 : 0, reinterpret_cast<nrldpc_stream_t>(stream)),
              "perform_gpu_ldpc_decoding");
    }

    // NRLDPC_HOST_AUTO (default), NRLDPC_HOST_COPY or NRLDPC_HOST_DIRECT: how
    // perform_gpu_ldpc_decoding moves fp32 LLRs and bits (same results).
    void set_host_transfer(int mode) { check(nrldpc_set_host_transfer(h_, mode), "set_host_transfer"); }

    // Device-resident variant (no copies).
    void decode(const float* d_llr, uint8_t* d_packed, int n_cw, int n_iterations,
                cudaStream_t stream, bool early_stop = false) {
        check(nrldpc_decode(h_, d_llr, d_packed, n_cw, n_iterations, early_stop ? 1 : 0, nullptr,
                            nullptr, reinterpret_cast<nrldpc_stream_t>(stream)),
              "nrldpc_decode");
    }

private:
    nrldpc_handle* h_ = nullptr;
    int n_bp_ = 0, packed_bytes_ = 0;
};

// ---- the reference's own call shape -------------------------------------------------
// For a caller that keeps its structs: the same arguments as the reference's
//   template <typename T> void perform_gpu_ldpc_decoding(dev_mem<T>* d, host_mem<T>* h,
//       const cuda_grid* g, int n_iterations, int stream_index)   (src/gpu_decoder_top.h:13-18)
// reading the members that call reads: h->llr_cuda[s] and h->mem_size_llr_cuda
// (pinned LLRs of the stream's batch), h->hd_packed_cuda[s] (pinned packed
// output), d->streams[s].  `g` is not needed (the decoder sizes its own
// launch).  compat::setup replaces the reference's setup_dev_memory +
// setup_gpu_grid + put_h_compact_and_params_in_constant_memory: one decoder
// per stream, since the reference keeps one process-wide code.
namespace compat {

inline std::vector<std::unique_ptr<Decoder>>& decoders() {
    static std::vector<std::unique_ptr<Decoder>> d;
    return d;
}
inline float& char_llr_scale() {  // LLR = q * scale for the char (CHAR_PRC) build
    static float scale = 1.0f;
    return scale;
}

inline void setup(const nrldpc_ldpc_params& p, int n_streams, int max_cw_per_stream, float alpha = 0.75f,
                  int device = 0) {
    auto& d = decoders();
    d.clear();
    for (int s = 0; s < n_streams; s++) d.emplace_back(new Decoder(p, max_cw_per_stream, alpha, device));
}

namespace detail {
inline void run(Decoder& dec, const float* llr, char* out, int n_cw, int it, cudaStream_t st) {
    dec.perform_gpu_ldpc_decoding(llr, reinterpret_cast<uint8_t*>(out), n_cw, it, st);
}
template <typename T>
typename std::enable_if<sizeof(T) == 1>::type run(Decoder& dec, const T* llr, char* out, int n_cw, int it,
                                                  cudaStream_t st) {
    dec.perform_gpu_ldpc_decoding_q(llr, 2, char_llr_scale(), reinterpret_cast<uint8_t*>(out), n_cw, it, st);
}
template <typename T>
typename std::enable_if<sizeof(T) == 2>::type run(Decoder& dec, const T* llr, char* out, int n_cw, int it,
                                                  cudaStream_t st) {
    dec.perform_gpu_ldpc_decoding_q(llr, 1, 1.0f, reinterpret_cast<uint8_t*>(out), n_cw, it, st);
}
}  // namespace detail

template <typename DevMem, typename HostMem, typename Grid>
void perform_gpu_ldpc_decoding(DevMem* d, HostMem* h, const Grid* /*g*/, int n_iterations, int stream_index) {
    auto& decs = decoders();
    if (stream_index < 0 || stream_index >= static_cast<int>(decs.size()))
        throw std::runtime_error("perform_gpu_ldpc_decoding: no decoder for this stream (compat::setup)");
    Decoder& dec = *decs[stream_index];
    const auto* llr = h->llr_cuda[stream_index];
    const int n_cw = static_cast<int>(h->mem_size_llr_cuda / (static_cast<long>(dec.n_bp()) * sizeof(*llr)));
    detail::run(dec, llr, h->hd_packed_cuda[stream_index], n_cw, n_iterations, d->streams[stream_index]);
}

}  // namespace compat
}  // namespace nrldpc
