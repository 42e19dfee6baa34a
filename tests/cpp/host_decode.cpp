// A reference-style C++ caller of the decoder through include/nr_gpu_ldpc_gb300.hpp,
// shaped like the reference's test_throughput (src/main.cpp:147-171):
// setup_ldpc -> one Decoder per stream -> perform_gpu_ldpc_decoding on pinned
// host buffers -> synchronize.
//   host_decode <A> <n_iter> <llr.f32> <out.u8> [host transfer mode]
// reads n codewords of fp32 LLRs (file size / (4 * N_bp)) and writes their
// packed hard decisions; the mode is NRLDPC_HOST_AUTO (default), _COPY or
// _DIRECT.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "nr_gpu_ldpc_gb300.hpp"

int main(int argc, char** argv) {
    if (argc != 5 && argc != 6) {
        std::fprintf(stderr, "usage: %s A n_iter llr.f32 out.u8 [mode]\n", argv[0]);
        return 2;
    }
    const int A = std::atoi(argv[1]), n_iter = std::atoi(argv[2]);
    try {
        const nrldpc_ldpc_params p = nrldpc::setup_ldpc(A, 1.0f / 3.0f, n_iter);
        FILE* f = std::fopen(argv[3], "rb");
        if (!f) return 3;
        std::fseek(f, 0, SEEK_END);
        const long bytes = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        const int n_cw = static_cast<int>(bytes / (4L * p.N_before_puncture));
        float* llr = nullptr;
        uint8_t* packed = nullptr;
        cudaMallocHost(&llr, static_cast<size_t>(bytes));  // pinned, like h->llr_cuda[s]
        if (std::fread(llr, 1, static_cast<size_t>(bytes), f) != static_cast<size_t>(bytes)) return 4;
        std::fclose(f);
        nrldpc::Decoder dec(p, n_cw);
        if (argc == 6) dec.set_host_transfer(std::atoi(argv[5]));
        cudaMallocHost(&packed, static_cast<size_t>(n_cw) * dec.packed_bytes());
        cudaStream_t stream;
        cudaStreamCreate(&stream);
        dec.perform_gpu_ldpc_decoding(llr, packed, n_cw, p.n_iterations, stream);
        const cudaError_t err = cudaStreamSynchronize(stream);
        if (err != cudaSuccess) {
            std::fprintf(stderr, "decode failed on the GPU: %s\n", cudaGetErrorString(err));
            return 6;
        }
        FILE* g = std::fopen(argv[4], "wb");
        if (!g) return 5;
        std::fwrite(packed, 1, static_cast<size_t>(n_cw) * dec.packed_bytes(), g);
        std::fclose(g);
        std::printf("decoded %d codewords: bg %d Z %d N_bp %d\n", n_cw, p.bg_index, p.Z, p.N_before_puncture);
        cudaStreamDestroy(stream);
        cudaFreeHost(llr);
        cudaFreeHost(packed);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
