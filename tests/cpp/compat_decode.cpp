// A caller written against the reference's own decode call shape
// (perform_gpu_ldpc_decoding(dev_mem<T>*, host_mem<T>*, const cuda_grid*,
// n_iterations, stream_index), src/gpu_decoder_top.h:13-18) through
// nrldpc::compat: its structs carry the members that call reads.
//   compat_decode <llr.f32> <out.u8>
// decodes the file's codewords twice, split over two streams.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "nr_gpu_ldpc_gb300.hpp"

template <typename T>
struct HostBuffers {  // the host_mem members the decode call reads
    T** llr_cuda;
    int mem_size_llr_cuda;
    char** hd_packed_cuda;
    int mem_size_hd_cuda_packed;
};
template <typename T>
struct DeviceState {  // the dev_mem member it reads
    cudaStream_t* streams;
};
struct Grid {};

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    try {
        const nrldpc_ldpc_params p = nrldpc::setup_ldpc(8424, 1.0f / 3.0f, 10);
        FILE* f = std::fopen(argv[1], "rb");
        if (!f) return 3;
        std::fseek(f, 0, SEEK_END);
        const long bytes = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        const int n_cw = static_cast<int>(bytes / (4L * p.N_before_puncture));
        const int n_streams = 2, per_stream = (n_cw + 1) / 2;
        nrldpc::compat::setup(p, n_streams, per_stream);
        const int packed = (p.N_before_puncture + 7) / 8;
        float* llr[2];
        char* out[2];
        cudaStream_t streams[2];
        for (int s = 0; s < n_streams; s++) {
            cudaMallocHost(&llr[s], static_cast<size_t>(per_stream) * p.N_before_puncture * 4);
            cudaMallocHost(&out[s], static_cast<size_t>(per_stream) * packed);
            cudaStreamCreate(&streams[s]);
        }
        std::vector<float> all(static_cast<size_t>(bytes) / 4);
        if (std::fread(all.data(), 1, static_cast<size_t>(bytes), f) != static_cast<size_t>(bytes)) return 4;
        std::fclose(f);
        int counts[2] = {per_stream, n_cw - per_stream};
        for (int s = 0; s < n_streams; s++)
            std::memcpy(llr[s], all.data() + static_cast<size_t>(s) * per_stream * p.N_before_puncture,
                        static_cast<size_t>(counts[s]) * p.N_before_puncture * 4);
        DeviceState<float> d{streams};
        Grid g;
        for (int s = 0; s < n_streams; s++) {
            HostBuffers<float> h{llr, counts[s] * p.N_before_puncture * 4, out, counts[s] * packed};
            nrldpc::compat::perform_gpu_ldpc_decoding(&d, &h, &g, p.n_iterations, s);
        }
        const cudaError_t err = cudaDeviceSynchronize();
        if (err != cudaSuccess) {
            std::fprintf(stderr, "decode failed on the GPU: %s\n", cudaGetErrorString(err));
            return 6;
        }
        FILE* o = std::fopen(argv[2], "wb");
        if (!o) return 5;
        for (int s = 0; s < n_streams; s++) std::fwrite(out[s], 1, static_cast<size_t>(counts[s]) * packed, o);
        std::fclose(o);
        for (int s = 0; s < n_streams; s++) {
            cudaFreeHost(llr[s]);
            cudaFreeHost(out[s]);
            cudaStreamDestroy(streams[s]);
        }
        nrldpc::compat::decoders().clear();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
