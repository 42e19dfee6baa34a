// Decode entry point that performs no device (or host heap) allocation.
//
// Some callers cannot call cudaMalloc at decode time: a 5G physical-layer
// pipeline reserves all device memory when it starts and must not allocate
// while it processes slots (an allocation can block and synchronise the
// device and blow the slot's deadline), and code embedded in another
// runtime's memory manager may not own raw device memory at all.  Those
// callers cannot create an nrldpc_handle (its init allocates the check-node
// scratch and staging buffers).  nrldpc_decode_noalloc serves them: the caller
// passes only its input and output buffers, and the decoder's scratch lives in
// a fixed static device array of this file.
//
// Scratch: kNoAllocScratchBytes (96 MiB) for the check-node state of the
// persistent decode CTAs, enough for two CTAs per SM of a 152-SM GB300 at the
// largest code (BG1, Z = 384: 282,624 bytes per CTA), plus 256 bytes of
// counters.  The array is reserved on a GPU when the CUDA runtime loads this
// file's device module there, and held until the process exits: with lazy
// module loading (CUDA's default) when a call of this file first touches the
// array on that GPU (this entry point or nrldpc_noalloc_device_error); with
// CUDA_MODULE_LOADING=EAGER at context creation, on every GPU the process
// uses, whether or not it ever calls this entry point.
//
// Set-up: the first successful call on each device (the current device)
// looks up the array's device address with cudaGetSymbolAddress and
// configures the kernel's shared-memory limit; make that first call before
// any stream capture.  A set-up that fails is not remembered: the next call
// tries again.  All calls share the one array, which keeps the previous
// call's contents: the scheduler counter is cleared on every call (the
// check-node state is written before it is read), but calls that overlap on
// the GPU -- on different streams without ordering, or from several host
// threads -- race on the scratch and give wrong results.  Serialise them.
//
// Errors found on the device (a bounded wait that ran out) are kept in the
// array's error word until nrldpc_noalloc_device_error reads and clears it.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "../../include/nr_gpu_ldpc_gb300.h"
#include "nrldpc_internal.h"

namespace nrldpc {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(96) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_state[kNoAllocScratchBytes];
static __device__ __align__(256) int g_noalloc_counters[64];  // [0] scheduler, [1] error flag

struct DeviceSetup {
    bool done;
    uint32_t* state;
    int* counters;
    int sm_count;
    size_t smem_optin;
    size_t smem_per_sm;
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

int setup_device(int dev, DeviceSetup** out) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& s = g_setup[dev];
    if (!s.done) {
        void* p = nullptr;
        void* q = nullptr;
        cudaDeviceProp prop;
        if (cudaGetSymbolAddress(&p, g_noalloc_state) != cudaSuccess ||
            cudaGetSymbolAddress(&q, g_noalloc_counters) != cudaSuccess ||
            cudaGetDeviceProperties(&prop, dev) != cudaSuccess ||
            decode_kernel_attributes(prop.sharedMemPerBlockOptin) != cudaSuccess) {
            cudaGetLastError();  // leave no sticky launch-side error behind; retried next call
            return NRLDPC_ERR_CUDA;
        }
        s.state = static_cast<uint32_t*>(p);
        s.counters = static_cast<int*>(q);
        s.sm_count = prop.multiProcessorCount;
        s.smem_optin = prop.sharedMemPerBlockOptin;
        s.smem_per_sm = prop.sharedMemPerMultiprocessor;
        s.done = true;
    }
    *out = &s;
    return NRLDPC_OK;
}

// Shared by the decode and its timeout self-test: wait_limit / extra_tx are
// zero in every decode.
int noalloc_decode(int bg, int z, float alpha, const float* d_llr, uint8_t* d_packed, int n_cw, int n_iter,
                   int early_stop, cudaStream_t st, int wait_limit, uint32_t extra_tx) {
    if (n_cw < 0 || n_iter < 1 || (early_stop != 0 && early_stop != 1) || !(alpha > 0.0f))
        return NRLDPC_ERR_INVALID_ARG;
    CodeTable tab;
    if (!make_nr_table(bg, z, &tab)) return NRLDPC_ERR_BAD_CONFIG;
    if (n_cw == 0) return NRLDPC_OK;
    if (!d_llr || !d_packed) return NRLDPC_ERR_INVALID_ARG;
    if (reinterpret_cast<uintptr_t>(d_llr) % 16 != 0) return NRLDPC_ERR_ALIGNMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return NRLDPC_ERR_NO_DEVICE;
    DeviceSetup* s = nullptr;
    const int rc = setup_device(dev, &s);
    if (rc) return rc;
    int cpb = std::max(1, kMaxThreads / z);
    while (cpb > 1 && decode_smem_bytes(tab, cpb) > s->smem_optin) cpb--;
    cpb = std::min(cpb, 48);
    const size_t smem = decode_smem_bytes(tab, cpb);
    if (smem > s->smem_optin) return NRLDPC_ERR_BAD_CONFIG;
    const int threads = (cpb * z + 31) / 32 * 32;
    const int minb = (2 * (smem + 1024) <= s->smem_per_sm) ? 2 : 1;
    const int per_sm = decode_max_ctas_per_sm(false, minb, threads, smem);
    const size_t slot_bytes = static_cast<size_t>(cpb) * tab.rows * tab.z * kStateBytesPerRow;
    const size_t slots = kNoAllocScratchBytes / slot_bytes;
    if (slots < 1) return NRLDPC_ERR_SCRATCH_TOO_SMALL;
    DecodeArgs a{};
    a.llr = d_llr;
    a.packed = d_packed;
    a.state = s->state;
    a.work_counter = s->counters;
    a.error_flag = s->counters + 1;
    a.n_cw = n_cw;
    a.n_iter = n_iter;
    a.cpb = cpb;
    a.n_groups = (n_cw + cpb - 1) / cpb;
    a.early_stop = early_stop;
    a.alpha = alpha;
    a.wait_limit = wait_limit;
    a.extra_tx = extra_tx;
    const long max_grid = std::min<long>(std::max(per_sm, 1) * static_cast<long>(s->sm_count),
                                         static_cast<long>(slots));
    const int grid = static_cast<int>(std::min<long>(a.n_groups, max_grid));
    // only the scheduler counter: the error word stays set until it is read
    if (cudaMemsetAsync(s->counters, 0, sizeof(int), st) != cudaSuccess) return NRLDPC_ERR_CUDA;
    return launch_decode(tab, a, nullptr, grid, threads, smem, false, minb, st) == cudaSuccess ? NRLDPC_OK
                                                                                       : NRLDPC_ERR_CUDA;
}

}  // namespace
}  // namespace nrldpc

using namespace nrldpc;

extern "C" int nrldpc_decode_noalloc(int bg, int z, float alpha, const float* d_llr,
                                     uint8_t* d_packed, int n_cw, int n_iter, int early_stop,
                                     nrldpc_stream_t stream) {
    return noalloc_decode(bg, z, alpha, d_llr, d_packed, n_cw, n_iter, early_stop,
                          reinterpret_cast<cudaStream_t>(stream), 0, 0);
}

// Reads the error word of the current device's static scratch with a
// synchronous symbol copy (no allocation) and clears it when set.
extern "C" int nrldpc_noalloc_device_error(void) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_noalloc_counters, sizeof(int), sizeof(int)) != cudaSuccess)
        return NRLDPC_ERR_CUDA;
    if (v) {
        const int zero = 0;
        if (cudaMemcpyToSymbol(g_noalloc_counters, &zero, sizeof(int), sizeof(int)) != cudaSuccess)
            return NRLDPC_ERR_CUDA;
    }
    return v ? NRLDPC_ERR_TIMEOUT : NRLDPC_OK;
}

extern "C" int nrldpc_selftest_noalloc_wait_timeout(int bg, int z, const float* d_llr, uint8_t* d_packed,
                                                    int n_cw, nrldpc_stream_t stream) {
    // 16 bytes expected and no copy issued, 1024 wait iterations
    return noalloc_decode(bg, z, 0.75f, d_llr, d_packed, n_cw, 1, 0, reinterpret_cast<cudaStream_t>(stream),
                          1024, 16);
}
