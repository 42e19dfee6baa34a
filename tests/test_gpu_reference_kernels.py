"""The reference's own CUDA kernels on the GPU as the parity pin.

src/ldpc_kernels.cu, unmodified, compiled for sm_103a with nvcc's default
flags (the reference's CMake build sets none: --fmad=true) into
oracle/_ref/ref_kernels_bg1.cubin, run by oracle/ref_gpu_harness.cpp in the
launch sequence of perform_gpu_ldpc_decoding (src/gpu_decoder_top.cu:25-49)
with the constant memory the reference's own setup writes, for its own
configuration (BG1, Z = 384).  The decoder's packed hard decisions and fp32
posteriors equal that binary's, bit for bit, and so do the oracle's; the
oracle with the reference's dt = R_temp - RCache fused into one
multiply-add differs, so the comparison does see a contraction where one
happens (the reference binary makes none there).

The cubin and the constant image are built where the reference tree exists
and travel with the repository copy; without them this test skips."""
import time

import numpy as np
import pytest
import torch

from nr_gpu_ldpc_gb300 import Decoder, codes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _llrs():
    z = 384
    oc = O.OracleCode(codes.base_matrix(1, codes.set_index(z)), z)
    parts = []
    for k, eb in enumerate((1.5, 1.75, 2.0, 2.5)):
        llr, _ = oc.gen_llr(22, 300 + k, 0, np.full(4, codes.noise_sigma(eb, 1 / 3), np.float32), 2)
        parts.append(llr)
    llr = np.concatenate(parts)
    # adversarial entries as in the golden fixtures: +-0, a tie, a large magnitude
    llr[0, 800:804] = [0.0, -0.0, 1500.0, -1500.0]
    llr[1, 900] = llr[1, 901]
    return oc, llr


@pytest.mark.skipif(not O.RefGPU.available(), reason="the reference's kernels were not built (no reference tree)")
@pytest.mark.parametrize("n_iter", [1, 2, 5, 10])
def test_decoder_equals_the_reference_binary(gpu, n_iter):
    oc, llr = _llrs()
    rpk, rapp = O.RefGPU().decode(llr, n_iter, want_app=True)
    dec = Decoder(bg=1, z=384, max_batch=len(llr))
    pk, app = dec.decode(torch.from_numpy(llr).to(gpu), n_iter, want_app=True)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(pk.cpu().numpy(), rpk)
    np.testing.assert_array_equal(app.cpu().numpy().view(np.uint32), rapp.view(np.uint32))
    opk, oapp, _ = oc.minsum_f32(llr, n_iter, want_app=True, threads=4)
    np.testing.assert_array_equal(opk, rpk)
    np.testing.assert_array_equal(oapp.view(np.uint32), rapp.view(np.uint32))
    if n_iter >= 2:  # from the second iteration on, a fused dt would show
        O.set_fma_dt(True)
        try:
            _, fapp, _ = oc.minsum_f32(llr, n_iter, want_app=True, threads=4)
        finally:
            O.set_fma_dt(False)
        assert (fapp.view(np.uint32) != rapp.view(np.uint32)).sum() > 0


@pytest.mark.skipif(not O.RefGPU.available(), reason="the reference's kernels were not built (no reference tree)")
def test_decoder_outpaces_the_reference_binary_on_the_same_gpu(gpu):
    """446 BG1 Z=384 codewords (the most one stream of the reference holds in
    fp32), 10 iterations, LLRs resident, device time: the reference's own
    kernels against this decoder (measured 2.33 vs 0.69 ms, 3.4x)."""
    n = 446
    dec = Decoder(bg=1, z=384, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(2.0, 1 / 3), device=gpu)
    llr, _ = dec.gen_llr(7, 0, sig)
    ref_ms = O.RefGPU().time_ms(llr.cpu().numpy(), 10, warmup=3, reps=10)
    for _ in range(3):
        dec.decode(llr, 10)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        dec.decode(llr, 10)
    e1.record()
    torch.cuda.synchronize()
    ours_ms = e0.elapsed_time(e1) / 10
    print(f"reference kernels {ref_ms:.3f} ms, this decoder {ours_ms:.3f} ms per {n} codewords")
    assert ours_ms * 2.0 < ref_ms, (ours_ms, ref_ms)
    dec.close()


@pytest.mark.skipif(not O.RefGPU.available(), reason="the reference's kernels were not built (no reference tree)")
def test_testbench_latency_against_the_reference_binary(gpu):
    """The reference testbench's latency measurement (test_latency,
    src/main.cpp:147-156) on its configuration: one 40-codeword BG1 Z=384
    batch (n_cw_per_mcw * n_mcw), 5 iterations, pinned host buffers with the
    copies inside the timing, host clock, best of 50 calls: the reference's
    own kernels against this decoder's host-buffer call, same bits out.
    Measured 179 us for the reference's kernels and 190 us here: at one
    codeword per SM this decoder walks a codeword's 46 base rows in sequence
    on one SM (164 us of kernel time), where each of the reference's 11
    launches spreads the batch over a CTA per base row.  The bound below
    guards against a regression of that gap; the throughput design wins from
    a few hundred codewords on (3.4x at 446)."""
    n, n_iter = 40, 5
    dec = Decoder(bg=1, z=384, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(2.0, 1 / 3), device=gpu)
    llr, _ = dec.gen_llr(9, 0, sig)
    llr_np = llr.cpu().numpy()
    ref = O.RefGPU()
    ref_best, ref_med = ref.latency_us(llr_np, n_iter)
    rpk, _ = ref.decode(llr_np, n_iter)
    h_llr = torch.from_numpy(llr_np).pin_memory()
    h_out = torch.empty((n, dec.packed_bytes), dtype=torch.uint8).pin_memory()
    s = torch.cuda.Stream()
    for _ in range(5):
        dec.decode_host(h_llr, h_out, n_iter, stream=s)
        torch.cuda.synchronize()
    us = []
    for _ in range(50):
        t0 = time.perf_counter()
        dec.decode_host(h_llr, h_out, n_iter, stream=s)
        torch.cuda.synchronize()
        us.append(1e6 * (time.perf_counter() - t0))
    us.sort()
    print(f"latency of 40 codewords, 5 iterations: reference kernels best {ref_best:.1f} us "
          f"(median {ref_med:.1f}), this decoder best {us[0]:.1f} us (median {us[25]:.1f})")
    np.testing.assert_array_equal(h_out.numpy(), rpk)
    assert us[0] < 1.25 * ref_best, (us[0], ref_best)
    dec.close()

