"""The allocation-free decode entry point (nrldpc_decode_noalloc).

It exists for callers that cannot call cudaMalloc while decoding -- e.g. a
physical-layer pipeline that reserves all device memory up front and may not
allocate in its slot loop -- and therefore cannot hold a decoder handle.  Its
scratch is a fixed static device array shared by all calls, so these tests
call it twice in a row on different batches (the second call sees the first
call's leftovers) and check each result against the handle-based
nrldpc_decode, bit for bit, and against the oracle directly; one batch is
large enough that every persistent CTA reuses its scratch slot for several
codeword groups; and a bounded wait that runs out is reported by
nrldpc_noalloc_device_error.  Collected last, so a stop-at-first-failure run
has run every other test before it; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from nr_gpu_ldpc_gb300 import Decoder, _lib, codes
from oracle.oracle import OracleCode

pytestmark = pytest.mark.gpu
NRLDPC_ERR_TIMEOUT = -6


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def noalloc_decode(bg, z, llr, n_iter, early=0, alpha=0.75):
    lib = _lib.load()
    out = torch.empty((llr.shape[0], (llr.shape[1] + 7) // 8), dtype=torch.uint8, device=llr.device)
    rc = lib.nrldpc_decode_noalloc(bg, z, alpha, C.c_void_p(llr.data_ptr()), C.c_void_p(out.data_ptr()),
                                   llr.shape[0], n_iter, early, _stream())
    _lib.check("nrldpc_decode_noalloc", rc)
    return out


@pytest.mark.parametrize("bg,z,n,ebn0", [(1, 384, 300, 1.75), (2, 128, 200, 2.0), (1, 36, 70, 2.5)])
def test_noalloc_matches_handle_decode_twice(bg, z, n, ebn0):
    assert torch.cuda.is_available()
    dec = Decoder(bg=bg, z=z, max_batch=n)
    rate = dec.kb / (dec.cols - 2)
    for call, seed in enumerate((11, 12)):
        sig = torch.full((n,), codes.noise_sigma(ebn0 + 0.25 * call, rate), device="cuda")
        llr, _ = dec.gen_llr(seed, 1000 * call, sig)
        want = dec.decode(llr, 8)
        got = noalloc_decode(bg, z, llr, 8)
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"call {call + 1} differs from nrldpc_decode"
        want_es = dec.decode(llr, 8, early_stop=True)
        got_es = noalloc_decode(bg, z, llr, 8, early=1)
        torch.cuda.synchronize()
        assert torch.equal(got_es, want_es), f"early-stop call {call + 1} differs"
    assert _lib.load().nrldpc_noalloc_device_error() == 0
    dec.close()


@pytest.mark.parametrize("bg,z,n", [(1, 384, 24), (2, 128, 30)])
def test_noalloc_matches_oracle_twice(bg, z, n):
    """Against the oracle's restatement of the reference min-sum (not only
    against the handle decode, which shares the kernel), two calls in a row."""
    oc = OracleCode(codes.base_matrix(bg, codes.set_index(z)), z)
    kb = 22 if bg == 1 else 10
    rate = kb / (oc.cols - 2)
    for call in range(2):
        sigma = np.full(n, codes.noise_sigma(1.6 + 0.3 * call, rate), np.float32)
        llr, _ = oc.gen_llr(kb, 40 + call, 0, sigma, 2)
        got = noalloc_decode(bg, z, torch.from_numpy(llr).cuda(), 6, early=call)
        torch.cuda.synchronize()
        want, _, _ = oc.minsum_f32(llr, 6, early_stop=bool(call), threads=4)
        assert np.array_equal(got.cpu().numpy(), want), f"call {call + 1} differs from the oracle"


def test_noalloc_reuses_scratch_slots_across_many_groups():
    """2048 BG1 Z=384 codewords: far more codeword groups than persistent
    CTAs, so every CTA's scratch slot carries several codewords in turn."""
    n = 2048
    dec = Decoder(bg=1, z=384, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(1.7, 1 / 3), device="cuda")
    llr, _ = dec.gen_llr(5, 0, sig)
    for early in (0, 1):
        want = dec.decode(llr, 10, early_stop=bool(early))
        got = noalloc_decode(1, 384, llr, 10, early=early)
        torch.cuda.synchronize()
        assert torch.equal(got, want), f"early_stop={early}"
    dec.close()


def test_noalloc_reports_a_wait_that_ran_out():
    """The self-test's copy barrier expects bytes no copy delivers, so every
    CTA's bounded wait runs out; the error word reports it once, and the next
    decode is exact again."""
    lib = _lib.load()
    z, n = 384, 8
    oc = OracleCode(codes.base_matrix(1, codes.set_index(z)), z)
    llr, _ = oc.gen_llr(22, 78, 0, np.full(n, codes.noise_sigma(2.0, 1 / 3), np.float32), 2)
    d_llr = torch.from_numpy(llr).cuda()
    out = torch.zeros((n, oc.n_bytes), dtype=torch.uint8, device="cuda")
    assert lib.nrldpc_noalloc_device_error() == 0
    assert lib.nrldpc_selftest_noalloc_wait_timeout(1, z, C.c_void_p(d_llr.data_ptr()),
                                                    C.c_void_p(out.data_ptr()), n, _stream()) == 0
    torch.cuda.synchronize()
    assert lib.nrldpc_noalloc_device_error() == NRLDPC_ERR_TIMEOUT
    assert lib.nrldpc_noalloc_device_error() == 0
    got = noalloc_decode(1, z, d_llr, 5)
    torch.cuda.synchronize()
    want, _, _ = oc.minsum_f32(llr, 5)
    assert np.array_equal(got.cpu().numpy(), want)
    assert lib.nrldpc_noalloc_device_error() == 0


def test_noalloc_rejects_bad_arguments():
    lib = _lib.load()
    x = torch.zeros((2, 68 * 384 + 4), device="cuda")
    out = torch.zeros((2, 4000), dtype=torch.uint8, device="cuda")
    s = _stream()
    assert lib.nrldpc_decode_noalloc(1, 17, 0.75, C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()),
                                     2, 5, 0, s) == -2
    assert lib.nrldpc_decode_noalloc(1, 384, 0.75, C.c_void_p(x.data_ptr() + 4),
                                     C.c_void_p(out.data_ptr()), 2, 5, 0, s) == -4
    assert lib.nrldpc_decode_noalloc(1, 384, 0.75, None, C.c_void_p(out.data_ptr()), 2, 5, 0, s) == -1
