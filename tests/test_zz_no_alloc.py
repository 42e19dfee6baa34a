"""The allocation-free decode entry point (nrldpc_decode_noalloc).

It exists for callers that cannot call cudaMalloc while decoding -- e.g. a
physical-layer pipeline that reserves all device memory up front and may not
allocate in its slot loop -- and therefore cannot hold a decoder handle.  Its
scratch is a fixed static device array shared by all calls, so this test
calls it twice in a row on different batches (the second call sees the first
call's leftovers) and checks each result against the handle-based
nrldpc_decode, bit for bit.  Collected last, so a stop-at-first-failure run
has run every other test before it; it also passes alone in a fresh process.
"""
import ctypes as C

import pytest
import torch

from nr_gpu_ldpc_gb300 import Decoder, _lib, codes

pytestmark = pytest.mark.gpu


def noalloc_decode(bg, z, llr, n_iter, early=0, alpha=0.75):
    lib = _lib.load()
    out = torch.empty((llr.shape[0], (llr.shape[1] + 7) // 8), dtype=torch.uint8, device=llr.device)
    rc = lib.nrldpc_decode_noalloc(bg, z, alpha, C.c_void_p(llr.data_ptr()), C.c_void_p(out.data_ptr()),
                                   llr.shape[0], n_iter, early,
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream))
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


def test_noalloc_rejects_bad_arguments():
    lib = _lib.load()
    x = torch.zeros((2, 68 * 384 + 4), device="cuda")
    out = torch.zeros((2, 4000), dtype=torch.uint8, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.nrldpc_decode_noalloc(1, 17, 0.75, C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()),
                                     2, 5, 0, s) == -2
    assert lib.nrldpc_decode_noalloc(1, 384, 0.75, C.c_void_p(x.data_ptr() + 4),
                                     C.c_void_p(out.data_ptr()), 2, 5, 0, s) == -4
    assert lib.nrldpc_decode_noalloc(1, 384, 0.75, None, C.c_void_p(out.data_ptr()), 2, 5, 0, s) == -1
