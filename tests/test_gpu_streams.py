"""Several handles on several streams at once, as the reference's n_streams
pattern uses them (src/main.cpp:160-170: one batch per stream issued back to
back, one synchronize): every stream's host-buffer decode equals the same
handle's device decode and the oracle, whatever the other streams do."""
import numpy as np
import pytest
import torch

from nr_gpu_ldpc_gb300 import Decoder, codes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["auto", "copy", "direct"])
def test_one_handle_per_stream_concurrently(gpu, mode):
    n_streams, n_cw, z = 6, 40, 64
    decs = [Decoder(bg=1, z=z, max_batch=n_cw) for _ in range(n_streams)]
    streams = [torch.cuda.Stream() for _ in range(n_streams)]
    sig = torch.full((n_cw,), codes.noise_sigma(1.5, 22 / 66), device=gpu)
    llr_h, out_h, want = [], [], []
    for k, d in enumerate(decs):
        d.set_host_transfer(mode)
        llr, _ = d.gen_llr(seed=5, cw_base=1000 * k, sigma=sig)
        want.append(d.decode(llr, 5).cpu())
        llr_h.append(llr.cpu().pin_memory())
        out_h.append(torch.empty((n_cw, d.packed_bytes), dtype=torch.uint8).pin_memory())
    torch.cuda.synchronize()
    for _ in range(3):
        for k, d in enumerate(decs):
            out_h[k].zero_()
        for k, d in enumerate(decs):
            d.decode_host(llr_h[k], out_h[k], 5, stream=streams[k])
        torch.cuda.synchronize()
        for k in range(n_streams):
            assert torch.equal(out_h[k], want[k]), (mode, k)
    oc = O.OracleCode(codes.base_matrix(1, codes.set_index(z)), z)
    opk, _, _ = oc.minsum_f32(llr_h[2].numpy(), 5)
    np.testing.assert_array_equal(out_h[2].numpy(), opk)
    for d in decs:
        d.close()
