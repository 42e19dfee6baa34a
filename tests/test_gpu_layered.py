"""Layered (row-sequential) schedule on the GPU against the oracle's layered
decoder, bit for bit: packed hard decisions, posterior bits and iteration
counts, with and without early stop, plain (alpha) and weighted."""
import numpy as np
import pytest
import torch

from nr_gpu_ldpc_gb300 import Decoder, codes
from oracle.oracle import OracleCode

pytestmark = pytest.mark.gpu


def _bits(a):
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


def _setup(bg, z, n, ebn0, seed=5, max_batch=None):
    dec = Decoder(bg=bg, z=z, max_batch=max_batch or n)
    dec.set_schedule("layered")
    oc = OracleCode(codes.base_matrix(bg, codes.set_index(z)), z)
    rate = dec.kb / (dec.cols - 2)
    sig = np.full(n, codes.noise_sigma(ebn0, rate), np.float32)
    llr, cw = oc.gen_llr(dec.kb, seed, 0, sig, 2)
    return dec, oc, llr, cw


@pytest.mark.parametrize("bg,z,n", [(1, 384, 6), (2, 128, 9), (1, 64, 13), (2, 15, 30), (1, 2, 50)])
@pytest.mark.parametrize("early", [False, True])
def test_layered_matches_oracle(gpu, bg, z, n, early):
    dec, oc, llr, _ = _setup(bg, z, n, 1.2)
    pk, app, it = dec.decode(torch.from_numpy(llr).to(gpu), 7, early_stop=early, want_app=True, want_iters=True)
    torch.cuda.synchronize()
    opk, oapp, oit = oc.layered_f32(llr, 7, early_stop=early, want_app=True)
    np.testing.assert_array_equal(pk.cpu().numpy(), opk)
    np.testing.assert_array_equal(_bits(app.cpu().numpy()), _bits(oapp))
    np.testing.assert_array_equal(it.cpu().numpy(), oit)
    assert dec.device_error() == 0


def test_layered_early_stop_mixture(gpu):
    """Eb/N0 spread so codewords stop at different iterations (per-slot stop
    inside multi-codeword CTAs at Z=64)."""
    dec = Decoder(bg=1, z=64, max_batch=96)
    dec.set_schedule("layered")
    oc = OracleCode(codes.base_matrix(1, codes.set_index(64)), 64)
    sig = np.linspace(0.55, 0.95, 96).astype(np.float32)
    llr, _ = oc.gen_llr(22, 77, 0, sig, 2)
    pk, it = dec.decode(torch.from_numpy(llr).to(gpu), 12, early_stop=True, want_iters=True)
    torch.cuda.synchronize()
    opk, _, oit = oc.layered_f32(llr, 12, early_stop=True)
    np.testing.assert_array_equal(it.cpu().numpy(), oit)
    np.testing.assert_array_equal(pk.cpu().numpy(), opk)
    assert len(np.unique(oit)) >= 3


def test_layered_weighted_matches_oracle(gpu):
    dec, oc, llr, _ = _setup(1, 96, 8, 1.0)
    rng = np.random.default_rng(3)
    w = rng.uniform(0.5, 1.0, (4, dec.n_edges)).astype(np.float32)
    dec.set_weights(w)
    for early in (False, True):
        pk, app, it = dec.decode(torch.from_numpy(llr).to(gpu), 6, early_stop=early, weighted=True,
                                 want_app=True, want_iters=True)
        torch.cuda.synchronize()
        opk, oapp, oit = oc.layered_f32(llr, 6, w=w, early_stop=early, want_app=True)
        np.testing.assert_array_equal(pk.cpu().numpy(), opk)
        np.testing.assert_array_equal(_bits(app.cpu().numpy()), _bits(oapp))
        np.testing.assert_array_equal(it.cpu().numpy(), oit)


def test_layered_adversarial_inputs(gpu):
    """Signed zeros, infinities, NaN and magnitudes above 1000 in the LLRs."""
    z = 32
    dec = Decoder(bg=2, z=z, max_batch=8)
    dec.set_schedule("layered")
    oc = OracleCode(codes.base_matrix(2, codes.set_index(z)), z)
    rng = np.random.default_rng(9)
    llr = rng.normal(0.5, 2.0, (8, dec.n_bp)).astype(np.float32)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 2000.0, -1500.0], np.float32)
    mask = rng.random(llr.shape) < 0.05
    llr[mask] = rng.choice(specials, mask.sum())
    for early in (False, True):
        pk, app, it = dec.decode(torch.from_numpy(llr).to(gpu), 5, early_stop=early, want_app=True,
                                 want_iters=True)
        torch.cuda.synchronize()
        opk, oapp, oit = oc.layered_f32(llr, 5, early_stop=early, want_app=True)
        np.testing.assert_array_equal(pk.cpu().numpy(), opk)
        np.testing.assert_array_equal(_bits(app.cpu().numpy()), _bits(oapp))
        np.testing.assert_array_equal(it.cpu().numpy(), oit)


def test_layered_converges_faster_than_flooding(gpu):
    """Full 4096-codeword BG1 Z=384 batch at 2.0 dB: the layered schedule
    needs fewer iterations on average and loses no frame the flooding decoder
    gets right (a size-independent property; the oracle checks a sample)."""
    n = 4096
    dec = Decoder(bg=1, z=384, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(2.0, 22 / 66), device=gpu)
    llr, cw = dec.gen_llr(17, 0, sig)
    pf, itf = dec.decode(llr, 20, early_stop=True, want_iters=True)
    dec.set_schedule("layered")
    pl, itl = dec.decode(llr, 20, early_stop=True, want_iters=True)
    cf = dec.count_errors(pf, cw)
    cl = dec.count_errors(pl, cw)
    torch.cuda.synchronize()
    assert itl.float().mean().item() < 0.75 * itf.float().mean().item()
    assert int(cl[1]) <= int(cf[1])
    oc = OracleCode(codes.base_matrix(1, codes.set_index(384)), 384)
    sample = [0, 1234, 4095]
    opk, _, oit = oc.layered_f32(llr[sample].cpu().numpy(), 20, early_stop=True)
    np.testing.assert_array_equal(pl[sample].cpu().numpy(), opk)
    np.testing.assert_array_equal(itl[sample].cpu().numpy(), oit)
