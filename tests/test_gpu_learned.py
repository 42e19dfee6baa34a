"""Learned weighted min-sum on the GPU: forward, adjoint and Adam kernels
against the CPU oracle, and the weighted decoder against the oracle."""
import numpy as np
import pytest
import torch

from nr_gpu_ldpc_gb300 import Decoder, codes
from nr_gpu_ldpc_gb300.learned import Trainer
from oracle.oracle import OracleCode

pytestmark = pytest.mark.gpu


def _data(bg, z, n, seed, ebn0=1.5):
    oc = OracleCode(codes.base_matrix(bg, codes.set_index(z)), z)
    kb = codes.KB_MAX[bg]
    sig = np.full(n, codes.noise_sigma(ebn0, kb / (oc.cols - 2)), np.float32)
    llr, cw = oc.gen_llr(kb, seed, 0, sig, 2)
    return oc, llr, cw


@pytest.mark.parametrize("bg,z", [(2, 16), (1, 12), (2, 128)])
def test_forward_loss_and_adjoint_match_oracle(gpu, bg, z):
    T, n = 4, 6
    oc, llr, cw = _data(bg, z, n, 3 + z)
    # perturb the punctured zeros so no two |Q| tie exactly
    rng = np.random.default_rng(z)
    llr[:, :2 * z] = rng.normal(0, 0.3, (n, 2 * z)).astype(np.float32)
    w = rng.uniform(0.55, 0.95, (T, oc.n_edges)).astype(np.float32)
    tr = Trainer(bg=bg, z=z, n_iter=T, batch=n, chunk=n)
    wd = torch.from_numpy(w).to(gpu)
    loss, grad = tr.loss_and_grad(torch.from_numpy(llr).to(gpu), torch.from_numpy(cw).to(gpu), wd)
    oloss, ograd, _ = oc.wms_loss_grad(llr, cw, T, w.astype(np.float64))
    assert abs(loss - oloss) <= 1e-5 * abs(oloss)
    g = grad.cpu().numpy()
    rel = np.linalg.norm(g - ograd) / np.linalg.norm(ograd)
    assert rel < 2e-3, rel
    assert np.corrcoef(g.ravel(), ograd.ravel())[0, 1] > 0.9999


def test_forward_posterior_is_the_weighted_decoder(gpu):
    bg, z, T, n = 1, 64, 5, 5
    oc, llr, cw = _data(bg, z, n, 9)
    w = np.random.default_rng(2).uniform(0.6, 0.9, (T, oc.n_edges)).astype(np.float32)
    tr = Trainer(bg=bg, z=z, n_iter=T, batch=n, chunk=n)
    app = torch.empty((n, oc.n_bp), device=gpu)
    tr.forward(torch.from_numpy(llr).to(gpu), torch.from_numpy(cw).to(gpu), 1.0, app=app,
               weights=torch.from_numpy(w).to(gpu))
    torch.cuda.synchronize()
    opk, oapp, _ = oc.wms_decode_f32(llr, T, w, want_app=True)
    np.testing.assert_array_equal(app.cpu().numpy().view(np.uint32), oapp.view(np.uint32))
    dec = Decoder(bg=bg, z=z, max_batch=n)
    dec.set_weights(w)
    pk, dapp = dec.decode(torch.from_numpy(llr).to(gpu), T, weighted=True, want_app=True)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(pk.cpu().numpy(), opk)
    np.testing.assert_array_equal(dapp.cpu().numpy().view(np.uint32), oapp.view(np.uint32))


@pytest.mark.parametrize("bg,z", [(1, 384), (2, 128)])
def test_weighted_decode_with_early_stop_matches_oracle(gpu, bg, z):
    n, T = 12, 8
    oc, llr, cw = _data(bg, z, n, 21, ebn0=2.0)
    w = np.random.default_rng(5).uniform(0.6, 0.95, (6, oc.n_edges)).astype(np.float32)
    dec = Decoder(bg=bg, z=z, max_batch=n)
    dec.set_weights(w)  # 6 rows: iterations 7 and 8 reuse the last row
    pk, app, its = dec.decode(torch.from_numpy(llr).to(gpu), T, early_stop=True, weighted=True,
                              want_app=True, want_iters=True)
    torch.cuda.synchronize()
    opk, oapp, oits = oc.wms_decode_f32(llr, T, w, early_stop=True, want_app=True)
    np.testing.assert_array_equal(its.cpu().numpy(), oits)
    np.testing.assert_array_equal(pk.cpu().numpy(), opk)
    np.testing.assert_array_equal(app.cpu().numpy().view(np.uint32), oapp.view(np.uint32))


@pytest.mark.parametrize("layered", [False, True])
def test_signed_weights_match_oracle(gpu, layered):
    """Negative and zero weights: every message is the product w * sign * min,
    as the oracle computes it."""
    n, T = 10, 6
    oc, llr, _ = _data(1, 64, n, 8, ebn0=2.0)
    rng = np.random.default_rng(9)
    w = rng.uniform(-0.9, 0.95, (T, oc.n_edges)).astype(np.float32)
    w[:, ::17] = 0.0
    dec = Decoder(bg=1, z=64, max_batch=n)
    if layered:
        dec.set_schedule("layered")
    dec.set_weights(w)
    pk, app, its = dec.decode(torch.from_numpy(llr).to(gpu), T, early_stop=True, weighted=True,
                              want_app=True, want_iters=True)
    torch.cuda.synchronize()
    if layered:
        opk, oapp, oits = oc.layered_f32(llr, T, w=w, early_stop=True, want_app=True)
    else:
        opk, oapp, oits = oc.wms_decode_f32(llr, T, w, early_stop=True, want_app=True)
    np.testing.assert_array_equal(its.cpu().numpy(), oits)
    np.testing.assert_array_equal(pk.cpu().numpy(), opk)
    np.testing.assert_array_equal(app.cpu().numpy().view(np.uint32), oapp.view(np.uint32))


def test_adam_step_matches_numpy(gpu):
    tr = Trainer(bg=2, z=8, n_iter=2, batch=4, chunk=4, lr=1e-2)
    rng = np.random.default_rng(0)
    g = rng.normal(size=tr.w.shape)
    tr.grad.copy_(torch.from_numpy(g))
    w0 = tr.w.cpu().numpy().copy()
    from nr_gpu_ldpc_gb300 import _lib
    from nr_gpu_ldpc_gb300.decoder import _dev_ptr, _stream_ptr
    lib = _lib.load()
    for step in (1, 2):
        assert lib.nrldpc_adam_step(tr.w.numel(), _dev_ptr(tr.w), _dev_ptr(tr.grad), _dev_ptr(tr.m),
                                    _dev_ptr(tr.v), step, 1e-2, 0.9, 0.999, 1e-8, 0.0,
                                    _stream_ptr(None)) == 0
    torch.cuda.synchronize()
    m = v = 0.0
    w = w0.astype(np.float64)
    for step in (1, 2):
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        w = np.maximum(w - 1e-2 * (m / (1 - 0.9 ** step)) / (np.sqrt(v / (1 - 0.999 ** step)) + 1e-8), 0.0)
    np.testing.assert_allclose(tr.w.cpu().numpy(), w, rtol=1e-5, atol=1e-6)


def test_short_training_lowers_the_loss(gpu):
    tr = Trainer(bg=2, z=32, n_iter=5, batch=2048, chunk=1024, lr=5e-3, seed=7)
    hist = tr.train(25)
    assert np.mean(hist[-5:]) < np.mean(hist[:5])
    assert np.isfinite(hist).all()


@pytest.mark.parametrize("bg,z", [(2, 16), (1, 12), (2, 64)])
def test_layered_forward_and_adjoint_match_oracle(gpu, bg, z):
    T, n = 4, 6
    oc, llr, cw = _data(bg, z, n, 11 + z)
    rng = np.random.default_rng(z + 1)
    llr[:, :2 * z] = rng.normal(0, 0.3, (n, 2 * z)).astype(np.float32)
    w = rng.uniform(0.55, 0.95, (T, oc.n_edges)).astype(np.float32)
    tr = Trainer(bg=bg, z=z, n_iter=T, batch=n, chunk=n, schedule="layered")
    wd = torch.from_numpy(w).to(gpu)
    loss, grad = tr.loss_and_grad(torch.from_numpy(llr).to(gpu), torch.from_numpy(cw).to(gpu), wd)
    # the oracle's forward in the decoder's fp32 rounding: same argmins and
    # signs as the GPU (an f64 forward flips near-tied argmins of the
    # sequential in-place updates); loss and adjoint in double
    oloss, ograd, _ = oc.wms_loss_grad(llr, cw, T, w.astype(np.float64), layered=True, f32_forward=True)
    assert abs(loss - oloss) <= 1e-5 * abs(oloss)
    g = grad.cpu().numpy()
    rel = np.linalg.norm(g - ograd) / np.linalg.norm(ograd)
    assert rel < 2e-4, rel
    assert np.corrcoef(g.ravel(), ograd.ravel())[0, 1] > 0.9999


def test_layered_forward_posterior_is_the_layered_decoder(gpu):
    bg, z, T, n = 1, 64, 5, 5
    oc, llr, cw = _data(bg, z, n, 19)
    w = np.random.default_rng(4).uniform(0.6, 0.9, (T, oc.n_edges)).astype(np.float32)
    tr = Trainer(bg=bg, z=z, n_iter=T, batch=n, chunk=n, schedule="layered")
    app = torch.empty((n, oc.n_bp), device=gpu)
    tr.forward(torch.from_numpy(llr).to(gpu), torch.from_numpy(cw).to(gpu), 1.0, app=app,
               weights=torch.from_numpy(w).to(gpu))
    torch.cuda.synchronize()
    opk, oapp, _ = oc.layered_f32(llr, T, w=w, want_app=True)
    np.testing.assert_array_equal(app.cpu().numpy().view(np.uint32), oapp.view(np.uint32))


def test_layered_short_training_lowers_the_loss(gpu):
    tr = Trainer(bg=2, z=32, n_iter=4, batch=2048, chunk=1024, lr=5e-3, seed=3, schedule="layered")
    hist = tr.train(25)
    assert np.mean(hist[-5:]) < np.mean(hist[:5])
    assert np.isfinite(hist).all()


def test_weight_rows_limit(gpu):
    from nr_gpu_ldpc_gb300 import _lib
    dec = Decoder(bg=2, z=16, max_batch=4)
    with pytest.raises(_lib.NrLdpcError):
        dec.set_weights(np.full((17, dec.n_edges), 0.75, np.float32))
    dec.set_weights(np.full((16, dec.n_edges), 0.75, np.float32))  # the maximum is accepted


def test_trained_weights_gain_over_plain(gpu):
    """What the trained network adds (committed weights/bg1_L6, BG1 Z=384,
    1.8 dB, 16384 seeded codewords, early stop): the learned layered decoder
    at <= 6 iterations has a lower FER than the same layered decoder with the
    plain alpha = 0.75 and than plain flooding min-sum at 10 iterations."""
    from nr_gpu_ldpc_gb300.learned import load_weights
    n = 8192
    dec = Decoder(bg=1, z=384, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(1.8, 22 / 66), device=gpu)
    sets = [dec.gen_llr(seed=404, cw_base=k * n, sigma=sig) for k in range(2)]

    def fer(schedule, weights, iters):
        dec.set_schedule(schedule)
        if weights is not None:
            dec.set_weights(load_weights(weights))
        counts = torch.zeros(2, dtype=torch.int64, device=gpu)
        for llr, cw in sets:
            pk = dec.decode(llr, iters, early_stop=True, weighted=weights is not None)
            dec.count_errors(pk, cw, counts=counts)
        torch.cuda.synchronize()
        return int(counts[1]) / (2 * n)

    learned = fer("layered", "bg1_L6", 6)
    plain_layered = fer("layered", None, 6)
    plain_flooding = fer("flooding", None, 10)
    assert learned < 0.2 * plain_layered and learned < 0.2 * plain_flooding, (learned, plain_layered, plain_flooding)
    assert plain_flooding <= 1e-2  # the operating point: plain min-sum at 10 iterations has FER <= 1e-2


def test_trained_bg2_weights_gain_over_plain(gpu):
    """What the training configuration's own network adds (committed
    weights/bg2_T8: BG2 Z=128, flooding, 8 iterations, trained on the GPU on
    Eb/N0 U[1,3] dB): at 2.0 dB, 16384 seeded codewords, early stop, its FER
    is well below that of the same decoder with the plain alpha = 0.75
    (measured 0.040 against 0.107)."""
    from nr_gpu_ldpc_gb300.learned import load_weights
    n = 16384
    dec = Decoder(bg=2, z=128, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(2.0, dec.kb / (dec.cols - 2)), device=gpu)
    llr, cw = dec.gen_llr(seed=505, cw_base=0, sigma=sig)

    def fer(weights):
        if weights is not None:
            dec.set_weights(weights)
        counts = torch.zeros(2, dtype=torch.int64, device=gpu)
        pk = dec.decode(llr, 8, early_stop=True, weighted=weights is not None)
        dec.count_errors(pk, cw, counts=counts)
        torch.cuda.synchronize()
        return int(counts[1]) / n

    learned, plain = fer(load_weights("bg2_T8")), fer(None)
    assert plain > 0.03 and learned < 0.6 * plain, (learned, plain)
    dec.close()
