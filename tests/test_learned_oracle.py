"""Learned weighted min-sum: the oracle's adjoint against finite differences
(CPU).  Random continuous LLRs (no punctured zeros) keep the piecewise-linear
min/sign structure away from ties, so central differences are exact up to
the smooth softplus terms."""
import numpy as np

from nr_gpu_ldpc_gb300 import codes
from oracle.oracle import OracleCode


def _case(bg=2, z=6, n=3, T=3, seed=0):
    oc = OracleCode(codes.base_matrix(bg, codes.set_index(z)), z)
    rng = np.random.default_rng(seed)
    kb = codes.KB_MAX[bg]
    info = rng.integers(0, 2, (n, kb * z)).astype(np.uint8)
    cw = np.stack([oc.encode(kb, i) for i in info])
    bits = np.unpackbits(cw, axis=1, bitorder="little")[:, :oc.n_bp].astype(np.float32)
    llr = ((1 - 2 * bits) * 1.2 + rng.normal(0, 1.3, bits.shape)).astype(np.float32)
    w = rng.uniform(0.5, 1.0, (T, oc.n_edges))
    return oc, llr, cw, w


def test_adjoint_matches_finite_differences():
    oc, llr, cw, w = _case()
    T = w.shape[0]
    loss, grad, _ = oc.wms_loss_grad(llr, cw, T, w)
    rng = np.random.default_rng(1)
    idx = [(int(rng.integers(T)), int(rng.integers(oc.n_edges))) for _ in range(25)]
    checked = 0
    for t, e in idx:
        fd = []
        for eps in (1e-5, 5e-6):
            wp, wm = w.copy(), w.copy()
            wp[t, e] += eps
            wm[t, e] -= eps
            lp, _, _ = oc.wms_loss_grad(llr, cw, T, wp, want_grad=False)
            lm, _, _ = oc.wms_loss_grad(llr, cw, T, wm, want_grad=False)
            fd.append((lp - lm) / (2 * eps))
        if abs(fd[0] - fd[1]) > 1e-6 * max(1.0, abs(fd[0])) * 1e3:
            continue  # a min/sign switch inside the stencil: not differentiable here
        np.testing.assert_allclose(grad[t, e], fd[0], rtol=2e-4, atol=1e-9)
        checked += 1
    assert checked >= 20
    assert np.abs(grad).max() > 0


def test_weighted_decode_f32_equals_plain_at_constant_weight():
    """w[t][e] = 0.75 everywhere is the reference decoder exactly."""
    oc, llr, cw, _ = _case(bg=1, z=8, n=2, T=4)
    w = np.full((4, oc.n_edges), 0.75, np.float32)
    p1, a1, _ = oc.wms_decode_f32(llr, 4, w, want_app=True)
    p2, a2, _ = oc.minsum_f32(llr, 4, want_app=True)
    np.testing.assert_array_equal(p1, p2)
    np.testing.assert_array_equal(a1.view(np.uint32), a2.view(np.uint32))


def test_loss_posterior_equals_f64_decoder_at_constant_weight():
    oc, llr, cw, _ = _case(bg=2, z=8, n=2, T=3)
    w = np.full((3, oc.n_edges), 0.75)
    _, _, app = oc.wms_loss_grad(llr, cw, 3, w, want_grad=False)
    _, a64, _ = oc.minsum_f64(llr.astype(np.float64), 3)
    np.testing.assert_allclose(app, a64, rtol=1e-12, atol=1e-12)


def test_layered_adjoint_matches_finite_differences():
    """The layered weighted min-sum adjoint (rows reversed, per-edge dloss/dR
    carried between iterations) against central differences."""
    oc, llr, cw, w = _case(bg=2, z=6, n=3, T=3, seed=4)
    T = w.shape[0]
    loss, grad, _ = oc.wms_loss_grad(llr, cw, T, w, layered=True)
    rng = np.random.default_rng(2)
    checked = 0
    for _ in range(30):
        t, e = int(rng.integers(T)), int(rng.integers(oc.n_edges))
        fd = []
        for eps in (1e-5, 5e-6):
            wp, wm = w.copy(), w.copy()
            wp[t, e] += eps
            wm[t, e] -= eps
            lp, _, _ = oc.wms_loss_grad(llr, cw, T, wp, want_grad=False, layered=True)
            lm, _, _ = oc.wms_loss_grad(llr, cw, T, wm, want_grad=False, layered=True)
            fd.append((lp - lm) / (2 * eps))
        if abs(fd[0] - fd[1]) > 1e-6 * max(1.0, abs(fd[0])) * 1e3:
            continue
        np.testing.assert_allclose(grad[t, e], fd[0], rtol=2e-4, atol=1e-9)
        checked += 1
    assert checked >= 24
    assert np.abs(grad).max() > 0


def test_layered_loss_posterior_equals_layered_f32_decoder():
    """The f64 layered forward at constant weight 0.75 agrees with the fp32
    layered decoder to fp32 accuracy."""
    oc, llr, cw, _ = _case(bg=1, z=8, n=2, T=3, seed=6)
    w = np.full((3, oc.n_edges), 0.75)
    _, _, app = oc.wms_loss_grad(llr, cw, 3, w, want_grad=False, layered=True)
    _, a32, _ = oc.layered_f32(llr, 3, want_app=True)
    np.testing.assert_allclose(app, a32, rtol=1e-4, atol=1e-4)


def test_layered_f32_forward_matches_layered_decoder():
    """The fp32-forward variant of the layered loss reproduces the fp32
    layered decoder's posterior bit for bit (it is the GPU forward)."""
    oc, llr, cw, w = _case(bg=1, z=8, n=2, T=3, seed=8)
    w32 = w.astype(np.float32)
    _, _, app = oc.wms_loss_grad(llr, cw, 3, w32.astype(np.float64), want_grad=False, layered=True,
                                 f32_forward=True)
    _, a32, _ = oc.layered_f32(llr, 3, w=w32, want_app=True)
    np.testing.assert_array_equal(app.astype(np.float32).view(np.uint32), a32.view(np.uint32))
