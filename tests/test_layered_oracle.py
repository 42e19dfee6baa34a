"""The oracle's layered decoder (CPU): consistency properties that pin it
without a reference counterpart (the reference decodes flooding only)."""
import numpy as np

from nr_gpu_ldpc_gb300 import codes
from oracle.oracle import OracleCode


def _code(bg, z):
    return OracleCode(codes.base_matrix(bg, codes.set_index(z)), z)


def test_constant_weights_equal_alpha():
    oc = _code(1, 32)
    sig = np.full(6, codes.noise_sigma(1.0, 22 / 66), np.float32)
    llr, _ = oc.gen_llr(22, 3, 0, sig, 2)
    w = np.full((3, len(oc.base[oc.base >= 0])), 0.75, np.float32)
    a = oc.layered_f32(llr, 6, alpha=0.75, want_app=True)
    b = oc.layered_f32(llr, 6, w=w, want_app=True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


def test_noiseless_codeword_stops_after_one_iteration():
    oc = _code(2, 24)
    sig = np.full(4, 0.3, np.float32)
    llr, cw = oc.gen_llr(10, 8, 0, sig, 2)
    pk, _, it = oc.layered_f32(llr, 10, early_stop=True)
    np.testing.assert_array_equal(pk, cw)
    assert (it == 1).all()
    for row in pk:
        assert oc.syndrome_weight(row) == 0


def test_one_iteration_first_row_equals_flooding_message():
    """Iteration 1 of row 0 sees only channel LLRs in both schedules, so a
    code with a single check row decodes identically."""
    base = np.array([[0, 1, 2, 3]], np.int32)
    oc = OracleCode(base, 4)
    llr = np.random.default_rng(1).normal(0.4, 1.0, (5, 16)).astype(np.float32)
    a = oc.minsum_f32(llr, 1, want_app=True)
    b = oc.layered_f32(llr, 1, want_app=True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_allclose(a[1], b[1], rtol=1e-6, atol=1e-6)


def test_layered_needs_fewer_iterations():
    oc = _code(1, 64)
    sig = np.full(40, codes.noise_sigma(1.8, 22 / 66), np.float32)
    llr, cw = oc.gen_llr(22, 21, 0, sig, 2)
    _, _, itf = oc.minsum_f32(llr, 25, early_stop=True)
    pk, _, itl = oc.layered_f32(llr, 25, early_stop=True)
    assert itl.mean() < 0.75 * itf.mean()
    assert (np.unpackbits(pk ^ cw, axis=1, bitorder="little")[:, :22 * 64].any(1)).sum() <= 1
