"""Base graphs, lifting sizes and the structural encoder (host side, no GPU)."""
import ctypes as C

import numpy as np
import pytest

from nr_gpu_ldpc_gb300 import codes
from oracle.oracle import OracleCode


def test_edge_counts_and_degrees():
    for bg, edges, rdeg, cdeg in ((1, 316, 19, 30), (2, 197, 10, 23)):
        for ils in range(8):
            h = codes.base_matrix(bg, ils)
            m = h != -1
            assert m.sum() == edges
            assert m.sum(1).max() == rdeg and m.sum(0).max() == cdeg
            kb = codes.KB_MAX[bg]
            # extension rows end in their own degree-1 column with shift 0
            for r in range(4, h.shape[0]):
                c = np.nonzero(m[r])[0][-1]
                assert c == kb + r and m[:, c].sum() == 1 and h[r, c] == 0


def test_lifting_sizes():
    assert len(codes.LIFTING_SIZES) == 51
    assert codes.set_index(384) == 1 and codes.set_index(320) == 2 and codes.set_index(2) == 0
    with pytest.raises(codes.LdpcConfigError):
        codes.set_index(17)


def test_c_library_tables_match_python(cuda_lib):
    out = np.zeros(46 * 68, np.int32)
    rows, cols = C.c_int(), C.c_int()
    for bg in (1, 2):
        for ils in range(8):
            assert cuda_lib.nrldpc_base_matrix(bg, ils, out.ctypes.data_as(C.c_void_p),
                                               C.byref(rows), C.byref(cols)) == 0
            h = out[:rows.value * cols.value].reshape(rows.value, cols.value)
            np.testing.assert_array_equal(h, codes.base_matrix(bg, ils))
    for z, ils in codes.LIFTING_SIZES.items():
        assert cuda_lib.nrldpc_set_index(z) == ils
    assert cuda_lib.nrldpc_set_index(17) == -1


@pytest.mark.parametrize("bg", [1, 2])
def test_encoder_syndrome_all_lifting_sizes(bg):
    rng = np.random.default_rng(bg)
    kb = codes.KB_MAX[bg]
    for z in codes.LIFTING_SIZES:
        oc = OracleCode(codes.base_matrix(bg, codes.set_index(z)), z)
        info = rng.integers(0, 2, kb * z).astype(np.uint8)
        cw = oc.encode(kb, info)
        bits = np.unpackbits(cw, bitorder="little")
        np.testing.assert_array_equal(bits[:kb * z], info)
        assert oc.syndrome_weight(cw) == 0, (bg, z)
        flipped = cw.copy()
        flipped[0] ^= 1
        assert oc.syndrome_weight(flipped) > 0


def test_encoder_wifi_matrix():
    oc = OracleCode(codes.wifi_base(), 96)
    info = np.random.default_rng(3).integers(0, 2, 12 * 96).astype(np.uint8)
    assert oc.syndrome_weight(oc.encode(12, info)) == 0


def test_noise_sigma_matches_formula():
    # sigma = sqrt((1/R) / 10^(EbN0/10) / 2), computed in float32
    for eb in (0.5, 1.0, 2.5):
        want = np.sqrt(np.float32(1 / (1 / 3)) / np.float32(10 ** (eb / 10)) / 2)
        assert abs(codes.noise_sigma(eb, 1 / 3) - want) < 1e-6
