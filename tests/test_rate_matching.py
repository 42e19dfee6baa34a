"""Rate matching / de-rate-matching oracle (TS 38.212 5.4.2.1 bit selection,
5.4.2.2 bit interleaving): the O(1) index maps against literal walks of the
standard's loops, and decode round trips with filler bits fixed by +inf
LLRs."""
import numpy as np
import pytest

from nr_gpu_ldpc_gb300 import codes
from oracle import oracle as O


def standard_walk(z, ncb, k_prime, kb_z, k0, e):
    """The standard's loop: k = 0, j = 0; while k < E: if d[(k0+j) mod Ncb] is
    not NULL: e_k = that bit, k++; j++."""
    null = set(range(k_prime - 2 * z, kb_z - 2 * z))
    out, j = [], 0
    while len(out) < e:
        idx = (k0 + j) % ncb
        if idx not in null:
            out.append(idx)
        j += 1
    return out


@pytest.mark.parametrize("bg,z", [(1, 384), (2, 128), (1, 52), (2, 15)])
def test_index_map_matches_standard_loop(bg, z):
    kb = codes.KB_MAX[bg]
    ncb = (66 if bg == 1 else 50) * z
    rng = np.random.default_rng(z)
    for rv in range(4):
        k0 = O.rm_k0(bg, z, rv)
        assert k0 == [0, 17 if bg == 1 else 13, 33 if bg == 1 else 25, 56 if bg == 1 else 43][rv] * z
        for f in (0, 1, z - 1, 3 * z + 5):
            kp = kb * z - f
            e = int(rng.integers(z, 2 * ncb))
            want = standard_walk(z, ncb, kp, kb * z, k0, e)
            got = [O.rm_index(z, ncb, kb * z, kp, k0, k) for k in range(e)]
            assert got == want, (rv, f, e)


def standard_interleave(e_bits, qm):
    """The standard's loop: for j < E/Qm: for i < Qm: f[i + j*Qm] = e[i*E/Qm + j]."""
    n = len(e_bits)
    f = [None] * n
    for j in range(n // qm):
        for i in range(qm):
            f[i + j * qm] = e_bits[i * (n // qm) + j]
    return f


@pytest.mark.parametrize("qm", [1, 2, 4, 6, 8, 10])
def test_interleaver_matches_standard_loop(qm):
    for e in (qm * 7, qm * 331, qm * 1000):
        want = standard_interleave(list(range(e)), qm)
        got = [O.interleave_src(e, qm, p) for p in range(e)]
        assert got == want
        assert sorted(got) == list(range(e))


def test_modulation_order_is_validated():
    oc = O.OracleCode(codes.base_matrix(2, codes.set_index(64)), 64)
    for qm, e in ((3, 1200), (4, 1202), (12, 1200)):
        with pytest.raises(RuntimeError):
            O.gen_rm_llr(oc, 10, 2, 1, 0, np.full(1, 0.5, np.float32), 640, e, 0, qm)
        with pytest.raises(RuntimeError):
            O.derate_match(oc, 10, 2, np.zeros((1, e), np.float32), 640, e, 0, qm)


def test_interleaving_permutes_the_transmission():
    """Same codeword and noise per position: the qm = 4 transmission carries at
    position p the rate-matched bit that qm = 1 carries at interleave_src(p)."""
    oc = O.OracleCode(codes.base_matrix(1, codes.set_index(64)), 64)
    e = 4 * 800
    l1, c1 = O.gen_rm_llr(oc, 22, 1, 7, 0, np.full(1, 1e-3, np.float32), 0, e, 0, 1)
    l4, c4 = O.gen_rm_llr(oc, 22, 1, 7, 0, np.full(1, 1e-3, np.float32), 0, e, 0, 4)
    np.testing.assert_array_equal(c1, c4)
    src = np.array([O.interleave_src(e, 4, p) for p in range(e)])
    np.testing.assert_array_equal(np.sign(l4[0]), np.sign(l1[0][src]))
    assert not np.array_equal(np.sign(l4[0]), np.sign(l1[0]))


@pytest.mark.parametrize("bg,z,rate,qm", [(1, 384, 0.5, 1), (2, 128, 0.33, 2), (1, 64, 0.8, 8), (2, 96, 0.2, 6),
                                          (1, 96, 0.6, 4), (2, 64, 0.4, 10)])
def test_rate_matched_round_trip(bg, z, rate, qm):
    kb = codes.KB_MAX[bg]
    oc = O.OracleCode(codes.base_matrix(bg, codes.set_index(z)), z)
    n = 6
    kp = kb * z - 37  # 37 filler bits
    ncb = oc.n_bp - 2 * z
    # rv 0 at the target rate; rv 1..3 (retransmission versions, which skip
    # systematic columns) with E covering the whole buffer once or more; E a
    # whole number of modulation symbols
    e = np.array([round(kp / rate)] * 2 + [ncb - 37, ncb - 37 + 500, 2 * ncb, ncb], np.int32)
    e = (e + qm - 1) // qm * qm
    rv = np.array([0, 0, 1, 2, 3, 3], np.int32)
    llr_e, cw = O.gen_rm_llr(oc, kb, bg, 42, 0, np.full(n, 0.3, np.float32), kp, e, rv, qm)
    mother = O.derate_match(oc, kb, bg, llr_e, kp, e, rv, qm)
    assert np.isinf(mother[:, kp:kb * z]).all() and (mother[:, kp:kb * z] > 0).all()
    assert (mother[:, :2 * z] == 0).all()
    bits = np.unpackbits(cw, axis=1, bitorder="little")[:, :oc.n_bp]
    assert (bits[:, kp:kb * z] == 0).all()
    sent = mother != 0
    sent[:, kp:kb * z] = False
    assert ((mother < 0) == bits.astype(bool))[sent].mean() > 0.999  # sigma 0.3: clean channel
    packed, _, _ = oc.minsum_f32(mother, 20)
    got = np.unpackbits(packed, axis=1, bitorder="little")[:, :kp]
    np.testing.assert_array_equal(got, bits[:, :kp])
