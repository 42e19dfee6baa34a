"""The project's channel (Philox info bits, structural encoder, Box-Muller
AWGN) against the reference's own pipeline (rand() info bits, OAI encoder,
drand48 Marsaglia AWGN: src/encoding_tools.cpp:13-99, src/nr_ldpc.cpp:655-913)
run on the CPU from oracle/_ref.  Same decoder, same Eb/N0 -> frame error
rates agree within 95% binomial confidence.  Needs the reference tree (skips
where oracle/_ref was not built)."""
import numpy as np
import pytest

from nr_gpu_ldpc_gb300 import codes
from nr_gpu_ldpc_gb300.evaluate import clopper_pearson
from oracle.oracle import OracleCode, RefEmu


@pytest.mark.skipif(not RefEmu.available("bg1"), reason="oracle/_ref needs the reference tree")
@pytest.mark.parametrize("ebn0", [1.5, 1.6, 1.7])
def test_fer_matches_reference_channel_pipeline(ebn0):
    """One point of the FER curve per Eb/N0 in the waterfall."""
    n, it = 240, 10
    H = codes.base_matrix(1, 1)
    oc = OracleCode(H, 384)
    ref = RefEmu(H, 384)
    llr_r, info_r = ref.transmit_llr(8424, 1 / 3, n, ebn0, 69012 + int(ebn0 * 100), 8448, 26112)
    pk, _, _ = oc.minsum_f32(llr_r, it, threads=8)
    bits = np.unpackbits(pk, axis=1, bitorder="little")[:, :8448]
    fe_ref = int((bits != info_r).any(axis=1).sum())
    sig = np.full(n, codes.noise_sigma(ebn0, 1 / 3), np.float32)
    llr_o, cw = oc.gen_llr(22, 777 + int(ebn0 * 100), 0, sig, 2)
    pk, _, _ = oc.minsum_f32(llr_o, it, threads=8)
    fe_own = int((np.unpackbits(pk ^ cw, axis=1, bitorder="little")[:, :8448]).any(axis=1).sum())
    lo_r, hi_r = clopper_pearson(fe_ref, n)
    lo_o, hi_o = clopper_pearson(fe_own, n)
    assert 0 < fe_ref < n and 0 < fe_own < n, (fe_ref, fe_own)  # in the waterfall
    assert lo_r <= fe_own / n <= hi_r or lo_o <= fe_ref / n <= hi_o, (fe_ref, fe_own)
    # the per-bit LLR statistics agree too: mean and spread of the sent LLRs
    sent_r = np.abs(llr_r[:, 768:])
    sent_o = np.abs(llr_o[:, 768:])
    assert abs(sent_r.mean() - sent_o.mean()) < 0.02 * sent_r.mean()
    assert abs(sent_r.std() - sent_o.std()) < 0.02 * sent_r.std()
