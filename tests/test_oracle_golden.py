"""Pin the CPU oracle to the reference's own code through the committed
fixtures (tests/golden/golden.json, made by tests/golden/make_golden.py from
the reference's kernels, setup_ldpc and channel pipeline run on the CPU)."""
import hashlib
import os

import numpy as np
import pytest

from nr_gpu_ldpc_gb300 import codes
from oracle.oracle import OracleCode
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def case_code(case):
    if case["code"] == "nr":
        return codes.base_matrix(case["bg"], codes.set_index(case["z"]))
    return codes.wifi_base()


def regen(case):
    oc = OracleCode(case_code(case), case["z"])
    sig = np.full(case["n_cw"], case["sigma"], np.float32)
    llr, cw = oc.gen_llr(case["kb"], case["seed"], case["cw_base"], sig, case["n_punct_cols"])
    return oc, llr, cw


@pytest.mark.parametrize("idx", range(15))
def test_oracle_matches_reference_kernels(golden, idx):
    case = golden["cases"][idx]
    oc, llr, cw = regen(case)
    assert sha(llr) == case["llr_sha256"], "seeded generator drifted from the fixture"
    assert sha(cw) == case["cw_sha256"]
    if "llr" in case:
        np.testing.assert_array_equal(llr, np.array(case["llr"], np.float32))
    for it, res in case["results"].items():
        packed, app, _ = oc.minsum_f32(llr, int(it), want_app=True)
        assert sha(packed) == res["packed_sha256"], f"{case['name']} I={it}: hard decisions"
        assert sha(app) == res["app_sha256"], f"{case['name']} I={it}: posterior bits"
        errs = np.unpackbits(packed ^ cw, axis=1, bitorder="little")[:, :case["kb"] * case["z"]].sum(1)
        assert errs.tolist() == res["info_bit_errors"]
        if "packed_hex" in res:
            assert [p.tobytes().hex() for p in packed] == res["packed_hex"]
            np.testing.assert_array_equal(app, np.array(res["app"], np.float32))


def test_golden_case_count(golden):
    assert len(golden["cases"]) == 15


def test_oracle_on_reference_channel_pipeline(golden):
    """LLRs made by the reference's OAI encoder + drand48 AWGN (BG1, A=8424)."""
    pipe = golden["ref_pipeline"]
    llr = np.load(os.path.join(GOLDEN, "ref_pipeline_bg1_z384_llr.npy"))
    assert sha(llr) == pipe["llr_sha256"]
    oc = OracleCode(codes.base_matrix(1, 1), 384)
    info = np.frombuffer(bytes.fromhex(pipe["info_packed_hex"]), np.uint8)
    for it, res in pipe["results"].items():
        packed, app, _ = oc.minsum_f32(llr, int(it), want_app=True)
        assert sha(packed) == res["packed_sha256"]
        assert sha(app) == res["app_sha256"]
    # the reference encoder's codeword satisfies every check of the decoder's table
    packed10, _, _ = oc.minsum_f32(llr, 10)
    if np.array_equal(packed10[0][:info.size], info):
        assert oc.syndrome_weight(packed10[0]) == 0


def test_setup_ldpc_mirror(golden):
    for row in golden["setup_ldpc"]:
        p = codes.setup_ldpc(row["A"], row["rate"], 5)
        got = dict(A=p.A, bg_index=p.bg_index, Z=p.Z, K=p.K, N=p.N, H_rows=p.H_rows, H_cols=p.H_cols,
                   n_nz_in_row=p.n_nz_in_row, n_nz_in_col=p.n_nz_in_col, n_iterations=p.n_iterations,
                   N_before_puncture=p.N_before_puncture, H00=int(p.H[0, 0]))
        for k, v in got.items():
            assert v == row[k], (row["A"], row["rate"], k, v, row[k])


def test_fp64_twin_agrees_where_fp32_is_stable():
    """The FP64 transcription gives the same hard decisions at low iteration
    counts and posteriors within 1e-5 relative (floor 1) where no min/sign
    decision flipped."""
    z = 64
    oc = OracleCode(codes.base_matrix(1, codes.set_index(z)), z)
    sig = np.full(4, codes.noise_sigma(2.0, 1 / 3), np.float32)
    llr, _ = oc.gen_llr(22, 5, 0, sig, 2)
    for it in (1, 2, 3):
        p32, a32, _ = oc.minsum_f32(llr, it, want_app=True)
        p64, a64, _ = oc.minsum_f64(llr.astype(np.float64), it)
        rel = np.abs(a32 - a64) / np.maximum(np.abs(a64), 1.0)
        assert np.quantile(rel, 0.999) < 1e-5
        assert (p32 != p64).sum() <= 2


def test_fused_dt_switch_is_off_by_default_and_changes_posteriors(golden):
    """The oracle's fused-dt switch (what a contracting compiler would make of
    the reference's dt line; the reference's own binary was measured not to
    contract it) is off unless asked for: with it on, the posteriors of a
    BG1 Z=384 fixture differ from the reference's from the second iteration,
    and with it off again they match."""
    from oracle import oracle as O
    case = next(c for c in golden["cases"] if c["code"] == "nr" and c["bg"] == 1 and c["z"] == 384
                and "5" in c["results"] and "app_sha256" in c["results"]["5"])
    oc, llr, _ = regen(case)
    want = case["results"]["5"]["app_sha256"]
    try:
        O.set_fma_dt(True)
        _, app_fused, _ = oc.minsum_f32(llr, 5, want_app=True)
    finally:
        O.set_fma_dt(False)
    _, app, _ = oc.minsum_f32(llr, 5, want_app=True)
    assert sha(app) == want
    assert sha(app_fused) != want
