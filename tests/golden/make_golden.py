"""Generate the golden fixtures from the reference's own code.

Runs only where the reference tree is present (it needs oracle/_ref, built by
``make -C oracle REF=<reference tree>``; the tree is taken from the first
argument or NRLDPC_REF_ROOT, else the Makefile's default).  Every expected value below comes from
the reference's source executed on the CPU:

* decode results: src/ldpc_kernels.cu kernels replayed in the launch order of
  src/gpu_decoder_top.cu:25-49 (oracle/ref_harness.cpp);
* ``setup_ldpc`` fields: src/nr_ldpc.cpp:31-230;
* the reference channel pipeline: src/encoding_tools.cpp transmit/calculate_llr
  with the vendored OAI encoder (src/nr_ldpc.cpp:655-913).

Inputs for the decode cases are drawn with the project's seeded generator
(Philox4x32-10 + Box-Muller, reproduced by the oracle and the GPU); each case
records the SHA-256 of its LLR bytes so a test can prove it regenerated the
same input.  Large outputs are stored as SHA-256 of the packed hard decisions
and of the fp32 posterior bytes; small cases store them in full.

Usage: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
from nr_gpu_ldpc_gb300 import codes  # noqa: E402
from oracle.oracle import OracleCode, RefEmu, build  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def hd_from_app(app: np.ndarray) -> np.ndarray:
    """Reference hard decision (ldpc_kernels.cu:463-467): APP > 0 -> 0 else 1,
    packed LSB-first per codeword."""
    hd = (~(app > 0)).astype(np.uint8)
    return np.packbits(hd, axis=1, bitorder="little")


def decode_case(name, code_kind, bg, z, ebn0, n_cw, iters_list, seed, full=False):
    if code_kind == "nr":
        base = codes.base_matrix(bg, codes.set_index(z))
        kb, punct = codes.KB_MAX[bg], 2
        rows, cols = base.shape
        rate = kb / (cols - 2)
    else:
        base = codes.wifi_base()
        kb, punct = codes.WIFI_KB, 0
        rate = 0.5
    oc = OracleCode(base, z)
    sigma = codes.noise_sigma(ebn0, rate)
    llr, cw = oc.gen_llr(kb, seed, 0, np.full(n_cw, sigma, np.float32), punct)
    ref = RefEmu(base, z)
    case = dict(name=name, code=code_kind, bg=bg, z=z, ebn0_db=ebn0, rate_for_sigma=rate,
                sigma=sigma, seed=seed, cw_base=0, n_cw=n_cw, kb=kb, n_punct_cols=punct,
                llr_sha256=sha(llr), cw_sha256=sha(cw), results={})
    if full:
        case["llr"] = llr.tolist()
    for it in iters_list:
        packed, app = ref.decode(llr, it, want_app=True)
        if z % 8:
            packed = hd_from_app(app)  # the reference pack kernel needs Z % 8 == 0
        else:
            assert np.array_equal(packed, hd_from_app(app))
        n_info = kb * z
        bits = np.unpackbits(packed ^ cw, axis=1, bitorder="little")[:, :n_info]
        res = dict(packed_sha256=sha(packed), app_sha256=sha(app),
                   info_bit_errors=bits.sum(1).tolist())
        if full:
            res["packed_hex"] = [p.tobytes().hex() for p in packed]
            res["app"] = app.tolist()
        case["results"][str(it)] = res
    print(name, {k: v["info_bit_errors"] for k, v in case["results"].items()})
    return case


def main():
    build((sys.argv[1] if len(sys.argv) > 1 else None) or os.environ.get("NRLDPC_REF_ROOT") or None)
    for kind in ("bg1", "bg2", "wifi"):
        if not RefEmu.available(kind):
            raise SystemExit("oracle/_ref missing: the reference tree is required")
    cases = []
    # the reference's own configuration: BG1, Z = 384 (src/main.cpp:62-69)
    for eb, seed in ((1.0, 101), (1.75, 102), (2.5, 103)):
        cases.append(decode_case(f"bg1_z384_eb{eb}", "nr", 1, 384, eb, 4, [1, 2, 5, 10], seed))
    cases.append(decode_case("bg2_z128_eb2.0", "nr", 2, 128, 2.0, 4, [1, 2, 5, 8, 10], 201))
    cases.append(decode_case("bg2_z384_eb1.5", "nr", 2, 384, 1.5, 2, [3, 10], 202))
    cases.append(decode_case("bg1_z64_eb2.0", "nr", 1, 64, 2.0, 4, [2, 10], 203))
    cases.append(decode_case("bg1_z320_eb2.0", "nr", 1, 320, 2.0, 2, [4, 10], 204))
    cases.append(decode_case("bg2_z96_eb3.0", "nr", 2, 96, 3.0, 4, [5, 10], 205))
    cases.append(decode_case("bg1_z208_eb1.5", "nr", 1, 208, 1.5, 2, [10], 206))
    cases.append(decode_case("bg2_z36_eb2.5", "nr", 2, 36, 2.5, 4, [6], 207))
    cases.append(decode_case("wifi_z96_eb2.0", "wifi", 0, 96, 2.0, 4, [5], 301))
    cases.append(decode_case("wifi_z96_eb4.0", "wifi", 0, 96, 4.0, 4, [5], 302))
    # small cases stored in full (readable)
    cases.append(decode_case("bg1_z2_eb1.0", "nr", 1, 2, 1.0, 2, [1, 3], 401, full=True))
    cases.append(decode_case("bg2_z3_eb0.5", "nr", 2, 3, 0.5, 2, [2, 4], 402, full=True))
    cases.append(decode_case("bg2_z8_eb2.0", "nr", 2, 8, 2.0, 2, [1, 5], 403, full=True))

    # setup_ldpc over a sweep of payload sizes and rates
    ref1 = RefEmu(codes.base_matrix(1, 1), 384)
    setup = []
    for A in (24, 100, 292, 293, 500, 1000, 2000, 3000, 3824, 3825, 4000, 6000, 8000, 8424):
        for rate in (0.2, 1 / 3, 0.5, 2 / 3, 0.75, 0.9):
            try:
                codes.setup_ldpc(A, rate, 5)
            except codes.LdpcConfigError:
                continue  # no lifting size: the reference reads an uninitialized iLS here
            row = ref1.setup_ldpc(A, rate, 5)
            row["rate"] = rate
            setup.append(row)

    # the reference channel pipeline (OAI encoder, drand48 AWGN), BG1 A=8424
    llr, info = ref1.transmit_llr(8424, 1 / 3, 1, 1.5, 69012, 8448, 26112)
    np.save(os.path.join(OUT, "ref_pipeline_bg1_z384_llr.npy"), llr.astype(np.float32))
    ref1 = RefEmu(codes.base_matrix(1, 1), 384)
    pipe = dict(A=8424, rate=1 / 3, ebn0_db=1.5, srand_seed=69012, n_cw=1,
                info_packed_hex=np.packbits(info.astype(np.uint8), axis=1,
                                            bitorder="little")[0].tobytes().hex(),
                llr_sha256=sha(llr), results={})
    for it in (5, 10):
        packed, app = ref1.decode(llr, it, want_app=True)
        pipe["results"][str(it)] = dict(packed_sha256=sha(packed), app_sha256=sha(app))

    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(dict(cases=cases, setup_ldpc=setup, ref_pipeline=pipe), f)
    print("wrote", len(cases), "decode cases,", len(setup), "setup_ldpc rows")


if __name__ == "__main__":
    main()
