"""Mixed-code batches on the GPU: rate-matched generation, de-rate-matching and
one-launch decoding of uneven (BG, Z, E, filler) mixes, each job checked
against the CPU oracle bit for bit."""
import numpy as np
import pytest
import torch

from nr_gpu_ldpc_gb300 import Decoder, _lib, codes
from nr_gpu_ldpc_gb300.batch import Batch, make_jobs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ZS = (64, 96, 128, 192, 256, 320, 384)


def _mix(n, seed, zs=ZS, small=False, qms=(1,)):
    rng = np.random.default_rng(seed)
    bg = rng.integers(1, 3, n)
    z = rng.choice(zs, n)
    kb = np.where(bg == 1, 22, 10)
    filler = rng.integers(0, 40, n)
    kp = kb * z - filler
    rate = rng.uniform(0.25, 0.8, n) if not small else rng.uniform(0.3, 0.6, n)
    e = np.maximum((kp / rate).astype(np.int64), 2 * z + 8)
    rv = rng.choice([0, 0, 0, 1, 2, 3], n)
    ncb = np.where(bg == 1, 66, 50) * z
    e = np.where(rv > 0, np.maximum(e, ncb), e)  # retransmission versions: cover the buffer
    qm = rng.choice(qms, n)
    e = (e + qm - 1) // qm * qm  # a whole number of modulation symbols
    eb = rng.uniform(1.0, 3.0, n)
    rate_eff = kp / e
    sigma = np.sqrt((1.0 / rate_eff) / (2.0 * 10 ** (eb / 10))).astype(np.float32)
    return make_jobs(bg, z, kp, e, rv, sigma, qm)


def _oracle(bg, z):
    return O.OracleCode(codes.base_matrix(bg, codes.set_index(z)), z)


def test_generate_derate_decode_against_oracle(gpu):
    """Every job bit-exact with the oracle through generation (rate matching,
    bit interleaving for modulation orders 1-10, channel), de-rate-matching
    and decoding."""
    jobs, n_llr, n_e, n_out = _mix(30, 3, qms=(1, 2, 4, 6, 8, 10))
    assert len(set(jobs["qm"].tolist())) == 6
    b = Batch(max_jobs=64)
    b.set_jobs(jobs)
    llr_e = torch.zeros(n_e, device=gpu)
    cw = torch.zeros(n_out, dtype=torch.uint8, device=gpu)
    b.gen(99, 5000, llr_e, cw)
    llr = torch.full((n_llr,), 7.0, device=gpu)
    b.derate(llr_e, llr)
    packed = torch.zeros(n_out, dtype=torch.uint8, device=gpu)
    iters = torch.zeros(len(jobs), dtype=torch.int32, device=gpu)
    b.decode(llr, packed, 10, early_stop=True, iters=iters)
    torch.cuda.synchronize()
    h_e, h_cw, h_llr = llr_e.cpu().numpy(), cw.cpu().numpy(), llr.cpu().numpy()
    h_pk, h_it = packed.cpu().numpy(), iters.cpu().numpy()
    for i, j in enumerate(jobs):
        bg, z = int(j["bg"]), int(j["z"])
        oc = _oracle(bg, z)
        kb = codes.KB_MAX[bg]
        e = int(j["e"])
        qm = int(j["qm"])
        le, c = O.gen_rm_llr(oc, kb, bg, 99, 5000 + i, j["sigma"], int(j["k_prime"]), e, int(j["rv"]), qm)
        np.testing.assert_array_equal(h_e[j["e_offset"]:j["e_offset"] + e].view(np.uint32), le[0].view(np.uint32))
        np.testing.assert_array_equal(h_cw[j["out_offset"]:j["out_offset"] + oc.n_bytes], c[0])
        m = O.derate_match(oc, kb, bg, le, int(j["k_prime"]), e, int(j["rv"]), qm)
        got = h_llr[j["llr_offset"]:j["llr_offset"] + oc.n_bp]
        np.testing.assert_array_equal(got.view(np.uint32), m[0].view(np.uint32))
        pk, _, it = oc.minsum_f32(m, 10, early_stop=True)
        np.testing.assert_array_equal(h_pk[j["out_offset"]:j["out_offset"] + oc.n_bytes], pk[0])
        assert h_it[i] == it[0]


def test_modulation_order_validation(gpu):
    b = Batch(max_jobs=4)
    ok, *_ = make_jobs([1], 64, e=3000, qm=4)
    b.set_jobs(ok)
    for qm, e in ((3, 3000), (4, 3002), (12, 3000), (-2, 3000)):
        bad, *_ = make_jobs([1], 64, e=e, qm=qm)
        with pytest.raises(_lib.NrLdpcError):
            b.set_jobs(bad)


def test_mixed_batch_equals_per_code_decoders(gpu):
    """One launch over a mixed list gives what each code's own handle gives;
    the graph is replayed with new buffers on the second call."""
    jobs, n_llr, _, n_out = make_jobs(np.array([1, 2, 1, 2, 1, 2] * 5), np.array([384, 128, 64, 96, 320, 384] * 5))
    b = Batch(max_jobs=64)
    b.set_jobs(jobs)
    g = torch.Generator(device=gpu).manual_seed(4)
    for call in range(2):
        llr = torch.randn(n_llr, device=gpu, generator=g) * 3 + 1
        packed = torch.zeros(n_out, dtype=torch.uint8, device=gpu)
        b.decode(llr, packed, 6)
        torch.cuda.synchronize()
        for (bg, z) in {(int(j["bg"]), int(j["z"])) for j in jobs}:
            sel = [i for i, j in enumerate(jobs) if j["bg"] == bg and j["z"] == z]
            dec = Decoder(bg=bg, z=z, max_batch=len(sel))
            x = torch.stack([llr[jobs[i]["llr_offset"]:jobs[i]["llr_offset"] + dec.n_bp] for i in sel])
            want = dec.decode(x.contiguous(), 6)
            torch.cuda.synchronize()
            for k, i in enumerate(sel):
                o = int(jobs[i]["out_offset"])
                assert torch.equal(packed[o:o + dec.packed_bytes], want[k]), (call, bg, z)


def test_codewords_per_cta_does_not_change_results(gpu):
    jobs, n_llr, _, n_out = make_jobs(np.full(40, 2), 64)
    llr = torch.randn(n_llr, device=gpu) * 2 + 1.5
    outs = []
    for cpb in (1, 2, 6):
        b = Batch(max_jobs=64)
        b.set_cw_per_cta(2, 64, cpb)
        assert b.get_cw_per_cta(2, 64) == cpb
        b.set_jobs(jobs)
        p = torch.zeros(n_out, dtype=torch.uint8, device=gpu)
        b.decode(llr, p, 8, early_stop=True)
        outs.append(p)
    torch.cuda.synchronize()
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], outs[2])


@pytest.mark.parametrize("bg,z", [(1, 256), (2, 320), (2, 96), (1, 64)])
def test_sub_rows_per_thread_do_not_change_results(gpu, bg, z):
    """Threads per codeword Z (one sub-row each) or Z/2 (two each), at
    several codewords per CTA, early stop off and on: the same bits and
    iteration counts, on warp-aligned (Z/2 a multiple of 32) and unaligned
    (Z/2 = 48) slots."""
    jobs, n_llr, _, n_out = make_jobs(np.full(150, bg), z)
    b = Batch(max_jobs=150)
    llr = torch.randn(n_llr, device=gpu, generator=torch.Generator(device=gpu).manual_seed(z)) * 2.5 + 1.2
    ref = None
    for spt in (1, 2):
        b.set_sub_rows_per_thread(bg, z, spt)
        b.set_cw_per_cta(bg, z, 0)
        top = b.get_cw_per_cta(bg, z)
        for cpb in sorted({1, top}):
            b.set_cw_per_cta(bg, z, cpb)
            assert b.get_sub_rows_per_thread(bg, z) == spt and b.get_cw_per_cta(bg, z) == cpb
            b.set_jobs(jobs)
            got = []
            for early in (False, True):
                p = torch.zeros(n_out, dtype=torch.uint8, device=gpu)
                it = torch.zeros(len(jobs), dtype=torch.int32, device=gpu)
                b.decode(llr, p, 8, early_stop=early, iters=it)
                got += [p, it]
            torch.cuda.synchronize()
            if ref is None:
                ref = got
            for a, c in zip(ref, got):
                assert torch.equal(a, c), (spt, cpb)
    b.close()


def test_sub_rows_per_thread_in_a_mixed_batch(gpu):
    """Two sub-rows per thread for some codes of a mixed list (the CTA then
    has the threads of its widest work item): every job equals its code's
    own handle."""
    jobs, n_llr, _, n_out = make_jobs(np.array([1, 2, 1, 2, 1, 2] * 4), np.array([256, 128, 320, 96, 384, 256] * 4))
    b = Batch(max_jobs=64)
    for bg, z in ((1, 256), (2, 96), (1, 320)):
        b.set_sub_rows_per_thread(bg, z, 2)
    with pytest.raises(_lib.NrLdpcError):
        b.set_sub_rows_per_thread(1, 13, 2)  # odd Z has no half
    b.set_jobs(jobs)
    llr = torch.randn(n_llr, device=gpu, generator=torch.Generator(device=gpu).manual_seed(8)) * 3 + 1
    packed = torch.zeros(n_out, dtype=torch.uint8, device=gpu)
    b.decode(llr, packed, 6, early_stop=True)
    torch.cuda.synchronize()
    for (bg, z) in {(int(j["bg"]), int(j["z"])) for j in jobs}:
        sel = [i for i, j in enumerate(jobs) if j["bg"] == bg and j["z"] == z]
        dec = Decoder(bg=bg, z=z, max_batch=len(sel))
        x = torch.stack([llr[jobs[i]["llr_offset"]:jobs[i]["llr_offset"] + dec.n_bp] for i in sel])
        want = dec.decode(x.contiguous(), 6, early_stop=True)
        torch.cuda.synchronize()
        for k, i in enumerate(sel):
            o = int(jobs[i]["out_offset"])
            assert torch.equal(packed[o:o + dec.packed_bytes], want[k]), (bg, z)
    b.close()


def test_autotuner_picks_an_admissible_point(gpu):
    """Each code alone: the tuner times every admissible (sub-rows per
    thread, codewords per CTA) and returns the fastest of them."""
    from nr_gpu_ldpc_gb300.autotune import tune
    res = tune(zs=(96,), bgs=(2,), reps=1, waves=1, verbose=False)
    (e,) = res["entries"]
    tried = {(t["sub_rows_per_thread"], t["cw_per_cta"]) for t in e["tried"]}
    assert {1, 2} <= {spt for spt, _ in tried}
    assert (e["sub_rows_per_thread"], e["cw_per_cta"]) in tried
    assert all(cpb * (96 // spt) <= 384 for spt, cpb in tried)
    assert e["us_per_cw"] == min(t["us_per_cw"] for t in e["tried"])


def test_workload_tuner_keeps_a_tried_point_per_code(gpu):
    """On a job list: every code present gets a point it was timed at, and
    the tuned batch is no slower than the default one by more than timing
    noise."""
    from nr_gpu_ldpc_gb300.autotune import tune_workload
    bg = np.array([1, 2] * 60)
    z = np.array([64, 128, 256, 96] * 30)
    kp = np.where(bg == 1, 22, 10) * z
    e = (kp * 2.5).astype(np.int64)
    sigma = np.full(len(bg), 0.8, np.float32)
    res = tune_workload(bg, z, kp, e, sigma, n_iter=4, reps=1, verbose=False)
    assert {(x["bg"], x["z"]) for x in res["entries"]} == {(int(a), int(c)) for a, c in zip(bg, z)}
    for x in res["entries"]:
        assert (x["sub_rows_per_thread"], x["cw_per_cta"]) in {(t["sub_rows_per_thread"], t["cw_per_cta"])
                                                              for t in x["tried"]} | {(1, 0)}
    assert res["batch_ms_tuned"] <= res["batch_ms_default"]


def test_uneven_8192_codeword_mix(gpu):
    """The mixed workload at full size: 8192 codewords, BG1/BG2, Z from
    {64..384}, rate matching with filler, Eb/N0 1-3 dB, early stop, 10
    iterations: the error counter agrees with a host count, every frame whose
    decoder stopped early decoded correctly, and a sample matches the oracle."""
    jobs, n_llr, n_e, n_out = _mix(8192, 11)
    b = Batch(max_jobs=8192)
    b.set_jobs(jobs)
    llr_e = torch.empty(n_e, device=gpu)
    cw = torch.empty(n_out, dtype=torch.uint8, device=gpu)
    b.gen(5, 0, llr_e, cw)
    llr = torch.empty(n_llr, device=gpu)
    b.derate(llr_e, llr)
    packed = torch.empty(n_out, dtype=torch.uint8, device=gpu)
    iters = torch.empty(8192, dtype=torch.int32, device=gpu)
    b.decode(llr, packed, 10, early_stop=True, iters=iters)
    counts = b.count_errors(packed, cw)
    torch.cuda.synchronize()
    h_llr, h_pk, h_it, h_cw = llr.cpu().numpy(), packed.cpu().numpy(), iters.cpu().numpy(), cw.cpu().numpy()
    frame_err = np.zeros(8192, bool)
    for i, j in enumerate(jobs):
        o, kp = int(j["out_offset"]), int(j["k_prime"])
        d = np.unpackbits(h_pk[o:o + (kp + 7) // 8] ^ h_cw[o:o + (kp + 7) // 8], bitorder="little")[:kp]
        frame_err[i] = d.any()
    assert int(counts[1]) == frame_err.sum()
    assert not frame_err[h_it < 10].any()  # stopped early => satisfied every check => decoded
    assert (h_it < 10).sum() > 8192 // 4
    for i in np.random.default_rng(0).choice(8192, 12, replace=False):
        j = jobs[i]
        oc = _oracle(int(j["bg"]), int(j["z"]))
        m = h_llr[j["llr_offset"]:j["llr_offset"] + oc.n_bp]
        pk, _, it = oc.minsum_f32(m, 10, early_stop=True)
        np.testing.assert_array_equal(h_pk[j["out_offset"]:j["out_offset"] + oc.n_bytes], pk[0])
        assert h_it[i] == it[0]


def test_crc_kernel_matches_oracle(gpu):
    import ctypes as C
    from nr_gpu_ldpc_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(1)
    for ctype, poly in enumerate((O.CRC24A, O.CRC24B, O.CRC16)):
        for n_bits in (8, 13, 1000, 8448):
            stride = (n_bits + 7) // 8 + 3
            data = rng.integers(0, 256, (37, stride), dtype=np.uint8)
            d = torch.from_numpy(data).to(gpu)
            rem = torch.empty(37, dtype=torch.int32, device=gpu)
            assert lib.nrldpc_crc(C.c_void_p(d.data_ptr()), 37, stride, n_bits, ctype,
                                  C.c_void_p(rem.data_ptr()),
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
            torch.cuda.synchronize()
            want = [O.crc(data[i], n_bits, poly) for i in range(37)]
            assert (rem.cpu().numpy().astype(np.uint32) == np.array(want, np.uint32)).all()
