"""GPU decode parity through the C-ABI: golden fixtures made from the
reference's own kernels, the oracle on seeded and adversarial inputs, and
size-independent properties at the full 4096-codeword BG1 Z=384 batch."""
import ctypes as C
import hashlib
import os

import numpy as np
import pytest
import torch

from nr_gpu_ldpc_gb300 import Decoder, _lib, codes
from oracle.oracle import OracleCode

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_decoder(case_or_bg, z=None, max_batch=64, **kw):
    if isinstance(case_or_bg, dict):
        case = case_or_bg
        if case["code"] == "wifi":
            return Decoder(z=case["z"], base=codes.wifi_base(), max_batch=max_batch, **kw)
        return Decoder(bg=case["bg"], z=case["z"], max_batch=max_batch, **kw)
    return Decoder(bg=case_or_bg, z=z, max_batch=max_batch, **kw)


def bits_nan_canonical(a: np.ndarray) -> np.ndarray:
    """fp32 bit patterns with every NaN mapped to one pattern (IEEE 754
    leaves NaN payloads unspecified: the GPU returns 0x7fffffff, x86 0x7fc00000)."""
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


def oracle_for(dec: Decoder):
    base = codes.wifi_base() if dec.cols == 24 else codes.base_matrix(dec.bg, codes.set_index(dec.z))
    return OracleCode(base, dec.z)


@pytest.mark.parametrize("idx", range(15))
def test_golden_fixture(golden, gpu, idx):
    """Hard decisions and posterior bits equal the reference kernels'."""
    case = golden["cases"][idx]
    dec = make_decoder(case)
    oc = oracle_for(dec)
    sig = np.full(case["n_cw"], case["sigma"], np.float32)
    llr, cw = oc.gen_llr(case["kb"], case["seed"], case["cw_base"], sig, case["n_punct_cols"])
    assert sha(llr) == case["llr_sha256"]
    d_llr = torch.from_numpy(llr).to(gpu)
    for it, res in case["results"].items():
        packed, app = dec.decode(d_llr, int(it), want_app=True)
        torch.cuda.synchronize()
        assert sha(packed.cpu().numpy()) == res["packed_sha256"], f"{case['name']} I={it}"
        assert sha(app.cpu().numpy()) == res["app_sha256"], f"{case['name']} I={it} posterior"
    assert dec.device_error() == 0


def test_reference_channel_pipeline_fixture(golden, gpu):
    """LLRs from the reference's own OAI encoder + drand48 AWGN pipeline."""
    pipe = golden["ref_pipeline"]
    llr = np.load(os.path.join(GOLDEN, "ref_pipeline_bg1_z384_llr.npy"))
    dec = Decoder(bg=1, z=384, max_batch=4)
    for it, res in pipe["results"].items():
        packed, app = dec.decode(torch.from_numpy(llr).to(gpu), int(it), want_app=True)
        torch.cuda.synchronize()
        assert sha(packed.cpu().numpy()) == res["packed_sha256"]
        assert sha(app.cpu().numpy()) == res["app_sha256"]


@pytest.mark.parametrize("bg,z", [(1, 384), (2, 128), (1, 96), (2, 7), (1, 15), (2, 384), (1, 2)])
def test_generator_bit_identical_to_oracle(gpu, bg, z):
    dec = make_decoder(bg, z, max_batch=16)
    oc = oracle_for(dec)
    sig = np.linspace(0.6, 1.3, 9).astype(np.float32)
    llr, cw = oc.gen_llr(dec.kb, 1234567, 99, sig, 2)
    g_llr, g_cw = dec.gen_llr(1234567, 99, torch.from_numpy(sig).to(gpu), 2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(g_llr.cpu().numpy().view(np.uint32), llr.view(np.uint32))
    np.testing.assert_array_equal(g_cw.cpu().numpy(), cw)
    for i in range(cw.shape[0]):
        assert oc.syndrome_weight(cw[i]) == 0


@pytest.mark.parametrize("bg,z,cpb", [(1, 384, 0), (2, 128, 0), (1, 64, 0), (1, 64, 1), (1, 64, 4),
                                      (2, 3, 0), (2, 52, 0), (1, 176, 0), (2, 240, 0)])
def test_random_and_adversarial_llrs(gpu, bg, z, cpb):
    """Heavy-tailed LLRs with exact zeros, -0.0, +-inf, NaN and magnitudes
    above the 1000.0 two-min start value."""
    dec = make_decoder(bg, z, max_batch=32, cw_per_cta=cpb)
    oc = oracle_for(dec)
    rng = np.random.default_rng(z * 10 + bg)
    n = 11
    llr = (rng.standard_t(3, size=(n, dec.n_bp)) * 3 + 0.8).astype(np.float32)
    llr[:, :2 * z] = 0.0
    m = rng.random(llr.shape)
    llr[m < 0.002] = -0.0
    llr[(m > 0.002) & (m < 0.003)] = np.inf
    llr[(m > 0.003) & (m < 0.0035)] = -np.inf
    llr[(m > 0.0035) & (m < 0.004)] = np.nan
    llr[(m > 0.004) & (m < 0.01)] *= 5000.0
    d = torch.from_numpy(llr).to(gpu)
    for it in (1, 3, 7):
        pk, app = dec.decode(d, it, want_app=True)
        torch.cuda.synchronize()
        opk, oapp, _ = oc.minsum_f32(llr, it, want_app=True)
        np.testing.assert_array_equal(pk.cpu().numpy(), opk)
        np.testing.assert_array_equal(bits_nan_canonical(app.cpu().numpy()), bits_nan_canonical(oapp))


@pytest.mark.parametrize("bg,z,ebn0", [(1, 384, 2.0), (2, 128, 2.0), (1, 64, 2.5), (2, 20, 3.0)])
def test_early_stop_parity(gpu, bg, z, ebn0):
    dec = make_decoder(bg, z, max_batch=64)
    oc = oracle_for(dec)
    rate = dec.kb / (dec.cols - 2)
    sig = np.full(24, codes.noise_sigma(ebn0, rate), np.float32)
    llr, cw = oc.gen_llr(dec.kb, 77, 0, sig, 2)
    pk, app, its = dec.decode(torch.from_numpy(llr).to(gpu), 12, early_stop=True, want_app=True,
                              want_iters=True)
    torch.cuda.synchronize()
    opk, oapp, oits = oc.minsum_f32(llr, 12, early_stop=True, want_app=True)
    np.testing.assert_array_equal(its.cpu().numpy(), oits)
    np.testing.assert_array_equal(pk.cpu().numpy(), opk)
    np.testing.assert_array_equal(app.cpu().numpy().view(np.uint32), oapp.view(np.uint32))
    assert (oits < 12).any()
    for i in np.nonzero(oits < 12)[0]:
        assert oc.syndrome_weight(opk[i]) == 0


def test_host_buffer_call_matches_device_call(gpu):
    dec = Decoder(bg=1, z=384, max_batch=40)
    sig = torch.full((40,), codes.noise_sigma(1.75, 1 / 3), device=gpu)
    llr, _ = dec.gen_llr(5, 0, sig)
    ref = dec.decode(llr, 10)
    h_llr = llr.cpu().pin_memory()
    h_out = torch.empty((40, dec.packed_bytes), dtype=torch.uint8).pin_memory()
    s = torch.cuda.Stream()
    dec.decode_host(h_llr, h_out, 10, stream=s)
    s.synchronize()
    assert torch.equal(h_out, ref.cpu())


def test_errors_and_empty_batch(gpu):
    dec = Decoder(bg=2, z=64, max_batch=8)
    llr = torch.zeros((9, dec.n_bp), device=gpu)
    with pytest.raises(_lib.NrLdpcError) as e:
        dec.decode(llr, 5)
    assert e.value.status == -5
    out = dec.decode(llr[:0], 5)
    assert out.shape == (0, dec.packed_bytes)
    flat = torch.zeros(dec.n_bp * 2 + 1, device=gpu)
    with pytest.raises(_lib.NrLdpcError) as e:
        dec.decode(flat[1:].view(2, dec.n_bp), 5)
    assert e.value.status == -4
    with pytest.raises(_lib.NrLdpcError) as e:
        Decoder(bg=1, z=17)
    assert e.value.status == -2
    lib = _lib.load()
    assert lib.nrldpc_decode(None, None, None, 1, 1, 0, None, None, None) == -1
    with pytest.raises(_lib.NrLdpcError):
        dec.decode(llr[:2], 0)


def test_full_size_batch_properties(gpu):
    """4096 BG1 Z=384 codewords: noiseless codewords decode to themselves in
    two iterations, high-SNR batches decode without errors, and sampled
    codewords match the oracle bit for bit."""
    n = 4096
    dec = Decoder(bg=1, z=384, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(3.0, 1 / 3), device=gpu)
    llr, cw = dec.gen_llr(31, 1000, sig)
    bits = torch.from_numpy(np.unpackbits(cw.cpu().numpy(), axis=1, bitorder="little")).to(gpu)
    clean = (1.0 - 2.0 * bits.float()) * 8.0
    clean[:, :768] = 0.0
    pk = dec.decode(clean.contiguous(), 2)
    counts = dec.count_errors(pk, cw)
    torch.cuda.synchronize()
    assert counts.tolist() == [0, 0]
    pk = dec.decode(llr, 10)
    counts = dec.count_errors(pk, cw)
    torch.cuda.synchronize()
    assert counts.tolist() == [0, 0]
    oc = oracle_for(dec)
    idx = [0, 1, 2047, 4095]
    opk, _, _ = oc.minsum_f32(llr[idx].cpu().numpy(), 10)
    np.testing.assert_array_equal(pk[idx].cpu().numpy(), opk)


def test_count_errors_against_numpy(gpu):
    dec = Decoder(bg=2, z=9, max_batch=64)
    rng = np.random.default_rng(0)
    a = rng.integers(0, 256, (50, dec.packed_bytes), dtype=np.uint8)
    b = a.copy()
    b[rng.random(b.shape) < 0.01] ^= 0x10
    counts = dec.count_errors(torch.from_numpy(a).to(gpu), torch.from_numpy(b).to(gpu), n_info=77)
    torch.cuda.synchronize()
    diff = np.unpackbits(a ^ b, axis=1, bitorder="little")[:, :77].sum(1)
    assert counts.tolist() == [int(diff.sum()), int((diff > 0).sum())]


@pytest.mark.parametrize("qtype", ["f16", "i8"])
def test_reduced_precision_host_transfer(gpu, qtype):
    """fp16 / int8 LLRs over the host link decode exactly like the fp32
    decode of the widened values (the oracle on the same values)."""
    dec = Decoder(bg=2, z=128, max_batch=24)
    oc = oracle_for(dec)
    sig = np.full(24, codes.noise_sigma(2.0, 0.2), np.float32)
    llr, _ = oc.gen_llr(10, 8, 0, sig, 2)
    if qtype == "f16":
        q = torch.from_numpy(llr.astype(np.float16))
        wide, scale = q.float().numpy(), 1.0
    else:
        scale = 0.25
        q = torch.from_numpy(np.clip(np.round(llr / scale), -128, 127).astype(np.int8))
        wide = (q.numpy().astype(np.float32) * np.float32(scale)).astype(np.float32)
    out = torch.empty((24, dec.packed_bytes), dtype=torch.uint8).pin_memory()
    s = torch.cuda.Stream()
    dec.decode_host_q(q.pin_memory(), out, 8, scale=scale, stream=s)
    s.synchronize()
    want, _, _ = oc.minsum_f32(wide, 8)
    np.testing.assert_array_equal(out.numpy(), want)


def test_host_call_in_chunks_back_to_back(gpu):
    """A batch of several CTA rounds goes through the chunked host pipeline
    (copies of chunk k+1 overlap the decode of chunk k); two calls queued
    back to back on one stream with different inputs both come out right."""
    n = 1500  # 304-codeword rounds at BG1 Z=384: chunks of 304, 608, 588
    dec = Decoder(bg=1, z=384, max_batch=n)
    dec.set_host_transfer("copy")
    sig = torch.full((n,), codes.noise_sigma(1.6, 1 / 3), device=gpu)
    llr_a, _ = dec.gen_llr(41, 0, sig)
    llr_b, _ = dec.gen_llr(42, 0, sig)
    ref_a, ref_b = dec.decode(llr_a, 7).cpu(), dec.decode(llr_b, 7).cpu()
    h_a, h_b = llr_a.cpu().pin_memory(), llr_b.cpu().pin_memory()
    out_a = torch.empty((n, dec.packed_bytes), dtype=torch.uint8).pin_memory()
    out_b = torch.empty_like(out_a).pin_memory()
    s = torch.cuda.Stream()
    dec.decode_host(h_a, out_a, 7, stream=s)
    dec.decode_host(h_b, out_b, 7, stream=s)
    s.synchronize()
    assert torch.equal(out_a, ref_a) and torch.equal(out_b, ref_b)
    q = llr_a.cpu().to(torch.float16)
    out_q = torch.empty_like(out_a).pin_memory()
    dec.decode_host_q(q.pin_memory(), out_q, 7, stream=s)
    s.synchronize()
    assert torch.equal(out_q, dec.decode(q.to(gpu).float(), 7).cpu())
    # int8 with a scale: widened on the GPU on whichever lane decodes the chunk
    scale = 0.125
    q8 = torch.clamp(torch.round(llr_b.cpu() / scale), -128, 127).to(torch.int8)
    out_8 = torch.empty_like(out_a).pin_memory()
    dec.decode_host_q(q8.pin_memory(), out_8, 7, scale=scale, stream=s)
    s.synchronize()
    assert torch.equal(out_8, dec.decode((q8.to(gpu).float() * scale).contiguous(), 7).cpu())


@pytest.mark.parametrize("bg,z,n,early", [(1, 384, 700, False), (1, 384, 700, True), (2, 52, 333, True)])
def test_host_transfer_modes_agree(gpu, bg, z, n, early):
    """'direct' (the decoder reads pinned host LLRs and writes the packed bits
    back itself), 'copy' (staged chunks) and 'auto' all give the device
    call's bits, also from views into the middle of pinned buffers; 'direct'
    refuses pageable buffers."""
    dec = Decoder(bg=bg, z=z, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(1.7, dec.kb / (dec.cols - 2)), device=gpu)
    llr, _ = dec.gen_llr(61, 0, sig)
    ref = dec.decode(llr, 8, early_stop=early).cpu()
    h_llr = llr.cpu().pin_memory()
    s = torch.cuda.Stream()
    for mode in ("direct", "copy", "auto"):
        dec.set_host_transfer(mode)
        out = torch.full((n, dec.packed_bytes), 0xAB, dtype=torch.uint8).pin_memory()
        dec.decode_host(h_llr, out, 8, early_stop=early, stream=s)
        s.synchronize()
        assert torch.equal(out, ref), mode
        out.fill_(0xAB)
        dec.decode_host(h_llr[3:], out[3:], 8, early_stop=early, stream=s)
        s.synchronize()
        assert torch.equal(out[3:], ref[3:]) and (out[:3] == 0xAB).all(), mode
    dec.set_host_transfer("direct")
    with pytest.raises(_lib.NrLdpcError) as e:
        dec.decode_host(llr.cpu(), torch.empty((n, dec.packed_bytes), dtype=torch.uint8), 8, stream=s)
    assert e.value.status == -1
    with pytest.raises(_lib.NrLdpcError):
        dec.set_host_transfer(3)


def test_posterior_within_1e5_of_fp64_transcription(gpu):
    """GPU posteriors against the oracle's FP64 min-sum at 1-3 iterations:
    within 1e-5 relative (floor 1) for 99.9% of positions, hard decisions
    differing only where an fp32 rounding flipped a min or a sign."""
    dec = Decoder(bg=1, z=384, max_batch=4)
    oc = oracle_for(dec)
    sig = np.full(4, codes.noise_sigma(2.0, 1 / 3), np.float32)
    llr, _ = oc.gen_llr(22, 71, 0, sig, 2)
    for it in (1, 2, 3):
        pk, app = dec.decode(torch.from_numpy(llr).to(gpu), it, want_app=True)
        torch.cuda.synchronize()
        p64, a64, _ = oc.minsum_f64(llr.astype(np.float64), it)
        rel = np.abs(app.cpu().numpy() - a64) / np.maximum(np.abs(a64), 1.0)
        assert np.quantile(rel, 0.999) < 1e-5, (it, np.quantile(rel, 0.999))
        assert (np.unpackbits(pk.cpu().numpy() ^ p64, axis=1)).sum() <= 8


ALL_Z = sorted({a << j for a in (2, 3, 5, 7, 9, 11, 13, 15) for j in range(8) if a << j <= 384})


@pytest.mark.parametrize("bg", [1, 2])
def test_every_lifting_size_against_oracle(gpu, bg):
    """All 51 lifting sizes of the base graph (every shift table, Z from 2 to
    384, cw_per_cta from 1 to 48): flooding with early stop and layered
    decodes of seeded codewords equal the oracle bit for bit."""
    for z in ALL_Z:
        n = 3
        dec = Decoder(bg=bg, z=z, max_batch=n)
        oc = oracle_for(dec)
        rate = dec.kb / (dec.cols - 2)
        sig = np.linspace(codes.noise_sigma(1.2, rate), codes.noise_sigma(2.2, rate), n).astype(np.float32)
        llr, _ = oc.gen_llr(dec.kb, 500 + z, 0, sig, 2)
        d_llr = torch.from_numpy(llr).to(gpu)
        pk, it = dec.decode(d_llr, 4, early_stop=True, want_iters=True)
        dec.set_schedule("layered")
        pl = dec.decode(d_llr, 3)
        torch.cuda.synchronize()
        opk, _, oit = oc.minsum_f32(llr, 4, early_stop=True, threads=3)
        np.testing.assert_array_equal(pk.cpu().numpy(), opk, err_msg=f"flooding bg{bg} z{z}")
        np.testing.assert_array_equal(it.cpu().numpy(), oit, err_msg=f"iterations bg{bg} z{z}")
        opl, _, _ = oc.layered_f32(llr, 3, threads=3)
        np.testing.assert_array_equal(pl.cpu().numpy(), opl, err_msg=f"layered bg{bg} z{z}")
        dec.close()


def test_bounded_wait_reports_timeout(gpu):
    """The wait for a group's LLR copy is bounded.  The self-test entry point
    tells the copy barrier to expect 16 bytes more than the copies deliver
    and issues no copy, so no CTA's wait can complete: each gives up after its limit, the kernel
    records the timeout and returns, the host reads it (and reading clears
    it), and the same handle then decodes bit-exactly again."""
    lib = _lib.load()
    z, n = 384, 8
    oc = OracleCode(codes.base_matrix(1, codes.set_index(z)), z)
    llr, _ = oc.gen_llr(22, 77, 0, np.full(n, codes.noise_sigma(2.0, 1 / 3), np.float32), 2)
    dec = make_decoder(1, z, max_batch=n)
    d_llr = torch.from_numpy(llr).to(gpu)
    out = torch.zeros((n, dec.packed_bytes), dtype=torch.uint8, device=gpu)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.nrldpc_selftest_wait_timeout(dec._h, C.c_void_p(d_llr.data_ptr()), C.c_void_p(out.data_ptr()),
                                            n, stream) == 0
    torch.cuda.synchronize()
    assert dec.device_error() == -6  # NRLDPC_ERR_TIMEOUT: the LLR-load wait ran out
    assert dec.device_error() == 0
    packed = dec.decode(d_llr, 5)
    torch.cuda.synchronize()
    want, _, _ = oc.minsum_f32(llr, 5)
    assert np.array_equal(packed.cpu().numpy(), want)
    assert dec.device_error() == 0
    dec.close()


@pytest.mark.parametrize("schedule", ["flooding", "layered-learned"])
def test_early_stop_parity_across_the_waterfall(gpu, schedule):
    """Early stop where it matters most: 96 BG1 Z=384 codewords spread over
    the waterfall (1.7-1.9 dB), many of which converge after a few to many
    iterations and fail their syndrome checks at late rows first -- the
    state in which the decoder switches from the row-by-row syndrome pass to
    the bit-sliced one.  Iteration counts, hard decisions and posteriors
    equal the oracle's (plain flooding min-sum, or the layered decoder with
    the trained weights bg1_L6)."""
    from nr_gpu_ldpc_gb300.learned import load_weights
    z, n = 384, 96
    dec = make_decoder(1, z, max_batch=n)
    oc = oracle_for(dec)
    sig = np.array([codes.noise_sigma(eb, 1 / 3) for eb in np.linspace(1.7, 1.9, n)], np.float32)
    llr, _ = oc.gen_llr(dec.kb, 4242, 0, sig, 2)
    d = torch.from_numpy(llr).to(gpu)
    if schedule == "flooding":
        pk, app, its = dec.decode(d, 15, early_stop=True, want_app=True, want_iters=True)
        torch.cuda.synchronize()
        opk, oapp, oits = oc.minsum_f32(llr, 15, early_stop=True, want_app=True, threads=4)
    else:
        w = load_weights("bg1_L6")
        dec.set_schedule("layered")
        dec.set_weights(w)
        pk, app, its = dec.decode(d, 6, early_stop=True, weighted=True, want_app=True, want_iters=True)
        torch.cuda.synchronize()
        opk, oapp, oits = oc.layered_f32(llr, 6, w=w, early_stop=True, want_app=True, threads=4)
    np.testing.assert_array_equal(its.cpu().numpy(), oits)
    np.testing.assert_array_equal(pk.cpu().numpy(), opk)
    np.testing.assert_array_equal(app.cpu().numpy().view(np.uint32), oapp.view(np.uint32))
    assert len(np.unique(oits)) >= 2  # codewords stop at different iterations
    dec.close()
