"""Code-block segmentation (TS 38.212 5.2.2): the C-ABI rules against the
oracle's restatement (CPU), and the GPU bit moves + CRC24B attach / check
against the oracle's blocks (GPU)."""
import ctypes as C

import numpy as np
import pytest

from nr_gpu_ldpc_gb300 import _lib
from oracle import oracle as O


def _c_info(B, bg):
    g = _lib.SegmentInfoC()
    rc = _lib.load(build_if_missing=True).nrldpc_segment(B, bg, C.byref(g))
    return rc, {f: getattr(g, f) for f, _ in g._fields_}


@pytest.mark.parametrize("bg", [1, 2])
def test_segment_rules_match_oracle(cuda_lib, bg):
    rng = np.random.default_rng(bg)
    sizes = list(range(24, 1200, 37)) + list(rng.integers(1200, 60000, 300))
    checked = 0
    for B in sizes:
        B = int(B)
        want = O.segment_info(B, bg)
        rc, got = _c_info(B, bg)
        if want is None:
            assert rc != 0
            continue
        assert rc == 0 and got == want, (B, got, want)
        checked += 1
    assert checked > 60


def test_segment_known_cases(cuda_lib):
    assert _c_info(8448, 1)[1] == {"B": 8448, "C": 1, "L": 0, "k_prime": 8448, "k": 8448, "zc": 384,
                                   "kb": 22, "filler": 0, "bg": 1}
    rc, g = _c_info(16848, 1)  # two full BG1 blocks of 8424 data + 24 CRC bits
    assert rc == 0 and (g["C"], g["k_prime"], g["zc"], g["filler"]) == (2, 8448, 384, 0)
    rc, g = _c_info(500, 2)  # BG2, Kb = 8 for 192 < B <= 560
    assert rc == 0 and (g["C"], g["kb"], g["zc"], g["k"]) == (1, 8, 64, 640)


@pytest.mark.gpu
@pytest.mark.parametrize("B,bg", [(16848, 1), (8448, 1), (12096, 2), (100000 - 100000 % 8 + 8, 1)])
def test_gpu_segment_desegment_round_trip(gpu, B, bg):
    import torch
    from nr_gpu_ldpc_gb300 import segmentation as S
    info = O.segment_info(B, bg)
    if info is None:
        pytest.skip("not a segmentable size")
    rng = np.random.default_rng(B)
    tb_bits = rng.integers(0, 2, B).astype(np.uint8)
    tb = torch.from_numpy(np.packbits(tb_bits, bitorder="little")).to(gpu)
    stride = (info["k"] + 7) // 8 + 4
    blocks = torch.full((info["C"], stride), 0xA5, dtype=torch.uint8, device=gpu)
    S.segment(tb, info, blocks)
    torch.cuda.synchronize()
    want = O.cb_segment(tb_bits, info)
    got = np.unpackbits(blocks.cpu().numpy(), axis=1, bitorder="little")[:, :info["k_prime"]]
    np.testing.assert_array_equal(got, want)
    back = torch.zeros_like(tb)
    rem = S.desegment(blocks, info, back)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(np.unpackbits(back.cpu().numpy(), bitorder="little")[:B], tb_bits)
    if info["L"]:
        assert (rem.cpu().numpy() == 0).all()
        blocks[info["C"] - 1, 3] ^= 0x10  # corrupt the last block
        rem = S.desegment(blocks, info, back)
        torch.cuda.synchronize()
        r = rem.cpu().numpy()
        assert (r[:-1] == 0).all() and r[-1] != 0
