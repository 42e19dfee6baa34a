"""Code description: 5G NR base graphs, lifting sizes and ``setup_ldpc``.

Host-side logic only (no GPU).  ``setup_ldpc`` mirrors the reference's
``ldpc_params setup_ldpc(int A, float rate, int n_iterations)``
(src/nr_ldpc.cpp:31-230, struct at src/types.h:38-55) field for field,
including its quirks:

* ``Z_min = K' / K_b`` is an integer division and Z_c is the smallest set
  entry >= Z_min (src/nr_ldpc.cpp:85-106), so K_b * Z_c can fall short of K'.
* C > 1 (segmentation) is reported, not supported (src/nr_ldpc.cpp:76-81).

Table shifts are stored unreduced; ``lifted_base(bg, z)`` applies
V mod Z (TS 38.212 5.3.2).  The reference kernels subtract Z once
(src/ldpc_kernels.cu:126-130), which equals V mod Z whenever V < Z -- true
for every Z the reference runs (Z = 384, iLS 1).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import base_graphs as _bg

BASE_Z = (2, 3, 5, 7, 9, 11, 13, 15)
BG_SHAPE = {1: _bg.BG1_SHAPE, 2: _bg.BG2_SHAPE}
BG_EDGES = {1: _bg.BG1_EDGES, 2: _bg.BG2_EDGES}
KB_MAX = {1: 22, 2: 10}          # systematic base columns
WIFI_SHAPE = _bg.WIFI_SHAPE
WIFI_KB = 12

#: every lifting size of TS 38.212 Table 5.3.2-1 with its set index iLS
LIFTING_SIZES = {}
for _ils, _a in enumerate(BASE_Z):
    _z = _a
    while _z <= 384:
        LIFTING_SIZES[_z] = _ils
        _z *= 2
LIFTING_SIZES = dict(sorted(LIFTING_SIZES.items()))


class LdpcConfigError(ValueError):
    """Invalid base graph / lifting size / code parameters."""


def set_index(z: int) -> int:
    """Lifting-size set index iLS of Z (TS 38.212 Table 5.3.2-1)."""
    try:
        return LIFTING_SIZES[int(z)]
    except KeyError:
        raise LdpcConfigError(f"Z={z} is not a 5G NR lifting size") from None


def base_matrix(bg: int, ils: int) -> np.ndarray:
    """Dense base matrix of shifts (unreduced V, -1 = zero block)."""
    if bg not in BG_SHAPE:
        raise LdpcConfigError(f"base graph must be 1 or 2, got {bg}")
    if not 0 <= ils < 8:
        raise LdpcConfigError(f"iLS must be 0..7, got {ils}")
    rows, cols = BG_SHAPE[bg]
    h = np.full((rows, cols), -1, dtype=np.int32)
    for r, c, v in BG_EDGES[bg]:
        h[r, c] = v[ils]
    return h


def lifted_base(bg: int, z: int) -> np.ndarray:
    """Base matrix for (BG, Z) with shifts reduced mod Z (-1 kept)."""
    h = base_matrix(bg, set_index(z)).copy()
    m = h >= 0
    h[m] %= int(z)
    return h


def wifi_base() -> np.ndarray:
    """802.11n 12x24 rate-1/2 base matrix (the reference Overview.md example)."""
    h = np.full(WIFI_SHAPE, -1, dtype=np.int32)
    for r, c, v in _bg.WIFI_EDGES:
        h[r, c] = v
    return h


@dataclass
class LdpcParams:
    """Mirror of the reference's ``ldpc_params`` (src/types.h:38-55)."""
    A: int
    rate: float
    bg_index: int
    Z: int
    K: int
    N: int
    H_rows: int
    H_cols: int
    H: np.ndarray = field(repr=False)
    n_nz_in_row: int
    n_nz_in_col: int
    h_element_count_per_row: np.ndarray = field(repr=False)
    h_element_count_per_col: np.ndarray = field(repr=False)
    n_iterations: int
    N_before_puncture: int
    i_ls: int
    C: int
    K_b: int


def setup_ldpc(A: int, rate: float, n_iterations: int) -> LdpcParams:
    """Parameterize the code as the reference does (src/nr_ldpc.cpp:31-230)."""
    A = int(A)
    rate = float(np.float32(rate))
    l = 24 if A > 3824 else 16                                   # :37
    B = A + l
    if (A <= 292) or (A < 3824 and rate <= 0.67) or (rate <= 0.25):  # :45
        bg, k_cb = 2, 3840
        k_b = 10 if B > 640 else 9 if B > 560 else 8 if B > 192 else 6
    else:
        bg, k_cb, k_b = 1, 8448, 22
    if B <= k_cb:                                                # :66-75
        C, b_prime = 1, B
    else:
        C = math.ceil(B // (k_cb - 24))
        b_prime = B + C * 24
    k_prime = b_prime // C
    z_min = k_prime // k_b                                       # :85
    z_c, i_ls = 1000, None
    for i, a in enumerate(BASE_Z):                               # :93-106
        t = a
        for _ in range(8):
            v = t if t < 385 else 0
            t *= 2
            if v >= z_min and v < z_c:
                z_c, i_ls = v, i
    if i_ls is None:
        raise LdpcConfigError(f"no lifting size >= {z_min} (A={A})")
    K = 22 * z_c if bg == 1 else 10 * z_c
    N = 66 * z_c if bg == 1 else 50 * z_c
    rows, cols = BG_SHAPE[bg]
    H = base_matrix(bg, i_ls)
    nz = H != -1
    per_row = nz.sum(1).astype(np.int8)
    per_col = nz.sum(0).astype(np.int8)
    return LdpcParams(A=A, rate=rate, bg_index=bg, Z=z_c, K=K, N=N, H_rows=rows, H_cols=cols,
                      H=H, n_nz_in_row=int(per_row.max()), n_nz_in_col=int(per_col.max()),
                      h_element_count_per_row=per_row, h_element_count_per_col=per_col,
                      n_iterations=int(n_iterations), N_before_puncture=N + 2 * z_c,
                      i_ls=i_ls, C=C, K_b=k_b)


def compact_rows(h: np.ndarray):
    """``h_compact1`` order: per base row, nonzero (col, V) in ascending column
    order (src/setup_exp.cu:241-250)."""
    return [[(int(c), int(h[r, c])) for c in np.nonzero(h[r] != -1)[0]] for r in range(h.shape[0])]


def compact_cols(h: np.ndarray):
    """``h_compact2`` order: per base column, nonzero (row, V) in ascending row
    order (src/setup_exp.cu:261-270)."""
    return [[(int(r), int(h[r, c])) for r in np.nonzero(h[:, c] != -1)[0]] for c in range(h.shape[1])]


def noise_sigma(ebn0_db: float, code_rate: float) -> float:
    """sigma for BPSK at Eb/N0 (dB), as src/encoding_tools.cpp:27-38 (float)."""
    f = np.float32
    energy_per_bit = f(1) / f(code_rate)
    eb_n0 = f(np.power(f(10.0), f(ebn0_db) / f(10)))
    n0 = f(energy_per_bit / eb_n0)
    return float(f(np.sqrt(f(n0 / f(2)))))
