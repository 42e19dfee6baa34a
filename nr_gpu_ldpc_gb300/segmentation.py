"""Transport-block code-block segmentation (3GPP TS 38.212 5.2.2) over the
C-ABI: the segmentation rules on the host (nrldpc_segment), the bit moves and
per-block CRC24B attach / check on the GPU (nrldpc_cb_segment,
nrldpc_cb_desegment).  The reference computes the number of code blocks but
decodes C = 1 only (src/nr_ldpc.cpp:64-81)."""
from __future__ import annotations

import ctypes as C
from typing import Optional

import torch

from . import _lib
from .decoder import _dev_ptr, _stream_ptr


def segment_info(B: int, bg: int) -> dict:
    """C, L, K', K, Zc, Kb, filler of a transport block of B bits (TB CRC
    included) for base graph bg."""
    lib = _lib.load()
    g = _lib.SegmentInfoC()
    _lib.check("nrldpc_segment", lib.nrldpc_segment(int(B), int(bg), C.byref(g)))
    return {f: getattr(g, f) for f, _ in g._fields_}


def _info_c(info: dict):
    g = _lib.SegmentInfoC()
    for f, _ in g._fields_:
        setattr(g, f, int(info[f]))
    return g


def segment(tb: torch.Tensor, info: dict, blocks: torch.Tensor, stream=None) -> torch.Tensor:
    """Packed transport block (uint8, device) -> C packed code blocks, one per
    row of `blocks` ([C, stride] uint8, device), CRC24B attached when C > 1."""
    lib = _lib.load()
    g = _info_c(info)
    _lib.check("nrldpc_cb_segment", lib.nrldpc_cb_segment(_dev_ptr(tb), C.byref(g), _dev_ptr(blocks),
                                                          blocks.shape[1], _stream_ptr(stream)))
    return blocks


def desegment(blocks: torch.Tensor, info: dict, tb: torch.Tensor, crc_rem: Optional[torch.Tensor] = None,
              stream=None):
    """Decoded code blocks -> packed transport block; returns the per-block
    CRC24B remainders (int32 [C], 0 = pass) when C > 1."""
    lib = _lib.load()
    g = _info_c(info)
    if info["L"] > 0 and crc_rem is None:
        crc_rem = torch.empty(info["C"], dtype=torch.int32, device=blocks.device)
    _lib.check("nrldpc_cb_desegment",
               lib.nrldpc_cb_desegment(_dev_ptr(blocks), blocks.shape[1], C.byref(g), _dev_ptr(tb),
                                       _dev_ptr(crc_rem), _stream_ptr(stream)))
    return crc_rem
