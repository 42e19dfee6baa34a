"""Python host API over the C-ABI (device memory and streams from PyTorch).

``Decoder`` owns one ``nrldpc_handle``: a lifted code (5G NR BG1/BG2 at a
lifting size Z, or a custom QC base matrix) with its device scratch.  All
GPU work goes through ``libnrldpc_gb300.so``; nothing here computes on the
CPU.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import _lib
from .codes import KB_MAX


def _stream_ptr(stream: Optional[torch.cuda.Stream]) -> C.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _dev_ptr(t: Optional[torch.Tensor]):
    return None if t is None else C.c_void_p(t.data_ptr())


class Decoder:
    """Flooding normalized min-sum decoder on one GPU.

    Parameters mirror the reference's setup (src/nr_ldpc.cpp:31,
    src/setup_exp.cu:102-166,286-313): base graph ``bg`` and lifting size
    ``z``, at most ``max_batch`` codewords per call, ``alpha`` (the
    reference's literal 0.75).  ``base`` gives a custom base matrix instead.
    """

    def __init__(self, bg: int = 1, z: int = 384, max_batch: int = 4096, alpha: float = 0.75,
                 device: int = 0, cw_per_cta: int = 0, base: Optional[np.ndarray] = None):
        lib = _lib.load()
        if cw_per_cta == 0 and base is None:
            from .autotune import load_table
            cpb, spt = load_table(device).get((bg, z), (0, 1))
            cw_per_cta = cpb if spt == 1 else 0  # this decoder runs one sub-row per thread
        cfg = _lib.ConfigC(bg=bg if base is None else 0, z=z, max_batch=max_batch, alpha=alpha,
                           device=device, cw_per_cta=cw_per_cta)
        h = C.c_void_p()
        if base is None:
            _lib.check("nrldpc_init", lib.nrldpc_init(C.byref(cfg), C.byref(h)))
            self.kb = KB_MAX[bg]
        else:
            b = np.ascontiguousarray(base, dtype=np.int32)
            _lib.check("nrldpc_init_custom",
                       lib.nrldpc_init_custom(b.ctypes.data_as(C.c_void_p), b.shape[0], b.shape[1],
                                              C.byref(cfg), C.byref(h)))
            self.kb = b.shape[1] - b.shape[0]
        self._h = h
        self._lib = lib
        self.bg, self.z, self.max_batch, self.alpha = bg, z, max_batch, alpha
        self.device = torch.device("cuda", device)
        vals = [C.c_int() for _ in range(6)]
        _lib.check("nrldpc_geometry", lib.nrldpc_geometry(h, *[C.byref(v) for v in vals]))
        self.rows, self.cols, _, self.n_edges, self.n_bp, self.packed_bytes = [v.value for v in vals]
        self.n_info = self.kb * self.z
        self.schedule = "flooding"

    def close(self):
        if getattr(self, "_h", None):
            self._lib.nrldpc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- decode ---------------------------------------------------------------------
    def _check_llr(self, llr: torch.Tensor) -> int:
        if llr.device.type != "cuda" or llr.dtype != torch.float32 or not llr.is_contiguous():
            raise ValueError("llr must be a contiguous float32 CUDA tensor")
        n = llr.numel() // self.n_bp
        if llr.numel() != n * self.n_bp:
            raise ValueError(f"llr size must be a multiple of n_bp={self.n_bp}")
        return n

    def decode(self, llr: torch.Tensor, n_iter: int, early_stop: bool = False,
               want_app: bool = False, want_iters: bool = False, weighted: bool = False,
               out: Optional[torch.Tensor] = None, stream: Optional[torch.cuda.Stream] = None):
        """Decode [n_cw, n_bp] device LLRs; returns packed hard decisions
        [n_cw, packed_bytes] (uint8, device), plus app / iters if asked."""
        n = self._check_llr(llr)
        packed = out if out is not None else torch.empty((n, self.packed_bytes), dtype=torch.uint8,
                                                          device=llr.device)
        app = torch.empty((n, self.n_bp), dtype=torch.float32, device=llr.device) if want_app else None
        iters = torch.empty(n, dtype=torch.int32, device=llr.device) if want_iters else None
        fn = self._lib.nrldpc_decode_weighted if weighted else self._lib.nrldpc_decode
        _lib.check("nrldpc_decode", fn(self._h, _dev_ptr(llr), _dev_ptr(packed), n, int(n_iter),
                                       int(bool(early_stop)), _dev_ptr(app), _dev_ptr(iters),
                                       _stream_ptr(stream)))
        res = [packed]
        if want_app:
            res.append(app)
        if want_iters:
            res.append(iters)
        return res[0] if len(res) == 1 else tuple(res)

    def decode_host(self, llr_host: torch.Tensor, packed_host: torch.Tensor, n_iter: int,
                    early_stop: bool = False, stream: Optional[torch.cuda.Stream] = None):
        """Reference-shaped call: host LLRs in, host packed bits out, H2D +
        decode + D2H queued on one stream (asynchronous; sync the stream)."""
        if llr_host.device.type != "cpu" or packed_host.device.type != "cpu":
            raise ValueError("host tensors expected")
        n = llr_host.numel() // self.n_bp
        _lib.check("nrldpc_decode_host_async",
                   self._lib.nrldpc_decode_host_async(self._h, C.c_void_p(llr_host.data_ptr()),
                                                      C.c_void_p(packed_host.data_ptr()), n,
                                                      int(n_iter), int(bool(early_stop)),
                                                      _stream_ptr(stream)))

    def decode_host_q(self, llr_q_host: torch.Tensor, packed_host: torch.Tensor, n_iter: int,
                      scale: float = 1.0, early_stop: bool = False,
                      stream: Optional[torch.cuda.Stream] = None):
        """Host call with fp16 (torch.float16) or int8 (LLR = q * scale) LLRs."""
        if llr_q_host.dtype == torch.float16:
            qtype = 1
        elif llr_q_host.dtype == torch.int8:
            qtype = 2
        else:
            raise ValueError("fp16 or int8 LLRs expected")
        n = llr_q_host.numel() // self.n_bp
        _lib.check("nrldpc_decode_host_async_q",
                   self._lib.nrldpc_decode_host_async_q(self._h, C.c_void_p(llr_q_host.data_ptr()), qtype,
                                                        float(scale), C.c_void_p(packed_host.data_ptr()),
                                                        n, int(n_iter), int(bool(early_stop)),
                                                        _stream_ptr(stream)))

    def set_host_transfer(self, mode) -> None:
        """How decode_host moves fp32 data: 'copy' (staged chunk copies),
        'direct' (the decoder reads the LLRs from pinned host memory and
        writes the bits back itself) or 'auto' (default: 'direct' for pinned
        buffers on a GPU with a coherent host link up to 4 rounds of
        resident CTAs, else 'copy')."""
        code = {"auto": 0, "copy": 1, "direct": 2}.get(mode, mode)
        _lib.check("nrldpc_set_host_transfer", self._lib.nrldpc_set_host_transfer(self._h, int(code)))

    # ---- schedule -------------------------------------------------------------------
    FLOODING, LAYERED = 0, 1

    def set_schedule(self, schedule) -> None:
        """'flooding' (the reference's, default) or 'layered' (row-sequential,
        in-place posterior; no reference counterpart)."""
        code = {"flooding": 0, "layered": 1}.get(schedule, schedule)
        _lib.check("nrldpc_set_schedule", self._lib.nrldpc_set_schedule(self._h, int(code)))
        self.schedule = "layered" if code == 1 else "flooding"

    # ---- learned weights ------------------------------------------------------------
    def set_weights(self, w) -> None:
        w = np.ascontiguousarray(np.asarray(w, dtype=np.float32).reshape(-1, self.n_edges))
        _lib.check("nrldpc_set_weights",
                   self._lib.nrldpc_set_weights(self._h, w.ctypes.data_as(C.c_void_p), w.shape[0]))

    # ---- channel --------------------------------------------------------------------
    def gen_llr(self, seed: int, cw_base: int, sigma: torch.Tensor, n_punct_cols: Optional[int] = None,
                want_cw: bool = True, llr_out: Optional[torch.Tensor] = None,
                cw_out: Optional[torch.Tensor] = None, stream=None):
        """Seeded codewords + AWGN LLRs on the GPU ([n] sigma on the device)."""
        n = sigma.numel()
        if n_punct_cols is None:
            n_punct_cols = 2 if self.kb in (22, 10) and self.cols in (68, 52) else 0
        llr = llr_out if llr_out is not None else torch.empty((n, self.n_bp), dtype=torch.float32,
                                                              device=self.device)
        cw = None
        if want_cw:
            cw = cw_out if cw_out is not None else torch.empty((n, self.packed_bytes),
                                                               dtype=torch.uint8, device=self.device)
        _lib.check("nrldpc_gen_llr",
                   self._lib.nrldpc_gen_llr(self._h, int(seed), int(cw_base), n, _dev_ptr(sigma),
                                            int(n_punct_cols), _dev_ptr(llr), _dev_ptr(cw),
                                            _stream_ptr(stream)))
        return llr, cw

    def count_errors(self, packed: torch.Tensor, cw_packed: torch.Tensor, n_info: Optional[int] = None,
                     counts: Optional[torch.Tensor] = None, stream=None) -> torch.Tensor:
        """Accumulate [bit errors, frame errors] over the info bits into a
        device int64[2] tensor (returned)."""
        n = packed.shape[0]
        if counts is None:
            counts = torch.zeros(2, dtype=torch.int64, device=packed.device)
        _lib.check("nrldpc_count_errors",
                   self._lib.nrldpc_count_errors(self._h, _dev_ptr(packed), _dev_ptr(cw_packed), n,
                                                 int(self.n_info if n_info is None else n_info),
                                                 _dev_ptr(counts), _stream_ptr(stream)))
        return counts

    def device_error(self) -> int:
        return self._lib.nrldpc_device_error(self._h)
