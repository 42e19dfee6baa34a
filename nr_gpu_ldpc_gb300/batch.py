"""Mixed-code batches over the C-ABI: any mix of 5G NR (BG, Z), rate-matched
lengths and filler bits in one job list, decoded by one persistent launch
(replayed from a CUDA graph) that pulls codeword groups from a device work
queue.  The reference decodes one compiled-in code per process
(src/globals.h:15) and has no rate matching (src/main.cpp:64-65)."""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import _lib
from .codes import BG_SHAPE, KB_MAX
from .decoder import _dev_ptr, _stream_ptr

JOB_DTYPE = np.dtype([("bg", "<i4"), ("z", "<i4"), ("k_prime", "<i4"), ("e", "<i4"), ("rv", "<i4"),
                      ("sigma", "<f4"), ("qm", "<i4"), ("reserved", "<i4"), ("llr_offset", "<i8"),
                      ("e_offset", "<i8"), ("out_offset", "<i8")])
assert JOB_DTYPE.itemsize == 56


def make_jobs(bg, z, k_prime=0, e=0, rv=0, sigma=1.0, qm=1):
    """Job array with contiguous layouts: mother LLRs (4-float aligned),
    rate-matched LLRs, packed outputs.  qm: modulation order of the bit
    interleaver (e must be a multiple of it).  Returns (jobs, n_llr, n_e,
    n_out)."""
    bg = np.asarray(bg, np.int32)
    n = bg.size
    z = np.broadcast_to(np.asarray(z, np.int32), (n,))
    jobs = np.zeros(n, JOB_DTYPE)
    jobs["bg"], jobs["z"] = bg, z
    jobs["k_prime"] = np.broadcast_to(k_prime, (n,))
    jobs["rv"] = np.broadcast_to(rv, (n,))
    jobs["sigma"] = np.broadcast_to(sigma, (n,))
    jobs["qm"] = np.broadcast_to(qm, (n,))
    cols = np.where(bg == 1, BG_SHAPE[1][1], BG_SHAPE[2][1])
    kb = np.where(bg == 1, KB_MAX[1], KB_MAX[2])
    nbp = cols * z
    kp = np.where(jobs["k_prime"] == 0, kb * z, jobs["k_prime"])
    ee = np.broadcast_to(np.asarray(e), (n,)).astype(np.int64)
    ee = np.where(ee == 0, nbp - 2 * z - (kb * z - kp), ee)
    jobs["e"] = np.broadcast_to(e, (n,))
    llr_len = (nbp + 3) // 4 * 4
    jobs["llr_offset"] = np.concatenate([[0], np.cumsum(llr_len)[:-1]])
    jobs["e_offset"] = np.concatenate([[0], np.cumsum(ee)[:-1]])
    pb = (nbp + 7) // 8
    jobs["out_offset"] = np.concatenate([[0], np.cumsum(pb)[:-1]])
    return jobs, int(llr_len.sum()), int(ee.sum()), int(pb.sum())


MIXED_ZS = (64, 96, 128, 192, 256, 320, 384)


def mixed_workload(n: int = 8192, seed: int = 2024):
    """The uneven-batch workload: n codewords, BG1 or BG2 uniformly, Z uniform
    in {64, ..., 384}, up to 39 filler bits, code rate K'/E uniform in
    [0.25, 0.8] (E at least 2Z + 8), Eb/N0 uniform in 1-3 dB.  Returns
    (bg, z, k_prime, e, sigma) arrays."""
    rng = np.random.default_rng(seed)
    bg = rng.integers(1, 3, n)
    z = rng.choice(MIXED_ZS, n)
    kb = np.where(bg == 1, 22, 10)
    kp = kb * z - rng.integers(0, 40, n)
    e = np.maximum((kp / rng.uniform(0.25, 0.8, n)).astype(np.int64), 2 * z + 8)
    eb = rng.uniform(1.0, 3.0, n)
    sigma = np.sqrt((e / kp) / (2.0 * 10 ** (eb / 10))).astype(np.float32)
    return bg, z, kp, e, sigma


class Batch:
    def __init__(self, max_jobs: int, alpha: float = 0.75, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        _lib.check("nrldpc_batch_create", self.lib.nrldpc_batch_create(device, max_jobs, alpha, C.byref(h)))
        self._h = h
        self.device = torch.device("cuda", device)
        self.jobs = None
        from .autotune import load_table
        for (bg, z), (cpb, spt) in load_table(device).items():  # tuned geometry, if any
            try:
                self.set_sub_rows_per_thread(bg, z, spt)
                self.set_cw_per_cta(bg, z, cpb)
            except _lib.NrLdpcError:
                pass

    def close(self):
        if getattr(self, "_h", None):
            self.lib.nrldpc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_cw_per_cta(self, bg: int, z: int, cpb: int):
        _lib.check("nrldpc_batch_set_cw_per_cta", self.lib.nrldpc_batch_set_cw_per_cta(self._h, bg, z, cpb))

    def get_cw_per_cta(self, bg: int, z: int) -> int:
        v = C.c_int()
        _lib.check("nrldpc_batch_get_cw_per_cta", self.lib.nrldpc_batch_get_cw_per_cta(self._h, bg, z, C.byref(v)))
        return v.value

    def set_sub_rows_per_thread(self, bg: int, z: int, spt: int):
        """Threads per codeword = Z / spt (spt 1 or 2); apply before set_jobs."""
        _lib.check("nrldpc_batch_set_sub_rows_per_thread",
                   self.lib.nrldpc_batch_set_sub_rows_per_thread(self._h, bg, z, spt))

    def get_sub_rows_per_thread(self, bg: int, z: int) -> int:
        v = C.c_int()
        _lib.check("nrldpc_batch_get_sub_rows_per_thread",
                   self.lib.nrldpc_batch_get_sub_rows_per_thread(self._h, bg, z, C.byref(v)))
        return v.value

    def set_jobs(self, jobs: np.ndarray):
        jobs = np.ascontiguousarray(jobs, JOB_DTYPE)
        _lib.check("nrldpc_batch_set_jobs",
                   self.lib.nrldpc_batch_set_jobs(self._h, jobs.ctypes.data_as(C.c_void_p), jobs.size))
        self.jobs = jobs

    def gen(self, seed: int, cw_base: int, llr_e: torch.Tensor, cw: Optional[torch.Tensor], stream=None):
        _lib.check("nrldpc_batch_gen", self.lib.nrldpc_batch_gen(self._h, int(seed), int(cw_base), _dev_ptr(llr_e),
                                                                 _dev_ptr(cw), _stream_ptr(stream)))

    def derate(self, llr_e: torch.Tensor, llr: torch.Tensor, stream=None):
        _lib.check("nrldpc_batch_derate",
                   self.lib.nrldpc_batch_derate(self._h, _dev_ptr(llr_e), _dev_ptr(llr), _stream_ptr(stream)))

    def decode(self, llr: torch.Tensor, packed: torch.Tensor, n_iter: int, early_stop: bool = False,
               iters: Optional[torch.Tensor] = None, stream=None):
        _lib.check("nrldpc_batch_decode",
                   self.lib.nrldpc_batch_decode(self._h, _dev_ptr(llr), _dev_ptr(packed), int(n_iter),
                                                int(bool(early_stop)), _dev_ptr(iters), _stream_ptr(stream)))

    def count_errors(self, packed: torch.Tensor, cw: torch.Tensor, counts: Optional[torch.Tensor] = None,
                     stream=None) -> torch.Tensor:
        if counts is None:
            counts = torch.zeros(2, dtype=torch.int64, device=self.device)
        _lib.check("nrldpc_batch_count_errors",
                   self.lib.nrldpc_batch_count_errors(self._h, _dev_ptr(packed), _dev_ptr(cw), _dev_ptr(counts),
                                                      _stream_ptr(stream)))
        return counts
