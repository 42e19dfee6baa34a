"""Learned weighted min-sum: GPU training loop and weight files.

The model replaces the reference's fixed normalization (alpha = 0.75,
src/ldpc_kernels.cu:164,295) by a weight per (iteration, base edge), shared
by every lifted copy of the edge and by every lifting size.  Training runs
entirely on the GPU through the C-ABI: seeded codewords and AWGN LLRs
(nrldpc_gen_llr), the unrolled forward (nrldpc_wms_forward), its adjoint
(nrldpc_wms_backward) and Adam (nrldpc_adam_step).  The loss is the BCE of
the posterior LLRs after every unrolled iteration (mean over iterations,
codewords and columns).
"""
from __future__ import annotations

import ctypes as C
import json
import os
from typing import Optional

import numpy as np
import torch

from . import _lib
from .decoder import Decoder, _dev_ptr, _stream_ptr

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")


def sigma_from_ebn0(ebn0_db: torch.Tensor, rate: float) -> torch.Tensor:
    """sigma = sqrt((1/R) / (2 * 10^(EbN0/10))) per codeword (float32)."""
    return torch.sqrt((1.0 / rate) / (2.0 * torch.pow(10.0, ebn0_db / 10.0))).to(torch.float32)


class Trainer:
    """Trains w[n_iter][n_edges] for one base graph at one lifting size,
    under the flooding (the reference's) or the layered schedule."""

    def __init__(self, bg: int = 2, z: int = 128, n_iter: int = 8, batch: int = 16384,
                 chunk: int = 4096, lr: float = 1e-3, ebn0_range=(1.0, 3.0), w_init: float = 0.75,
                 seed: int = 1, device: int = 0, schedule: str = "flooding"):
        self.dec = Decoder(bg=bg, z=z, max_batch=chunk, device=device)
        self.dec.set_schedule(schedule)
        self.schedule = schedule
        self.lib = _lib.load()
        self.bg, self.z, self.T, self.batch, self.chunk = bg, z, n_iter, batch, chunk
        self.lr, self.ebn0_range, self.seed = lr, ebn0_range, seed
        self.rate = self.dec.kb / (self.dec.cols - 2)
        dev = self.dec.device
        E = self.dec.n_edges
        self.w = torch.full((n_iter, E), w_init, dtype=torch.float32, device=dev)
        self.m = torch.zeros_like(self.w)
        self.v = torch.zeros_like(self.w)
        self.grad = torch.zeros((n_iter, E), dtype=torch.float64, device=dev)
        self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
        nbytes = C.c_size_t()
        _lib.check("nrldpc_wms_workspace_bytes",
                   self.lib.nrldpc_wms_workspace_bytes(self.dec._h, chunk, n_iter, C.byref(nbytes)))
        self.ws = torch.empty(nbytes.value, dtype=torch.uint8, device=dev)
        self.step_count = 0
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(seed)

    # ---- primitives ---------------------------------------------------------------------
    def forward(self, llr: torch.Tensor, cw: torch.Tensor, scale: float, app: Optional[torch.Tensor] = None,
                weights: Optional[torch.Tensor] = None):
        w = self.w if weights is None else weights
        _lib.check("nrldpc_wms_forward",
                   self.lib.nrldpc_wms_forward(self.dec._h, _dev_ptr(llr), _dev_ptr(cw), llr.shape[0],
                                               self.T, _dev_ptr(w), _dev_ptr(self.ws), float(scale),
                                               _dev_ptr(self.loss), _dev_ptr(app), _stream_ptr(None)))

    def backward(self, n_cw: int, weights: Optional[torch.Tensor] = None):
        w = self.w if weights is None else weights
        _lib.check("nrldpc_wms_backward",
                   self.lib.nrldpc_wms_backward(self.dec._h, n_cw, self.T, _dev_ptr(w), _dev_ptr(self.ws),
                                                _dev_ptr(self.grad), _stream_ptr(None)))

    def loss_and_grad(self, llr: torch.Tensor, cw: torch.Tensor, weights: Optional[torch.Tensor] = None):
        """Loss and dloss/dw of one batch (mean over iterations, codewords, columns)."""
        self.loss.zero_()
        self.grad.zero_()
        n = llr.shape[0]
        self.forward(llr, cw, 1.0 / (self.T * n * self.dec.n_bp), weights=weights)
        self.backward(n, weights=weights)
        torch.cuda.synchronize()
        return float(self.loss.item()), self.grad.clone()

    # ---- training -----------------------------------------------------------------------
    def step(self) -> float:
        self.loss.zero_()
        self.grad.zero_()
        scale = 1.0 / (self.T * self.batch * self.dec.n_bp)
        lo, hi = self.ebn0_range
        for k in range(0, self.batch, self.chunk):
            n = min(self.chunk, self.batch - k)
            eb = lo + (hi - lo) * torch.rand(n, generator=self.gen, device=self.dec.device)
            sig = sigma_from_ebn0(eb, self.rate)
            base = (self.seed << 40) + self.step_count * self.batch + k
            llr, cw = self.dec.gen_llr(seed=self.seed, cw_base=base, sigma=sig)
            self.forward(llr, cw, scale)
            self.backward(n)
        self.step_count += 1
        _lib.check("nrldpc_adam_step",
                   self.lib.nrldpc_adam_step(self.w.numel(), _dev_ptr(self.w), _dev_ptr(self.grad),
                                             _dev_ptr(self.m), _dev_ptr(self.v), self.step_count,
                                             float(self.lr), 0.9, 0.999, 1e-8, 0.0, _stream_ptr(None)))
        return float(self.loss.item())

    def train(self, steps: int, log_every: int = 0):
        hist = []
        for i in range(steps):
            hist.append(self.step())
            if log_every and (i % log_every == 0 or i == steps - 1):
                print(f"step {i:5d} loss {hist[-1]:.6f}", flush=True)
        return hist

    def weights(self) -> np.ndarray:
        return self.w.detach().cpu().numpy()

    def save(self, path: str, meta: Optional[dict] = None):
        np.save(path + ".npy", self.weights())
        info = dict(bg=self.bg, z=self.z, n_iter=self.T, batch=self.batch, lr=self.lr, schedule=self.schedule,
                    ebn0_range=list(self.ebn0_range), seed=self.seed, steps=self.step_count)
        info.update(meta or {})
        with open(path + ".json", "w") as f:
            json.dump(info, f, indent=1)


def load_weights(name: str) -> np.ndarray:
    """Committed trained weights, e.g. ``bg1_T8`` -> weights/bg1_T8.npy."""
    return np.load(os.path.join(WEIGHTS_DIR, name + ".npy"))
