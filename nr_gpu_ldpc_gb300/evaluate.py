"""FER/BER measurement on the GPU with Clopper-Pearson confidence intervals.

Codewords, channel and decoding all run on the GPU (nrldpc_gen_llr,
nrldpc_decode[_weighted], nrldpc_count_errors); only the four counters come
back.  The reference counts errors over the info bits of each codeword
(src/encoding_tools.cpp:112-155); so does this.

    python -m nr_gpu_ldpc_gb300.evaluate --bg 1 --z 384 --ebn0 1.5 2.0 --iters 10 \
        [--weights bg1_T8] [--schedule layered] [--frames 100000] [--early-stop]

    python -m nr_gpu_ldpc_gb300.evaluate --compare   # the learned-vs-plain table:
        BG1 Z=384, batch 16384, Eb/N0 1.0..2.0 dB, early stop on: plain
        flooding min-sum at 10 iterations, the learned layered decoder
        (weights/bg1_L6) at 4, 5, 6 iterations, the layered decoder without
        weights at 6, until 100 frame errors or 2^20 frames per point.
"""
from __future__ import annotations

import argparse
import json
import math
from typing import Optional

import numpy as np
import torch

from .decoder import Decoder
from .learned import load_weights, sigma_from_ebn0


def _beta_ppf(q: float, a: float, b: float) -> float:
    """Quantile of Beta(a, b) by bisection on the regularized incomplete beta
    (scipy when available)."""
    try:
        from scipy.stats import beta
        return float(beta.ppf(q, a, b))
    except ImportError:  # pragma: no cover - scipy is present in both images
        lo, hi = 0.0, 1.0
        from math import lgamma, exp, log
        def cdf(x, n=2000):
            xs = np.linspace(0, x, n)
            f = np.exp((a - 1) * np.log(np.maximum(xs, 1e-300)) + (b - 1) * np.log(np.maximum(1 - xs, 1e-300))
                       + lgamma(a + b) - lgamma(a) - lgamma(b))
            return float(np.trapz(f, xs))
        for _ in range(60):
            mid = (lo + hi) / 2
            lo, hi = (mid, hi) if cdf(mid) < q else (lo, mid)
        return (lo + hi) / 2


def clopper_pearson(k: int, n: int, conf: float = 0.95):
    """Exact binomial confidence interval for k successes in n trials."""
    if n == 0:
        return 0.0, 1.0
    a = (1 - conf) / 2
    lo = 0.0 if k == 0 else _beta_ppf(a, k, n - k + 1)
    hi = 1.0 if k == n else _beta_ppf(1 - a, k + 1, n - k)
    return lo, hi


def measure(dec: Decoder, ebn0_db: float, n_iter: int, frames: int, batch: int = 8192,
            early_stop: bool = False, weighted: bool = False, seed: int = 1,
            max_frame_errors: Optional[int] = None) -> dict:
    """Decode `frames` seeded codewords at one Eb/N0; return counts and rates."""
    rate = dec.kb / (dec.cols - 2) if dec.cols in (68, 52) else dec.kb / dec.cols
    dev = dec.device
    counts = torch.zeros(2, dtype=torch.int64, device=dev)
    iters_sum = torch.zeros(1, dtype=torch.int64, device=dev)
    out = torch.empty((batch, dec.packed_bytes), dtype=torch.uint8, device=dev)
    done = 0
    while done < frames:
        n = min(batch, frames - done)
        sig = sigma_from_ebn0(torch.full((n,), float(ebn0_db), device=dev), rate)
        llr, cw = dec.gen_llr(seed=seed, cw_base=(int(ebn0_db * 1000) << 32) + done, sigma=sig)
        pk, its = dec.decode(llr, n_iter, early_stop=early_stop, weighted=weighted, want_iters=True,
                             out=out[:n])
        dec.count_errors(pk, cw, counts=counts)
        iters_sum += its.sum()
        done += n
        if max_frame_errors is not None and int(counts[1].item()) >= max_frame_errors:
            break
    be, fe = (int(x) for x in counts.tolist())
    lo, hi = clopper_pearson(fe, done)
    return {"ebn0_db": ebn0_db, "frames": done, "frame_errors": fe, "bit_errors": be,
            "fer": fe / done, "fer_ci95": [lo, hi], "ber": be / (done * dec.n_info),
            "avg_iters": int(iters_sum.item()) / done}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--bg", type=int, default=1)
    ap.add_argument("--z", type=int, default=384)
    ap.add_argument("--ebn0", type=float, nargs="+", default=[1.5, 1.75, 2.0])
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--frames", type=int, default=65536)
    ap.add_argument("--early-stop", action="store_true")
    ap.add_argument("--weights", default=None, help="committed weight file name (weights/<name>.npy)")
    ap.add_argument("--schedule", default="flooding", choices=["flooding", "layered"])
    ap.add_argument("--compare", action="store_true", help="the learned-vs-plain FER table")
    args = ap.parse_args()
    if args.compare:
        compare()
        return
    dec = Decoder(bg=args.bg, z=args.z, max_batch=8192)
    dec.set_schedule(args.schedule)
    if args.weights:
        dec.set_weights(load_weights(args.weights))
    for eb in args.ebn0:
        r = measure(dec, eb, args.iters, args.frames, early_stop=args.early_stop,
                    weighted=args.weights is not None)
        print(json.dumps(r), flush=True)


def compare(ebn0=(1.0, 1.25, 1.5, 1.6, 1.7, 1.8, 1.9, 2.0), max_frames: int = 1 << 20, min_errors: int = 100,
            batch: int = 16384):
    """FER of plain min-sum (flooding, 10 iterations) against the learned
    layered decoder at 4/5/6 iterations and the layered decoder without
    weights, early stop on; one JSON line per (decoder, Eb/N0)."""
    dec = Decoder(bg=1, z=384, max_batch=batch)
    configs = [("plain flooding", "flooding", None, 10), ("learned layered", "layered", "bg1_L6", 4),
               ("learned layered", "layered", "bg1_L6", 5), ("learned layered", "layered", "bg1_L6", 6),
               ("layered alpha 0.75", "layered", None, 6)]
    for name, sched, weights, iters in configs:
        dec.set_schedule(sched)
        if weights:
            dec.set_weights(load_weights(weights))
        for eb in ebn0:
            r = measure(dec, eb, iters, max_frames, batch=batch, early_stop=True, weighted=weights is not None,
                        max_frame_errors=min_errors)
            r.update(decoder=name, schedule=sched, weights=weights or "alpha 0.75", iters_max=iters)
            print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
