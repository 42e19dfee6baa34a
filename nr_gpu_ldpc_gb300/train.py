"""Train learned weighted min-sum weights on the GPU and save them.

    python -m nr_gpu_ldpc_gb300.train --bg 2 --z 128 --iters 8 --batch 16384 \
        --steps 400 --lr 1e-3 --out nr_gpu_ldpc_gb300/weights/bg2_T8

Defaults follow the training configuration the project is specified on:
8 unrolled iterations, weights initialised to 0.75, 16384 seeded codewords
per step at Eb/N0 uniform in [1, 3] dB, BCE on the posterior LLRs, Adam with
learning rate 1e-3.  --schedule layered trains the row-sequential decoder
(its own forward and adjoint kernels) instead of the flooding one.
"""
from __future__ import annotations

import argparse
import time

from .learned import Trainer


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--bg", type=int, default=2)
    ap.add_argument("--z", type=int, default=128)
    ap.add_argument("--iters", type=int, default=8)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--chunk", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--ebn0", type=float, nargs=2, default=[1.0, 3.0])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--schedule", default="flooding", choices=["flooding", "layered"])
    ap.add_argument("--out", required=True)
    args = ap.parse_args()
    tr = Trainer(bg=args.bg, z=args.z, n_iter=args.iters, batch=args.batch, chunk=args.chunk,
                 lr=args.lr, ebn0_range=tuple(args.ebn0), seed=args.seed, schedule=args.schedule)
    t0 = time.time()
    hist = tr.train(args.steps, log_every=max(1, args.steps // 20))
    dt = time.time() - t0
    tr.save(args.out, meta={"final_loss": hist[-1], "first_loss": hist[0], "seconds": dt,
                            "loss_every_10": hist[::10]})
    print(f"saved {args.out}.npy after {args.steps} steps in {dt:.1f} s, loss {hist[0]:.5f} -> {hist[-1]:.5f}")


if __name__ == "__main__":
    main()
