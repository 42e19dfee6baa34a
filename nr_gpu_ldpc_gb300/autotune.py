"""Autotuner for codewords per CTA, per (BG, Z).

The decode CTA holds `cw_per_cta` codewords of one code (threads = cw_per_cta
* Z, at most 384; two fp32 posterior buffers over each codeword's core columns
in shared memory, two CTAs per SM).
Fewer codewords per CTA balance early-stopping codewords better; more keep
the SM busier.  For each code this times the persistent batch decode of a
homogeneous job list at every admissible value and keeps the fastest; the
table is stored per GPU model and applied by ``Batch``/``Decoder``.

    python -m nr_gpu_ldpc_gb300.autotune [--z 64 96 128 ...] [--iters 10] [--out PATH]
"""
from __future__ import annotations

import argparse
import json
import os
from typing import Optional

import numpy as np
import torch

TUNING_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning")


def table_path(device: int = 0) -> str:
    name = torch.cuda.get_device_name(device).replace(" ", "_")
    return os.path.join(TUNING_DIR, f"{name}.json")


def load_table(device: int = 0) -> dict:
    """{(bg, z): cw_per_cta} for this GPU model, or {} if not tuned."""
    try:
        path = table_path(device)
    except Exception:
        return {}
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        d = json.load(f)
    return {(e["bg"], e["z"]): e["cw_per_cta"] for e in d["entries"]}


def tune(zs=(64, 96, 128, 192, 256, 320, 384), bgs=(1, 2), n_iter: int = 10, ebn0: float = 2.0,
         early_stop: bool = True, device: int = 0, reps: int = 5, verbose: bool = True):
    from .batch import Batch, make_jobs
    from .learned import sigma_from_ebn0
    dev = torch.device("cuda", device)
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    entries = []
    for bg in bgs:
        for z in zs:
            probe = Batch(max_jobs=1, device=device)
            max_cpb = probe.get_cw_per_cta(bg, z)
            probe.close()
            n = sms * max_cpb * 8
            rate = (22 if bg == 1 else 10) / (66 if bg == 1 else 50)
            sig = float(sigma_from_ebn0(torch.tensor([ebn0]), rate)[0])
            jobs, n_llr, n_e, n_out = make_jobs(np.full(n, bg), z, sigma=sig)
            best = None
            for cpb in sorted({1, 2, 3, 4, 6, 8, 12, max_cpb}):
                if cpb > max_cpb:
                    continue
                b = Batch(max_jobs=n, device=device)
                b.set_cw_per_cta(bg, z, cpb)
                b.set_jobs(jobs)
                llr_e = torch.empty(n_e, device=dev)
                cw = torch.empty(n_out, dtype=torch.uint8, device=dev)
                b.gen(3, 0, llr_e, cw)
                llr = torch.empty(n_llr, device=dev)
                b.derate(llr_e, llr)
                out = torch.empty(n_out, dtype=torch.uint8, device=dev)
                b.decode(llr, out, n_iter, early_stop)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    b.decode(llr, out, n_iter, early_stop)
                e1.record()
                torch.cuda.synchronize()
                us = e0.elapsed_time(e1) * 1e3 / reps / n
                if verbose:
                    print(f"bg{bg} z{z} cw_per_cta {cpb}: {us:.4f} us/cw", flush=True)
                if best is None or us < best[1]:
                    best = (cpb, us)
                b.close()
            entries.append({"bg": bg, "z": z, "cw_per_cta": best[0], "us_per_cw": best[1]})
    return {"device": torch.cuda.get_device_name(device), "n_iter": n_iter, "ebn0_db": ebn0,
            "early_stop": early_stop, "entries": entries}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--z", type=int, nargs="+", default=[64, 96, 128, 192, 256, 320, 384])
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    res = tune(tuple(args.z), n_iter=args.iters)
    path = args.out or table_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(res, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
