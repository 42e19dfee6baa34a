"""Autotuner of the mixed-batch launch geometry per (BG, Z): codewords per
CTA and threads per codeword.

The decode CTA holds `cw_per_cta` codewords of one code, each taken by
Z / spt threads that own spt sub-rows apiece (spt = 1 or 2, "sub-rows per
thread"; at most 384 threads per CTA; two fp32 posterior buffers over each
codeword's core columns in shared memory).  Fewer codewords per CTA balance
early-stopping codewords better; more keep the SM busier; two sub-rows per
thread halve the threads a codeword needs at the cost of more work per
thread.  The batch's CTA has the threads of its widest work item, so the
best point for a code depends on what it is decoded with:

* ``tune`` times each code alone (a homogeneous batch, whose CTA is as wide
  as that code's work items) at every admissible (spt, cw_per_cta);
* ``tune_workload`` tunes a given job list, coordinate by coordinate: for
  each code present (largest work first) every admissible point is timed on
  the whole batch with the other codes at their current points.

The table is stored per GPU model and applied by ``Batch`` (both knobs) and
``Decoder`` (codewords per CTA, where the tuned point has one sub-row per
thread).

    python -m nr_gpu_ldpc_gb300.autotune [--z 64 96 ...] [--iters 10] [--out PATH]
    python -m nr_gpu_ldpc_gb300.autotune --workload mixed [--out PATH]
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np
import torch

TUNING_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning")


def table_path(device: int = 0) -> str:
    name = torch.cuda.get_device_name(device).replace(" ", "_")
    return os.path.join(TUNING_DIR, f"{name}.json")


def load_table(device: int = 0) -> dict:
    """{(bg, z): (cw_per_cta, sub_rows_per_thread)} for this GPU model, or {}
    if not tuned."""
    try:
        path = table_path(device)
    except Exception:
        return {}
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        d = json.load(f)
    return {(e["bg"], e["z"]): (e["cw_per_cta"], e.get("sub_rows_per_thread", 1)) for e in d["entries"]}


def candidates(max_cpb: int):
    """Codewords-per-CTA values tried up to the largest admissible one."""
    return sorted(c for c in {1, 2, 3, 4, 6, 8, 12, max_cpb} if c <= max_cpb)


def _points(batch, bg: int, z: int, spts=(1, 2)):
    """Every admissible (spt, cw_per_cta) of one code."""
    pts = []
    for spt in spts:
        if z % spt:
            continue
        batch.set_sub_rows_per_thread(bg, z, spt)
        batch.set_cw_per_cta(bg, z, 0)
        pts += [(spt, c) for c in candidates(batch.get_cw_per_cta(bg, z))]
    return pts


def _time_decode(batch, llr, out, n_iter: int, early_stop: bool, reps: int) -> float:
    """Milliseconds per decode of the loaded job list (CUDA events)."""
    batch.decode(llr, out, n_iter, early_stop)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        batch.decode(llr, out, n_iter, early_stop)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune(zs=(64, 96, 128, 192, 256, 320, 384), bgs=(1, 2), n_iter: int = 10, ebn0: float = 2.0,
         early_stop: bool = True, device: int = 0, reps: int = 5, spts=(1, 2), waves: int = 8,
         verbose: bool = True):
    """Each code alone: a homogeneous batch of `waves` CTA rounds timed at
    every admissible point; the fastest is kept."""
    from .batch import Batch, make_jobs
    from .learned import sigma_from_ebn0
    dev = torch.device("cuda", device)
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    entries = []
    for bg in bgs:
        for z in zs:
            b = Batch(max_jobs=1, device=device)
            pts = _points(b, bg, z, spts)
            b.set_sub_rows_per_thread(bg, z, 1)
            b.set_cw_per_cta(bg, z, 0)
            n = sms * b.get_cw_per_cta(bg, z) * waves
            b.close()
            rate = (22 if bg == 1 else 10) / (66 if bg == 1 else 50)
            sig = float(sigma_from_ebn0(torch.tensor([ebn0]), rate)[0])
            jobs, n_llr, n_e, n_out = make_jobs(np.full(n, bg), z, sigma=sig)
            b = Batch(max_jobs=n, device=device)
            b.set_jobs(jobs)
            llr_e = torch.empty(n_e, device=dev)
            cw = torch.empty(n_out, dtype=torch.uint8, device=dev)
            b.gen(3, 0, llr_e, cw)
            llr = torch.empty(n_llr, device=dev)
            b.derate(llr_e, llr)
            out = torch.empty(n_out, dtype=torch.uint8, device=dev)
            tried = []
            for spt, cpb in pts:
                b.set_sub_rows_per_thread(bg, z, spt)
                b.set_cw_per_cta(bg, z, cpb)
                b.set_jobs(jobs)
                us = _time_decode(b, llr, out, n_iter, early_stop, reps) * 1e3 / n
                tried.append({"sub_rows_per_thread": spt, "cw_per_cta": cpb, "us_per_cw": us})
                if verbose:
                    print(f"bg{bg} z{z} spt {spt} cw_per_cta {cpb}: {us:.4f} us/cw", flush=True)
            b.close()
            best = min(tried, key=lambda t: t["us_per_cw"])
            entries.append({"bg": bg, "z": z, "sub_rows_per_thread": best["sub_rows_per_thread"],
                            "cw_per_cta": best["cw_per_cta"], "us_per_cw": best["us_per_cw"], "tried": tried})
    return {"device": torch.cuda.get_device_name(device), "mode": "each code alone", "n_iter": n_iter,
            "ebn0_db": ebn0, "early_stop": early_stop, "entries": entries}


def tune_workload(bg, z, k_prime, e, sigma, n_iter: int = 10, early_stop: bool = True, device: int = 0,
                  reps: int = 3, spts=(1, 2), passes: int = 1, start=None, verbose: bool = True):
    """A given job list (arrays of BG, Z, K', E, sigma), coordinate by
    coordinate: for each code present, largest total work first, every
    admissible point timed on the whole batch with the other codes at their
    current points (`start`: {(bg, z): (cpb, spt)}, else the defaults)."""
    from .batch import Batch, make_jobs
    dev = torch.device("cuda", device)
    jobs, n_llr, n_e, n_out = make_jobs(bg, z, k_prime, e, 0, sigma)
    b = Batch(max_jobs=len(jobs), device=device)
    codes = sorted({(int(x), int(y)) for x, y in zip(bg, z)},
                   key=lambda c: -sum(1 for x, y in zip(bg, z) if (x, y) == c) * c[1] * (316 if c[0] == 1 else 197))
    cur = {}
    for c in codes:
        cpb, spt = (start or {}).get(c, (0, 1))
        b.set_sub_rows_per_thread(*c, spt)
        b.set_cw_per_cta(*c, cpb)
        cur[c] = (b.get_sub_rows_per_thread(*c), b.get_cw_per_cta(*c))
    b.set_jobs(jobs)
    llr_e = torch.empty(n_e, device=dev)
    cw = torch.empty(n_out, dtype=torch.uint8, device=dev)
    b.gen(9, 0, llr_e, cw)
    llr = torch.empty(n_llr, device=dev)
    b.derate(llr_e, llr)
    out = torch.empty(n_out, dtype=torch.uint8, device=dev)
    base_ms = _time_decode(b, llr, out, n_iter, early_stop, reps)
    tried = {c: [] for c in codes}
    best_ms = base_ms
    for _ in range(passes):
        for c in codes:
            for spt, cpb in _points(b, *c, spts):
                b.set_sub_rows_per_thread(*c, spt)
                b.set_cw_per_cta(*c, cpb)
                b.set_jobs(jobs)
                ms = _time_decode(b, llr, out, n_iter, early_stop, reps)
                tried[c].append({"sub_rows_per_thread": spt, "cw_per_cta": cpb, "batch_ms": ms})
                if verbose:
                    print(f"bg{c[0]} z{c[1]} spt {spt} cw_per_cta {cpb}: batch {ms:.4f} ms", flush=True)
                if ms < best_ms:
                    best_ms, cur[c] = ms, (spt, cpb)
            b.set_sub_rows_per_thread(c[0], c[1], cur[c][0])
            b.set_cw_per_cta(c[0], c[1], cur[c][1])
    b.close()
    entries = [{"bg": c[0], "z": c[1], "sub_rows_per_thread": cur[c][0], "cw_per_cta": cur[c][1],
                "tried": tried[c]} for c in sorted(codes)]
    return {"device": torch.cuda.get_device_name(device), "mode": "workload", "n_iter": n_iter,
            "early_stop": early_stop, "codewords": len(jobs), "batch_ms_default": base_ms,
            "batch_ms_tuned": best_ms, "entries": entries}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--z", type=int, nargs="+", default=[64, 96, 128, 192, 256, 320, 384])
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--workload", choices=["mixed"], default=None,
                    help="tune on the uneven 8192-codeword mix instead of each code alone")
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    if args.workload == "mixed":
        from .batch import mixed_workload
        res = tune_workload(*mixed_workload(), n_iter=args.iters)
        res["workload"] = "8192 codewords, BG1/BG2, Z in {64..384}, rate-matched, Eb/N0 U[1,3] dB"
    else:
        res = tune(tuple(args.z), n_iter=args.iters)
    path = args.out or table_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(res, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
