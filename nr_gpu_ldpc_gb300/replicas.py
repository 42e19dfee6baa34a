"""Replicas across GPUs: codewords are independent, so N processes (one per
GPU) each decode their own contiguous share of a batch with no collective on
the data path.  The only exchanges are host-side reductions of a few
counters (bit errors, frame errors, frames, iterations) and of step times.

The reference has no multi-GPU path (device 0 only,
src/cuda_gpu_wrapper/gpu_setup.cu:122); this module is what a job that
spreads a batch over several GPUs needs around the single-GPU decoder.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def shard(n_total: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous share (start, count) of n_total codewords for one rank;
    shares differ by at most one codeword and cover the batch exactly."""
    if world < 1 or not 0 <= rank < world or n_total < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(n_total, world)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def reduce_counts(counts, group=None) -> torch.Tensor:
    """Sum int64 counters over ranks (CPU tensors work with gloo; CUDA
    tensors with nccl).  Returns the reduced tensor (a copy)."""
    t = torch.as_tensor(counts, dtype=torch.int64).clone()
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


def max_over_ranks(value: float, device=None, group=None) -> float:
    """Largest value over ranks (the whole job's step time is its slowest rank's)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
