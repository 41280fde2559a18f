"""Replica bookkeeping for runs on N GPUs of one node (torchrun, one process
per GPU).

The transport path has no exchange step: every rank renders its own view
(its own seed and RNG view index) and the ranks meet only to agree on the
timing.  The whole job's rate is all ranks' samples over the slowest rank's
time.  With `dist` None (one process) every helper is the identity.
"""
from __future__ import annotations

import os


def rank_info() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment"""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def view_seed(base_seed: int, rank: int) -> int:
    """seed of the view a rank renders: one independent replica per rank"""
    return base_seed + rank


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def max_over_ranks(x: float, dist, device: str = "cuda") -> float:
    """the largest value of x over the ranks (timings: the slowest rank)"""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(samples_per_rank: float, seconds_max: float, world: int) -> float:
    """all ranks' samples over the slowest rank's time (weak scaling: the
    per-rank work is fixed as the world grows)"""
    return world * samples_per_rank / seconds_max


def split_samples(spp: int, rank: int, world: int) -> tuple[int, int]:
    """(first sample, count) of a rank's share of one view's spp samples per
    pixel: contiguous ranges of the view's sample stream"""
    base, extra = divmod(spp, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def sum_over_ranks(t, dist):
    """in-place all-reduce sum of a tensor (per-pixel sums of a view whose
    samples were split across ranks, or gradients of the adjoint)"""
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t
