"""Replica bookkeeping for runs over several GPUs of one node.

The evaluation path has no exchange step: every rank evaluates its own copy of the workload
(whole meshes or requests per GPU), so the only cross-rank operations are the start/stop
barrier and the timing reduction (the slowest rank's time), as the benchmark contract asks.
The collective runs on whatever backend the process group uses (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

import os


def world() -> tuple[int, int, int]:
    """(rank, local rank, world size) from the torchrun environment (1 process: 0, 0, 1)."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def init(backend: str):
    """Joins the process group when there is more than one rank; returns torch.distributed or
    None."""
    if world()[2] <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend)
    return dist


def max_over_ranks(dist, value: float, device="cpu") -> float:
    """The largest `value` over all ranks (the whole job ends with its slowest rank)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, ranks: int, seconds: float) -> float:
    """Whole-job throughput: every rank processed `units_per_rank` units in `seconds` (the
    slowest rank's time)."""
    return ranks * units_per_rank / seconds
