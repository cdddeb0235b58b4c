"""Independent replicas on N GPUs of one node (one process per GPU, launched by torchrun).

The hot path does not shard at one rank (the reference's multi-rank path exchanges halos, which this
build does not implement), so N GPUs run N independent sweeps of the same per-GPU workload
("scaling": "weak").  The only cross-rank operations are the timing barrier and the maximum of
the per-rank times; no collective touches the data path.
"""

from __future__ import annotations

import torch
import torch.distributed as dist


def barrier(world: int) -> None:
    if world > 1:
        dist.barrier()


def max_over_ranks(ms: float, world: int, device: str | torch.device = "cpu") -> float:
    """the slowest rank's time: the job's time"""
    if world <= 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank_step: int, steps: int, world: int, job_ms: float) -> float:
    """units of all ranks per second of the job's (slowest rank's) time"""
    return units_per_rank_step * steps * world / (job_ms * 1e-3)
