"""Replicas across GPUs: the step does not shard.

The reference's multi-GPU modes split one grid across devices (GSPMD or
shard_map with halo exchange); this implementation's path is single-GPU, so a
multi-GPU job runs independent replicas -- one simulation per rank, no data
exchange -- and only the timing is combined: the job's throughput is the sum
of all ranks' cell updates over the slowest rank's time.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def max_over_ranks(x: float, device=None) -> float:
    """Maximum of a per-rank float over the process group (identity without one)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    backend = dist.get_backend()
    dev = device if device is not None else (
        torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else "cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(cells_per_rank: int, steps: int, ms_local: float, world: int,
                   device=None) -> tuple[float, float]:
    """(Gcell-updates/s of the whole job, slowest rank's ms)."""
    ms = max_over_ranks(ms_local, device)
    return world * cells_per_rank * steps / (ms * 1e-3) / 1e9, ms
