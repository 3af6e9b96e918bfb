"""Data-parallel replicas: one process per GPU, each running whole circuits on its own
rows, with no collective inside a step.

The gate-application path shards only along independent units -- batch rows of a
``QuantumDevice`` and independent circuits -- so several GPUs run as replicas: every
rank simulates its own rows end to end (forward, measurement, adjoint backward) and the
only cross-rank traffic is host-side bookkeeping: a barrier around timed regions and the
maximum of the ranks' times.  These helpers hold that bookkeeping so that it can be
exercised by multi-process CPU runs (gloo) as well as by the benchmark (NCCL).
"""
from __future__ import annotations

import os
from typing import Optional, Tuple

import torch


def rank_env() -> Tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment (1 process if unset)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank environment: RANK={rank} WORLD_SIZE={world}")
    return rank, world, local


def init(backend: str, timeout_s: Optional[float] = None) -> bool:
    """Join the process group when more than one rank runs; returns True if it did.
    ``timeout_s`` bounds every collective (a rank that leaves or never arrives then
    surfaces as an error on the others instead of a hang)."""
    _, world, _ = rank_env()
    if world == 1:
        return False
    import datetime

    import torch.distributed as dist

    if not dist.is_initialized():
        kw = {"timeout": datetime.timedelta(seconds=timeout_s)} if timeout_s else {}
        dist.init_process_group(backend, **kw)
    return True


def shard(total: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous share (start, count) of ``total`` independent units for ``rank``; shares
    differ by at most one unit and cover every unit exactly once."""
    if total < 0 or world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad shard request: total={total} rank={rank} world={world}")
    base, extra = divmod(total, world)
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def rank_seed(base: int, rank: int) -> int:
    """Seed of a rank's synthetic inputs: distinct per rank, reproducible per run."""
    return base + 1000003 * rank


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value: float, device: Optional[torch.device] = None) -> float:
    """Largest ``value`` over the ranks (the job's time is its slowest replica's)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job rate: units processed by all ranks over the slowest rank's time."""
    if seconds <= 0:
        raise ValueError("seconds must be positive")
    return units_per_rank * world / seconds


def finish() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()
        dist.destroy_process_group()
