"""Process-group plumbing for running independent replicas of the solve on several GPUs.

The solve does not shard across GPUs in this library (one partition per GPU, no halo exchange):
N ranks run N independent replicas. The only cross-rank operations are a barrier around the
timed region and a max over ranks of the measured times (the slowest replica sets the job time).
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class Rank:
    rank: int = 0
    world: int = 1
    local_rank: int = 0
    initialized: bool = False


def init_from_env(backend: str | None = None) -> Rank:
    """Reads RANK/WORLD_SIZE/LOCAL_RANK (torchrun) and initialises torch.distributed when the
    world has more than one rank."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    if world <= 1:
        return Rank(0, 1, local, False)
    import torch
    import torch.distributed as td
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    if backend == "nccl":
        torch.cuda.set_device(local)
    td.init_process_group(backend=backend, rank=rank, world_size=world)
    return Rank(rank, world, local, True)


def barrier(r: Rank):
    if r.initialized:
        import torch.distributed as td
        td.barrier()


def max_over_ranks(r: Rank, value: float) -> float:
    if not r.initialized:
        return float(value)
    import torch
    import torch.distributed as td
    dev = "cuda" if td.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(r: Rank, value: float) -> float:
    if not r.initialized:
        return float(value)
    import torch
    import torch.distributed as td
    dev = "cuda" if td.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=td.ReduceOp.SUM)
    return float(t.item())


def finalize(r: Rank):
    if r.initialized:
        import torch.distributed as td
        td.destroy_process_group()
