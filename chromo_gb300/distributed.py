"""Replicas across ranks: one process per GPU, replicas only.

Replicas are independent simulations, so several GPUs share a workload by
splitting its replicas (contiguous blocks of whole chi ladders, so replica
exchange never crosses a rank) with no collective on the data path; the only
collectives are scalar reductions of timings and counts.  Launch with
``torch.distributed.run`` (RANK, WORLD_SIZE, LOCAL_RANK, MASTER_ADDR set);
NCCL on GPUs, gloo on CPU.
"""
import os
from typing import Tuple


def init(backend: str = "nccl") -> Tuple[int, int, int]:
    """(rank, world, local_rank) from the environment; joins the process group
    when world > 1 (and selects the local GPU for NCCL)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return rank, world, local


def shard(n_replicas: int, rank: int, world: int, ladder: int = 1) -> range:
    """Replicas of ``rank``: a contiguous block of whole ladders of ``ladder``
    replicas, blocks as equal as possible (the first ranks take one ladder
    more when they do not divide evenly)."""
    if ladder < 1 or n_replicas % ladder:
        raise ValueError("the ladder size must divide the number of replicas")
    n_lad = n_replicas // ladder
    base, extra = divmod(n_lad, world)
    start = rank * base + min(rank, extra)
    count = base + (1 if rank < extra else 0)
    return range(start * ladder, (start + count) * ladder)


def _device(backend: str):
    return "cuda" if backend == "nccl" else "cpu"


def allreduce(x: float, op: str, world: int, backend: str = "nccl") -> float:
    """Max or sum of a scalar over the ranks."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device(backend))
    dist.all_reduce(t, op={"max": dist.ReduceOp.MAX, "sum": dist.ReduceOp.SUM}[op])
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
