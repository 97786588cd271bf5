"""Process-group helpers for running the engine on several GPUs.

The force-and-integrate path has no exchange step between independent
systems, so N GPUs run N independent replicas (or disjoint shards of an
ensemble); the only collectives are the barrier and max/sum reductions that
bracket a timed region.  Works with NCCL on GPUs and gloo on CPUs.
"""
from __future__ import annotations

import os


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None):
    """Initialise torch.distributed from the torchrun environment when
    WORLD_SIZE > 1; returns (rank, world, local_rank)."""
    rank, world, local = env_rank()
    if world > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
    return rank, world, local


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier():
    d = _dist()
    if d is not None:
        d.barrier()


def _reduce(x: float, op: str) -> float:
    d = _dist()
    if d is None:
        return float(x)
    import torch
    dev = "cuda" if d.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=getattr(d.ReduceOp, op))
    return float(t.item())


def max_over_ranks(x: float) -> float:
    return _reduce(x, "MAX")


def sum_over_ranks(x: float) -> float:
    return _reduce(x, "SUM")


def shard(n_items: int, rank: int, world: int):
    """Contiguous block [lo, hi) of n_items owned by rank (ensemble systems)."""
    per, extra = divmod(n_items, world)
    lo = rank * per + min(rank, extra)
    hi = lo + per + (1 if rank < extra else 0)
    return lo, hi


def finalize():
    d = _dist()
    if d is not None:
        d.destroy_process_group()
