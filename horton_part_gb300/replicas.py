"""Job-level replicas over several GPUs (one process per GPU).

Molecules are independent, so the multi-GPU form of the partitioning loop
needs no collective on its data path: each rank owns whole jobs. The only
cross-rank steps are host-side: a barrier around timed regions and the
maximum (or sum) of per-rank scalars. In-molecule point sharding (which
would need an all-reduce of the per-atom moments every inner iteration) is
not built.

Launch with ``torchrun`` (RANK / WORLD_SIZE / LOCAL_RANK / MASTER_ADDR from
the environment); the backend is NCCL on GPUs and gloo on CPU.
"""

from __future__ import annotations

import os

__all__ = ["env", "init", "shard", "barrier", "reduce_max", "reduce_sum", "finalize"]


def env():
    """(world_size, rank, local_rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend=None):
    """Join the process group when WORLD_SIZE > 1; returns (world, rank, local)."""
    world, rank, local = env()
    if world > 1:
        import torch
        import torch.distributed as dist

        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return world, rank, local


def shard(items, rank, world):
    """The items owned by ``rank``: every world-th item starting at ``rank``
    (each item exactly once over all ranks; sizes differ by at most one)."""
    return list(items)[rank::world]


def _active():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier():
    dist = _active()
    if dist is not None:
        dist.barrier()


def _reduce(value, op):
    dist = _active()
    if dist is None:
        return float(value)
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def reduce_max(value):
    """Maximum of a per-rank scalar over all ranks (the value itself alone)."""
    dist = _active()
    return _reduce(value, dist.ReduceOp.MAX if dist else None)


def reduce_sum(value):
    dist = _active()
    return _reduce(value, dist.ReduceOp.SUM if dist else None)


def finalize():
    dist = _active()
    if dist is not None:
        dist.destroy_process_group()
