"""Replica bookkeeping for runs on several GPUs of one node.

The FEM path does not shard: one system runs on one GPU, and more GPUs run
independent replicas (the same solve, or disjoint groups of batched
instances) with no collective on the data path.  The only cross-rank steps
are the benchmark's barrier and the maximum of the per-rank times.  Ranks
are launched by torchrun; the environment gives RANK, WORLD_SIZE and
LOCAL_RANK.
"""
from __future__ import annotations

import os


def world():
    """(rank, world_size, local_rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str = "nccl"):
    """Join the process group when there is more than one rank."""
    import torch.distributed as dist
    rank, size, _ = world()
    if size > 1 and not dist.is_initialized():
        dist.init_process_group(backend)
    return rank, size


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(values, device=None):
    """Element-wise maximum of a list of floats over all ranks (the values
    themselves on a single rank).  `device` holds the exchange tensor: the
    rank's GPU under NCCL, the CPU under gloo."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def shard(n: int, rank: int, size: int) -> range:
    """Contiguous, balanced share [a, b) of n independent items for a rank."""
    a = (n * rank) // size
    b = (n * (rank + 1)) // size
    return range(a, b)


def finalize():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
