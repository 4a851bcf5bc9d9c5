"""Replica parallelism across processes: the reference's MPI pattern.

kim-jane/MCRG runs one independent chain per MPI rank, splits the sample
count with split_samples (src/definitions.cpp:79-87) and sums the moment
arrays with MPI_Allreduce(SUM) (src/mcrg.cpp:101-103).  Here every rank owns
one GPU and its own replicas (Philox replica word = global replica index),
and the exact integer moment sums are combined on the host with
torch.distributed (gloo or nccl process group).  The payload is a few KB, so
the sum is exchanged as Python integers (all_gather_object) and stays exact
beyond 64 bits.
"""
from __future__ import annotations

from .tmatrix import MomentSums


def split_samples(rank: int, n_processes: int, n_samples: int) -> int:
    """Samples owned by `rank`, as src/definitions.cpp:79-87 splits them
    (rank 0 takes the remainder, which can be <= 0)."""
    loc = -(-n_samples // n_processes)
    if rank == 0:
        loc = n_samples - (n_processes - 1) * loc
    return loc


def replica_ids(rank: int, world: int, n_replicas: int) -> list[int]:
    """Global replica indices owned by `rank` (round robin)."""
    return list(range(rank, n_replicas, world))


def allreduce_moments(m: MomentSums, group=None) -> MomentSums:
    """Exact sum of every rank's moment sums, returned on every rank."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return m
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, m, group=group)
    total = parts[0]
    for p in parts[1:]:
        total = total + p
    return total
