"""Data-parallel C&C-B sampling across processes, one GPU each.

Every rank replays the whole random stream of the requested samples from the
same numpy state (the replay is host-only and cheap) and samples only its slice
on its GPU; gathered in rank order, the slices are exactly the samples one
process would produce, and every rank's numpy generator ends where that single
process's would.  The only cross-rank traffic is the final gather of the
samples (a host-side collective over torch.distributed, gloo or NCCL).
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np

from . import _native


def shard(n_samples: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous slice of rank `rank`: (first, count); counts differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    per, rem = divmod(int(n_samples), world)
    first = rank * per + min(rank, rem)
    return first, per + (1 if rank < rem else 0)


def _rank_world(group) -> Tuple[int, int]:
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def gather_rows(local: np.ndarray, group=None) -> np.ndarray:
    """Concatenates every rank's rows in rank order (all ranks receive the result)."""
    import torch.distributed as dist

    rank, world = _rank_world(group)
    if world == 1:
        return local
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    return np.concatenate(parts, axis=0)


def gccb_sample_sharded(U: np.ndarray, input_state, weights, n_samples: int, group=None,
                        gather: bool = True) -> np.ndarray:
    """n_samples C&C-B samples (uniform losses when `weights` holds the particle-count
    weights) split over the ranks of `group`; returns all samples (gather=True) or
    this rank's slice."""
    rank, world = _rank_world(group)
    first, count = shard(n_samples, rank, world)
    local = _native.gccb_sample_slice(_native.as_matrix(U), input_state, weights, n_samples, first, count)
    return gather_rows(local, group) if gather else local
