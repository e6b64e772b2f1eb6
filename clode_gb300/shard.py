"""Member sharding of one ensemble over several GPUs (one process per GPU).

Ensemble members are independent, so a multi-GPU run is a contiguous split
of the member range with no exchange between ranks; results are gathered on
the host.  To make a sharded run identical to the unsharded one, each shard
must draw the random streams the full ensemble would give its members: the
reference seeds word k of the [j * nPts + i] state layout with ``seed + k``
(clode/cpp/CLODE.cpp:447-453), which depends on the global nPts, so
``shard_rng_state`` rebuilds that global layout for the shard's members.
"""
from __future__ import annotations

import numpy as np


def member_range(n_pts: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced [i0, i1) of members for ``rank`` out of ``world``."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of range for world size {world}")
    base, extra = divmod(n_pts, world)
    i0 = rank * base + min(rank, extra)
    return i0, i0 + base + (1 if rank < extra else 0)


def seeded_rng_state(seed: int, n_pts: int) -> np.ndarray:
    """The full ensemble's state after seed_rng(seed): word k = int32(seed + k), sign-extended."""
    k = np.arange(2 * n_pts, dtype=np.int64)
    v = ((int(seed) + k + 2**31) % 2**32) - 2**31
    return v.astype(np.int64).view(np.uint64)


def shard_rng_state(seed: int, n_pts: int, i0: int, i1: int) -> np.ndarray:
    """State words of members [i0, i1) of a seeded n_pts ensemble, in the shard's own layout."""
    full = seeded_rng_state(seed, n_pts).reshape(2, n_pts)
    return np.ascontiguousarray(full[:, i0:i1].ravel())


def gather_members(local: np.ndarray, group=None) -> np.ndarray:
    """Concatenate per-rank member rows (axis 0) in rank order on every rank."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, np.asarray(local), group=group)
    return np.concatenate(parts, axis=0)
