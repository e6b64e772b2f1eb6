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


def sharded_features(sim, x0: np.ndarray, pars: np.ndarray, tspan, seed: int, group=None,
                     per_member_tspan: bool = False) -> dict:
    """features() of one ensemble split over the ranks of a process group.

    Every rank passes the whole ensemble (``x0`` shaped (nPts, nVar), ``pars``
    (nPts, nPar), ``tspan`` a [t0, t1] pair or, with ``per_member_tspan``,
    (nPts, 2)) and its own feature simulator ``sim``, built on the rank's
    GPU with whatever solver, observer and engine options the run uses.  The
    rank integrates the contiguous member range ``member_range`` gives it,
    seeded with the random streams ``seed_rng(seed)`` gives those members in
    the whole ensemble, so that the gathered result equals the unsharded
    run's.  Results come back on every rank in member order: ``F`` (nPts,
    nFeatures), ``xf`` (nPts, nVar), ``tf`` and ``dt`` (nPts,), plus the
    rank's own range.  The only communication is the final gather of the
    results (``gather_members``); no data moves between ranks while they
    integrate.  Without an initialised process group it runs the whole
    ensemble on this rank.
    """
    import torch.distributed as dist

    x0 = np.asarray(x0, dtype=np.float64)
    pars = np.asarray(pars, dtype=np.float64)
    n = x0.shape[0]
    distributed = dist.is_available() and dist.is_initialized()
    rank = dist.get_rank(group) if distributed else 0
    world = dist.get_world_size(group) if distributed else 1
    i0, i1 = member_range(n, rank, world)
    m = i1 - i0
    if m > 0:
        sim.set_problem_data(np.ascontiguousarray(x0[i0:i1].flatten(order="F")),
                             np.ascontiguousarray(pars[i0:i1].flatten(order="F")))
        if per_member_tspan:
            sim.set_tspan_per_member(np.ascontiguousarray(np.asarray(tspan, dtype=np.float64)[i0:i1].ravel()))
        else:
            sim.set_tspan(list(np.asarray(tspan, dtype=np.float64)[:2]))
        sim.set_rng_state(shard_rng_state(seed, n, i0, i1))
        sim.features(True)
        nf = sim.get_n_features()
        local = {"F": np.asarray(sim.get_f()).reshape(nf, m).T,
                 "xf": np.asarray(sim.get_xf()).reshape(-1, m).T,
                 "tf": np.asarray(sim.get_tf()).reshape(m, 1),
                 "dt": np.asarray(sim.get_dt()).reshape(m, 1)}
    else:
        nf = sim.get_n_features()
        local = {"F": np.zeros((0, nf)), "xf": np.zeros((0, x0.shape[1])), "tf": np.zeros((0, 1)),
                 "dt": np.zeros((0, 1))}
    out = {"range": (i0, i1)}
    for k, v in local.items():
        g = gather_members(v, group) if distributed else v
        out[k] = g[:, 0] if k in ("tf", "dt") else g
    return out
