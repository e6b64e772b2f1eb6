"""``sharded_features`` (one ensemble split over ranks) with the GPU feature
simulator: the ranks of a 2- and a 3-rank split are run one after the other
in this process, each through the entry point with the process group's
rank and size set for it and the gather replaced by returning the rank's own
rows; their rows, concatenated in rank order, must equal the whole ensemble
run as one rank, bit for bit.  The model is stochastic (the lactotroph with
a noise current under stochastic Euler) and the ensemble size is not a
multiple of the ranks, so each shard must draw exactly the random streams
the whole ensemble gives its members.  The exchange between real ranks (the
gather over gloo) is covered on CPU ranks."""
import numpy as np
import pytest

from clode_gb300 import clode_cpp_wrapper as W, rhs_path, shard

pytestmark = pytest.mark.gpu

VARS = ["v", "n", "f", "c"]
PARS = ["gcal", "gsk", "gbk", "sig"]


def _sim():
    pi = W.ProblemInfo(rhs_path("lactotroph_noise.cl"), VARS, PARS, ["ica"], 1)
    op = W.ObserverParams(e_var_ix=3, f_var_ix=0, max_event_count=100000, nhood_radius=0.05,
                          x_up_threshold=0.3, x_down_threshold=0.2)
    sim = W.FeatureSimulatorBase(pi, "seuler", "nhood2", op, True, W.OpenCLResource(), "")
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=0.01, dtmax=1.0, abstol=1e-6, reltol=1e-6, max_steps=10000000))
    return sim


def _inputs(n):
    """The last n // 2 members repeat the parameters and spans of the first n // 2 (only the noise differs)."""
    r = np.random.default_rng(21)
    m = n - n // 2
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
    pars = np.stack([r.uniform(0.5, 3.0, m), np.full(m, 3.0), r.uniform(0.0, 2.0, m), np.full(m, 2.0)], axis=1)
    ts = np.stack([np.zeros(m), r.uniform(200.0, 800.0, m)], axis=1)
    return x0, np.concatenate([pars, pars])[:n], np.concatenate([ts, ts])[:n]


class _Rank:
    """torch.distributed as one rank of a group of `world` sees it."""

    def __init__(self, rank, world):
        self.rank, self.world = rank, world

    def is_available(self):
        return True

    def is_initialized(self):
        return True

    def get_rank(self, group=None):
        return self.rank

    def get_world_size(self, group=None):
        return self.world


@pytest.mark.parametrize("world", [2, 3])
def test_shards_on_the_gpu_equal_the_whole_ensemble(world, monkeypatch):
    import torch.distributed as dist

    n = 2001
    x0, pars, ts = _inputs(n)
    whole = shard.sharded_features(_sim(), x0, pars, ts, seed=9, per_member_tspan=True)
    assert whole["range"] == (0, n)

    monkeypatch.setattr(shard, "gather_members", lambda local, group=None: np.asarray(local))
    parts = []
    for rank in range(world):
        fake = _Rank(rank, world)
        for name in ("is_available", "is_initialized", "get_rank", "get_world_size"):
            monkeypatch.setattr(dist, name, getattr(fake, name))
        out = shard.sharded_features(_sim(), x0, pars, ts, seed=9, per_member_tspan=True)
        assert out["range"] == shard.member_range(n, rank, world)
        parts.append(out)
    for key in ("F", "xf", "tf", "dt"):
        got = np.concatenate([p[key] for p in parts], axis=0)
        assert got.shape == whole[key].shape
        assert np.array_equal(got, whole[key], equal_nan=True), key
    # the noise mattered: members with the same parameters and span but other streams differ
    h = n // 2
    assert np.mean(np.any(whole["xf"][:h] != whole["xf"][n - h:], axis=1)) > 0.9
