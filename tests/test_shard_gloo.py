"""Multi-GPU host logic on CPU ranks (gloo, world size 2): an ensemble split
into contiguous member shards, each shard seeded with the streams the full
ensemble would give its members, gathers to exactly the unsharded result.
The per-rank work is run by the CPU oracle, standing in for one GPU each:
through the helpers directly, and through ``sharded_features``, the
one-ensemble entry point, with an oracle-backed stand-in for each rank's
feature simulator."""
import os
import socket

import numpy as np
import pytest

from clode_gb300.shard import member_range, seeded_rng_state, shard_rng_state


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _scenario_inputs(n=96):
    rng = np.random.default_rng(17)
    pars = np.stack([rng.uniform(0.1, 2, n), np.zeros(n), rng.uniform(0.1, 1, n)], axis=1)
    return np.zeros((n, 1)), pars


def _run_members(x0, pars, rng_state):
    from oracle.build import OracleConfig
    from oracle.runner import OracleSimulator
    from clode_gb300 import rhs_path

    cfg = OracleConfig(rhs_path("ornstein_uhlenbeck.cl"), n_var=1, n_par=3, n_wiener=1, stepper="seuler",
                       single_precision=True)
    s = OracleSimulator(cfg, nthreads=1)
    s.set_solver_params(dt=1e-3, max_steps=2000)
    s.set_problem_data(x0, pars)
    s.rng[:] = rng_state
    s.set_tspan((0.0, 1.0))
    s.transient()
    return s.get_xf(), s.rng.reshape(2, -1).T.copy()


def _worker(rank, world, port, q):
    import torch.distributed as dist

    from clode_gb300.shard import gather_members

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x0, pars = _scenario_inputs()
        n = x0.shape[0]
        i0, i1 = member_range(n, rank, world)
        xf, rs = _run_members(x0[i0:i1], pars[i0:i1], shard_rng_state(123, n, i0, i1))
        xf_all = gather_members(xf)
        rs_all = gather_members(rs)
        if rank == 0:
            q.put((xf_all, rs_all))
    finally:
        dist.destroy_process_group()


def test_member_range_partitions():
    for n in (0, 1, 7, 100, 4096):
        for world in (1, 2, 3, 8):
            spans = [member_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(b - a for a, b in spans) - min(b - a for a, b in spans) <= 1


def test_shard_rng_state_matches_global_seeding():
    full = seeded_rng_state(-5, 10).reshape(2, 10)
    assert full[0, 0] == np.uint64(2**64 - 5)  # int32 -5 sign-extended (clode/cpp/CLODE.cpp:452)
    sh = shard_rng_state(-5, 10, 3, 7).reshape(2, 4)
    np.testing.assert_array_equal(sh, full[:, 3:7])


def test_two_gloo_ranks_reproduce_unsharded_run():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    x0, pars = _scenario_inputs()
    n = x0.shape[0]
    ref_xf, ref_rs = _run_members(x0, pars, seeded_rng_state(123, n))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    xf, rs = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    np.testing.assert_array_equal(xf, ref_xf)
    np.testing.assert_array_equal(rs, ref_rs)


class _OracleFeatureSim:
    """The slice of the feature simulator's interface that sharded_features
    uses, backed by the CPU oracle (a stand-in for one rank's GPU)."""

    def __init__(self):
        from clode_gb300 import rhs_path
        from oracle.build import OracleConfig
        from oracle.runner import OracleSimulator

        cfg = OracleConfig(rhs_path("lactotroph_noise.cl"), n_var=4, n_par=4, n_aux=1, n_wiener=1,
                           stepper="seuler", single_precision=True, observer="nhood2")
        self.s = OracleSimulator(cfg, nthreads=1)
        self.s.set_solver_params(dt=0.05, max_steps=1000000)
        self.s.set_observer_params(e_var_ix=3, f_var_ix=0, max_event_count=10000, nhood_radius=0.05)

    def set_problem_data(self, x0, pars):
        self.s.set_problem_data(np.asarray(x0).reshape(4, -1).T, np.asarray(pars).reshape(4, -1).T)

    def set_tspan_per_member(self, ts):
        self.s.set_tspan(np.asarray(ts).reshape(-1, 2))

    def set_tspan(self, ts):
        self.s.set_tspan(ts)

    def set_rng_state(self, words):
        self.s.rng[:] = words

    def features(self, reinit):
        self.s.features(reinit)

    def get_n_features(self):
        from oracle.runner import n_features
        return n_features("nhood2", 4, 1, 0)

    def get_f(self):
        return self.s.F.astype(np.float64)

    def get_xf(self):
        return self.s.xf.astype(np.float64)

    def get_tf(self):
        return self.s.get_tf()

    def get_dt(self):
        return self.s.get_dt()


def _noise_map(n=70):
    rng = np.random.default_rng(21)
    pars = np.stack([rng.uniform(0.5, 3.0, n), np.full(n, 3.0), rng.uniform(0.0, 2.0, n), np.full(n, 2.0)], axis=1)
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
    ts = np.stack([np.zeros(n), rng.uniform(100.0, 300.0, n)], axis=1)
    return x0, pars, ts


def _sharded_worker(rank, world, port, q):
    import torch.distributed as dist

    from clode_gb300.shard import sharded_features

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x0, pars, ts = _noise_map()
        out = sharded_features(_OracleFeatureSim(), x0, pars, ts, seed=77, per_member_tspan=True)
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


def test_sharded_features_entry_point_on_two_gloo_ranks():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from clode_gb300.shard import sharded_features

    x0, pars, ts = _noise_map()
    whole = sharded_features(_OracleFeatureSim(), x0, pars, ts, seed=77, per_member_tspan=True)
    assert whole["range"] == (0, x0.shape[0])
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_sharded_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    outs = dict(q.get(timeout=180) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert outs[0]["range"] == (0, 35) and outs[1]["range"] == (35, 70)
    for r in (0, 1):  # every rank holds the whole ensemble, equal to the unsharded run
        for k in ("F", "xf", "tf", "dt"):
            np.testing.assert_array_equal(outs[r][k], whole[k], err_msg=k)
