"""Multi-GPU host logic on CPU ranks (gloo, world size 2): an ensemble split
into contiguous member shards, each shard seeded with the streams the full
ensemble would give its members, gathers to exactly the unsharded result.
The per-rank work is run by the CPU oracle, standing in for one GPU each."""
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
