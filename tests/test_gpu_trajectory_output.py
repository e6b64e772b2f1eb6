"""Device regrouping of trajectories by member
(clode_sim_get_trajectory_by_member) and the per-member outputs built on it,
against the flat getters and the restatement of clODE's per-member loop
(oracle/trajectory_frontend.py, clode/trajectory.py:216-264).  Both read
the same device arrays, so every comparison is exact."""
import numpy as np
import pytest

from clode_gb300 import clode_cpp_wrapper as W, rhs_path
from clode_gb300.trajectory_output import get_trajectory
from oracle.trajectory_frontend import reference_get_trajectory, regroup_by_member

pytestmark = pytest.mark.gpu


def _lactotroph(single, n=300, max_store=400, nout=3):
    pi = W.ProblemInfo(rhs_path("lactotroph.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"], 0)
    sim = W.TrajectorySimulatorBase(pi, "dopri5", single, W.OpenCLResource(), "")
    sim.build_cl()
    rng = np.random.default_rng(11)
    pars = np.stack([rng.uniform(0.5, 3.0, n), np.full(n, 3.0), rng.uniform(0.0, 2.0, n)], axis=1)
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
    sim.set_solver_params(W.SolverParams(dt=0.1, dtmax=10.0, abstol=1e-6, reltol=1e-6, max_steps=100000,
                                         max_store=max_store, nout=nout))
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan([0.0, 150.0])
    sim.trajectory()
    return sim, pi


def _flat(sim, which):
    return {"t": sim.get_t(), "x": sim.get_x(), "dx": sim.get_dx(), "aux": sim.get_aux()}[which]


@pytest.mark.parametrize("single", [True, False])
def test_regroup_matches_flat_getters(single):
    sim, pi = _lactotroph(single)
    n, ms = 300, 400
    ns = sim.get_n_stored()
    assert ns.min() < ns.max() < ms  # ragged: adaptive steps differ per member
    for first, count, rows in ((0, n, None), (17, 101, 50), (299, 1, ms), (0, 0, 5)):
        got = sim.get_trajectory_by_member(first=first, count=count, rows=rows)
        r = got["t"].shape[1] if count else 0
        if rows is None and count:
            assert r == min(ms, int(ns[first:first + count].max()) + 1)
        assert np.array_equal(got["n_stored"], ns[first:first + count])
        for k, w in (("t", 1), ("x", 4), ("dx", 4), ("aux", 1)):
            want = regroup_by_member(_flat(sim, k), n, w, first, count, r)
            g = got[k].reshape(count, r, w)
            assert np.array_equal(g, want), k


def test_outputs_match_reference_loop():
    sim, pi = _lactotroph(True)
    ref = reference_get_trajectory(sim, pi.vars, pi.aux, 300, 400)
    ours = get_trajectory(sim)
    assert len(ours) == len(ref)
    for o, r in zip(ours, ref):
        assert np.array_equal(o.t, r["t"])
        assert o.x.dtype == r["x"].dtype
        assert np.array_equal(o.x, r["x"]) and np.array_equal(o.dx, r["dx"]) and np.array_equal(o.aux, r["aux"])


def test_regroup_in_several_chunks():
    # 65,536 OU members x 1,001 rows: 524 MB of doubles per array, staged in
    # 256 MB chunks, so every array takes two regroup launches
    n, steps, nout = 65536, 10000, 10
    pi = W.ProblemInfo(rhs_path("ornstein_uhlenbeck.cl"), ["x"], ["theta", "mu", "sigma"], [], 1)
    sim = W.TrajectorySimulatorBase(pi, "seuler", True, W.OpenCLResource(), "")
    sim.build_cl()
    rng = np.random.default_rng(5)
    pars = np.stack([rng.uniform(0.1, 2.0, n), np.zeros(n), rng.uniform(0.1, 1.0, n)], axis=1)
    sim.set_solver_params(W.SolverParams(dt=1e-3, max_steps=steps, max_store=steps // nout + 2, nout=nout))
    sim.set_problem_data(np.zeros(n), pars.flatten(order="F"))
    sim.seed_rng(1)
    sim.set_tspan([0.0, 100.0])
    sim.trajectory()
    ns = sim.get_n_stored()
    assert (ns == steps // nout).all()
    got = sim.get_trajectory_by_member()
    rows = got["t"].shape[1]
    assert rows == steps // nout + 1
    for k in ("t", "x", "dx"):
        want = regroup_by_member(_flat(sim, k), n, 1, 0, n, rows)[:, :, 0]
        assert np.array_equal(got[k].reshape(n, rows), want), k
    assert "aux" not in got


def test_regroup_rejects_bad_ranges():
    sim, _ = _lactotroph(True, n=40, max_store=50)
    with pytest.raises(Exception):
        sim.get_trajectory_by_member(first=30, count=11)
    with pytest.raises(Exception):
        sim.get_trajectory_by_member(rows=51)
    with pytest.raises(Exception):
        sim.get_trajectory_by_member(first=-1, count=3)


def test_getters_stay_within_the_stored_run():
    # max_store raised after the run: the getters return the rows the run's
    # buffers hold, never more, until the next run resizes them
    sim, _ = _lactotroph(True, n=40, max_store=50)
    t_before = sim.get_t()
    assert t_before.size == 50 * 40
    sim.set_solver_params(W.SolverParams(dt=0.1, dtmax=10.0, abstol=1e-6, reltol=1e-6, max_steps=100000,
                                         max_store=500, nout=3))
    assert np.array_equal(sim.get_t(), t_before)
    assert sim.get_x().size == 50 * 4 * 40
    with pytest.raises(Exception):
        sim.get_trajectory_by_member(rows=51)
    sim.trajectory()
    assert sim.get_t().size == 500 * 40


def test_trajectory_chunks_equal_the_repeated_calls():
    # the chunked helper against the calls a clODE user makes by hand:
    # trajectory over each part, then shift_x0
    from clode_gb300.trajectory_output import trajectory_chunks

    def make():
        pi = W.ProblemInfo(rhs_path("ornstein_uhlenbeck.cl"), ["x"], ["theta", "mu", "sigma"], [], 1)
        sim = W.TrajectorySimulatorBase(pi, "seuler", True, W.OpenCLResource(), "")
        n = 512
        rng = np.random.default_rng(9)
        pars = np.stack([rng.uniform(0.1, 2.0, n), np.zeros(n), rng.uniform(0.1, 1.0, n)], axis=1)
        sim.set_solver_params(W.SolverParams(dt=1e-3, max_steps=100000, max_store=205, nout=10))
        sim.set_problem_data(np.zeros(n), pars.flatten(order="F"))
        sim.seed_rng(4)
        return sim

    a, b = make(), make()
    got = list(trajectory_chunks(a, (0.0, 6.0), 3))
    assert [(t0, t1) for t0, t1, _ in got] == [(0.0, 2.0), (2.0, 4.0), (4.0, 6.0)]
    for t0, t1, rows in got:
        b.set_tspan([t0, t1])
        b.trajectory()
        want = b.get_trajectory_by_member()
        b.shift_x0()
        for k in ("n_stored", "t", "x", "dx"):
            assert np.array_equal(rows[k], want[k]), k
    assert np.array_equal(a.get_xf(), b.get_xf()) and np.array_equal(a.get_rng_state(), b.get_rng_state())
