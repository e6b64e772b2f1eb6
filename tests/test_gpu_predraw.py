"""Pre-drawn deviates of stochastic trajectory runs against deviates drawn in
the integration loop.

With the option ``predraw`` a stochastic trajectory run counts
each member's deviates, draws them in a launch of their own with four lanes
per member (jump-ahead of the member's stream, two passes per block of
candidates), and the trajectory launch reads them.  These tests run the same
ensembles with ``predraw`` on and off and require bitwise equal results —
stored rows, final states, final times, RNG words:

* the OU process in FP32 and FP64, both schedules;
* per-member time spans (members that take different numbers of deviates),
  including spans that end before they start, and runs cut short by
  max_steps and by max_store;
* two Wiener processes (two deviates per step, an odd number per member);
* two runs in a row (the second continues from the first's RNG words);
* short runs (a few deviates per member, the smallest blocks).
"""
import os

import numpy as np
import pytest

from clode_gb300 import clode_cpp_wrapper as W, rhs_path

pytestmark = pytest.mark.gpu

TWO_NOISE = """
void getRHS(const realtype t, const realtype x_[], const realtype p_[],
            realtype dx_[], realtype aux_[], const realtype w_[])
{
    dx_[0] = -p_[0] * x_[0] + p_[1] * w_[0];
    dx_[1] = -p_[0] * x_[1] + p_[1] * (w_[0] - w_[1]);
}
"""


def _sim(single, predraw, schedule=1, two=False, tmp=None):
    if two:
        path = os.path.join(tmp, "two_noise.cl")
        with open(path, "w") as f:
            f.write(TWO_NOISE)
        pi = W.ProblemInfo(path, ["x", "y"], ["theta", "sigma"], [], 2)
    else:
        pi = W.ProblemInfo(rhs_path("ornstein_uhlenbeck.cl"), ["x"], ["theta", "mu", "sigma"], [], 1)
    sim = W.TrajectorySimulatorBase(pi, "seuler", single, W.OpenCLResource(), "")
    sim.set_option("schedule", schedule)
    sim.set_option("predraw", predraw)
    sim.build_cl()
    return sim


def _run(sim, x0, pars, ts, sp, seed=11, runs=1):
    sim.set_solver_params(W.SolverParams(**sp))
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    if ts.ndim == 2:
        sim.set_tspan_per_member(ts.ravel())
    else:
        sim.set_tspan(list(ts))
    sim.seed_rng(seed)
    out = []
    for _ in range(runs):
        sim.trajectory()
        out.append({"t": np.asarray(sim.get_t()), "x": np.asarray(sim.get_x()), "dx": np.asarray(sim.get_dx()),
                    "n": np.asarray(sim.get_n_stored()), "xf": np.asarray(sim.get_xf()),
                    "tf": np.asarray(sim.get_tf()), "rng": sim.get_rng_state()})
        sim.shift_x0()
    return out


def _equal(a, b):
    for ra, rb in zip(a, b):
        for k in ra:
            x, y = ra[k], rb[k]
            same = (x == y) | (np.isnan(x) & np.isnan(y)) if x.dtype.kind == "f" else (x == y)
            assert same.all(), f"{k}: {np.size(same) - np.count_nonzero(same)} differ"


def _ou(n, seed=3):
    r = np.random.default_rng(seed)
    pars = np.stack([r.uniform(0.1, 2.0, n), np.zeros(n), r.uniform(0.1, 1.0, n)], axis=1)
    return np.zeros((n, 1)), pars


@pytest.mark.parametrize("single", [True, False], ids=["fp32", "fp64"])
@pytest.mark.parametrize("schedule", [0, 1], ids=["grid", "persistent"])
def test_ou_predrawn_equals_drawn_in_loop(single, schedule):
    x0, pars = _ou(4096)
    sp = dict(dt=1e-3, dtmax=1.0, abstol=1e-6, reltol=1e-3, max_steps=20000, max_store=2002, nout=10)
    on, off = _sim(single, 1, schedule), _sim(single, 0, schedule)
    a = _run(on, x0, pars, np.array([0.0, 20.0]), sp, runs=2)
    b = _run(off, x0, pars, np.array([0.0, 20.0]), sp, runs=2)
    _equal(a, b)
    assert on.get_option("predrawn") == 1 and off.get_option("predrawn") == 0


def test_per_member_spans_and_limits():
    n = 5000
    x0, pars = _ou(n, seed=4)
    r = np.random.default_rng(5)
    ts = np.stack([r.uniform(0.0, 1.0, n), r.uniform(1.0, 12.0, n)], axis=1)
    ts[::13, 1] = ts[::13, 0] - 0.5  # spans that end before they start: the initial deviate only
    sp = dict(dt=1e-3, dtmax=1.0, abstol=1e-6, reltol=1e-3, max_steps=9000, max_store=700, nout=7)
    a = _run(_sim(True, 1), x0, pars, ts, sp)
    b = _run(_sim(True, 0), x0, pars, ts, sp)
    _equal(a, b)
    # some members end on max_steps, some on max_store, some on t1
    assert len(np.unique(a[0]["n"])) > 3


def test_two_wiener_processes(tmp_path):
    n = 3000
    r = np.random.default_rng(6)
    x0 = r.normal(0, 1, (n, 2))
    pars = np.stack([r.uniform(0.5, 2.0, n), r.uniform(0.1, 1.0, n)], axis=1)
    sp = dict(dt=1e-3, dtmax=1.0, abstol=1e-6, reltol=1e-3, max_steps=5000, max_store=502, nout=10)
    a = _run(_sim(True, 1, two=True, tmp=str(tmp_path)), x0, pars, np.array([0.0, 5.0]), sp, runs=2)
    b = _run(_sim(True, 0, two=True, tmp=str(tmp_path)), x0, pars, np.array([0.0, 5.0]), sp, runs=2)
    _equal(a, b)


def test_short_runs():
    x0, pars = _ou(777, seed=8)
    sp = dict(dt=1e-2, dtmax=1.0, abstol=1e-6, reltol=1e-3, max_steps=100, max_store=20, nout=1)
    a = _run(_sim(True, 1), x0, pars, np.array([0.0, 0.05]), sp, runs=3)
    b = _run(_sim(True, 0), x0, pars, np.array([0.0, 0.05]), sp, runs=3)
    _equal(a, b)
