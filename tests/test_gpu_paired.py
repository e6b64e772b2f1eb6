"""Paired FP32 stage sums (option ``paired``) against the scalar ones.

In FP32 builds that allow contraction (``fmad`` 1, the benchmarked build) the
Dormand-Prince stage combinations take two state variables per instruction
(sm_100 paired FP32 multiply and fma), in a fixed contraction pattern; the
build that reproduces clODE bit for bit (``fmad`` 0) keeps its scalar stage
sums, because the device compiler fuses a paired multiply into a following
paired add even when contraction is off.

* ``fmad`` 0: the option changes nothing — results bitwise equal with it on
  and off (the lactotroph nhood2 map with the replayed and the integrated
  feature pass, Lorenz thresh2, a stored trajectory).
* ``fmad`` 1: paired and scalar stage sums are two roundings of the same
  arithmetic, which differ about as much as the fast build differs from the
  exact one.  That difference is the yardstick: the paired fast build may
  not move further from the scalar fast build than the scalar fast build
  lies from the exact build — in the share of members that take the same
  number of steps (Lorenz trajectories) or have the same spike counts (the
  lactotroph map), and in the median relative differences of step sizes,
  states and continuous features — while a wrong term in a paired stage
  would change every step size by a large factor.  The paired fast build
  itself is compared with the oracle in ``test_gpu_bench_build_parity``.
"""
import functools

import numpy as np
import pytest

import bench
from clode_gb300 import clode_cpp_wrapper as W, rhs_path

pytestmark = pytest.mark.gpu

N = 2048
FAST = dict(fmad=1, prec_div=0, ftz=1)


@functools.lru_cache(maxsize=None)
def _map():
    x0, pars, tspan = bench.make_workload(2048, 20261203, 1e3, 1e4)
    idx = np.sort(np.random.default_rng(11).choice(x0.shape[0], N, replace=False))
    return x0[idx], pars[idx], tspan[idx]


def _lactotroph(paired, replay, options=None):
    pi = W.ProblemInfo(rhs_path("lactotroph.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"], 0)
    sim = W.FeatureSimulatorBase(pi, "dopri5", "nhood2", W.ObserverParams(**bench.OBSERVER), True,
                                 W.OpenCLResource(), "")
    for k, v in dict(schedule=1, paired=paired, replay=replay, **(options or {})).items():
        sim.set_option(k, v)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(**bench.SOLVER))
    x0, pars, tspan = _map()
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan_per_member(tspan.ravel())
    sim.features(True)
    return sim


def _lorenz_problem():
    return W.ProblemInfo(rhs_path("lorenz.cl"), ["x", "y", "z"], ["rho", "sigma", "beta"], ["fx"], 0)


def _lorenz_inputs(n=1024, seed=5):
    r = np.random.default_rng(seed)
    x0 = np.ones((n, 3)) + r.normal(0, 1e-3, (n, 3))
    pars = np.stack([r.uniform(10, 60, n), r.uniform(5, 15, n), np.full(n, 8 / 3)], axis=1)
    return x0, pars


def _lorenz_features(paired, options=None):
    x0, pars = _lorenz_inputs()
    op = W.ObserverParams(e_var_ix=2, f_var_ix=2, max_event_count=100000, x_up_threshold=0.3,
                          x_down_threshold=0.2)
    sim = W.FeatureSimulatorBase(_lorenz_problem(), "dopri5", "thresh2", op, True, W.OpenCLResource(), "")
    for k, v in dict(schedule=1, paired=paired, **(options or {})).items():
        sim.set_option(k, v)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=1e-3, dtmax=1.0, abstol=1e-9, reltol=1e-6, max_steps=10000000))
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan([0.0, 60.0])
    sim.transient()
    sim.shift_tspan()
    sim.features(True)
    return sim


def _trajectory(paired, options=None, t1=10.0, store=4000, rtol=1e-6, atol=1e-9):
    x0, pars = _lorenz_inputs(512, seed=9)
    sim = W.TrajectorySimulatorBase(_lorenz_problem(), "dopri5", True, W.OpenCLResource(), "")
    for k, v in dict(paired=paired, **(options or {})).items():
        sim.set_option(k, v)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=1e-3, dtmax=1.0, abstol=atol, reltol=rtol, max_steps=10000000,
                                         max_store=store, nout=1))
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan([0.0, t1])
    sim.trajectory()
    out = {k: np.asarray(getattr(sim, "get_" + k)()) for k in ("t", "x", "dx", "aux", "n_stored", "xf")}
    assert out["n_stored"].max() < store  # not cut short by the buffer
    return out


def _outputs(sim):
    return {k: np.asarray(getattr(sim, "get_" + k)()) for k in ("f", "xf", "tf", "dt", "status")}


def _assert_bitwise(a, b):
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-6)


# ---- fmad 0: the option leaves the exact build unchanged

@pytest.mark.parametrize("replay", [1, 0])
def test_exact_build_lactotroph_map_unchanged(replay):
    a = _outputs(_lactotroph(1, replay))
    b = _outputs(_lactotroph(0, replay))
    assert np.isfinite(a["f"]).all()
    _assert_bitwise(a, b)


def test_exact_build_lorenz_thresh2_unchanged():
    a, b = _outputs(_lorenz_features(1)), _outputs(_lorenz_features(0))
    assert a["f"].size and np.isfinite(a["f"]).all()
    _assert_bitwise(a, b)


def test_exact_build_trajectory_unchanged():
    _assert_bitwise(_trajectory(1), _trajectory(0))


# ---- fmad 1: paired and scalar stage sums take the same steps
#
# Two roundings of the same arithmetic differ about as much as the fast build
# differs from the exact one (the contraction of a * b + c alone), so that
# difference is the yardstick: pairing may not move the results further from
# the scalar fast build than contraction moves the scalar fast build from
# the exact one (with small absolute floors), while a wrong term in a paired
# stage would change every step size by a large factor.

def _steps(a, b):
    """Share of members with the same stored-step count, and the median
    relative differences of the step sizes and states along their common
    steps."""
    ns_a, ns_b = a["n_stored"], b["n_stored"]
    n = ns_a.size
    same = ns_a == ns_b
    T_a, T_b = a["t"].reshape(-1, n), b["t"].reshape(-1, n)
    X_a, X_b = a["x"].reshape(-1, 3, n), b["x"].reshape(-1, 3, n)
    m = int(ns_a[same].min())
    h_a, h_b = np.diff(T_a[:m, same], axis=0), np.diff(T_b[:m, same], axis=0)
    return (same.mean(), float(np.median(_rel(h_a, h_b))),
            float(np.median(_rel(X_a[:m, :, same], X_b[:m, :, same]))),
            int(np.abs(ns_a.astype(np.int64) - ns_b).max()))


def test_fast_build_trajectory_same_steps():
    """Lorenz over [0, 2] with error estimates well above rounding (rtol 1e-4,
    atol 1e-6): one pair and an odd third variable per stage."""
    tol = dict(t1=2.0)
    opts = dict(FAST)
    paired = _trajectory(1, opts, **tol, rtol=1e-4, atol=1e-6)
    scalar = _trajectory(0, opts, **tol, rtol=1e-4, atol=1e-6)
    exact = _trajectory(0, {}, **tol, rtol=1e-4, atol=1e-6)
    assert paired["n_stored"].min() > 20
    got, ref = _steps(paired, scalar), _steps(scalar, exact)
    print(f"\npaired vs scalar fast: same counts {got[0]:.4f}, median rel dt {got[1]:.2e}, x {got[2]:.2e}, "
          f"max count diff {got[3]}; scalar fast vs exact: {ref[0]:.4f}, {ref[1]:.2e}, {ref[2]:.2e}, {ref[3]}")
    assert got[0] >= min(0.99, ref[0] - 0.03)
    assert got[1] <= max(1e-5, 3 * ref[1])
    assert got[2] <= max(1e-5, 3 * ref[2])
    assert got[3] <= max(2, 2 * ref[3])
    assert not np.array_equal(paired["x"], scalar["x"])  # the paired stage sums did run


def _map_diff(a, b):
    names = list(a.get_feature_names())
    Fa = np.asarray(a.get_f()).reshape(-1, N).T
    Fb = np.asarray(b.get_f()).reshape(-1, N).T
    counts = [names.index(c) for c in ("event count", "max peaks", "min peaks", "mean peaks")]
    steps = names.index("step count")
    cont = [names.index(f"{s} {v}") for v in ("v", "n", "f", "c") for s in ("max", "min", "mean")]
    agree = np.all(Fa[:, counts] == Fb[:, counts], axis=1)
    return (agree.mean(), float(np.median(_rel(Fa[agree][:, cont], Fb[agree][:, cont]))),
            float(np.median(_rel(Fa[:, steps], Fb[:, steps]))), float(np.mean(_rel(Fa[:, steps], Fb[:, steps]) < 0.01)))


def test_fast_build_lactotroph_map_close():
    paired = _lactotroph(1, 1, FAST)
    scalar = _lactotroph(0, 1, FAST)
    exact = _lactotroph(0, 1)
    got, ref = _map_diff(paired, scalar), _map_diff(scalar, exact)
    print(f"\npaired vs scalar fast: counts agree {got[0]:.4f}, median rel features {got[1]:.2e}, "
          f"steps {got[2]:.2e}, steps within 1 % {got[3]:.4f}; scalar fast vs exact: {ref[0]:.4f}, {ref[1]:.2e}, "
          f"{ref[2]:.2e}, {ref[3]:.4f}")
    assert got[0] >= min(0.99, ref[0] - 0.02)
    assert got[1] <= max(1e-5, 3 * ref[1])
    assert got[2] <= max(1e-4, 3 * ref[2])
    assert got[3] >= min(0.99, ref[3] - 0.02)
    # deterministic: a second paired run is bitwise the first
    again = _lactotroph(1, 1, FAST)
    assert np.array_equal(np.asarray(again.get_f()), np.asarray(paired.get_f()), equal_nan=True)
