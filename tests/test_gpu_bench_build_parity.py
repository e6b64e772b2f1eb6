"""The benchmarked build against the oracle, on the benchmark's own map.

bench.py times the lactotroph nhood2 map (2048 x 2048 grid of (gcal, gbk),
per-member time spans U[1e3, 1e4] ms, DP45 rtol = abstol = 1e-6 in FP32) with
the fast build: fmad on, division as reciprocal times numerator, denormals
flushed, the persistent schedule, and the register cap, block size, stepping
variant (one attempt per iteration or whole steps) and pass layout (separate
or fused observer initialisation) that the autotuner picks, with the members
taken longest time span first.  These tests run that build — and the exact
build beside it — on 4096 seeded members of the same map and compare every
member with the CPU oracle (FP32, the same inputs).

The criterion (the tolerance the comparison states):

* Event and spike counts (``event count``, ``max/min/mean peaks``) are exact
  for all but at most 1 % of the members.
* Every member whose counts differ is listed (printed) and must be a
  borderline member: its trajectory in the oracle brings a decision quantity
  of the observer close to its threshold — the nearest near-tangency
  ``margin`` (``tests/margins.py``: ball-exit distance, slope extremum or
  centre crossing, each relative to its own scale) is at most ten times the
  divergence ``delta`` between the two runs (the largest relative difference
  of the member's continuous features: extrema, means and ranges of the state
  variables) — and the divergence must be the member's own: the oracle's
  result for it moves by at least 1e-4 (relative, same features) under a
  rounding-size change: its initial voltage, or one of its parameters (gcal,
  gsk, gbk), moved by one FP32 ulp.  A parameter ulp changes the vector field
  at every evaluation by about a rounding error, as a different rounding of
  the arithmetic does; a change of the initial state alone can decay before
  the trajectory reaches the part of a burst where the spike count is
  decided.  (A one-ulp change of the tolerances leaves the oracle's result
  bitwise unchanged on these members, so it is no measure.)
  A member whose runs did not diverge (delta < 1e-4) must have exact counts.
* On members whose counts agree, the continuous features agree to a median
  relative difference of 1e-4.
"""
import functools

import numpy as np
import pytest

import bench
from tests.margins import nhood2_counts, nhood2_margins

pytestmark = pytest.mark.gpu

N = 4096
COUNTS = ("event count", "max peaks", "min peaks", "mean peaks")
CONTINUOUS = tuple(f"{s} {v}" for v in ("v", "n", "f", "c") for s in ("max", "min", "mean", "range"))
E_VAR, F_VAR = bench.OBSERVER["e_var_ix"], bench.OBSERVER["f_var_ix"]
BUILDS = {
    "bench": dict(fmad=1, prec_div=0, ftz=1, schedule=1),
    "exact": dict(schedule=1),
}


@functools.lru_cache(maxsize=None)
def _workload():
    x0, pars, tspan = bench.make_workload(2048, 20261203, 1e3, 1e4)
    idx = np.sort(np.random.default_rng(77).choice(x0.shape[0], N, replace=False))
    return x0[idx], pars[idx], tspan[idx]


@functools.lru_cache(maxsize=None)
def _oracle():
    """Oracle features at the inputs, and with the initial voltage and each
    parameter one FP32 ulp up and down (each member's own sensitivity)."""
    import os
    x0, pars, tspan = _workload()
    every = np.arange(N)
    F, _, _ = bench.run_cpu(x0, pars, tspan, every, os.cpu_count(), prefer_reference=False)
    moved = []
    for direction in (np.inf, -np.inf):
        xp = x0.copy()
        xp[:, 0] = float(np.nextafter(np.float32(x0[0, 0]), np.float32(direction)))
        moved.append(bench.run_cpu(xp, pars, tspan, every, os.cpu_count(), prefer_reference=False)[0])
        for col in range(pars.shape[1]):
            pp = pars.copy()
            pp[:, col] = np.nextafter(pars[:, col].astype(np.float32), np.float32(direction)).astype(np.float64)
            moved.append(bench.run_cpu(x0, pp, tspan, every, os.cpu_count(), prefer_reference=False)[0])
    return F, tuple(moved)


def _engine(build):
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path
    x0, pars, tspan = _workload()
    pi = W.ProblemInfo(rhs_path("lactotroph.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"], 0)
    sim = W.FeatureSimulatorBase(pi, "dopri5", "nhood2", W.ObserverParams(**bench.OBSERVER), True,
                                 W.OpenCLResource(), "")
    for k, v in BUILDS[build].items():
        sim.set_option(k, v)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(**bench.SOLVER))
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan_per_member(tspan.ravel())
    tuned = sim.autotune(N) if build == "bench" else None
    sim.features(True)
    F = np.asarray(sim.get_f()).reshape(-1, N).T
    return F, list(sim.get_feature_names()), tuned


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-6)


def _oracle_rows(members):
    """Every step of the oracle's run for these members (the feature pass's steps)."""
    from clode_gb300 import rhs_path
    from oracle.build import OracleConfig
    from oracle.runner import OracleSimulator
    x0, pars, tspan = _workload()
    F, _ = _oracle()
    cfg = OracleConfig(rhs_path("lactotroph.cl"), n_var=4, n_par=3, n_aux=1, stepper="dopri5",
                       single_precision=True)
    s = OracleSimulator(cfg)
    sp = dict(bench.SOLVER)
    sp.update(max_store=int(F[members, -4].max()) + 8, nout=1)  # "step count" column
    s.set_solver_params(**sp)
    s.set_problem_data(x0[members], pars[members])
    s.set_tspan(tspan[members])
    s.trajectory()
    n = len(members)
    T = s.t.reshape(-1, n)
    X = s.x.reshape(-1, 4, n)
    D = s.dx.reshape(-1, 4, n)
    return [(T[:s.n_stored[j] + 1, j], X[:s.n_stored[j] + 1, :, j], D[:s.n_stored[j] + 1, :, j])
            for j in range(n)]


@pytest.mark.parametrize("build", sorted(BUILDS))
def test_benchmark_map_counts_exact_except_listed_borderline_members(build):
    Fg, names, tuned = _engine(build)
    Fo, moved = _oracle()
    assert names[-4] == "step count"
    cc = [names.index(c) for c in COUNTS]
    cont = [names.index(c) for c in CONTINUOUS]
    mism = np.where(np.any(Fg[:, cc] != Fo[:, cc], axis=1))[0]
    print(f"\n{build} build{' (autotuned: ' + str(tuned) + ')' if tuned else ''}: "
          f"{mism.size} of {N} members differ in a count")
    assert mism.size <= 0.01 * N

    agree = np.setdiff1d(np.arange(N), mism)
    assert np.median(_rel(Fg[agree][:, cont], Fo[agree][:, cont])) < 1e-4

    if mism.size == 0:
        return
    x0, pars, tspan = _workload()
    delta = _rel(Fg[:, cont], Fo[:, cont]).max(axis=1)
    own = np.max([_rel(M[:, cont], Fo[:, cont]).max(axis=1) for M in moved], axis=0)
    rows = _oracle_rows(mism)
    bad = []
    print(" member   gcal    gbk     T1   oracle counts (events,max,min,mean peaks) -> engine   "
          "margin (ball, slope, centre)   delta   oracle 1-ulp (x0 or pars)")
    for i, (t, x, dx) in zip(mism, rows):
        t1 = np.float32(tspan[i, 1])
        radius, x_down = np.float32(bench.OBSERVER["nhood_radius"]), bench.OBSERVER["x_down_threshold"]
        # the re-evaluation from the oracle's rows reproduces the oracle's counts
        r = nhood2_counts(t, x, dx, t1, E_VAR, F_VAR, radius, x_down)
        assert r["event_steps"].size == Fo[i, names.index("event count")]
        if r["peaks"]:
            assert max(r["peaks"]) == Fo[i, names.index("max peaks")]
            assert min(r["peaks"]) == Fo[i, names.index("min peaks")]
        m = nhood2_margins(t, x, dx, t1, E_VAR, F_VAR, radius, x_down)
        print(f" {i:6d} {pars[i, 0]:6.3f} {pars[i, 2]:6.3f} {t1:7.1f}   {Fo[i, cc].tolist()} -> {Fg[i, cc].tolist()}"
              f"   {m['margin']:.2e} ({m['m_ball']:.1e}, {m['m_peak']:.1e}, {m['m_center']:.1e})"
              f"   {delta[i]:.2e}   {own[i]:.2e}")
        if not (delta[i] >= 1e-4 and m["margin"] <= 10 * delta[i] and own[i] >= 1e-4):
            bad.append(int(i))
    assert not bad, f"count mismatches outside the borderline criterion: members {bad}"
