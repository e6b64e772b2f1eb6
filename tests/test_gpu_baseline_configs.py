"""Parity on the workloads the engine is measured on, at their own sizes.

* Van der Pol, RK4 in FP64 (4096 members, mu ~ U[0.1, 5], x0, y0 ~ U[-2, 2];
  transient over [0, 200] then localmax features over [200, 1000], dt 0.01):
  bitwise equal to the oracle — final states, times, step sizes and every
  feature — with exactly 80,001 feature steps per member ending at
  t = 1000.0099999992724 (the reference's `t <= t1` loop with naive time
  accumulation from t0 = 200).
* Lorenz, DP45 rtol 1e-6, atol 1e-9 in FP32, thresh2 on z over [0, 500], on
  2048 seeded members of the 1024 x 1024 (sigma, rho) grid, against the FP64
  solution of clODE's own kernels at rtol 1e-10, atol 1e-13 (fixture
  ``tests/golden/lorenz_grid_fp64.npz``).  Members split cleanly by whether a
  1e-9 change of the initial state moves their FP64 result (about 70 % are
  chaotic and move by order one; the rest by less than 1e-7):
  - non-chaotic members: event counts exact; mean period within 5e-2
    relative (event times are resolved to a step, as in the reference), and
    no worse in the median than the reference's own FP32 arithmetic (the CPU
    oracle in FP32) plus 1e-4;
  - chaotic members: the distributions of mean period and event count over
    the members pass a two-sample Kolmogorov-Smirnov test against FP64 at
    alpha = 0.001, and so does the distribution of the members' errors
    against that of the FP32 oracle's errors.
* Lactotroph with an additive noise current (``lactotroph_noise``, sig = 2)
  under stochastic Euler, dt = 0.01, FP32, nhood2 on c / v, 128 points of the
  (gcal, gbk) map x 4 noise realisations, per-member spans U[1e3, 1e4] ms:
  the RNG words after the run equal the oracle's (the same normals are drawn
  in the same number); event counts equal for at least 85 % of the members
  and equal in distribution (KS, alpha = 0.001) with the same mean, mean
  periods equal in distribution, continuous features to a median relative
  difference of 1e-3 (noise-driven crossings, see the test).
"""
import functools
import json
import os

import numpy as np
import pytest

import bench
from tests.parity import Scenario, assert_bitwise, run_engine, run_oracle

pytestmark = pytest.mark.gpu

SEED = 20261203
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# ------------------------------------------------------------ Van der Pol --
def test_vdp_full_size_bitwise():
    rng = np.random.default_rng(SEED)
    n = 4096
    mu = rng.uniform(0.1, 5.0, n)
    x0 = rng.uniform(-2.0, 2.0, (n, 2))
    # max_event_count above the ~130 maxima of the fastest members: no run ends early
    sc = Scenario("van_der_pol.cl", 2, 1, x0, mu[:, None], stepper="rk4", observer="localmax", single=False,
                  sp=dict(dt=0.01, max_steps=10000000), op=dict(max_event_count=100000),
                  steps=[("transient", (0.0, 200.0)), ("shift_x0",), ("features", (200.0, 1000.0))])
    eng, ora = run_engine(sc, options={"schedule": 1}), run_oracle(sc)
    assert_bitwise(eng, ora)
    names = eng["feature_names"]
    F = eng["F_list"][0]
    assert (F[:, names.index("step count")] == 80001).all()
    # naive accumulation of dt from t0 = 200, as the reference does: 1000.0099999992724
    t = 200.0
    for _ in range(80001):
        t += 0.01
    assert (eng["tf"] == t).all() and abs(t - 1000.00999999927) < 1e-11
    # every member oscillates
    assert (F[:, names.index("mean IMI")] > 0).all()


# ----------------------------------------------------------------- Lorenz --
def _ks(a, b):
    a, b = np.sort(a), np.sort(b)
    v = np.concatenate([a, b])
    return float(np.abs(np.searchsorted(a, v, side="right") / a.size
                        - np.searchsorted(b, v, side="right") / b.size).max())


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-6)


@functools.lru_cache(maxsize=None)
def _lorenz_fixture():
    d = np.load(os.path.join(GOLDEN, "lorenz_grid_fp64.npz"))
    return {k: d[k] for k in d.files}


def _lorenz_scenario(x0, pars, single, tol):
    return Scenario("lorenz.cl", 3, 3, x0, pars, n_aux=1, stepper="dopri5", observer="thresh2", single=single,
                    sp=dict(dt=1e-3, dtmax=1.0, abstol=tol * 1e-3, reltol=tol, max_steps=10000000),
                    op=dict(e_var_ix=2, f_var_ix=2, max_event_count=100000, x_up_threshold=0.3,
                            x_down_threshold=0.2),
                    steps=[("features", (0.0, 500.0))], seed=None)


@pytest.mark.parametrize("build", ["exact", "bench"])
def test_lorenz_grid_fp32_against_fp64(build):
    d = _lorenz_fixture()
    cols = json.loads(str(d["meta"]))["perturbed_columns"]
    F64, x0, pars = d["F"], d["x0"], d["pars"]
    options = {"schedule": 1} if build == "exact" else dict(schedule=1, fmad=1, prec_div=0, ftz=1)
    eng = run_engine(_lorenz_scenario(x0, pars, True, 1e-6), options=options)
    names = eng["feature_names"]
    ev, per = names.index("event count"), names.index("mean period")
    assert cols[0] == per and cols[-1] == ev
    Fe = eng["F_list"][0]
    F32o = run_oracle(_lorenz_scenario(x0, pars, True, 1e-6))["F_list"][0]
    # members whose FP64 result moves under a 1e-9 change of the initial state
    cont = cols[1:-1]
    moved = np.maximum(_rel(d["F_up"][:, 1:-1], F64[:, cont]).max(1), _rel(d["F_down"][:, 1:-1], F64[:, cont]).max(1))
    chaotic = (moved > 1e-6) | (d["F_up"][:, -1] != F64[:, ev]) | (d["F_down"][:, -1] != F64[:, ev])
    quiet = ~chaotic
    print(f"\n{build}: {chaotic.sum()} chaotic, {quiet.sum()} non-chaotic members; "
          f"largest FP64 move of a non-chaotic member {moved[quiet].max():.1e}")
    assert 0.5 < chaotic.mean() < 0.9

    # non-chaotic: exact counts, periods to the step resolution
    bad = np.where(quiet & (Fe[:, ev] != F64[:, ev]))[0]
    for i in bad:
        print(f"  count differs: member {i} rho {pars[i, 0]:.3f} sigma {pars[i, 1]:.3f} "
              f"FP64 {F64[i, ev]:.0f} engine {Fe[i, ev]:.0f} FP32 oracle {F32o[i, ev]:.0f}")
    assert bad.size == 0
    two = quiet & (F64[:, ev] > 1)
    err_e, err_o = _rel(Fe[two, per], F64[two, per]), _rel(F32o[two, per], F64[two, per])
    print(f"  non-chaotic mean period rel. error: engine median {np.median(err_e):.2e} max {err_e.max():.2e}; "
          f"FP32 oracle median {np.median(err_o):.2e} max {err_o.max():.2e}")
    assert err_e.max() < 5e-2
    # both errors are the step granularity of the event times; the fast
    # build rounds differently (contracted multiply-adds, approximate
    # division) and so steps differently: its median within 10 % of the
    # FP32 oracle's
    assert np.median(err_e) <= 1.1 * np.median(err_o)

    # chaotic: distributions
    n = int(chaotic.sum())
    crit = 1.95 * np.sqrt(2.0 / n)
    for k in (per, ev):
        stat = _ks(Fe[chaotic, k], F64[chaotic, k])
        print(f"  chaotic {names[k]}: KS engine vs FP64 {stat:.3f} (critical {crit:.3f}); "
              f"FP32 oracle vs FP64 {_ks(F32o[chaotic, k], F64[chaotic, k]):.3f}")
        assert stat < crit, names[k]
    stat = _ks(_rel(Fe[chaotic, per], F64[chaotic, per]), _rel(F32o[chaotic, per], F64[chaotic, per]))
    print(f"  chaotic mean-period errors, engine vs FP32 oracle: KS {stat:.3f}")
    assert stat < crit


# ------------------------------------------------- lactotroph with noise --
NOISE_POINTS, REALISATIONS = 128, 4


@functools.lru_cache(maxsize=None)
def _noise_inputs():
    x0, pars, _ = bench.make_workload(2048, SEED, 1e3, 1e4)
    rng = np.random.default_rng(SEED + 4)
    pts = np.sort(rng.choice(pars.shape[0], NOISE_POINTS, replace=False))
    n = NOISE_POINTS * REALISATIONS
    p = np.repeat(pars[pts], REALISATIONS, axis=0)
    p = np.concatenate([p, np.full((n, 1), 2.0)], axis=1)  # sig = 2 (clode samples/lactotroph_noise.ode)
    t1 = rng.uniform(1e3, 1e4, n)
    return np.repeat(x0[pts], REALISATIONS, axis=0), p, np.stack([np.zeros(n), t1], axis=1)


def _noise_scenario():
    x, p, ts = _noise_inputs()
    return Scenario("lactotroph_noise.cl", 4, 4, x, p, n_aux=1, n_wiener=1,
                    stepper="seuler", observer="nhood2", single=True,
                    sp=dict(dt=0.01, max_steps=10000000),
                    op={k: v for k, v in bench.OBSERVER.items() if k != "max_event_timestamps"},
                    steps=[("features", None)], seed=SEED, tspan_pm=ts.ravel(),
                    var_names=["v", "n", "f", "c"], aux_names=["ica"])


def test_lactotroph_noise_seuler_against_oracle():
    sc = _noise_scenario()
    eng = run_engine(sc, options={"schedule": 1})
    from oracle.runner import OracleSimulator
    s = OracleSimulator(sc.oracle_config())
    s.set_solver_params(dt=0.01, dtmax=0.5, abstol=1e-6, reltol=1e-3, max_steps=10000000, max_store=1, nout=1)
    s.set_observer_params(**sc.op)
    s.set_problem_data(sc.x0, sc.pars)
    s.seed_rng(SEED)
    s.set_tspan(sc.tspan_pm)
    rng0 = s.rng.copy()
    s.features(True)
    Fo = s.get_F()
    # the same normals, drawn in the same number
    np.testing.assert_array_equal(eng["sim"].get_rng_state(), s.rng)
    assert not np.array_equal(s.rng, rng0)
    Fe = eng["F_list"][0]
    names = eng["feature_names"]
    ev, per = names.index("event count"), names.index("mean period")
    cont = [names.index(f"{a} {v}") for v in ("v", "n", "f", "c") for a in ("max", "min", "mean", "range")]
    n = Fe.shape[0]
    assert (Fo[:, ev] > 0).sum() > n // 10  # the noise map has events to count
    # With a noise current every step moves v by a random amount, so the
    # slope of v changes sign at most steps (the "peaks" count those sign
    # changes by the thousand) and the noisy trajectory grazes the
    # neighbourhood's boundary many times: an ulp of difference in exp or
    # log flips some of these decisions.  The oracle itself changes the event
    # count of about 2 % of these members when the initial voltage moves by
    # one ulp.  Event counts are therefore compared member by member for
    # most members and as distributions for all of them.
    exact = np.mean(Fe[:, ev] == Fo[:, ev])
    ks_ev, ks_per = _ks(Fe[:, ev], Fo[:, ev]), _ks(Fe[:, per], Fo[:, per])
    crit = 1.95 * np.sqrt(2.0 / n)  # two-sample KS, alpha = 0.001
    se = np.sqrt(Fe[:, ev].var() / n + Fo[:, ev].var() / n)
    delta = _rel(Fe[:, cont], Fo[:, cont]).max(axis=1)
    print(f"\nnoise map: event counts equal for {exact:.3f} of {n} members; KS events {ks_ev:.3f}, "
          f"mean period {ks_per:.3f} (critical {crit:.3f}); mean events {Fe[:, ev].mean():.3f} vs "
          f"{Fo[:, ev].mean():.3f}; continuous features: median rel. difference {np.median(delta):.1e}")
    assert exact >= 0.85
    assert ks_ev < crit and ks_per < crit
    assert abs(Fe[:, ev].mean() - Fo[:, ev].mean()) < 4 * se + 1e-12
    assert np.median(delta) < 1e-3
