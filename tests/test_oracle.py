"""The CPU oracle pinned before it is trusted:

  * against the golden fixtures made from clODE's own kernels compiled as C
    (tests/golden, runs everywhere);
  * against clODE's own kernels directly, over every stepper x observer x
    precision (only where the clODE sources are present);
  * against the known answers of the reference's test suite and samples.
"""
import itertools
import json
import os

import numpy as np
import pytest

from oracle.build import reference_available
from tests import known_answers as KA
from tests.golden.scenarios import scenarios
from tests.parity import Scenario, run_oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCEN = scenarios()


def compare_to_fixture(out: dict, name: str):
    fx = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(fx["meta"]))
    got = dict(out)
    if "F_list" in got:
        got["F"] = np.stack(got["F_list"])
    for k in fx.files:
        if k == "meta":
            continue
        a, b = np.asarray(got[k], dtype=np.float64), np.asarray(fx[k], dtype=np.float64)
        assert a.shape == b.shape, (k, a.shape, b.shape)
        if meta["exact"]:
            bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
            assert not bad.any(), f"{name}.{k}: {bad.sum()} values differ, e.g. {a[bad][:3]} vs {b[bad][:3]}"
        else:
            # tolerance from the fixture: the scenario calls exp/pow/log, whose
            # last bit depends on the math library; allow 5% of values to drift
            ok = np.isclose(a, b, rtol=meta["rtol"], atol=meta["rtol"] * 1e-3, equal_nan=True)
            assert ok.mean() >= 0.95, f"{name}.{k}: {(~ok).sum()} of {ok.size} outside rtol {meta['rtol']}"


@pytest.mark.parametrize("name", sorted(SCEN))
def test_port_matches_golden_fixture(name):
    sc, exact, rtol = SCEN[name]
    compare_to_fixture(run_oracle(sc, nthreads=2), name)


def test_golden_fixtures_present():
    for name in SCEN:
        assert os.path.exists(os.path.join(GOLDEN, name + ".npz")), name


needs_reference = pytest.mark.skipif(not reference_available(), reason="clODE sources not present")


@needs_reference
@pytest.mark.parametrize("stepper", ["euler", "heun", "rk4", "bs23", "dopri5", "seuler"])
@pytest.mark.parametrize("single", [False, True])
def test_port_bitwise_equals_reference_kernels(stepper, single):
    rng = np.random.default_rng(7)
    n = 16
    x0 = np.ones((n, 3)) + rng.normal(0, 1e-3, (n, 3))
    p = np.stack([rng.uniform(10, 60, n), rng.uniform(5, 15, n), np.full(n, 8 / 3)], axis=1)
    for observer, nse in itertools.product([None, "basic", "basicall", "localmax", "nhood1", "nhood2", "thresh2"],
                                           [0, 2]):
        if (observer is None or observer == "localmax") and nse:
            continue  # localmax with stored events makes the reference write out of bounds
        model = "lorenz.cl"
        sc = Scenario(model, 3, 3, x0, p, n_aux=1, n_wiener=0, stepper=stepper, observer=observer, single=single,
                      n_store_events=nse, seed=11,
                      sp=dict(dt=0.01, dtmax=0.5, abstol=1e-6, reltol=1e-4, max_steps=200000, max_store=300,
                              nout=3),
                      op=dict(e_var_ix=2, f_var_ix=0, max_event_count=1000, x_up_threshold=0.3,
                              x_down_threshold=0.2, nhood_radius=0.1),
                      steps=([("features", (0.0, 5.0)), ("shift_x0",), ("shift_tspan",), ("features", None)]
                             if observer else [("transient", (0.0, 5.0)), ("trajectory", (0.0, 5.0))]))
        a = run_oracle(sc, nthreads=1)
        b = run_oracle(sc, nthreads=1, reference=True)
        for k in ("xf", "tf", "dt", "t", "x", "dx", "n_stored"):
            if k in a:
                assert np.array_equal(a[k], b[k], equal_nan=True), (observer, nse, k)
        for fa, fb in zip(a.get("F_list", []), b.get("F_list", [])):
            assert np.array_equal(fa, fb, equal_nan=True), (observer, nse)


@needs_reference
def test_port_bitwise_equals_reference_stochastic():
    n = 32
    rng = np.random.default_rng(3)
    pars = np.stack([rng.uniform(0.1, 2, n), np.zeros(n), rng.uniform(0.1, 1, n)], axis=1)
    for single in (False, True):
        sc = Scenario("ornstein_uhlenbeck.cl", 1, 3, np.zeros((n, 1)), pars, n_wiener=1, stepper="seuler",
                      single=single, seed=5, sp=dict(dt=1e-3, max_steps=3000, max_store=400, nout=7),
                      steps=[("transient", (0.0, 1.0)), ("shift_x0",), ("trajectory", (0.0, 2.0))])
        a, b = run_oracle(sc, nthreads=1), run_oracle(sc, nthreads=1, reference=True)
        for k in ("xf", "tf", "dt", "t", "x", "dx", "n_stored"):
            assert np.array_equal(a[k], b[k]), k


def _oracle_runner(sc):
    return run_oracle(sc, nthreads=2)


@pytest.mark.parametrize("check", KA.ALL, ids=lambda f: f.__name__)
def test_port_known_answers(check):
    check(_oracle_runner)


@needs_reference
@pytest.mark.parametrize("check", [KA.lactotroph_published_transient, KA.sine_thresh2_timestamps],
                         ids=lambda f: f.__name__)
def test_reference_kernels_known_answers(check):
    # the reference compiled as C passes the same checks (pins the checks themselves)
    check(lambda sc: run_oracle(sc, nthreads=2, reference=True))
