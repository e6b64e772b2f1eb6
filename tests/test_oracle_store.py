"""The oracle's restatement of features with storage (oracle/clode_oracle.c
o_features_store) against the oracle's own features and trajectory runs,
on the CPU: the same features and final state, the trajectory run's rows,
and event counts equal to the observer's."""
import numpy as np

from clode_gb300 import rhs_path
from oracle.build import OracleConfig
from oracle.runner import OracleSimulator


def _lorenz(n=40, seed=3):
    rng = np.random.default_rng(seed)
    x0 = np.ones((n, 3)) + rng.normal(0, 1e-3, (n, 3))
    pars = np.stack([rng.uniform(10, 60, n), rng.uniform(5, 15, n), np.full(n, 8 / 3)], axis=1)
    return x0, pars


def _sim(cfg, x0, pars):
    s = OracleSimulator(cfg, nthreads=2)
    s.set_solver_params(dt=1e-3, max_steps=100000, max_store=3000, nout=5)
    s.set_observer_params(e_var_ix=2, f_var_ix=2, max_event_count=100000, x_up_threshold=0.3,
                          x_down_threshold=0.2)
    s.set_problem_data(x0, pars)
    s.set_tspan((0.0, 10.0))
    return s


def test_oracle_store_equals_features_and_trajectory():
    cfg = OracleConfig(rhs_path("lorenz.cl"), n_var=3, n_par=3, n_aux=1, stepper="rk4", single_precision=False,
                       observer="thresh2", n_store_events=0)
    x0, pars = _lorenz()
    a = _sim(cfg, x0, pars)
    a.features_store(event_rows=8, reinitialize=True)
    b = _sim(cfg, x0, pars)
    b.features(reinitialize=True)
    c = _sim(cfg, x0, pars)
    c.trajectory()
    assert np.array_equal(a.F, b.F) and np.array_equal(a.xf, b.xf) and np.array_equal(a.dt, b.dt)
    assert np.array_equal(a.n_stored, c.n_stored)
    for k in ("t", "x", "dx", "aux"):
        assert np.array_equal(getattr(a, k), getattr(c, k)), k
    assert a.n_events.max() > 1
    # events stored in order, zero past each member's count
    et = a.ev_t.reshape(8, -1)
    for i, ne in enumerate(a.n_events):
        k = min(int(ne), 8)
        assert (np.diff(et[:k, i]) > 0).all() and (et[k:, i] == 0).all()
