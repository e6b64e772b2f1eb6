"""The scenarios pinned by the golden fixtures in this directory.

Each fixture ``<name>.npz`` holds the inputs and the outputs of one scenario
computed by clODE's own kernel sources compiled as C (oracle/_ref, built by
oracle/build.py), made by ``make_golden.py``.  ``exact`` marks scenarios
whose arithmetic is + - * / and sqrt only, which any conforming IEEE
implementation reproduces bit for bit; the others call exp/pow/log and are
compared with the tolerance given here.
"""
import numpy as np

from tests.parity import Scenario

SEED = 20261203


def _vdp(n, seed):
    r = np.random.default_rng(seed)
    return r.uniform(-2, 2, (n, 2)), r.uniform(0.1, 5.0, (n, 1))


def _lorenz(n, seed):
    r = np.random.default_rng(seed)
    x0 = np.ones((n, 3)) + r.normal(0, 1e-3, (n, 3))
    return x0, np.stack([r.uniform(10, 60, n), r.uniform(5, 15, n), np.full(n, 8 / 3)], axis=1)


def _lacto(n, seed):
    r = np.random.default_rng(seed)
    p = np.stack([r.uniform(0.5, 3.0, n), np.full(n, 3.0), r.uniform(0, 2, n)], axis=1)
    return np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1)), p


def scenarios():
    out = {}
    x0, p = _vdp(64, SEED)
    out["vdp_rk4_fp64_localmax"] = (Scenario(
        "van_der_pol.cl", 2, 1, x0, p, stepper="rk4", observer="localmax", sp=dict(dt=0.01, max_steps=10000000),
        steps=[("transient", (0.0, 20.0)), ("shift_x0",), ("features", (20.0, 100.0))]), True, 0.0)
    x0, p = _lorenz(64, SEED)
    out["lorenz_heun_fp32_thresh2"] = (Scenario(
        "lorenz.cl", 3, 3, x0, p, n_aux=1, stepper="heun", observer="thresh2", single=True, n_store_events=2,
        sp=dict(dt=0.002), op=dict(e_var_ix=2, f_var_ix=2, max_event_count=100000, x_up_threshold=0.3,
                                   x_down_threshold=0.2),
        steps=[("features", (0.0, 20.0)), ("shift_x0",), ("shift_tspan",), ("features", None)]), True, 0.0)
    # rho in [5, 20]: no chaotic attractor, so last-bit differences of pow in
    # the step-size controller stay last-bit differences of the solution
    x0s, ps = _lorenz(64, SEED)
    ps[:, 0] = np.random.default_rng(SEED + 1).uniform(5, 20, 64)
    out["lorenz_dopri5_fp32_thresh2"] = (Scenario(
        "lorenz.cl", 3, 3, x0s, ps, n_aux=1, stepper="dopri5", observer="thresh2", single=True,
        sp=dict(dt=1e-3, dtmax=1.0, abstol=1e-9, reltol=1e-6), op=dict(e_var_ix=2, f_var_ix=2,
                                                                       max_event_count=100000,
                                                                       x_up_threshold=0.3, x_down_threshold=0.2),
        steps=[("features", (0.0, 20.0))]), False, 1e-3)
    out["lorenz_euler_fp64_nhood1"] = (Scenario(
        "lorenz.cl", 3, 3, x0, p, n_aux=1, stepper="euler", observer="nhood1", sp=dict(dt=0.001),
        op=dict(e_var_ix=2, f_var_ix=0, max_event_count=1000, nhood_radius=0.2),
        steps=[("features", (0.0, 20.0))]), True, 0.0)
    x0, p = _lacto(32, SEED)
    out["lactotroph_dopri5_fp32_nhood2"] = (Scenario(
        "lactotroph.cl", 4, 3, x0, p, n_aux=1, stepper="dopri5", observer="nhood2", single=True,
        sp=dict(dt=0.1, dtmax=1.0, abstol=1e-6, reltol=1e-6),
        op=dict(e_var_ix=3, f_var_ix=0, max_event_count=100000, nhood_radius=0.05, x_down_threshold=0.2),
        steps=[("features", (0.0, 2000.0))]), False, 1e-3)
    out["lactotroph_bs23_fp64_basicall"] = (Scenario(
        "lactotroph.cl", 4, 3, x0, p, n_aux=1, stepper="bs23", observer="basicall",
        sp=dict(dt=0.1, dtmax=5.0, abstol=1e-8, reltol=1e-6), steps=[("features", (0.0, 500.0))]), False, 1e-6)
    th = np.repeat(np.linspace(0.1, 2.0, 4), 8)
    sg = np.tile(np.linspace(0.1, 1.0, 4), 8)
    pou = np.stack([th, np.zeros(32), sg], axis=1)
    out["ou_seuler_fp32_trajectory"] = (Scenario(
        "ornstein_uhlenbeck.cl", 1, 3, np.zeros((32, 1)), pou, n_wiener=1, stepper="seuler", single=True,
        sp=dict(dt=1e-3, max_steps=2000, max_store=201, nout=10), seed=11,
        steps=[("trajectory", (0.0, 2.0))]), False, 1e-3)
    pth = np.tile([0.25, 8.0, 2.0, 10.0], (4, 1))
    out["thompson_a1_rk4_fp64_trajectory"] = (Scenario(
        "thompson_a1.cl", 2, 4, np.zeros((4, 2)), pth, n_aux=1, stepper="rk4",
        sp=dict(dt=0.01, dtmax=0.01, max_steps=20000, max_store=120, nout=5),
        steps=[("trajectory", (0.0, 5.0))]), True, 0.0)
    return out
