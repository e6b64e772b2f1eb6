"""The precise option against an FP64 reference solution.

``precise`` (no counterpart in the reference; not a parity build) keeps the
bulk of the integration in FP32 and adds: compensated time accumulation for
the fixed-step steppers, a compensated evaluation of the adaptive
controller's error estimate, compensated time-weighted means, and event
times refined inside the detecting step (cubic Hermite interpolation of the
step, root found in FP64) with event times and periods kept in FP64.

Each test states the error of the plain FP32 build and of the precise
build against an FP64 solution and requires the precise build's to be the
smaller one:

* Van der Pol (limit cycles, mu ~ U[0.5, 3]) and the non-chaotic members of
  the Lorenz (sigma, rho) grid (those whose FP64 result does not move under a
  1e-9 change of the initial state, ``tests/golden/lorenz_grid_fp64.npz``),
  DP45 rtol 1e-6 atol 1e-9 in FP32, thresh2: the mean period against the
  event times of the oracle's FP64 solution at rtol 1e-10, refined the same
  way (every stored step, in NumPy);
* Lorenz at rho = 15, RK4 with dt = the FP32 value of 1e-3 for 1e5 steps,
  thresh2: the number of steps, the final time and the time-weighted means
  against the engine's FP64 run of the same steps.
"""
import json
import os

import numpy as np
import pytest

from tests.parity import Scenario, run_engine, run_oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
T1 = 40.0


def _sc(model, x0, pars, single, tol, t1, stepper="dopri5", dt=1e-3, traj=False, max_store=1):
    nv, npar, naux, ev = (3, 3, 1, 2) if model == "lorenz.cl" else (2, 1, 0, 0)
    return Scenario(model, nv, npar, x0, pars, n_aux=naux, stepper=stepper,
                    observer=None if traj else "thresh2", single=single,
                    sp=dict(dt=dt, dtmax=1.0, abstol=tol * 1e-3, reltol=tol, max_steps=10000000,
                            max_store=max_store, nout=1),
                    op=dict(e_var_ix=ev, f_var_ix=ev, max_event_count=100000, x_up_threshold=0.3,
                            x_down_threshold=0.2),
                    steps=[("trajectory" if traj else "features", (0.0, t1))], seed=None)


def _hermite_crossing(t0, x0, d0, t1, x1, d1, level):
    """Time in [t0, t1] where the step's cubic Hermite interpolant equals level."""
    h = t1 - t0
    lo, hi = 0.0, 1.0
    f0 = x0 - level
    for _ in range(100):
        s = 0.5 * (lo + hi)
        s2, s3 = s * s, s * s * s
        v = (2 * s3 - 3 * s2 + 1) * x0 + (s3 - 2 * s2 + s) * h * d0 + (-2 * s3 + 3 * s2) * x1 + (s3 - s2) * h * d1
        if (v - level < 0) == (f0 < 0):
            lo = s
        else:
            hi = s
    return t0 + 0.5 * (lo + hi) * h


def _thresh2_mean_period(t, z, dz, t1, up=0.3, down=0.2):
    """Mean period of thresh2 (e = f, dx thresholds 0) from every step of a
    solution, event times refined as the precise option refines them
    (clode/cpp/observers/observer_threshold_2.clh event logic).  Returns
    (events, mean period)."""
    K = t.size - 1
    warm = 0
    while warm < K and t[warm] < t1:
        warm += 1
    zw, dw = z[1:warm + 1], dz[1:warm + 1]
    lo_, amp = zw.min(), zw.max() - zw.min()
    x_up, x_down, dx_up, dx_down = lo_ + up * amp, lo_ + down * amp, 0.0, dw.min()
    is_up = z[0] > x_up
    ev = []
    for k in range(2, K + 1):
        if is_up and z[k] <= x_down and dz[k] >= dx_down:
            is_up = False
        if not is_up and z[k] > x_up and dz[k] > dx_up:
            te = _hermite_crossing(t[k - 1], z[k - 1], dz[k - 1], t[k], z[k], dz[k], x_up) if z[k - 1] <= x_up else t[k]
            ev.append(te)
            is_up = True
    per = np.diff(ev)
    return len(ev), (per.mean() if per.size else 0.0)


def _period_errors(model, x0, pars, t1, e_var, max_store):
    """Mean-period errors of the plain and precise FP32 builds against the
    refined FP64 solution, over members with two or more events."""
    ora = run_oracle(_sc(model, x0, pars, False, 1e-10, t1, traj=True, max_store=max_store))
    assert ora["n_stored"].max() < max_store  # every step stored
    n_truth, per_truth = [], []
    for i in range(x0.shape[0]):
        k = int(ora["n_stored"][i]) + 1
        t, z, dz = ora["t"][i, :k], ora["x"][i, e_var, :k], ora["dx"][i, e_var, :k]
        ne, mp = _thresh2_mean_period(t, z, dz, t1)
        n_truth.append(ne)
        per_truth.append(mp)
    n_truth, per_truth = np.array(n_truth), np.array(per_truth)
    plain = run_engine(_sc(model, x0, pars, True, 1e-6, t1), options={"schedule": 1})
    precise = run_engine(_sc(model, x0, pars, True, 1e-6, t1), options={"schedule": 1, "precise": 1})
    names = plain["feature_names"]
    ev, per = names.index("event count"), names.index("mean period")
    Fp, Fq = plain["F_list"][0], precise["F_list"][0]
    assert (Fq[:, ev] == n_truth).all()  # the events of the FP64 solution
    m = n_truth >= 2
    e_plain = np.abs(Fp[m, per] - per_truth[m]) / per_truth[m]
    e_precise = np.abs(Fq[m, per] - per_truth[m]) / per_truth[m]
    print(f"\n{model}: mean period vs FP64 (refined events), {m.sum()} members: plain median "
          f"{np.median(e_plain):.2e} max {e_plain.max():.2e}; precise median {np.median(e_precise):.2e} "
          f"max {e_precise.max():.2e}")
    return m.sum(), e_plain, e_precise


def test_vdp_event_times_refined():
    n = 128
    r = np.random.default_rng(12)
    x0 = r.uniform(-2.0, 2.0, (n, 2))
    mu = r.uniform(0.5, 3.0, (n, 1))
    count, e_plain, e_precise = _period_errors("van_der_pol.cl", x0, mu, 100.0, 0, 60000)
    assert count >= 100
    assert np.median(e_precise) < 0.1 * np.median(e_plain)
    assert e_precise.max() < e_plain.max()


def test_lorenz_event_times_refined():
    d = np.load(os.path.join(GOLDEN, "lorenz_grid_fp64.npz"))
    cols = json.loads(str(d["meta"]))["perturbed_columns"]
    F64 = d["F"]
    rel = lambda a, b: np.abs(a - b) / np.maximum(np.abs(b), 1e-6)  # noqa: E731
    moved = np.maximum(rel(d["F_up"][:, 1:-1], F64[:, cols[1:-1]]).max(1),
                       rel(d["F_down"][:, 1:-1], F64[:, cols[1:-1]]).max(1))
    quiet = np.where((moved < 1e-6) & (d["F_up"][:, -1] == F64[:, 36]) & (d["F_down"][:, -1] == F64[:, 36])
                     & (F64[:, 36] >= 2))[0]
    sel = quiet[np.linspace(0, quiet.size - 1, min(96, quiet.size)).astype(int)]
    count, e_plain, e_precise = _period_errors("lorenz.cl", d["x0"][sel], d["pars"][sel], T1, 2, 30000)
    assert count >= 10
    assert np.median(e_precise) < 0.1 * np.median(e_plain)
    assert e_precise.max() < e_plain.max()


def test_compensated_time_and_means_fixed_step():
    n = 256
    r = np.random.default_rng(2)
    x0 = np.ones((n, 3)) + r.normal(0, 1e-3, (n, 3))
    pars = np.stack([np.full(n, 15.0), r.uniform(8, 12, n), np.full(n, 8 / 3)], axis=1)
    # dt is the FP32 value of 1e-3 in every run, so the FP64 run integrates the same steps
    dt = float(np.float32(1e-3))
    sc = lambda single: _sc("lorenz.cl", x0, pars, single, 1e-6, 100.0, stepper="rk4", dt=dt)  # noqa: E731
    ref = run_engine(sc(False), options={"schedule": 1})
    plain = run_engine(sc(True), options={"schedule": 1})
    precise = run_engine(sc(True), options={"schedule": 1, "precise": 1})
    names = ref["feature_names"]
    steps = names.index("step count")
    F64, Fp, Fq = ref["F_list"][0], plain["F_list"][0], precise["F_list"][0]
    print(f"\nsteps FP64 {F64[0, steps]:.0f} plain FP32 {Fp[0, steps]:.0f} precise FP32 {Fq[0, steps]:.0f}; "
          f"tf FP64 {ref['tf'][0]!r} plain {plain['tf'][0]!r} precise {precise['tf'][0]!r}")
    # the precise build takes the FP64 run's steps and ends at its time (to FP32 rounding)
    assert (Fq[:, steps] == F64[:, steps]).all()
    ulp = np.spacing(np.float32(100.0))
    assert (np.abs(precise["tf"] - ref["tf"]) <= ulp).all()
    assert np.abs(plain["tf"] - ref["tf"]).max() >= np.abs(precise["tf"] - ref["tf"]).max()
    # time-weighted means of x, y, z
    cols = [names.index(f"mean x{j}") for j in range(3)]
    e_plain = np.abs(Fp[:, cols] - F64[:, cols]) / np.abs(F64[:, cols])
    e_precise = np.abs(Fq[:, cols] - F64[:, cols]) / np.abs(F64[:, cols])
    print(f"means vs FP64: plain median {np.median(e_plain):.2e} max {e_plain.max():.2e}; "
          f"precise median {np.median(e_precise):.2e} max {e_precise.max():.2e}")
    assert np.median(e_precise) <= np.median(e_plain)
