"""Getters into a caller's buffer (``get_f(out=...)``, no reference
counterpart): the values equal those of the allocating getter, the buffer
may be larger than needed and may be page-locked host memory reused between
calls (which the conversion kernel writes directly); a buffer of the wrong
type or size is refused.  Inputs in page-locked host memory (read directly
by the conversion kernel) give the results of ordinary arrays."""
import numpy as np
import pytest

from clode_gb300 import clode_cpp_wrapper as W, rhs_path

pytestmark = pytest.mark.gpu


def _sim(n=3000):
    pi = W.ProblemInfo(rhs_path("lorenz.cl"), ["x", "y", "z"], ["rho", "sigma", "beta"], ["fx"], 0)
    op = W.ObserverParams(e_var_ix=2, f_var_ix=0, max_event_count=100000, x_up_threshold=0.3,
                          x_down_threshold=0.2)
    sim = W.FeatureSimulatorBase(pi, "dopri5", "thresh2", op, True, W.OpenCLResource(), "")
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=1e-3, dtmax=1.0, abstol=1e-9, reltol=1e-6, max_steps=1000000))
    r = np.random.default_rng(1)
    x0 = np.ones((n, 3)) + r.normal(0, 1e-3, (n, 3))
    pars = np.stack([r.uniform(10, 40, n), r.uniform(5, 15, n), np.full(n, 8 / 3)], axis=1)
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan([0.0, 20.0])
    sim.features(True)
    return sim


def test_get_f_into_caller_buffers():
    torch = pytest.importorskip("torch")
    sim = _sim()
    ref = sim.get_f()
    plain = np.full(ref.size + 17, np.nan)
    got = sim.get_f(out=plain)
    assert got.size == ref.size and np.shares_memory(got, plain)
    assert np.array_equal(got, ref, equal_nan=True)
    pinned = torch.empty(ref.size, dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(2):  # reused between calls
        pinned[:] = np.nan
        got = sim.get_f(out=pinned)
        assert np.array_equal(got, ref, equal_nan=True)


def test_get_f_refuses_unfit_buffers():
    sim = _sim(200)
    n = sim.get_f().size
    for bad in (np.zeros(n - 1), np.zeros(n, dtype=np.float32), np.zeros((n, 2))[:, 0]):
        with pytest.raises(ValueError):
            sim.get_f(out=bad)


def test_page_locked_inputs_give_the_same_results():
    torch = pytest.importorskip("torch")
    n = 3000
    r = np.random.default_rng(1)
    x0 = (np.ones((n, 3)) + r.normal(0, 1e-3, (n, 3))).flatten(order="F")
    pars = np.stack([r.uniform(10, 40, n), r.uniform(5, 15, n), np.full(n, 8 / 3)], axis=1).flatten(order="F")

    def pinned(a):
        b = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy()
        b[:] = a
        return b

    outs = []
    for x, p in ((x0, pars), (pinned(x0), pinned(pars))):
        sim = _sim(10)
        sim.set_problem_data(x, p)
        sim.set_tspan([0.0, 20.0])
        sim.features(True)
        outs.append((sim.get_f(), np.asarray(sim.get_x0()), np.asarray(sim.get_pars())))
    for a, b in zip(*outs):
        assert np.array_equal(a, b, equal_nan=True)
