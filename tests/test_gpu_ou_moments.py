"""Stochastic Euler on the Ornstein-Uhlenbeck process dx = theta (mu - x) dt
+ sigma dW: after many relaxation times the ensemble of realisations has the
stationary mean mu and the Euler-Maruyama stationary variance
sigma^2 / (theta (2 - theta dt)) (the exact process: sigma^2 / (2 theta)),
within the sampling error of the ensemble (the reference's OU example,
examples/Ornstein_Uhlenbeck.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("single", [True, False])
def test_ou_stationary_moments(single):
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path

    n_each = 32768
    thetas = np.array([0.5, 2.0])
    sigma, mu, dt = 0.8, 0.3, 1e-3
    pars = np.concatenate([np.tile([th, mu, sigma], (n_each, 1)) for th in thetas])
    n = pars.shape[0]
    pi = W.ProblemInfo(rhs_path("ornstein_uhlenbeck.cl"), ["x"], ["theta", "mu", "sigma"], [], 1)
    sim = W.SimulatorBase(pi, "seuler", single, W.OpenCLResource(), "")
    sim.set_option("schedule", 1)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=dt, max_steps=10000000))
    sim.set_problem_data(np.zeros(n), pars.flatten(order="F"))
    sim.seed_rng(2024)
    sim.set_tspan([0.0, 20.0])  # 10 relaxation times of the slower process
    sim.transient()
    xf = np.asarray(sim.get_xf())
    for k, th in enumerate(thetas):
        x = xf[k * n_each:(k + 1) * n_each]
        v_em = sigma ** 2 / (th * (2.0 - th * dt))
        v_exact = sigma ** 2 / (2.0 * th)
        m, s2 = x.mean(), x.var(ddof=1)
        # 5-sigma sampling bounds of the mean and of the sample variance
        assert abs(m - mu) < 5.0 * np.sqrt(v_em / n_each), (th, m)
        assert abs(s2 - v_em) < 5.0 * v_em * np.sqrt(2.0 / (n_each - 1)), (th, s2, v_em)
        # the discretisation bias is below the sampling error here
        assert abs(v_em - v_exact) < v_em * np.sqrt(2.0 / (n_each - 1))
