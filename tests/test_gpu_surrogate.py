"""The surrogate network's own tensor-core kernels against the NumPy oracle
(forward and gradients), its training, its screening, and what it gains over
integrating every point of a feature map with the plain engine."""
import time

import numpy as np
import pytest

from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu


def _net(K=4, H=4, seed=3):
    from clode_gb300.surrogate import MLP
    return MLP(K, H, 0, seed)


def test_tensor_core_forward_matches_oracle():
    net = _net()
    p = net.get_params()
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (1000, 2)).astype(np.float32)  # not a multiple of the 128-row tile
    mean, spread, heads = net.predict(x, heads=True)
    ref = MO.forward(p, x, 16)["out"]
    scale = np.abs(ref).max()
    # tolerance: BF16 activations; a value on a rounding tie may round the other way
    # when the GPU accumulates in FP32 and the oracle in float64
    np.testing.assert_allclose(heads, ref, rtol=2e-2, atol=2e-2 * scale)
    r4 = ref.reshape(-1, 4, 4)
    np.testing.assert_allclose(mean, r4.mean(axis=1), rtol=2e-2, atol=2e-2 * scale)


def test_gradients_match_oracle():
    net = _net(seed=5)
    p = net.get_params()
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (777, 2)).astype(np.float32)
    y = np.stack([np.sin(3 * x[:, 0]), np.cos(2 * x[:, 1]), x[:, 0] * x[:, 1], x[:, 0] ** 2], axis=1)
    y = y.astype(np.float32)
    loss, g = net.gradients(x, y)
    lref, gref, _ = MO.loss_and_gradients(p, x, y, 4, 4)
    assert abs(loss - lref) <= 1e-3 * abs(lref) + 1e-6
    parts = MO.split(g, 16)
    refs = MO.split(gref, 16)
    for name in parts:
        a, b = parts[name].ravel(), refs[name].ravel()
        err = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30)
        # tolerance: BF16 rounding of activations and back-propagated gradients
        assert err < 2e-2, (name, err)


def test_grid_prediction_matches_point_prediction():
    net = _net(seed=11)
    nx, ny = 300, 211  # not multiples of the 128-row tile
    gx = np.linspace(-1, 1, nx, dtype=np.float64)
    gy = np.linspace(-1, 1, ny, dtype=np.float64)
    X0, X1 = np.meshgrid(gx, gy, indexing="xy")
    x = np.stack([X0.ravel(), X1.ravel()], axis=1).astype(np.float32)
    mean, _ = net.predict(x)
    scale = np.array([2.0, -1.0, 0.5, 3.0], dtype=np.float32)
    offset = np.array([0.0, 1.0, -2.0, 0.25], dtype=np.float32)
    grid = net.predict_grid(nx, ny, scale, offset)
    # tolerance: the device computes the grid coordinates in FP32, the host in
    # float64 rounded once; an ulp of input moves the sine layer slightly
    np.testing.assert_allclose(grid, mean * scale + offset, rtol=0, atol=2e-2 * np.abs(mean).max() * 3.0)
    assert np.median(np.abs(grid - (mean * scale + offset))) < 1e-3 * np.abs(mean).max() * 3.0


def test_training_fits_a_smooth_map():
    net = _net(seed=7)
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, (65536, 2)).astype(np.float32)
    y = np.stack([np.sin(3 * x[:, 0]) * np.cos(2 * x[:, 1]), x[:, 0] * x[:, 1], np.exp(-x[:, 0] ** 2),
                  x[:, 1] ** 3], axis=1).astype(np.float32)
    hist = net.train(x, y, steps=1500, batch=2048, lr=2e-3)
    assert np.isfinite(hist).all()
    assert hist[-50:].mean() < 0.02 * hist[:5].mean()
    xt = rng.uniform(-1, 1, (4096, 2)).astype(np.float32)
    yt = np.stack([np.sin(3 * xt[:, 0]) * np.cos(2 * xt[:, 1]), xt[:, 0] * xt[:, 1], np.exp(-xt[:, 0] ** 2),
                   xt[:, 1] ** 3], axis=1)
    mean, spread = net.predict(xt)
    assert np.sqrt(np.mean((mean - yt) ** 2)) < 0.05


def test_screen_flags_the_discontinuity():
    net = _net(seed=9)
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (65536, 2)).astype(np.float32)
    y = np.repeat((x[:, :1] > 0).astype(np.float32), 4, axis=1)  # a step along x0 = 0
    net.train(x, y, steps=800, batch=2048, lr=2e-3)
    n = 64
    g = np.linspace(-1, 1, n)
    G0, G1 = np.meshgrid(g, g, indexing="xy")
    net.predict(np.stack([G0.ravel(), G1.ravel()], axis=1))
    flags = net.screen(n, n, np.full(4, 10.0), np.full(4, 0.25)).reshape(n, n)
    cols = np.nonzero(flags.any(axis=0))[0]
    assert cols.size > 0
    assert np.abs(g[cols]).max() < 0.2  # only next to the step
    assert flags[:, :20].sum() == 0 and flags[:, -20:].sum() == 0


def test_surrogate_screened_map_gains_over_plain_engine():
    """The trained network against the method without it: a 1024 x 1024
    lactotroph map (fixed tspan) computed point by point by the plain engine,
    and the same map surrogate-screened (257 x 257 integrated sub-grid, GPU
    training, prediction, calibrated cell screen, engine fallback on
    rejected cells)."""
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path
    from clode_gb300.surrogate import FeatureMapScreen

    W.get_logger().set_log_level(W.LogLevel.warn)
    pi = W.ProblemInfo(rhs_path("lactotroph.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"], 0)
    op = W.ObserverParams(e_var_ix=3, f_var_ix=0, max_event_count=1000000, nhood_radius=0.05, x_down_threshold=0.2)
    sim = W.FeatureSimulatorBase(pi, "dopri5", "nhood2", op, True, W.OpenCLResource(), "")
    sim.set_option("schedule", 1)
    sim.set_option("fmad", 1)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=0.1, dtmax=1.0, abstol=1e-6, reltol=1e-6, max_steps=10000000))
    names = None
    cols = None

    def integrate(gcal, gbk):
        nonlocal names, cols
        n = gcal.size
        pars = np.stack([gcal, np.full(n, 3.0), gbk], axis=1)
        x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
        sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
        sim.set_tspan([0.0, 3000.0])
        sim.features(True)
        if names is None:
            names = sim.get_feature_names()
            cols = [names.index(c) for c in ("max v", "min v", "mean v", "mean c")]
        F = np.asarray(sim.get_f()).reshape(-1, n).T
        return F[:, cols]

    nx = ny = 1024
    g0 = np.linspace(0.5, 3.0, nx)
    g1 = np.linspace(0.0, 2.0, ny)
    P0, P1 = np.meshgrid(g0, g1, indexing="xy")
    integrate(P0.ravel()[:1000], P1.ravel()[:1000])  # program build and warm-up
    t0 = time.perf_counter()
    plain = integrate(P0.ravel(), P1.ravel())
    t_plain = time.perf_counter() - t0

    scr = FeatureMapScreen(integrate, lo=(0.5, 0.0), hi=(3.0, 2.0), n_features=4, seed=1)
    res = scr.run(nx, ny, train_stride=4, steps=3000, batch=4096, tol=0.01, keep=0.99, n_calibration=16384)
    scale = plain.max(axis=0) - plain.min(axis=0)
    err = FeatureMapScreen.map_error(res.features, plain, scale)
    good = np.mean(err <= 0.01)
    integrated = res.integrated_fraction
    print(f"plain {t_plain:.2f} s, screened {res.timings['total_s']:.2f} s, integrated fraction "
          f"{integrated:.3f}, points within 1 % of range: {good:.4f}, timings {res.timings}")
    # the stated error (1 % of each feature's range) holds on the whole map ...
    assert good >= 0.98
    # ... while the engine integrates only part of it: the network's gain
    assert integrated < 0.5
    # the sub-grid and calibration points carry the engine's values exactly
    sampled = res.flags == res.SAMPLED
    np.testing.assert_array_equal(res.features[sampled], plain[sampled])
