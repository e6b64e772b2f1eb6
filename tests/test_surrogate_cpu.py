"""Host logic of the surrogate-screened feature map, on the CPU: the
sub-grid / calibration / fallback bookkeeping and the calibrated cell screen,
with an analytic map standing in for the engine and a stand-in network whose
error is known (no GPU involved)."""
import numpy as np
import pytest

from clode_gb300.surrogate import FeatureMapScreen, ScreenResult


def _map(p0, p1):
    """Smooth features with a jump along p0 + p1 = 1."""
    a = np.sin(3 * p0) * np.cos(2 * p1)
    b = np.where(p0 + p1 > 1.0, 1.0, 0.0) + 0.1 * p0
    return np.stack([a, b], axis=1)


class _FakeNet:
    """Predicts the map exactly except inside a disc, where it is off by 5 %
    of the feature range, and near the jump, where it smears the step."""

    def __init__(self, lo, hi):
        self.lo, self.hi = np.asarray(lo, float), np.asarray(hi, float)
        self.trained = 0

    def train(self, x, y, steps, batch, lr, seed):
        self.trained += steps
        return np.zeros(max(steps, 0), dtype=np.float32)

    def predict_grid(self, nx, ny, scale, offset):
        g0 = np.linspace(self.lo[0], self.hi[0], nx)
        g1 = np.linspace(self.lo[1], self.hi[1], ny)
        P0, P1 = np.meshgrid(g0, g1, indexing="xy")
        P0, P1 = P0.ravel(), P1.ravel()
        F = _map(P0, P1)
        F[:, 1] = 1.0 / (1.0 + np.exp(-(P0 + P1 - 1.0) / 0.02)) + 0.1 * P0  # smeared step
        disc = (P0 - 0.3) ** 2 + (P1 - 0.7) ** 2 < 0.01
        F[disc, 0] += 0.05 * 2.0
        return F.astype(np.float32)


def _screen(calls):
    def integrate(p0, p1):
        calls.append(p0.size)
        return _map(p0, p1)

    scr = FeatureMapScreen.__new__(FeatureMapScreen)
    scr.integrate = integrate
    scr.lo, scr.hi = np.array([0.0, 0.0]), np.array([1.0, 1.0])
    scr.K = 2
    scr.net = _FakeNet(scr.lo, scr.hi)
    scr.seed = 3
    return scr


@pytest.mark.parametrize("refine", [False, True])
def test_screened_map_bookkeeping_and_error(refine):
    calls = []
    scr = _screen(calls)
    nx, ny = 200, 150
    res = scr.run(nx, ny, train_stride=8, steps=40, batch=64, tol=0.01, keep=0.99, n_calibration=3000,
                  refine=refine)
    g0, g1 = np.linspace(0, 1, nx), np.linspace(0, 1, ny)
    P0, P1 = np.meshgrid(g0, g1, indexing="xy")
    exact = _map(P0.ravel(), P1.ravel())
    t = res.timings
    # the sub-grid includes the last lines; calibration points are interior
    assert t["training_points"] == len(np.unique(np.r_[0:nx:8, nx - 1])) * len(np.unique(np.r_[0:ny:8, ny - 1]))
    assert t["calibration_points"] == 3000
    # one engine call integrates the sub-grid and the calibration sample together
    assert calls[0] == t["training_points"] + 3000
    sampled = t["training_points"] + 3000 + t["lattice_points"] + t["calibration2_points"]
    assert t["integrated_points"] == sampled + t["fallback_points"]
    assert np.count_nonzero(res.flags == ScreenResult.SAMPLED) == sampled
    assert np.count_nonzero(res.flags == ScreenResult.FALLBACK) == t["fallback_points"]
    if not refine:
        assert t["lattice_points"] == 0 and t["calibration2_points"] == 0
    # every integrated point carries the engine's value
    integ = res.flags != ScreenResult.SURROGATE
    np.testing.assert_array_equal(res.features[integ], exact[integ].astype(np.float32))
    # the disc and the jump are integrated, the rest kept
    scale = exact.max(axis=0) - exact.min(axis=0)
    err = FeatureMapScreen.map_error(res.features, exact, scale)
    assert np.mean(err <= 0.01) >= 0.99
    disc = ((P0 - 0.3) ** 2 + (P1 - 0.7) ** 2 < 0.01).ravel()
    # cells with a corner in the disc are integrated; edge cells whose four
    # corners miss it may keep a few surrogate points (the calibrated error
    # bound above still holds)
    assert np.mean(res.flags[disc] != ScreenResult.SURROGATE) > 0.8
    assert 0.15 < res.integrated_fraction < 0.6


def test_calibration_search():
    rng = np.random.default_rng(0)
    r = rng.uniform(0, 1, 5000)
    v = rng.uniform(0, 1, 5000)
    err = np.where(r > 0.6, 0.5, 0.001)  # points with r above 0.6 are wrong
    tr, tv, frac = FeatureMapScreen._calibrate(r, v, err, 0.01, 0.99)
    acc = (r <= tr) & (v <= tv)
    assert np.mean(err[acc] <= 0.01) >= 0.99
    assert 0.55 < frac <= 0.62 and tv >= np.quantile(v, 0.99)
    assert FeatureMapScreen._calibrate(r, v, np.ones_like(r), 0.01, 0.99) == (-1.0, -1.0, 0.0)
