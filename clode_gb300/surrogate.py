"""Learned surrogate for large feature maps (no counterpart in clODE).

An MLP 2 -> 256 -> 256 -> 256 -> H heads x K features (BF16 tensor-core
layers with FP32 accumulation, trained on the GPU by this package's own
kernels, include/clode_gb300.h ``clode_mlp_*``) learns a feature map from a
coarse sub-grid that the ensemble engine integrates.  It then predicts the
full grid, and every point where the heads disagree or a feature jumps
between grid neighbours is integrated again by the plain engine, which stays
the fallback and the judge of the surrogate's error.

``FeatureMapScreen.run`` is the whole workflow; ``MLP`` is the network.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int)


def _fp(a):
    return None if a is None else a.ctypes.data_as(_F)


def _check(rc: int):
    N.check(rc)


class MLP:
    """The surrogate network on one GPU (handle of ``clode_mlp_create``)."""

    def __init__(self, n_outputs: int = 4, n_heads: int = 4, device: int = 0, seed: int = 0):
        self.K, self.H = n_outputs, n_heads
        self._h = C.c_void_p()
        _check(N.lib.clode_mlp_create(n_outputs, n_heads, device, seed, C.byref(self._h)))
        n = C.c_size_t(0)
        _check(N.lib.clode_mlp_param_count(self._h, C.byref(n)))
        self.n_params = n.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.lib.clode_mlp_destroy(h)
            self._h = C.c_void_p()

    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, dtype=np.float32)
        _check(N.lib.clode_mlp_get_params(self._h, _fp(out), out.size))
        return out

    def set_params(self, p) -> None:
        a = np.ascontiguousarray(p, dtype=np.float32)
        _check(N.lib.clode_mlp_set_params(self._h, _fp(a), a.size))

    def gradients(self, x, y):
        """Loss and gradient vector of one batch (no update)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_float(0.0)
        _check(N.lib.clode_mlp_gradients(self._h, _fp(x), _fp(y), x.shape[0], _fp(g), g.size, C.byref(loss)))
        return loss.value, g

    def train(self, x, y, steps: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        hist = np.zeros(max(steps, 1), dtype=np.float32)
        _check(N.lib.clode_mlp_train(self._h, _fp(x), _fp(y), x.shape[0], steps, batch, lr, seed, _fp(hist)))
        return hist[:steps]

    def predict(self, x, heads: bool = False):
        """Mean and spread (standard deviation) over the heads, (n, K) each."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        n = x.shape[0]
        mean = np.empty((n, self.K), dtype=np.float32)
        spread = np.empty((n, self.K), dtype=np.float32)
        hv = np.empty((n, self.H * self.K), dtype=np.float32) if heads else None
        _check(N.lib.clode_mlp_predict(self._h, _fp(x), n, _fp(mean), _fp(spread), _fp(hv)))
        return (mean, spread, hv) if heads else (mean, spread)

    def screen(self, nx: int, ny: int, spread_thr, jump_thr) -> np.ndarray:
        """Flags of the last prediction on an nx x ny grid: 1 = heads disagree, 2 = neighbour jump."""
        st = np.ascontiguousarray(spread_thr, dtype=np.float32)
        jt = np.ascontiguousarray(jump_thr, dtype=np.float32)
        flags = np.empty(nx * ny, dtype=np.int32)
        _check(N.lib.clode_mlp_screen(self._h, nx, ny, _fp(st), _fp(jt), flags.ctypes.data_as(_I)))
        return flags

    def timings(self):
        tr, pr = C.c_double(0), C.c_double(0)
        _check(N.lib.clode_mlp_timings(self._h, C.byref(tr), C.byref(pr)))
        return tr.value, pr.value


@dataclass
class ScreenResult:
    features: np.ndarray            # (ny*nx, K) screened map
    flags: np.ndarray               # per point: 0 surrogate value kept, else re-integrated
    timings: dict = field(default_factory=dict)
    loss: np.ndarray | None = None

    @property
    def fallback_fraction(self) -> float:
        return float(np.mean(self.flags != 0))


class FeatureMapScreen:
    """Surrogate-screened feature map of a 2-parameter grid.

    ``integrate(par0, par1) -> (n, K) features`` runs the plain engine on the
    given parameter points (a callable, so any model, stepper and observer
    can be screened).  ``lo``/``hi`` bound the two parameters.
    """

    def __init__(self, integrate, lo, hi, n_features: int, n_heads: int = 4, seed: int = 0, device: int = 0):
        self.integrate = integrate
        self.lo = np.asarray(lo, dtype=np.float64)
        self.hi = np.asarray(hi, dtype=np.float64)
        self.K = n_features
        self.net = MLP(n_features, n_heads, device, seed)
        self.seed = seed

    def _norm_x(self, p0, p1):
        x0 = 2.0 * (p0 - self.lo[0]) / (self.hi[0] - self.lo[0]) - 1.0
        x1 = 2.0 * (p1 - self.lo[1]) / (self.hi[1] - self.lo[1]) - 1.0
        return np.stack([x0, x1], axis=1).astype(np.float32)

    @staticmethod
    def rel_error(F, ref, scale):
        """Per point: the largest relative error over the features, relative to
        |ref| + 1e-3 * (feature scale) so features crossing zero stay defined."""
        return (np.abs(F - ref) / (np.abs(ref) + 1e-3 * scale)).max(axis=1)

    def calibrate(self, Xv, Fv, mu, sd, dx, dy, scale, tol, keep):
        """Thresholds on head spread and neighbour jump (normalised units) such
        that, on held-out integrated points, at least `keep` of the points the
        screen accepts have error <= tol; among those, the pair that accepts
        the most points.  Returns (spread_thr, jump_thr, accepted fraction)."""
        mean, spread = self.net.predict(Xv)
        err = self.rel_error(mean.astype(np.float64) * sd + mu, Fv, scale)
        s = spread.max(axis=1)
        j = np.zeros_like(s)
        for d in (np.array([dx, 0.0], np.float32), np.array([0.0, dy], np.float32)):
            for sign in (1.0, -1.0):
                mn, _ = self.net.predict(Xv + sign * d)
                j = np.maximum(j, np.abs(mn - mean).max(axis=1))
        qs = np.concatenate([np.linspace(0.0, 0.95, 20), [0.975, 0.99, 1.0]])
        s_cand = np.quantile(s, qs)
        j_cand = np.quantile(j, qs)
        best = (-1.0, -1.0, 0.0)
        for ts in s_cand:
            ok_s = s <= ts
            for tj in j_cand:
                acc = ok_s & (j <= tj)
                frac = acc.mean()
                if frac <= best[2] or not acc.any():
                    continue
                if np.mean(err[acc] <= tol) >= keep:
                    best = (float(ts), float(tj), float(frac))
        return best

    def run(self, nx: int, ny: int, train_stride: int = 8, steps: int = 3000, batch: int = 4096,
            lr: float = 2e-3, tol: float = 0.01, keep: float = 0.99, holdout: float = 0.1) -> ScreenResult:
        """Screened map of the nx x ny grid; `tol`/`keep`: the accepted
        surrogate values are calibrated to have error <= tol for a fraction
        `keep` of held-out integrated points."""
        t_all = time.perf_counter()
        g0 = np.linspace(self.lo[0], self.hi[0], nx)
        g1 = np.linspace(self.lo[1], self.hi[1], ny)
        P0, P1 = np.meshgrid(g0, g1, indexing="xy")  # point m = iy * nx + ix
        P0, P1 = P0.ravel(), P1.ravel()
        # 1. a coarse sub-grid integrated by the engine
        sub = np.zeros((ny, nx), dtype=bool)
        sub[::train_stride, ::train_stride] = True
        sub = sub.ravel()
        t0 = time.perf_counter()
        Fsub = np.asarray(self.integrate(P0[sub], P1[sub]), dtype=np.float64)
        t_train_data = time.perf_counter() - t0
        Xsub = self._norm_x(P0[sub], P1[sub])
        rng = np.random.default_rng(self.seed)
        val = rng.random(Xsub.shape[0]) < holdout
        mu, sd = Fsub[~val].mean(axis=0), Fsub[~val].std(axis=0) + 1e-12
        scale = np.abs(Fsub).max(axis=0)
        Y = ((Fsub[~val] - mu) / sd).astype(np.float32)
        # 2. training on the GPU, learning rate halved over four phases
        t0 = time.perf_counter()
        losses = []
        for ph in range(4):
            losses.append(self.net.train(Xsub[~val], Y, steps=steps // 4, batch=batch, lr=lr / 2 ** ph,
                                         seed=self.seed + ph))
        loss = np.concatenate(losses)
        t_train = time.perf_counter() - t0
        # 3. calibration of the screen on the held-out integrated points
        t0 = time.perf_counter()
        dx, dy = 2.0 / max(nx - 1, 1), 2.0 / max(ny - 1, 1)
        ts, tj, acc = self.calibrate(Xsub[val], Fsub[val], mu, sd, dx, dy, scale, tol, keep)
        t_cal = time.perf_counter() - t0
        # 4. prediction of the full grid and screening
        t0 = time.perf_counter()
        mean, spread = self.net.predict(self._norm_x(P0, P1))
        flags = self.net.screen(nx, ny, np.full(self.K, ts), np.full(self.K, tj))
        if ts < 0:
            flags[:] = 4  # no threshold met the error bar: everything is integrated
        t_predict = time.perf_counter() - t0
        F = mean.astype(np.float64) * sd + mu
        # the integrated sub-grid points are known exactly
        F[sub] = Fsub
        flags[sub] = 0
        # 4. fallback: the plain engine on every flagged point
        t0 = time.perf_counter()
        redo = np.nonzero(flags)[0]
        if redo.size:
            F[redo] = np.asarray(self.integrate(P0[redo], P1[redo]), dtype=np.float64)
        t_fallback = time.perf_counter() - t0
        total = time.perf_counter() - t_all
        return ScreenResult(F, flags, loss=loss, timings={
            "train_data_s": t_train_data, "train_s": t_train, "calibrate_s": t_cal, "predict_screen_s": t_predict,
            "fallback_s": t_fallback, "total_s": total, "points": nx * ny,
            "points_per_s": nx * ny / total, "fallback_points": int(redo.size),
            "integrated_points": int(redo.size + sub.sum()), "spread_thr": ts, "jump_thr": tj,
            "calibrated_accept_fraction": acc})
