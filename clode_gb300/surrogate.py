"""Learned surrogate for large feature maps (no counterpart in clODE).

An MLP 2 -> 256 (sine) -> 256 -> 256 -> H heads x K features (BF16
tensor-core layers with FP32 accumulation, trained on the GPU by this
package's own kernels, include/clode_gb300.h ``clode_mlp_*``) learns a
feature map from a coarse sub-grid that the ensemble engine integrates.  It
then predicts the full grid; the cells of the sub-grid where the network
misses the integrated corners, or where the corners reveal a discontinuity,
are integrated again by the plain engine, which stays the fallback and the
reference for the surrogate's error.

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

    WIDTH = 256

    def __init__(self, n_outputs: int = 4, n_heads: int = 4, device: int = 0, seed: int = 0,
                 input_scale: float | None = None):
        """`input_scale`: the first (sine) layer's frequencies are drawn from
        U(-input_scale, input_scale) for inputs normalised to [-1, 1]
        (default: the library's, 20)."""
        self.K, self.H = n_outputs, n_heads
        self._h = C.c_void_p()
        _check(N.lib.clode_mlp_create(n_outputs, n_heads, device, seed, C.byref(self._h)))
        n = C.c_size_t(0)
        _check(N.lib.clode_mlp_param_count(self._h, C.byref(n)))
        self.n_params = n.value
        if input_scale is not None:
            p = self.get_params()
            rng = np.random.default_rng(seed)
            p[:2 * self.WIDTH] = rng.uniform(-input_scale, input_scale, 2 * self.WIDTH)
            self.set_params(p)

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

    def predict_grid(self, nx: int, ny: int, scale=None, offset=None) -> np.ndarray:
        """Mean over the heads on the nx x ny grid of inputs in [-1, 1]^2
        (point iy * nx + ix), generated on the device; returns
        mean * scale + offset as float32, shape (nx * ny, K)."""
        out = np.empty((nx * ny, self.K), dtype=np.float32)
        sc = None if scale is None else np.ascontiguousarray(scale, dtype=np.float32)
        of = None if offset is None else np.ascontiguousarray(offset, dtype=np.float32)
        _check(N.lib.clode_mlp_predict_grid(self._h, nx, ny, _fp(sc), _fp(of), _fp(out)))
        return out

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
    flags: np.ndarray               # per point: SURROGATE, FALLBACK or SAMPLED
    timings: dict = field(default_factory=dict)
    loss: np.ndarray | None = None

    SURROGATE, FALLBACK, SAMPLED = 0, 1, 2

    @property
    def fallback_fraction(self) -> float:
        return float(np.mean(self.flags == self.FALLBACK))

    @property
    def integrated_fraction(self) -> float:
        return float(np.mean(self.flags != self.SURROGATE))


class FeatureMapScreen:
    """Surrogate-screened feature map of a 2-parameter grid.

    ``integrate(par0, par1) -> (n, K) features`` runs the plain engine on the
    given parameter points (a callable, so any model, stepper and observer
    can be screened).  ``lo``/``hi`` bound the two parameters.

    Error measure: a point's error is the largest over the K features of
    |surrogate - engine| / (the feature's range over the map), so "1 %" means
    one percent of the feature's span.

    Screening is by cells of the integrated sub-grid: a cell's points take
    the network's values when the network reproduces the four integrated
    corners to within ``r`` and the corners themselves vary by at most ``v``
    (no discontinuity crosses the cell's corners); otherwise every point of
    the cell is integrated.  ``r`` and ``v`` are calibrated on a random sample
    of integrated interior points so that a fraction ``keep`` of the accepted
    sample points is within ``tol``.
    """

    def __init__(self, integrate, lo, hi, n_features: int, n_heads: int = 4, seed: int = 0, device: int = 0,
                 input_scale: float | None = None):
        self.integrate = integrate
        self.lo = np.asarray(lo, dtype=np.float64)
        self.hi = np.asarray(hi, dtype=np.float64)
        self.K = n_features
        self.net = MLP(n_features, n_heads, device, seed, input_scale=input_scale)
        self.seed = seed

    def _norm_x(self, p0, p1):
        x0 = 2.0 * (p0 - self.lo[0]) / (self.hi[0] - self.lo[0]) - 1.0
        x1 = 2.0 * (p1 - self.lo[1]) / (self.hi[1] - self.lo[1]) - 1.0
        return np.stack([x0, x1], axis=1).astype(np.float32)

    @staticmethod
    def map_error(F, ref, scale):
        """Per point: max over features of |F - ref| / scale (scale = feature range)."""
        return (np.abs(np.asarray(F, np.float64) - ref) / np.maximum(scale, 1e-30)).max(axis=1)

    @staticmethod
    def _calibrate(r, v, err, tol, keep):
        """Thresholds (r_max, v_max) on the sample's cell statistics such that
        at least `keep` of the accepted sample points have err <= tol; the pair
        accepting the most points.  r_max runs over every sample value (prefix
        sums in r order), v_max over quantiles of v.  Returns (r_max, v_max,
        accepted fraction), (-1, -1, 0) when no pair qualifies."""
        n = r.size
        best = (-1.0, -1.0, 0.0)
        if n == 0:
            return best
        good = err <= tol
        order = np.argsort(r, kind="stable")
        r_s, v_s, g_s = r[order], v[order], good[order]
        last_of_tie = np.r_[r_s[1:] != r_s[:-1], True]
        qs = np.concatenate([np.linspace(0.0, 0.95, 39), [0.975, 0.99, 1.0]])
        for tv in np.unique(np.quantile(v, qs)):
            m = v_s <= tv
            acc = np.cumsum(m)
            ok = np.cumsum(m & g_s)
            valid = last_of_tie & (acc > 0) & (ok >= keep * acc)
            if not valid.any():
                continue
            idx = np.nonzero(valid)[0]
            j = idx[np.argmax(acc[idx])]
            frac = float(acc[j]) / n
            if frac > best[2]:
                best = (float(r_s[j]), float(tv), frac)
        return best

    @staticmethod
    def _cell_stats(E, P, scale):
        """Per cell of a lattice of exact values E and predictions P (both
        [rows, cols, K], NaN where unknown): the network's worst miss on the
        four corners and the corners' spread, in units of the feature range.
        Cells with an unknown corner get NaN (never accepted)."""
        R = (np.abs(P - E) / scale).max(axis=2)
        c = lambda A: (A[:-1, :-1], A[:-1, 1:], A[1:, :-1], A[1:, 1:])
        r_cell = np.maximum.reduce(c(R))
        v_cell = ((np.maximum.reduce(c(E)) - np.minimum.reduce(c(E))) / scale).max(axis=2)
        return r_cell, v_cell

    def run(self, nx: int, ny: int, train_stride: int = 8, steps: int = 3000, batch: int = 4096,
            lr: float = 2e-3, tol: float = 0.01, keep: float = 0.99, n_calibration: int = 65536,
            refine: bool = False) -> ScreenResult:
        """Screened map of the nx x ny grid (point m = iy * nx + ix); features
        are float32 (the FP32 engine's values are exact in float32).

        With `refine`, a rejected cell is not integrated whole: its midpoint
        lattice is integrated, the cell splits into four sub-cells, and those
        are screened again with thresholds calibrated on a second sample drawn
        from the rejected cells; only the points of rejected sub-cells fall
        back to the engine."""
        t_all = time.perf_counter()
        K = self.K
        g0 = np.linspace(self.lo[0], self.hi[0], nx)
        g1 = np.linspace(self.lo[1], self.hi[1], ny)
        # 1. the sub-grid (every train_stride-th line and the last one) integrated by the engine
        sx = np.unique(np.r_[0:nx:train_stride, nx - 1])
        sy = np.unique(np.r_[0:ny:train_stride, ny - 1])
        SX, SY = np.meshgrid(sx, sy, indexing="xy")
        sub = (SY * nx + SX).ravel()
        # the calibration sample (random interior points, used in step 5) is
        # drawn now and integrated in the same engine call as the sub-grid:
        # one large launch instead of a second small one
        is_sub = np.zeros(nx * ny, dtype=bool)
        is_sub[sub] = True
        rng = np.random.default_rng(self.seed + 101)
        want = min(n_calibration, nx * ny - sub.size)
        cal = np.zeros(0, dtype=np.int64)
        while cal.size < want:
            cand = rng.integers(0, nx * ny, size=2 * (want - cal.size) + 16)
            cal = np.unique(np.r_[cal, cand[~is_sub[cand]]])
        if cal.size > want:
            cal = rng.choice(cal, size=want, replace=False)
        t0 = time.perf_counter()
        Fboth = np.asarray(self.integrate(np.r_[g0[SX.ravel()], g0[cal % nx]], np.r_[g1[SY.ravel()], g1[cal // nx]]),
                           dtype=np.float64)
        Fsub, Fcal = Fboth[:sub.size], Fboth[sub.size:]
        t_train_data = time.perf_counter() - t0
        lo, hi = Fsub.min(axis=0), Fsub.max(axis=0)
        scale = np.maximum(hi - lo, 1e-30)
        mu, sd = (hi + lo) / 2.0, scale / 2.0
        Xsub = self._norm_x(g0[SX.ravel()], g1[SY.ravel()])
        Y = ((Fsub - mu) / sd).astype(np.float32)
        # 2. training on the GPU, learning rate halved over four phases
        t0 = time.perf_counter()
        losses = [self.net.train(Xsub, Y, steps=steps // 4, batch=batch, lr=lr / 2 ** ph, seed=self.seed + ph)
                  for ph in range(4)]
        loss = np.concatenate(losses)
        t_train = time.perf_counter() - t0
        # 3. prediction of the full grid (inputs generated and outputs rescaled on the device)
        t0 = time.perf_counter()
        F = self.net.predict_grid(nx, ny, sd, mu)
        t_predict = time.perf_counter() - t0
        # the lattice of the sub-grid lines and their midlines, for the refinement
        sx2 = np.unique(np.r_[sx, (sx[:-1] + sx[1:]) // 2])
        sy2 = np.unique(np.r_[sy, (sy[:-1] + sy[1:]) // 2])
        refine = refine and sx.size > 1 and sy.size > 1
        P2 = F.reshape(ny, nx, K)[np.ix_(sy2, sx2)].astype(np.float64) if refine else None
        # 4. cell statistics from the integrated corners
        t0 = time.perf_counter()
        Fs = Fsub.reshape(sy.size, sx.size, K)
        Ps = F.reshape(ny, nx, K)[np.ix_(sy, sx)].astype(np.float64)
        R = (np.abs(Ps - Fs) / scale).max(axis=2)
        corners = lambda A: (A[:-1, :-1], A[:-1, 1:], A[1:, :-1], A[1:, 1:])
        if sx.size > 1 and sy.size > 1:
            r_cell = np.maximum.reduce(corners(R))
            v_cell = ((np.maximum.reduce(corners(Fs)) - np.minimum.reduce(corners(Fs))) / scale).max(axis=2)
        else:  # a single grid line: no cells, everything is integrated
            r_cell = np.full((1, 1), np.inf)
            v_cell = np.full((1, 1), np.inf)
        cx = np.clip(np.searchsorted(sx, np.arange(nx), side="right") - 1, 0, r_cell.shape[1] - 1)
        cy = np.clip(np.searchsorted(sy, np.arange(ny), side="right") - 1, 0, r_cell.shape[0] - 1)
        flags = np.full(nx * ny, ScreenResult.SURROGATE, dtype=np.int8)
        flags[sub] = ScreenResult.SAMPLED
        F[sub] = Fsub
        t_cells = time.perf_counter() - t0
        # 5. calibration: the screen's thresholds from the sample's exact values
        t0 = time.perf_counter()
        tr, tv, acc = -1.0, -1.0, 0.0
        if cal.size:
            ix, iy = cal % nx, cal // nx
            err_cal = self.map_error(F[cal], Fcal, scale)
            tr, tv, acc = self._calibrate(r_cell[cy[iy], cx[ix]], v_cell[cy[iy], cx[ix]], err_cal, tol, keep)
            F[cal] = Fcal
            flags[cal] = ScreenResult.SAMPLED
        t_cal = time.perf_counter() - t0
        # 6. cells that fail the screen
        t0 = time.perf_counter()
        reject_cell = ~((r_cell <= tr) & (v_cell <= tv))
        reject = reject_cell[cy[:, None], cx[None, :]].ravel() & (flags == ScreenResult.SURROGATE)
        redo = np.nonzero(reject)[0]
        t_refine, tr2, tv2, acc2, n_lattice, n_cal2 = 0.0, -1.0, -1.0, 0.0, 0, 0
        if refine and redo.size:
            # 6a. the midpoint lattice of every rejected cell
            t1 = time.perf_counter()
            ry, rx = np.nonzero(reject_cell)
            xs3 = np.stack([sx[rx], (sx[rx] + sx[rx + 1]) // 2, sx[rx + 1]], axis=1)
            ys3 = np.stack([sy[ry], (sy[ry] + sy[ry + 1]) // 2, sy[ry + 1]], axis=1)
            lat = np.unique((ys3[:, :, None] * nx + xs3[:, None, :]).ravel())
            new_pts = lat[flags[lat] == ScreenResult.SURROGATE]
            if new_pts.size:
                F[new_pts] = np.asarray(self.integrate(g0[new_pts % nx], g1[new_pts // nx]), dtype=np.float64)
                flags[new_pts] = ScreenResult.SAMPLED
            n_lattice = int(new_pts.size)
            E2 = np.full((sy2.size, sx2.size, K), np.nan)
            li, lj = np.searchsorted(sx2, lat % nx), np.searchsorted(sy2, lat // nx)
            E2[lj, li] = F[lat]
            r2_cell, v2_cell = self._cell_stats(E2, P2, scale)
            cx2 = np.clip(np.searchsorted(sx2, np.arange(nx), side="right") - 1, 0, sx2.size - 2)
            cy2 = np.clip(np.searchsorted(sy2, np.arange(ny), side="right") - 1, 0, sy2.size - 2)
            # 6b. second calibration sample, from the rejected cells' remaining points
            cand = np.nonzero(reject & (flags == ScreenResult.SURROGATE))[0]
            cal2 = rng.choice(cand, size=min(max(n_calibration // 2, 1), cand.size), replace=False) \
                if cand.size else np.zeros(0, dtype=np.int64)
            if cal2.size:
                ix2, iy2 = cal2 % nx, cal2 // nx
                Fc2 = np.asarray(self.integrate(g0[ix2], g1[iy2]), dtype=np.float64)
                err2 = self.map_error(F[cal2], Fc2, scale)
                r2s, v2s = r2_cell[cy2[iy2], cx2[ix2]], v2_cell[cy2[iy2], cx2[ix2]]
                known = np.isfinite(r2s) & np.isfinite(v2s)
                tr2, tv2, acc2 = self._calibrate(r2s[known], v2s[known], err2[known], tol, keep)
                F[cal2] = Fc2
                flags[cal2] = ScreenResult.SAMPLED
            n_cal2 = int(cal2.size)
            # 6c. keep the sub-cells that pass
            sub_ok = (r2_cell <= tr2) & (v2_cell <= tv2)
            keep_pt = sub_ok[cy2[:, None], cx2[None, :]].ravel()
            redo = np.nonzero(reject & (flags == ScreenResult.SURROGATE) & ~keep_pt)[0]
            t_refine = time.perf_counter() - t1
        # 7. fallback: the plain engine on every point that is still rejected
        if redo.size:
            F[redo] = np.asarray(self.integrate(g0[redo % nx], g1[redo // nx]), dtype=np.float64)
            flags[redo] = ScreenResult.FALLBACK
        t_fallback = time.perf_counter() - t0 - t_refine
        total = time.perf_counter() - t_all
        return ScreenResult(F, flags, loss=loss, timings={
            "train_data_s": t_train_data, "train_s": t_train, "predict_s": t_predict, "cells_s": t_cells,
            "calibrate_s": t_cal, "fallback_s": t_fallback, "total_s": total, "points": nx * ny,
            "points_per_s": nx * ny / total, "training_points": int(sub.size), "calibration_points": int(cal.size),
            "fallback_points": int(redo.size), "integrated_points": int(np.count_nonzero(flags)),
            "r_max": tr, "v_max": tv, "calibrated_accept_fraction": acc, "rejected_cells": int(reject_cell.sum()),
            "cells": int(reject_cell.size), "refine_s": t_refine, "lattice_points": n_lattice,
            "calibration2_points": n_cal2, "r2_max": tr2, "v2_max": tv2, "calibrated_accept_fraction2": acc2,
            "feature_scale": scale.tolist()})


def _speed(steps: int, batch: int, grid: int, seed: int) -> dict:
    """Training-step and grid-prediction timings of the network on synthetic
    smooth targets (262,144 training rows)."""
    net = MLP(4, 4, 0, seed)
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (262144, 2)).astype(np.float32)
    y = np.stack([np.sin(3 * x[:, 0]) * np.cos(2 * x[:, 1]), x[:, 0] * x[:, 1], np.exp(-x[:, 0] ** 2),
                  x[:, 1] ** 3], axis=1).astype(np.float32)
    net.train(x, y, steps=5, batch=batch)  # kernel attributes, graph capture
    hist = net.train(x, y, steps=steps, batch=batch)
    train_ms, _ = net.timings()
    net.predict_grid(64, 64)
    t0 = time.perf_counter()
    net.predict_grid(grid, grid)
    wall = time.perf_counter() - t0
    _, pred_ms = net.timings()
    return {"steps": steps, "batch": batch, "train_ms": train_ms, "us_per_step": 1e3 * train_ms / max(steps, 1),
            "loss_first": float(hist[0]), "loss_last": float(hist[-1]), "grid": grid,
            "predict_ms": pred_ms, "predict_wall_ms": 1e3 * wall,
            "predict_points_per_s": grid * grid / (pred_ms / 1e3)}


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="surrogate network training and prediction speed")
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--grid", type=int, default=2048)
    ap.add_argument("--seed", type=int, default=1)
    a = ap.parse_args()
    print(json.dumps(_speed(a.steps, a.batch, a.grid, a.seed)))
