"""Test infrastructure (the oracle), not product code.

Drives the CPU checkers built by ``oracle/build.py`` (the C restatement or
clODE's own kernels compiled as C) with the host-side semantics of clODE's
simulator classes, so a test can replay any call sequence on the CPU:

* device-side state is kept in the kernels' own layout: SoA vectors
  ``[j * nPts + i]`` in working precision, RNG state ``[2 * nPts]`` u64,
  per-member ``dt`` and ``tf`` (clode/cpp/CLODE.cpp:174-242);
* ``dt`` is filled with ``sp.dt`` only when nPts changes (CLODE.cpp:201-227),
  so adaptive runs continue from the last step size;
* ``seed_rng(seed)`` writes ``seed + k`` for k in [0, 2*nPts) (CLODE.cpp:447-453);
* ``features()`` runs the observer initialisation first when it has not run
  since the feature buffer was resized (clode/cpp/CLODEfeatures.cpp:143-259);
* ``shift_x0`` copies xf into x0, ``shift_tspan`` moves [t0,t1] to
  [t1, 2 t1 - t0] (CLODE.cpp:495-515).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import OracleConfig, build_port, build_reference


def n_features(observer: str, n_var: int, n_aux: int, n_store_events: int) -> int:
    """Feature count per observer: the length of each getObserverInfo_* name
    list (clode/cpp/observers/observer_*.clh)."""
    if observer == "basic":
        return 6
    if observer == "basicall":
        return 5 * n_var + 3 * n_aux + 1
    if observer == "localmax":
        return 6 + 5 * n_var + 3 * n_aux + 4 * n_store_events + 2
    if observer == "nhood1":
        return 6 + 5 * n_var + 3 * n_aux + 2 + 3
    if observer == "nhood2":
        return 6 + 7 * n_var + 3 * n_aux + n_store_events + 2 + 3
    if observer == "thresh2":
        return 18 + 5 * n_var + 3 * n_aux + 2 * n_store_events + 2 + 3
    raise ValueError(observer)


def _params_types(single: bool):
    real = C.c_float if single else C.c_double

    class SolverParams(C.Structure):
        _fields_ = [("dt", real), ("dtmax", real), ("abstol", real), ("reltol", real),
                    ("max_steps", C.c_uint), ("max_store", C.c_uint), ("nout", C.c_uint)]

    class ObserverParams(C.Structure):
        _fields_ = [("eVarIx", C.c_uint), ("fVarIx", C.c_uint), ("maxEventCount", C.c_uint),
                    ("maxEventTimestamps", C.c_uint), ("minXamp", real), ("minIMI", real),
                    ("nHoodRadius", real), ("xUpThresh", real), ("xDownThresh", real),
                    ("dxUpThresh", real), ("dxDownThresh", real), ("eps_dx", real)]

    return SolverParams, ObserverParams


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags.c_contiguous
    return a.ctypes.data_as(C.c_void_p)


class OracleSimulator:
    """CPU replay of one clODE simulator object.

    ``kind`` is "transient", "features" or "trajectory"; ``reference=True``
    uses clODE's own kernels compiled as C (only where its sources exist).
    Member arrays passed in and returned are shaped (nPts, n) in float64.
    """

    def __init__(self, cfg: OracleConfig, reference: bool = False, nthreads: int | None = None):
        self.cfg = cfg
        self.reference = reference
        self.path = build_reference(cfg) if reference else build_port(cfg)
        self.lib = C.CDLL(self.path)
        self.real = np.float32 if cfg.single_precision else np.float64
        self.nthreads = nthreads or os.cpu_count() or 1
        SP, OP = _params_types(cfg.single_precision)
        self.sp = SP(0.1, 0.5, 1e-6, 1e-3, 1000000, 1000000, 1)
        self.op = OP(0, 0, 100, cfg.n_store_events, 0.0, 0.0, 0.05, 0.2, 0.2, 0.0, 0.0, 0.0)
        self.op.maxEventTimestamps = cfg.n_store_events
        self.nPts = 0
        self.tspan = np.array([0.0, 1000.0], dtype=self.real)
        self.tspan_stride = 0
        self.observer_initialized = False
        self.F_elements = -1
        self.odata = None

    # ------------------------------------------------------------ set-up --
    def set_solver_params(self, dt=0.1, dtmax=0.5, abstol=1e-6, reltol=1e-3, max_steps=1000000,
                          max_store=1000000, nout=1):
        for k, v in dict(dt=dt, dtmax=dtmax, abstol=abstol, reltol=reltol, max_steps=max_steps,
                         max_store=max_store, nout=nout).items():
            setattr(self.sp, k, v)

    def set_observer_params(self, e_var_ix=0, f_var_ix=0, max_event_count=100, min_amp=0.0, min_imi=0.0,
                            nhood_radius=0.05, x_up_threshold=0.2, x_down_threshold=0.2,
                            dx_up_threshold=0.0, dx_down_threshold=0.0, eps_dx=0.0):
        op = self.op
        op.eVarIx, op.fVarIx, op.maxEventCount = e_var_ix, f_var_ix, max_event_count
        op.minXamp, op.minIMI, op.nHoodRadius = min_amp, min_imi, nhood_radius
        op.xUpThresh, op.xDownThresh = x_up_threshold, x_down_threshold
        op.dxUpThresh, op.dxDownThresh, op.eps_dx = dx_up_threshold, dx_down_threshold, eps_dx

    def set_tspan(self, tspan):
        """One [t0, t1] for every member, or a pair per member: shaped
        (nPts, 2), or flat [t0_0, t1_0, t0_1, t1_1, ...] as the engine's
        set_tspan_per_member takes it."""
        ts = np.asarray(tspan, dtype=np.float64)
        if ts.ndim == 1 and ts.size > 2:
            ts = ts.reshape(-1, 2)
        if ts.ndim == 1:
            self.tspan = np.ascontiguousarray(ts[:2].astype(self.real))
            self.tspan_stride = 0
        else:
            self.tspan = np.ascontiguousarray(ts.reshape(-1, 2).astype(self.real).ravel())
            self.tspan_stride = 2

    def _soa(self, a: np.ndarray, ncol: int) -> np.ndarray:
        a = np.asarray(a, dtype=np.float64).reshape(-1, ncol)
        return np.ascontiguousarray(a.T.astype(self.real).ravel())

    def set_problem_data(self, x0: np.ndarray, pars: np.ndarray):
        x0 = np.asarray(x0, dtype=np.float64).reshape(-1, self.cfg.n_var)
        n = x0.shape[0]
        if n != self.nPts:
            self.nPts = n
            self.rng = np.zeros(2 * n, dtype=np.uint64)
            self.dt = np.full(n, self.sp.dt, dtype=self.real)
            self.tf = np.zeros(n, dtype=self.real)
            self.xf = np.zeros(n * self.cfg.n_var, dtype=self.real)
            self.seed_rng(None)
        self.x0 = self._soa(x0, self.cfg.n_var)
        self.pars = self._soa(pars, max(self.cfg.n_par, 1)) if self.cfg.n_par > 0 else np.zeros(1, self.real)

    def seed_rng(self, seed: int | None = None):
        if seed is None:
            self.rng[:] = np.random.default_rng().integers(0, 2**63, size=2 * self.nPts, dtype=np.uint64)
        else:
            k = np.arange(2 * self.nPts, dtype=np.int64)
            v = ((int(seed) + k + 2**31) % 2**32) - 2**31  # int32 arithmetic, sign-extended
            self.rng[:] = v.astype(np.int64).view(np.uint64)

    def shift_x0(self):
        self.x0 = self.xf.copy()

    def shift_tspan(self):
        ts = self.tspan.astype(np.float64).reshape(-1, 2)
        new = np.stack([ts[:, 1], ts[:, 1] + (ts[:, 1] - ts[:, 0])], axis=1)
        self.set_tspan(new[0] if self.tspan_stride == 0 else new)

    # -------------------------------------------------------------- runs --
    def _range(self, i0, i1):
        return (0 if i0 is None else i0), (self.nPts if i1 is None else i1)

    def transient(self, i0=None, i1=None):
        a, b = self._range(i0, i1)
        self.lib.o_transient(self.nPts, a, b, self.nthreads, _ptr(self.tspan), self.tspan_stride, _ptr(self.x0),
                             _ptr(self.pars), C.byref(self.sp), _ptr(self.xf), _ptr(self.rng), _ptr(self.dt),
                             _ptr(self.tf))

    def _resize_features(self):
        nf = n_features(self.cfg.observer, self.cfg.n_var, self.cfg.n_aux, self.cfg.n_store_events)
        if nf * self.nPts != self.F_elements:
            self.F_elements = nf * self.nPts
            self.n_features = nf
            self.F = np.zeros(self.F_elements, dtype=self.real)
            self.odata = np.zeros(self.nPts * self.lib.o_odata_size(), dtype=np.uint8)
            self.observer_initialized = False

    def initialize_observer(self, i0=None, i1=None):
        self._resize_features()
        a, b = self._range(i0, i1)
        self.lib.o_init_observer(self.nPts, a, b, self.nthreads, _ptr(self.tspan), self.tspan_stride,
                                 _ptr(self.x0), _ptr(self.pars), C.byref(self.sp), _ptr(self.rng), _ptr(self.dt),
                                 _ptr(self.odata), C.byref(self.op))
        self.observer_initialized = True

    def features(self, reinitialize: bool | None = None, i0=None, i1=None):
        if reinitialize is not None:
            self.observer_initialized = not reinitialize
        self._resize_features()
        if not self.observer_initialized:
            self.initialize_observer(i0, i1)
        a, b = self._range(i0, i1)
        self.lib.o_features(self.nPts, a, b, self.nthreads, _ptr(self.tspan), self.tspan_stride, _ptr(self.x0),
                            _ptr(self.pars), C.byref(self.sp), _ptr(self.xf), _ptr(self.rng), _ptr(self.dt),
                            _ptr(self.tf), _ptr(self.odata), C.byref(self.op), _ptr(self.F))

    def trajectory(self, i0=None, i1=None):
        a, b = self._range(i0, i1)
        ms = int(self.sp.max_store)
        n, nv, na = self.nPts, self.cfg.n_var, self.cfg.n_aux
        # one extra row: the reference writes row max_store (clode/cpp/trajectory.cl:76,86-93)
        self.t = np.zeros((ms + 1) * n, dtype=self.real)
        self.x = np.zeros((ms + 1) * n * nv, dtype=self.real)
        self.dx = np.zeros((ms + 1) * n * nv, dtype=self.real)
        self.aux = np.zeros(max((ms + 1) * n * na, 1), dtype=self.real)
        self.n_stored = np.zeros(n, dtype=np.int32)
        self.lib.o_trajectory(n, a, b, self.nthreads, _ptr(self.tspan), self.tspan_stride, _ptr(self.x0),
                              _ptr(self.pars), C.byref(self.sp), _ptr(self.xf), _ptr(self.rng), _ptr(self.dt),
                              _ptr(self.tf), _ptr(self.t), _ptr(self.x), _ptr(self.dx), _ptr(self.aux),
                              _ptr(self.n_stored))

    def features_store(self, event_rows: int, reinitialize: bool | None = None):
        """features() that also stores the trajectory rows and the first
        event_rows event states (o_features_store, the port only)."""
        if self.reference:
            raise RuntimeError("features with storage exist in the port only")
        if reinitialize is not None:
            self.observer_initialized = not reinitialize
        self._resize_features()
        if not self.observer_initialized:
            self.initialize_observer()
        ms = int(self.sp.max_store)
        n, nv, na = self.nPts, self.cfg.n_var, self.cfg.n_aux
        self.t = np.zeros((ms + 1) * n, dtype=self.real)
        self.x = np.zeros((ms + 1) * n * nv, dtype=self.real)
        self.dx = np.zeros((ms + 1) * n * nv, dtype=self.real)
        self.aux = np.zeros(max((ms + 1) * n * na, 1), dtype=self.real)
        self.n_stored = np.zeros(n, dtype=np.int32)
        self.ev_t = np.zeros(max(event_rows * n, 1), dtype=self.real)
        self.ev_x = np.zeros(max(event_rows * n * nv, 1), dtype=self.real)
        self.ev_dx = np.zeros(max(event_rows * n * nv, 1), dtype=self.real)
        self.ev_aux = np.zeros(max(event_rows * n * na, 1), dtype=self.real)
        self.n_events = np.zeros(n, dtype=np.int32)
        self.lib.o_features_store(n, 0, n, self.nthreads, _ptr(self.tspan), self.tspan_stride, _ptr(self.x0),
                                  _ptr(self.pars), C.byref(self.sp), _ptr(self.xf), _ptr(self.rng), _ptr(self.dt),
                                  _ptr(self.tf), _ptr(self.odata), C.byref(self.op), _ptr(self.F), _ptr(self.t),
                                  _ptr(self.x), _ptr(self.dx), _ptr(self.aux), _ptr(self.n_stored), int(event_rows),
                                  _ptr(self.ev_t), _ptr(self.ev_x), _ptr(self.ev_dx), _ptr(self.ev_aux),
                                  _ptr(self.n_events))

    # ----------------------------------------------------------- getters --
    def get_xf(self) -> np.ndarray:
        return self.xf.astype(np.float64).reshape(self.cfg.n_var, self.nPts).T.copy()

    def get_x0(self) -> np.ndarray:
        return self.x0.astype(np.float64).reshape(self.cfg.n_var, self.nPts).T.copy()

    def get_F(self) -> np.ndarray:
        return self.F.astype(np.float64).reshape(self.n_features, self.nPts).T.copy()

    def get_dt(self) -> np.ndarray:
        return self.dt.astype(np.float64)

    def get_tf(self) -> np.ndarray:
        return self.tf.astype(np.float64)
