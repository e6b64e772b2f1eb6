"""Shared harness of the parity tests: one scenario, run twice on the same
seeded inputs — through the engine's drop-in API (``clode_cpp_wrapper``,
i.e. through the C ABI) and through the CPU oracle — then compared.

A scenario is a model, a stepper/observer/precision choice, the ensemble
data and a call sequence such as
``[("transient", (0, 20)), ("shift_x0",), ("features", (20, 100))]``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from clode_gb300 import rhs_path
from oracle.build import OracleConfig
from oracle.runner import OracleSimulator


@dataclass
class Scenario:
    rhs: str
    n_var: int
    n_par: int
    x0: np.ndarray
    pars: np.ndarray
    steps: list
    n_aux: int = 0
    n_wiener: int = 0
    stepper: str = "rk4"
    observer: str | None = None
    single: bool = False
    n_store_events: int = 0
    sp: dict = field(default_factory=dict)
    op: dict = field(default_factory=dict)
    seed: int | None = 1234
    tspan_pm: np.ndarray | None = None
    var_names: list | None = None
    aux_names: list | None = None

    @property
    def kind(self) -> str:
        if self.observer:
            return "features"
        if any(s[0] == "trajectory" for s in self.steps):
            return "trajectory"
        return "transient"

    def oracle_config(self) -> OracleConfig:
        return OracleConfig(rhs_path(self.rhs), n_var=self.n_var, n_par=self.n_par, n_aux=self.n_aux,
                            n_wiener=self.n_wiener, stepper=self.stepper, single_precision=self.single,
                            observer=self.observer, n_store_events=self.n_store_events)


SP_DEFAULT = dict(dt=0.1, dtmax=0.5, abstol=1e-6, reltol=1e-3, max_steps=1000000, max_store=1000000, nout=1)
OP_DEFAULT = dict(e_var_ix=0, f_var_ix=0, max_event_count=100, min_amp=0.0, min_imi=0.0, nhood_radius=0.05,
                  x_up_threshold=0.2, x_down_threshold=0.2, dx_up_threshold=0.0, dx_down_threshold=0.0, eps_dx=0.0)


def _collect(out: dict, get_xf, get_tf, get_dt):
    out["xf"] = get_xf()
    out["tf"] = get_tf()
    out["dt"] = get_dt()


def run_oracle(sc: Scenario, nthreads: int | None = None, reference: bool = False) -> dict:
    """Run the scenario on the CPU: the C restatement, or (reference=True)
    clODE's own kernels compiled as C, where the clODE sources exist."""
    s = OracleSimulator(sc.oracle_config(), nthreads=nthreads, reference=reference)
    sp = dict(SP_DEFAULT, **sc.sp)
    s.set_solver_params(**sp)
    if sc.observer:
        s.set_observer_params(**dict(OP_DEFAULT, **sc.op))
    s.set_problem_data(sc.x0, sc.pars)
    if sc.seed is not None:
        s.seed_rng(sc.seed)
    out: dict = {}
    for step in sc.steps:
        op = step[0]
        if op in ("transient", "features", "trajectory", "initialize_observer"):
            if len(step) > 1 and step[1] is not None:
                s.set_tspan(step[1])
            if sc.tspan_pm is not None and (len(step) == 1 or step[1] is None):
                s.set_tspan(sc.tspan_pm)
            if op == "transient":
                s.transient()
            elif op == "features":
                s.features(step[2] if len(step) > 2 else None)
                out.setdefault("F_list", []).append(s.get_F())
            elif op == "initialize_observer":
                s.initialize_observer()
            else:
                s.trajectory()
                n, nv, ms = s.nPts, sc.n_var, int(s.sp.max_store)
                out["t"] = s.t[: ms * n].astype(np.float64).reshape(ms, n).T.copy()
                out["x"] = s.x[: ms * n * nv].astype(np.float64).reshape(ms, nv, n).transpose(2, 1, 0).copy()
                out["dx"] = s.dx[: ms * n * nv].astype(np.float64).reshape(ms, nv, n).transpose(2, 1, 0).copy()
                out["n_stored"] = s.n_stored.copy()
        elif op == "shift_x0":
            s.shift_x0()
        elif op == "shift_tspan":
            s.shift_tspan()
        elif op == "seed":
            s.seed_rng(step[1])
        else:
            raise ValueError(op)
        _collect(out, s.get_xf, s.get_tf, s.get_dt)
    out["x0"] = s.get_x0()
    return out


def run_engine(sc: Scenario, options: dict | None = None) -> dict:
    from clode_gb300 import clode_cpp_wrapper as W
    pi = W.ProblemInfo(rhs_path(sc.rhs), sc.var_names or [f"x{j}" for j in range(sc.n_var)],
                       [f"p{j}" for j in range(sc.n_par)], sc.aux_names or [f"a{j}" for j in range(sc.n_aux)],
                       sc.n_wiener)
    res = W.OpenCLResource()
    if sc.kind == "features":
        op = W.ObserverParams(**{("min_amp" if k == "min_amp" else k): v for k, v in dict(OP_DEFAULT, **sc.op).items()},
                              max_event_timestamps=sc.n_store_events)
        sim = W.FeatureSimulatorBase(pi, sc.stepper, sc.observer, op, sc.single, res, "")
    elif sc.kind == "trajectory":
        sim = W.TrajectorySimulatorBase(pi, sc.stepper, sc.single, res, "")
    else:
        sim = W.SimulatorBase(pi, sc.stepper, sc.single, res, "")
    for k, v in (options or {}).items():
        sim.set_option(k, v)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(**dict(SP_DEFAULT, **sc.sp)))
    x0 = np.asarray(sc.x0, dtype=np.float64).reshape(-1, sc.n_var)
    pars = np.asarray(sc.pars, dtype=np.float64).reshape(x0.shape[0], -1)
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    if sc.seed is not None:
        sim.seed_rng(sc.seed)
    n = x0.shape[0]
    out: dict = {"stats": [], "status": []}
    for step in sc.steps:
        op = step[0]
        if op in ("transient", "features", "trajectory", "initialize_observer"):
            if len(step) > 1 and step[1] is not None:
                sim.set_tspan(list(step[1]))
            if sc.tspan_pm is not None and (len(step) == 1 or step[1] is None):
                sim.set_tspan_per_member(np.asarray(sc.tspan_pm, dtype=np.float64))
            if op == "transient":
                sim.transient()
            elif op == "features":
                if len(step) > 2 and step[2] is not None:
                    sim.features(step[2])
                else:
                    sim.features()
                nf = sim.get_n_features()
                out.setdefault("F_list", []).append(np.asarray(sim.get_f()).reshape(nf, n).T.copy())
                out["feature_names"] = sim.get_feature_names()
            elif op == "initialize_observer":
                sim.initialize_observer()
            else:
                sim.trajectory()
                ms = sim.get_solver_params().max_store
                out["t"] = np.asarray(sim.get_t()).reshape(ms, n).T.copy()
                out["x"] = np.asarray(sim.get_x()).reshape(ms, sc.n_var, n).transpose(2, 1, 0).copy()
                out["dx"] = np.asarray(sim.get_dx()).reshape(ms, sc.n_var, n).transpose(2, 1, 0).copy()
                out["n_stored"] = np.asarray(sim.get_n_stored())
            out["stats"].append(sim.get_stats())
            out["status"].append(sim.get_status())
        elif op == "shift_x0":
            sim.shift_x0()
        elif op == "shift_tspan":
            sim.shift_tspan()
        elif op == "seed":
            sim.seed_rng(step[1])
        else:
            raise ValueError(op)
        out["xf"] = np.asarray(sim.get_xf()).reshape(sc.n_var, n).T.copy()
        out["tf"] = np.asarray(sim.get_tf())
        out["dt"] = np.asarray(sim.get_dt())
    out["x0"] = np.asarray(sim.get_x0()).reshape(sc.n_var, n).T.copy()
    out["sim"] = sim
    return out


def mismatch_fraction(a: np.ndarray, b: np.ndarray, rtol: float, atol: float) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ok = np.isclose(a, b, rtol=rtol, atol=atol, equal_nan=True)
    return 1.0 - ok.mean() if ok.size else 0.0


def assert_bitwise(eng: dict, ora: dict, keys=("xf", "tf", "dt")):
    for k in keys:
        a, b = eng[k], ora[k]
        assert a.shape == b.shape, (k, a.shape, b.shape)
        bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
        assert not bad.any(), f"{k}: {bad.sum()} of {bad.size} differ; first {np.argwhere(bad)[:3].tolist()} " \
                              f"engine {a[bad][:3]} oracle {b[bad][:3]}"
    for i, (fa, fb) in enumerate(zip(eng.get("F_list", []), ora.get("F_list", []))):
        bad = ~((fa == fb) | (np.isnan(fa) & np.isnan(fb)))
        assert not bad.any(), f"F[{i}]: {bad.sum()} of {bad.size} differ; first {np.argwhere(bad)[:3].tolist()} " \
                              f"engine {fa[bad][:3]} oracle {fb[bad][:3]}"
