#!/usr/bin/env python
"""Feature-map throughput of the GB300 ensemble engine.

Workload (one "step"): the lactotroph electrical-activity model on a G x G
grid of (gcal, gbk) (default G = 2048, 4,194,304 members), gsk = 3,
x0 = (-60, 0, 0, 0.1), per-member time span [0, T_i] with T_i ~ U[1e3, 1e4] ms
(seeded), Dormand-Prince 5(4) with rtol = abstol = 1e-6 in FP32, and the
two-pass neighbourhood observer (nhood2) on c (event) and v (features): a
full observer initialisation pass followed by the feature pass, i.e. a
feature map computed from scratch.

Lines printed (one JSON line on rank 0):
  value  - grid points per second, device time of the ensemble kernel with
           the inputs resident in HBM (CUDA events on the launching stream)
  e2e    - the same metric through the public API with host buffers:
           set_problem_data + per-member tspan upload (H2D), features(),
           get_f() (D2H), wall clock
  cpu_baseline - the CPU oracle (a C restatement of clODE's kernels; clODE's
           own kernels compiled as C where its sources exist) on a bounded
           random sample of the same members, on all host cores; the same
           sample gives the engine's error against the CPU.

``--impl reference`` times only the CPU implementation (the reference arm).
Under torchrun each rank runs its own full grid on its own GPU (weak
scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "feature-map points/s (lactotroph nhood2 map, plain FP32 engine); RHS evals/s"
N_VAR, N_PAR, N_AUX = 4, 3, 1
FLOPS_PER_RHS = 43              # + - * / in the lactotroph RHS (3 exp counted apart)
FLOPS_PER_ATTEMPT = 62 * N_VAR + 10   # DP45 stage combinations and error norm
FLOPS_PER_STEP_OBS = 5 * N_VAR + 3 * N_AUX + 6  # nhood2 per-step extrema and means
# DRAM bytes (read + write) per member of one map (warm-up launch + feature
# launch): ncu dram__bytes_{read,write}.sum of both launches of the default
# build on the 512 x 512 case (262,144 members: 76.6 MB + 519.6 MB), scaled
# by members; the traffic is per-member state, so it grows in proportion
DRAM_BYTES_PER_MEMBER = (36643072 + 39959552 + 216447488 + 303181824) / 262144
# DRAM bytes (read + write) per recorded step of the recording and of the
# replay launches of a replayed map, by row layout (replay_split 0: whole
# rows of 1288 bytes per warp; 1: the event fields, 776 bytes): ncu
# dram__bytes_{read,write}.sum of all six launches of each kind (three maps
# of two launch pairs) on the 512 x 512 case, divided by the three maps'
# steps (3 x 1,463,676,130); the traffic is the stored rows, so it grows
# with the steps
DRAM_BYTES_PER_STEP = {
    0: {"record": (18436688896 + 183303534848) / (3 * 1463676130),
        "replay": (191494637312 + 1435273472) / (3 * 1463676130)},
    1: {"record": (10699342336 + 110497920768) / (3 * 1463676130),
        "replay": (113871344384 + 1407749888) / (3 * 1463676130)},
}


def measured_hbm_peak() -> tuple[float, str]:
    """The HBM copy rate of MEASURED_PEAKS.json (GB/s), else the 6.8 TB/s fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
        return float(peaks["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s"


def make_workload(grid: int, seed: int, tmin: float, tmax: float, rank: int = 0):
    g1 = np.linspace(0.5, 3.0, grid)
    g2 = np.linspace(0.0, 2.0, grid)
    gcal, gbk = np.meshgrid(g1, g2, indexing="xy")
    n = grid * grid
    pars = np.stack([gcal.ravel(), np.full(n, 3.0), gbk.ravel()], axis=1)
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
    rng = np.random.default_rng(seed + rank)
    t1 = rng.uniform(tmin, tmax, n)
    tspan = np.stack([np.zeros(n), t1], axis=1)
    return x0, pars, tspan


SOLVER = dict(dt=0.1, dtmax=1.0, abstol=1e-6, reltol=1e-6, max_steps=10000000, max_store=1, nout=1)
OBSERVER = dict(e_var_ix=3, f_var_ix=0, max_event_count=1000000, max_event_timestamps=0, nhood_radius=0.05,
                x_up_threshold=0.3, x_down_threshold=0.2)


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(k)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_sample_indices(n: int, count: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed ^ 0x5EED)
    return np.sort(rng.choice(n, size=min(count, n), replace=False))


def run_cpu(x0, pars, tspan, idx, nthreads: int, prefer_reference: bool = True, single: bool = True,
            tol: float | None = None):
    """Oracle on the members idx; returns (F rows, seconds, kind).  `single`
    and `tol` (rtol = abstol) select the precision and tolerance; the default
    is the workload's own (FP32, 1e-6)."""
    from clode_gb300 import rhs_path
    from oracle.build import OracleConfig, reference_available
    from oracle.runner import OracleSimulator

    cfg = OracleConfig(rhs_path("lactotroph.cl"), n_var=N_VAR, n_par=N_PAR, n_aux=N_AUX, stepper="dopri5",
                       single_precision=single, observer="nhood2", n_store_events=0)
    use_ref = prefer_reference and reference_available()
    s = OracleSimulator(cfg, reference=use_ref, nthreads=nthreads)
    sp = dict(SOLVER)
    if tol is not None:
        sp.update(abstol=tol, reltol=tol)
    s.set_solver_params(**sp)
    s.set_observer_params(**{k: v for k, v in OBSERVER.items() if k != "max_event_timestamps"})
    s.set_problem_data(x0[idx], pars[idx])
    s.set_tspan(tspan[idx])
    t0 = time.perf_counter()
    s.features(True)
    secs = time.perf_counter() - t0
    return s.get_F(), secs, ("reference" if use_ref else "port")


# screened feature sets: the extent of v and c (continuous over the map),
# and the same with nhood2's event and spike counts and mean period, which
# jump where the number of spikes per burst or the oscillation changes
SURROGATE_FEATURES = ("mean v", "max v", "min v", "mean c", "event count", "max peaks", "mean peaks", "mean period")
SURROGATE_SETS = {"counts": SURROGATE_FEATURES, "extent": SURROGATE_FEATURES[:4]}


def bench_surrogate(args, tuned_options: dict) -> dict:
    """Surrogate-screened vs plain feature map on the same GPU.

    Map: lactotroph, G2 x G2 grid of (gcal, gbk) (default 4096 x 4096), fixed
    tspan [0, 3000] ms (the surrogate learns a function of the two parameters),
    DP45 rtol 1e-6 FP32, nhood2.  Two screens of the same plain map: the
    eight features of SURROGATE_FEATURES (extent of v and c, event count,
    max and mean spikes per event, mean period) and the first four alone.
    Plain: every point integrated by the engine (timed once, all eight
    features).  Screened: a 513 x 513 sub-grid integrated, the network
    trained on it on the GPU, the full grid predicted, 65,536 random interior
    points integrated to calibrate the cell screen, every point of a rejected
    cell integrated again.  Error of a point: max over the screen's features
    of |screened - plain| / (the feature's range over the plain map),
    reported over the whole map, over 65,536 seeded held-out points, and per
    feature.
    """
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path
    from clode_gb300.surrogate import FeatureMapScreen

    pi = W.ProblemInfo(rhs_path("lactotroph.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"], 0)
    op = W.ObserverParams(**OBSERVER)
    sim = W.FeatureSimulatorBase(pi, "dopri5", "nhood2", op, True, W.OpenCLResource(), "")
    for k, v in tuned_options.items():
        sim.set_option(k, v)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(**SOLVER))
    cols = []

    def integrate(gcal, gbk):
        n = gcal.size
        pars = np.stack([gcal, np.full(n, 3.0), gbk], axis=1)
        x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
        sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
        sim.set_tspan([0.0, 3000.0])
        sim.features(True)
        if not cols:
            names = sim.get_feature_names()
            cols.extend(names.index(c) for c in SURROGATE_FEATURES)
        return np.asarray(sim.get_f()).reshape(-1, n).T[:, cols]

    G = args.surrogate_grid
    g0, g1 = np.linspace(0.5, 3.0, G), np.linspace(0.0, 2.0, G)
    P0, P1 = np.meshgrid(g0, g1, indexing="xy")
    P0, P1 = P0.ravel(), P1.ravel()
    integrate(P0[:4096], P1[:4096])  # build and warm-up
    t0 = time.perf_counter()
    plain_all = integrate(P0, P1)
    t_plain = time.perf_counter() - t0
    stride = args.surrogate_stride if args.surrogate_stride > 0 else max(G // 512, 1)
    rng = np.random.default_rng(args.seed ^ 0xC0DE)
    held = rng.choice(G * G, size=min(65536, G * G), replace=False)
    out = {"workload": f"lactotroph nhood2 map {G}x{G}, tspan [0,3000] ms",
           "training": {"steps": args.surrogate_steps, "batch": args.surrogate_batch, "stride": stride,
                        "refine": bool(args.surrogate_refine)},
           "error_measure": "max over the screen's features of |screened - plain| / feature range over the plain map",
           "points": G * G, "plain_points_per_s": G * G / t_plain, "plain_s": t_plain}
    for key, feats in SURROGATE_SETS.items():
        sel = [SURROGATE_FEATURES.index(f) for f in feats]
        plain = plain_all[:, sel]
        scr = FeatureMapScreen(lambda a, b: integrate(a, b)[:, sel], lo=(0.5, 0.0), hi=(3.0, 2.0),
                               n_features=len(feats), seed=1)
        res = scr.run(G, G, train_stride=stride, steps=args.surrogate_steps, batch=args.surrogate_batch,
                      tol=0.01, keep=0.99, n_calibration=65536, refine=bool(args.surrogate_refine))
        scale = plain.max(axis=0) - plain.min(axis=0)
        err = FeatureMapScreen.map_error(res.features, plain, scale)
        per_feature = np.abs(np.asarray(res.features, np.float64) - plain) / np.maximum(scale, 1e-30)
        out[key] = {
            "features": list(feats),
            "screened_points_per_s": res.timings["points_per_s"],
            "speedup_vs_plain": t_plain / res.timings["total_s"], "integrated_fraction": res.integrated_fraction,
            "fallback_fraction": res.fallback_fraction,
            "map": {"within_1pct": float(np.mean(err <= 0.01)), "err_median": float(np.median(err)),
                    "err_p99": float(np.quantile(err, 0.99)), "err_max": float(err.max())},
            "heldout": {"points": int(held.size), "within_1pct": float(np.mean(err[held] <= 0.01)),
                        "err_median": float(np.median(err[held])), "err_p99": float(np.quantile(err[held], 0.99))},
            "within_1pct_per_feature": {f: float(np.mean(per_feature[:, j] <= 0.01)) for j, f in enumerate(feats)},
            "final_loss": float(res.loss[-20:].mean()) if res.loss is not None and res.loss.size else None,
            "timings_s": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in res.timings.items()
                          if k != "feature_scale"},
        }
        del scr
    # the headline screen: the one with the counts
    out.update({k: out["counts"][k] for k in ("screened_points_per_s", "speedup_vs_plain", "fallback_fraction",
                                              "integrated_fraction", "map", "heldout")})
    return out


def bench_trajectory(args, tuned_options: dict) -> dict:
    """Stored trajectories of the Ornstein-Uhlenbeck process (the reference's
    stochastic example): theta = linspace(0.1, 2, 16) x sigma = linspace(0.1,
    1, 16) parameter points x 256 realisations = 65,536 members, x0 = 0,
    mu = 0, seeded RNG, stochastic Euler dt = 1e-3 over [0, 100] (100,000
    steps), a row (t, x, dx) stored every 10 steps: 10,001 rows, 7.87 GB
    written in FP32.  Reports member-steps/s and the write bandwidth of the
    trajectory launch against the measured HBM copy bandwidth."""
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path

    pi = W.ProblemInfo(rhs_path("ornstein_uhlenbeck.cl"), ["x"], ["theta", "mu", "sigma"], [], 1)
    sim = W.TrajectorySimulatorBase(pi, "seuler", True, W.OpenCLResource(), "")
    for k in ("schedule", "block_size", "fmad", "prec_div", "ftz"):
        if k in tuned_options:
            sim.set_option(k, tuned_options[k])
    sim.build_cl()
    steps, nout = args.trajectory_steps, 10
    sim.set_solver_params(W.SolverParams(dt=1e-3, dtmax=1.0, abstol=1e-6, reltol=1e-3, max_steps=steps,
                                         max_store=steps // nout + 2, nout=nout))
    th, sg = np.meshgrid(np.linspace(0.1, 2.0, 16), np.linspace(0.1, 1.0, 16), indexing="xy")
    pts = np.stack([th.ravel(), np.zeros(256), sg.ravel()], axis=1)
    pars = np.repeat(pts, 256, axis=0)
    n = pars.shape[0]
    sim.set_problem_data(np.zeros(n), pars.flatten(order="F"))
    sim.set_tspan([0.0, steps * 1e-3])
    times, draws = [], []
    for rep in range(3):
        sim.seed_rng(args.seed + rep)
        sim.trajectory()
        times.append(sim.last_kernel_ms())
        draws.append(sim.get_option("predraw_ms"))
    rows = int(np.asarray(sim.get_n_stored()).max()) + 1
    ms = float(min(times))
    written = rows * n * 3 * 4
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    gbs = written / (ms / 1e3) / 1e9
    frontend = bench_trajectory_frontend(W, pi, pars, tuned_options, args) if args.trajectory_frontend else None
    return {"frontend": frontend,
            "workload": f"OU trajectories, 65536 members (256 parameter points x 256 realisations), seuler "
                        f"dt 1e-3 over [0, {steps * 1e-3:g}], (t, x, dx) stored every 10 steps, FP32",
            "members": n, "steps_per_member": steps, "rows": rows, "ms": ms, "ms_all": times,
            "predrawn": bool(sim.get_option("predrawn")), "predraw_ms": draws[int(np.argmin(times))],
            "member_steps_per_s": n * steps / (ms / 1e3),
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                         "traffic": None, "algorithmic_bytes": written,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"}}


def bench_trajectory_frontend(W, pi, pars, tuned_options: dict, args) -> dict:
    """Per-member trajectory outputs on the host, the step after the
    trajectory kernel: clode_gb300.trajectory_output.get_trajectory (device
    regrouping, one copy per array, views) against the restatement of
    clODE's getters plus per-member loop (clode/trajectory.py:216-264) as the
    CPU baseline, on the first 8,192 members of the OU workload (32 parameter
    points x 256 realisations) over 20,000 steps: 2,001 rows of (t, x, dx)
    per member, 393 MB as float64."""
    from clode_gb300.trajectory_output import get_trajectory
    from oracle.trajectory_frontend import reference_get_trajectory

    n, steps, nout = 8192, 20000, 10
    sim = W.TrajectorySimulatorBase(pi, "seuler", True, W.OpenCLResource(), "")
    for k in ("schedule", "block_size", "fmad", "prec_div", "ftz"):
        if k in tuned_options:
            sim.set_option(k, tuned_options[k])
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=1e-3, dtmax=1.0, abstol=1e-6, reltol=1e-3, max_steps=steps,
                                         max_store=steps // nout + 2, nout=nout))
    sim.set_problem_data(np.zeros(n), pars[:n].flatten(order="F"))
    sim.set_tspan([0.0, steps * 1e-3])
    sim.seed_rng(args.seed)
    sim.trajectory()
    ours, ref = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        out = get_trajectory(sim)
        ours.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        want = reference_get_trajectory(sim, ["x"], [], n, steps // nout + 2)
        ref.append(time.perf_counter() - t0)
    same = all(np.array_equal(o.t, w["t"]) and np.array_equal(o.x, w["x"]) and np.array_equal(o.dx, w["dx"])
               for o, w in zip(out, want))
    rows = int(np.asarray(sim.get_n_stored()).max()) + 1
    nbytes = n * rows * 3 * 8
    return {"workload": f"per-member outputs of {n} OU trajectories x {rows} rows of (t, x, dx), float64",
            "members": n, "rows": rows, "bytes": nbytes, "s": min(ours), "gb_per_s": nbytes / min(ours) / 1e9,
            "identical_to_baseline": bool(same),
            "cpu_baseline": {"s": min(ref), "kind": "port", "cores": 1,
                             "sample": "clODE's getters + per-member loop (clode/trajectory.py:216-264), "
                                       "restated, over the same device arrays"},
            "speedup": min(ref) / min(ours)}


def bench_configs(args, tuned_options: dict) -> dict:
    """The two other deterministic workloads of the scope, timed on the device
    (CUDA events, observer initialisation included, best of 3):

    * Van der Pol, 4,096 members, mu ~ U[0.1, 5], (x0, y0) ~ U[-2, 2]^2
      (seeded), RK4 dt = 0.01 in FP64: transient [0, 200] (20,001 steps),
      then localmax features on x over [200, 1000] (80,001 steps).  Bound:
      the FP64 pipe (nominal 1.25 TFLOP/s on GB300).
    * Lorenz, 1024 x 1024 grid of sigma = linspace(5, 15) x rho =
      linspace(10, 60), beta = 8/3, x0 = (1, 1, 1) + N(0, 1e-6) (seeded),
      DP45 rtol 1e-6 atol 1e-9 dt0 1e-3 dtmax 1 in FP32 over [0, 500],
      thresh2 on z (up 0.3, down 0.2, at most 1e5 events).  Bound: the FP32
      pipe.  An absolute tolerance of 1e-9 is below FP32 resolution for
      some members (about one in 2.6e5): their step size falls to its floor
      and they run until max_steps, one lane alone for seconds while the
      rest of the map takes a fraction of that; max_steps is 1e6 here
      (the median member takes about 2.3e4 steps per pass) and the members
      that reach it are counted in the line.

    Flops are counted as for the lactotroph map: per RHS evaluation the
    model's + - * / (Van der Pol 5, Lorenz 9), per RK4 step 14 n + 3, per
    DP45 attempt 62 n + 10, per observer step 5 n + 3 n_aux + 6, with steps,
    attempts and evaluations counted on the device."""
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path

    out = {}
    # Van der Pol, RK4, FP64
    rng = np.random.default_rng(args.seed)
    n = 4096
    mu = rng.uniform(0.1, 5.0, n)
    x0 = rng.uniform(-2.0, 2.0, (n, 2))
    pi = W.ProblemInfo(rhs_path("van_der_pol.cl"), ["x", "y"], ["mu"], [], 0)
    sim = W.FeatureSimulatorBase(pi, "rk4", "localmax", W.ObserverParams(e_var_ix=0, f_var_ix=0,
                                                                        max_event_count=10000000),
                                 False, W.OpenCLResource(), "")
    for k in ("schedule", "block_size", "fmad"):
        if k in tuned_options:
            sim.set_option(k, tuned_options[k])
    sim.set_solver_params(W.SolverParams(dt=0.01, dtmax=0.01, max_steps=10000000))
    times, stats = [], None
    for _ in range(3):
        sim.set_problem_data(x0.flatten(order="F"), mu)
        sim.set_tspan([0.0, 200.0])
        sim.transient()
        ms, st = sim.last_kernel_ms(), sim.get_stats()
        sim.shift_x0()
        sim.set_tspan([200.0, 1000.0])
        sim.features(True)
        ms += sim.last_kernel_ms()
        st2 = sim.get_stats()
        times.append(ms)
        stats = {k: st[k] + st2[k] for k in ("steps", "rhs_evals")}
    flops = stats["rhs_evals"] * 5 + stats["steps"] * (14 * 2 + 3) + st2["steps"] * (5 * 2 + 6)
    ms = min(times)
    fp64_peak = 1.25
    out["vdp_rk4_fp64"] = {
        "members": n, "steps": stats["steps"], "rhs_evals": stats["rhs_evals"], "ms": ms,
        "points_per_s": n / (ms / 1e3), "rhs_evals_per_s": stats["rhs_evals"] / (ms / 1e3),
        "roofline": {"bound": "fp64", "achieved": flops / (ms / 1e3) / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": flops / (ms / 1e3) / 1e12 / fp64_peak,
                     "peak_source": "nominal GB300 FP64 rate (MEASURED_PEAKS.json has no FP64 figure)"}}

    # Lorenz, DP45, FP32, thresh2
    g = 1024
    sig, rho = np.meshgrid(np.linspace(5.0, 15.0, g), np.linspace(10.0, 60.0, g), indexing="xy")
    n = g * g
    x0 = np.ones((n, 3)) + rng.normal(0.0, 1e-3, (n, 3))
    pars = np.stack([rho.ravel(), sig.ravel(), np.full(n, 8.0 / 3.0)], axis=1)
    pi = W.ProblemInfo(rhs_path("lorenz.cl"), ["x", "y", "z"], ["rho", "sigma", "beta"], ["fx"], 0)
    sim = W.FeatureSimulatorBase(pi, "dopri5", "thresh2",
                                 W.ObserverParams(e_var_ix=2, f_var_ix=2, max_event_count=100000,
                                                  x_up_threshold=0.3, x_down_threshold=0.2),
                                 True, W.OpenCLResource(), "")
    for k, v in tuned_options.items():
        sim.set_option(k, v)
    sim.set_solver_params(W.SolverParams(dt=1e-3, dtmax=1.0, abstol=1e-9, reltol=1e-6, max_steps=1000000))
    # this map's own tuning (a cheap right-hand side: whether replaying the
    # stored steps pays is the autotuner's call), on the whole map
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan([0.0, 500.0])
    tuned_lorenz = sim.autotune(0)
    times = []
    for _ in range(3):
        sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))  # same size: dt continues
        sim.set_tspan([0.0, 500.0])
        sim.features(True)
        times.append(sim.last_kernel_ms())
    st = sim.get_stats()
    attempts = st["steps"] + st["rejected"]
    flops = st["rhs_evals"] * 9 + attempts * (62 * 3 + 10) + st["steps"] * (5 * 3 + 3 + 6)
    ms = min(times)
    peak = 152 * 128 * 2 * 2.07e9 / 1e12
    status = sim.get_status()
    out["lorenz_dp45_fp32"] = {
        "members": n, "steps": st["steps"], "rejected": st["rejected"], "rhs_evals": st["rhs_evals"], "ms": ms,
        "max_steps": 1000000, "members_at_max_steps": int(((status & 4) != 0).sum()),
        "members_hmin_fail": int(((status & 1) != 0).sum()), "autotune": tuned_lorenz,
        "points_per_s": n / (ms / 1e3), "rhs_evals_per_s": st["rhs_evals"] / (ms / 1e3),
        "roofline": {"bound": "fp32", "achieved": flops / (ms / 1e3) / 1e12, "peak": peak, "unit": "TFLOP/s",
                     "frac": flops / (ms / 1e3) / 1e12 / peak,
                     "peak_source": "nominal FP32 FMA rate 152 SMs x 128 lanes x 2 at 2070 MHz"}}
    return out


def bench_feature_store(args, tuned_options: dict) -> dict:
    """Features and stored trajectories in one pass (features_store) against
    the two runs it replaces (features, then trajectory): the lactotroph
    model on a 256 x 256 grid of (gcal, gbk), tspan [0, 3000] ms, DP45 rtol
    1e-6 FP32, nhood2; a row every 50 steps and the first 16 event states
    per member.  Device time of each call (observer initialisation
    included), best of 3."""
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path

    grid = 256
    x0, pars, _ = make_workload(grid, args.seed, args.tmin, args.tmax)
    pi = W.ProblemInfo(rhs_path("lactotroph.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"], 0)
    sp = W.SolverParams(dt=SOLVER["dt"], dtmax=SOLVER["dtmax"], abstol=1e-6, reltol=1e-6,
                        max_steps=SOLVER["max_steps"], max_store=1000, nout=50)
    op = W.ObserverParams(**OBSERVER)

    def setup(sim, traj=False):
        for k, v in tuned_options.items():
            if not (traj and k == "fuse_init"):
                sim.set_option(k, v)
        sim.set_solver_params(sp)
        sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
        sim.set_tspan([0.0, 3000.0])
        return sim

    store = setup(W.FeatureSimulatorBase(pi, "dopri5", "nhood2", op, True, W.OpenCLResource(), ""))
    plain = setup(W.FeatureSimulatorBase(pi, "dopri5", "nhood2", op, True, W.OpenCLResource(), ""))
    traj = setup(W.TrajectorySimulatorBase(pi, "dopri5", True, W.OpenCLResource(), ""), traj=True)
    t_store, t_sep = [], []
    for _ in range(3):  # each run continues from the step sizes the previous one ended with, in all three
        store.features_store(True, event_rows=16)
        t_store.append(store.last_kernel_ms())
        plain.features(True)
        ms = plain.last_kernel_ms()
        traj.trajectory()
        t_sep.append(ms + traj.last_kernel_ms())
    same_fast = bool(np.array_equal(store.get_n_stored(), traj.get_n_stored()))
    # identity of the stored rows, in the exact build (with fmad the compiler
    # may contract multiply-adds differently in the two kernels, so the fast
    # build's step sequences may part by a rounding)
    exact = {"fmad": 0, "prec_div": 1, "ftz": 0}
    store_x = setup(W.FeatureSimulatorBase(pi, "dopri5", "nhood2", op, True, W.OpenCLResource(), ""))
    traj_x = setup(W.TrajectorySimulatorBase(pi, "dopri5", True, W.OpenCLResource(), ""), traj=True)
    for sim in (store_x, traj_x):
        for k, v in exact.items():
            sim.set_option(k, v)
    store_x.features_store(True, event_rows=16)
    traj_x.trajectory()
    same = bool(np.array_equal(store_x.get_n_stored(), traj_x.get_n_stored())
                and np.array_equal(np.asarray(store_x.get_x()), np.asarray(traj_x.get_x())))
    return {"workload": f"lactotroph nhood2, {grid}x{grid} (gcal, gbk) grid, tspan [0, 3000] ms, DP45 rtol 1e-6 "
                        "FP32, a row every 50 steps, 16 event states per member",
            "members": grid * grid, "rows_max": int(store.get_n_stored().max()) + 1,
            "events_max": int(store.get_n_events().max()),
            "one_pass_ms": min(t_store), "two_runs_ms": min(t_sep), "speedup": min(t_sep) / min(t_store),
            "rows_identical_to_trajectory_run": same, "rows_identical_fast_build": same_fast}


def bench_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    x0, pars, tspan = make_workload(args.grid, args.seed, args.tmin, args.tmax)
    n = x0.shape[0]
    threads = os.cpu_count() or 1
    times, points, kind = [], 0, "port"
    for step in range(args.warmup + args.steps):
        idx = cpu_sample_indices(n, args.cpu_sample, args.seed + step)
        _, secs, kind = run_cpu(x0, pars, tspan, idx, threads)
        if step >= args.warmup:
            times.append(secs)
            points += idx.size
    value = points / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded lactotroph parameter grid)",
            "config": {"workload": workload_name(args.grid, args.tmin, args.tmax), "grid": args.grid},
            "cpu_baseline": {"value": value, "unit": "points/s", "cores": threads, "kind": kind,
                             "sample": f"{args.cpu_sample} random members of the grid per step"},
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def workload_name(grid, tmin, tmax):
    """The map's workload, worded the same in the lines of both arms."""
    return (f"lactotroph nhood2 feature map {grid}x{grid} = {grid * grid} points, per-member tspan "
            f"U[{tmin:g},{tmax:g}] ms, DP45 rtol=abstol=1e-6 FP32, observer init + features per step")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="clode_gb300", choices=["clode_gb300", "reference"])
    ap.add_argument("--grid", type=int, default=2048)
    ap.add_argument("--tmin", type=float, default=1e3)
    ap.add_argument("--tmax", type=float, default=1e4)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--cpu-sample", type=int, default=1024)
    ap.add_argument("--schedule", type=int, default=1)
    ap.add_argument("--block-size", type=int, default=128)
    ap.add_argument("--fmad", type=int, default=1)
    ap.add_argument("--prec-div", type=int, default=0)
    ap.add_argument("--ftz", type=int, default=1)
    ap.add_argument("--fast-math", type=int, default=0, help="approximate exp/pow/sqrt (NVRTC --use_fast_math)")
    ap.add_argument("--fast-exp", type=int, default=0, help="the model's FP32 exp within 2.5 ulp (own Cody-Waite exp)")
    ap.add_argument("--paired", type=int, default=None,
                    help="FP32 stage sums two variables per paired instruction (engine default 1)")
    ap.add_argument("--maxrreg", type=int, default=None)
    ap.add_argument("--blocks-per-sm", type=int, default=None)
    ap.add_argument("--split-attempts", type=int, default=None)
    ap.add_argument("--fuse-init", type=int, default=None)
    ap.add_argument("--step-block", type=int, default=None)
    ap.add_argument("--replay", type=int, default=None,
                    help="feature pass replays the warm-up's stored steps (engine default 1)")
    ap.add_argument("--replay-mb", type=float, default=None, help="record regions in MiB (engine default: automatic)")
    ap.add_argument("--precise", type=int, default=None, help="the engine's precision option (engine default 0)")
    ap.add_argument("--replay-split", type=int, default=None,
                    help="replay rows of the observer's event fields with the pass's sums taken while recording "
                         "(1, the engine default) or whole rows (0)")
    ap.add_argument("--replay-room", type=float, default=None,
                    help="region room kept for the members in flight, in mean member lengths (engine default 2.5)")
    ap.add_argument("--replay-fused", type=int, default=None,
                    help="recording and replay in one launch per launch pair (1) or two launches (0)")
    ap.add_argument("--replay-stages", type=int, default=None,
                    help="shared-memory row stages of the replay (-1 automatic, the engine default; 0: rows read "
                         "from global memory)")
    ap.add_argument("--autotune", type=int, default=4194304,
                    help="autotune on a strided sample of this many members first (0: off; the default, the "
                         "whole 2048 x 2048 map: a smaller sample mispredicts the map by a few percent)")
    ap.add_argument("--surrogate-grid", type=int, default=4096)
    ap.add_argument("--surrogate-steps", type=int, default=3000)
    ap.add_argument("--surrogate-batch", type=int, default=4096)
    ap.add_argument("--surrogate-refine", type=int, default=0)
    ap.add_argument("--surrogate-stride", type=int, default=0, help="training sub-grid stride (0: grid / 512)")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-trajectory", action="store_true")
    ap.add_argument("--trajectory-steps", type=int, default=100000)
    ap.add_argument("--order-by-span", type=int, default=None,
                    help="persistent lanes take the longest time spans first (engine default 1)")
    ap.add_argument("--configs", type=int, default=1,
                    help="1: also time the Van der Pol (RK4 FP64) and Lorenz (DP45 FP32) workloads")
    ap.add_argument("--feature-store", type=int, default=1,
                    help="1: also time features with storage against separate features and trajectory runs")
    ap.add_argument("--trajectory-frontend", type=int, default=1,
                    help="1: also time per-member trajectory outputs against clODE's per-member loop")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--shard", action="store_true",
                    help="under torchrun: the ranks split one map (strong scaling) instead of each timing its own")
    args = ap.parse_args()

    if args.impl == "reference":
        bench_reference_arm(args)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("gloo")

    from clode_gb300 import _native as N, clode_cpp_wrapper as W, rhs_path

    W.get_logger().set_log_level(W.LogLevel.warn)
    if args.shard:  # one map, members split contiguously over the ranks (clode_gb300.shard)
        from clode_gb300.shard import member_range
        x0, pars, tspan = make_workload(args.grid, args.seed, args.tmin, args.tmax)
        i0, i1 = member_range(x0.shape[0], rank, world)
        x0, pars, tspan = x0[i0:i1], pars[i0:i1], tspan[i0:i1]
    else:
        x0, pars, tspan = make_workload(args.grid, args.seed, args.tmin, args.tmax, rank)
    n = x0.shape[0]
    pi = W.ProblemInfo(rhs_path("lactotroph.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"], 0)
    res = W.OpenCLResource(0, local)
    op = W.ObserverParams(**OBSERVER)
    sim = W.FeatureSimulatorBase(pi, "dopri5", "nhood2", op, True, res, "")
    sim.set_option("fmad", args.fmad)
    sim.set_option("schedule", args.schedule)
    sim.set_option("block_size", args.block_size)
    for key, val in (("prec_div", args.prec_div), ("ftz", args.ftz), ("fast_math", args.fast_math),
                     ("fast_exp", args.fast_exp), ("paired", args.paired), ("split_attempts", args.split_attempts),
                     ("fuse_init", args.fuse_init), ("step_block", args.step_block),
                     ("maxrregcount", args.maxrreg), ("blocks_per_sm", args.blocks_per_sm),
                     ("order_by_span", args.order_by_span), ("replay", args.replay), ("replay_mb", args.replay_mb),
                     ("precise", args.precise), ("replay_stages", args.replay_stages),
                     ("replay_split", args.replay_split), ("replay_fused", args.replay_fused),
                     ("replay_room", args.replay_room)):
        if val is not None:
            sim.set_option(key, val)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(**SOLVER))
    x0_f = np.ascontiguousarray(x0.flatten(order="F"))
    pars_f = np.ascontiguousarray(pars.flatten(order="F"))
    ts_f = np.ascontiguousarray(tspan.ravel())
    sim.set_problem_data(x0_f, pars_f)
    sim.set_tspan_per_member(ts_f)
    tuned = sim.autotune(args.autotune) if args.autotune > 0 else None

    try:
        import torch
        flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
    except Exception:
        torch, flush = None, None

    def l2_flush():
        if flush is not None:
            flush.zero_()
            torch.cuda.synchronize(local)

    def barrier():
        if dist is not None:
            dist.barrier()

    # warm-up (includes the NVRTC build and first-touch of every buffer)
    for _ in range(args.warmup):
        sim.features(True)
    l2_flush()

    # device-timed steps, inputs resident in HBM
    launches0 = N.lib.clode_launch_count()
    kernel_ms, stats, split = [], [], []
    barrier()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            sim.features(True)
            kernel_ms.append(sim.last_kernel_ms())
            stats.append(sim.get_stats())
            split.append({k: sim.get_option(k) for k in ("replay_chunks", "replay_fallback", "replay_rewarm",
                                                          "replay_stages_used", "replay_regions_per_warp",
                                                          "replay_reallocs",
                                                          "replay_fused", "replay_split",
                                                          "replay_rows", "replay_row_bytes",
                                                          "replay_record_ms", "replay_replay_ms",
                                                          "replay_fallback_ms", "warmup_ms")})
            l2_flush()
        wall_dev = time.perf_counter() - t0
    barrier()
    launches_dev = N.lib.clode_launch_count() - launches0
    clk = clocks.summary()

    # end-to-end through the public API with host buffers: the inputs and the
    # features' destination in page-locked host memory, allocated once and
    # reused every step (the copies run at the host link's rate)
    def pinned(a):
        if torch is None or not torch.cuda.is_available():
            return np.array(a, dtype=np.float64)
        b = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy()
        b[:] = a.ravel()
        return b

    x0_h, pars_h, ts_h = pinned(x0_f), pinned(pars_f), pinned(ts_f)
    F_h = pinned(np.zeros(sim.get_n_features() * n))
    e2e_times, e2e_kernel, e2e_reallocs, e2e_dl = [], [], [], []
    h2d = x0_h.nbytes + pars_h.nbytes + ts_h.nbytes
    d2h = 0
    launches1 = N.lib.clode_launch_count()
    barrier()
    parts = np.zeros(4)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        sim.set_problem_data(x0_h, pars_h)
        t1 = time.perf_counter()
        sim.set_tspan_per_member(ts_h)
        t2 = time.perf_counter()
        sim.features(True)
        t3 = time.perf_counter()
        F = sim.get_f(out=F_h)
        t4 = time.perf_counter()
        e2e_times.append(t4 - t0)
        parts += np.array([t1 - t0, t2 - t1, t3 - t2, t4 - t3])
        e2e_kernel.append(sim.last_kernel_ms())
        e2e_reallocs.append(int(sim.get_option("replay_reallocs")))
        e2e_dl.append([round(sim.get_option(k), 2) for k in ("download_pin_ms", "download_ms", "download_wall_ms")])
        d2h = F.nbytes
    barrier()
    launches_e2e = N.lib.clode_launch_count() - launches1

    total_kernel_s = sum(kernel_ms) / 1e3
    value = args.steps * n / total_kernel_s
    e2e_value = args.steps * n / sum(e2e_times)
    if dist is not None:
        import torch
        t = torch.tensor([total_kernel_s, sum(e2e_times)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = args.grid * args.grid if args.shard else world * n
        value = args.steps * total / float(t[0])
        e2e_value = args.steps * total / float(t[1])

    st = stats[-1]
    ms = kernel_ms[-1]
    sp_ = split[-1]
    hbm_peak, hbm_src = measured_hbm_peak()
    replayed = sp_["replay_chunks"] > 0
    attempts = st["rhs_evals"] / 6.0
    info = W._device_infos()[local]
    sm_mhz = clk["sm_mhz"] or 1920.0
    peak_tflops = info.compute_units * 128 * 2 * sm_mhz * 1e6 / 1e12
    rhs_per_s = st["rhs_evals"] / (ms / 1e3)
    if replayed:
        # the recording warm-up launches integrate (stages, right-hand sides,
        # controller): FP32-bound; the replay launches read the stored rows
        # (per warp-wide row: the observer's fields of 32 lanes and two masks)
        # and run the observer: HBM-bound
        rec_ms = sp_["replay_record_ms"]
        flops = st["rhs_evals"] * FLOPS_PER_RHS + attempts * FLOPS_PER_ATTEMPT
        achieved_tflops = flops / (rec_ms / 1e3) / 1e12
        rep_bytes = sp_["replay_rows"] * sp_["replay_row_bytes"]
        roof_replay = None if sp_["replay_fused"] else {"bound": "hbm", "achieved": rep_bytes / (sp_["replay_replay_ms"] / 1e3) / 1e9,
                       "peak": hbm_peak, "unit": "GB/s",
                       "frac": rep_bytes / (sp_["replay_replay_ms"] / 1e3) / 1e9 / hbm_peak,
                       "traffic": DRAM_BYTES_PER_STEP[int(sp_["replay_split"])]["replay"] * st["steps"],
                       "algorithmic_bytes": rep_bytes, "rows": sp_["replay_rows"],
                       "row_bytes": sp_["replay_row_bytes"],
                       "peak_source": hbm_src,
                       "kernel": "clode_features_replay_staged" if sp_["replay_stages_used"] >= 2
                       else "clode_features_replay",
                       "ms": sp_["replay_replay_ms"]}
    else:
        rec_ms = ms
        flops = st["rhs_evals"] * FLOPS_PER_RHS + attempts * FLOPS_PER_ATTEMPT + st["steps"] * FLOPS_PER_STEP_OBS
        achieved_tflops = flops / (ms / 1e3) / 1e12
        roof_replay = None

    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": float(np.mean(kernel_ms)), "higher_is_better": True,
        "scaling": "strong" if args.shard else "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded lactotroph parameter grid, per-member time spans)",
        "config": {"workload": workload_name(args.grid, args.tmin, args.tmax),
                   "grid": args.grid, "points": n,
                   "schedule": "persistent" if sim.get_option("schedule") else "grid",
                   "block_size": args.block_size, "fmad": bool(args.fmad),
                   "variant": {k: v for k, v in (("prec_div", args.prec_div), ("ftz", args.ftz),
                                                 ("fast_math", args.fast_math), ("fast_exp", args.fast_exp),
                                                 ("paired", args.paired),
                                                 ("maxrregcount", args.maxrreg),
                                                 ("blocks_per_sm", args.blocks_per_sm)) if v is not None},
                   "registers": sim.kernel_registers("features_persistent" if sim.get_option("schedule") else "features"),
                   "autotune": tuned, "schedule_used": int(sim.get_option("schedule")),
                   "maxrregcount": int(sim.get_option("maxrregcount")),
                   "block_size_used": int(sim.get_option("block_size")),
                   "last_launch": {"grid": int(sim.get_option("last_grid")), "block": int(sim.get_option("last_block"))},
                   "l2": "256 MB buffer zeroed between timed steps; inputs 150 MB > L2"},
        "rhs_evals_per_s": rhs_per_s,
        "stats_per_step": st,
        "wall_ms_per_step_device_loop": 1e3 * wall_dev / args.steps,
        "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": peak_tflops, "unit": "TFLOP/s",
                     "frac": achieved_tflops / peak_tflops,
                     "traffic": ((DRAM_BYTES_PER_STEP[int(sp_["replay_split"])]["record"]
                                  + (DRAM_BYTES_PER_STEP[int(sp_["replay_split"])]["replay"]
                                     if sp_["replay_fused"] else 0)) * st["steps"]
                                 if replayed else DRAM_BYTES_PER_MEMBER * n),
                     "traffic_source": "ncu DRAM bytes of the 512 x 512 map, scaled by "
                                       + ("recorded steps" if replayed else "members"),
                     "peak_source": f"nominal FP32 FMA rate {info.compute_units} SMs x 128 lanes x 2 at the "
                                    f"median sampled SM clock {sm_mhz:.0f} MHz",
                     "kernel": ("clode_features_record_replay" if sp_["replay_fused"] else "clode_init_observer_record")
                     if replayed else "clode_init_observer + clode_features",
                     "ms": rec_ms, "flops_per_launch": flops},
        "roofline_replay": roof_replay,
        "replay": sp_,
        "e2e": {"value": e2e_value, "unit": "points/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * float(np.mean(e2e_times)),
                "ms_all": [round(1e3 * x, 2) for x in e2e_times],
                "features_device_ms": [round(x, 2) for x in e2e_kernel],
                "replay_reallocs": e2e_reallocs,
                "get_f_pin_device_wall_ms": e2e_dl,
                "wall_ms_per_call": dict(zip(("set_problem_data", "set_tspan_per_member", "features", "get_f"),
                                             (round(1e3 * x / max(args.steps, 1), 2) for x in parts)))},
        "gpu_launches": int(launches_dev + launches_e2e),
        "gpu_launches_detail": {"device_loop": int(launches_dev), "e2e_loop": int(launches_e2e)},
        "clocks": clk,
    }

    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        idx = cpu_sample_indices(n, args.cpu_sample, args.seed)
        Fc, secs, kind = run_cpu(x0, pars, tspan, idx, threads)
        nf = sim.get_n_features()
        Fg = np.asarray(F).reshape(nf, n).T[idx]
        names = sim.get_feature_names()
        ev = names.index("event count")
        per = names.index("mean period")
        rel = np.abs(Fg[:, per] - Fc[:, per]) / np.maximum(np.abs(Fc[:, per]), 1e-12)
        line["cpu_baseline"] = {"value": idx.size / secs, "unit": "points/s", "cores": threads, "kind": kind,
                                "sample": f"{idx.size} random members of the grid (seeded), one features run"}
        line["error_vs_cpu"] = {"members": int(idx.size),
                                "event_count_exact_frac": float(np.mean(Fg[:, ev] == Fc[:, ev])),
                                "mean_period_rel_err_median": float(np.median(rel)),
                                "mean_period_rel_err_p99": float(np.quantile(rel, 0.99))}
        # both FP32 results against an FP64 run with a 10^4 tighter tolerance
        F64, _, _ = run_cpu(x0, pars, tspan, idx, threads, prefer_reference=False, single=False, tol=1e-10)

        def _vs64(Fx):
            r = np.abs(Fx[:, per] - F64[:, per]) / np.maximum(np.abs(F64[:, per]), 1e-12)
            return {"event_count_exact_frac": float(np.mean(Fx[:, ev] == F64[:, ev])),
                    "mean_period_rel_err_median": float(np.median(r)),
                    "mean_period_rel_err_p99": float(np.quantile(r, 0.99)),
                    "frac_period_rel_err_above_1e-4": float(np.mean(r > 1e-4)),
                    "frac_period_rel_err_above_1e-2": float(np.mean(r > 1e-2))}

        # the engine's precise option (FP32 integration, compensated sums,
        # event times refined in FP64) on the same members and build options
        ps = W.FeatureSimulatorBase(pi, "dopri5", "nhood2", op, True, res, "")
        for key in ("fmad", "prec_div", "ftz", "fast_math", "fast_exp", "paired", "maxrregcount", "split_attempts",
                    "schedule", "block_size"):
            ps.set_option(key, sim.get_option(key))
        ps.set_option("precise", 1)
        ps.build_cl()
        ps.set_solver_params(W.SolverParams(**SOLVER))
        ps.set_problem_data(np.ascontiguousarray(x0[idx].flatten(order="F")),
                            np.ascontiguousarray(pars[idx].flatten(order="F")))
        ps.set_tspan_per_member(np.ascontiguousarray(tspan[idx].ravel()))
        ps.features(True)
        Fq = np.asarray(ps.get_f()).reshape(nf, idx.size).T
        del ps
        line["error_vs_fp64"] = {"reference_run": "CPU oracle, FP64, DP45 rtol = abstol = 1e-10, same members",
                                 "gpu_fp32": _vs64(Fg), "gpu_fp32_precise": _vs64(Fq), "cpu_fp32": _vs64(Fc)}
    opts = {k: sim.get_option(k) for k in ("schedule", "block_size", "maxrregcount", "fmad", "prec_div", "ftz",
                                           "fast_math", "fast_exp", "paired", "split_attempts", "fuse_init")}
    # the map's simulator (and the device memory of its stored steps) is not
    # needed by the workloads below
    del sim
    import gc
    gc.collect()
    if rank == 0 and not args.no_surrogate:
        try:
            line["surrogate"] = bench_surrogate(args, opts)
        except Exception as e:  # reported, not hidden: the plain line stands on its own
            line["surrogate"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and not args.no_trajectory:
        try:
            line["trajectory"] = bench_trajectory(args, opts)
        except Exception as e:
            line["trajectory"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and args.configs:
        try:
            line["configs"] = bench_configs(args, opts)
        except Exception as e:
            line["configs"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and args.feature_store:
        try:
            line["feature_store"] = bench_feature_store(args, opts)
        except Exception as e:
            line["feature_store"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
