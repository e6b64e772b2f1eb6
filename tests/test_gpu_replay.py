"""The replayed feature pass against the integrated one.

For the two-pass observers (nhood2, thresh2) on the persistent schedule the
engine, by default, stores every step of the feature pass during the warm-up
launch and replays them into the observer instead of integrating the
trajectory a second time.  These tests run the same ensembles with the
option ``replay`` on and off and require bitwise equal results — features,
final states, final times, step sizes, RNG words and status words — in the
cases that exercise each path of the replay:

* steppers fixed and adaptive, FP32 and FP64, per-member time spans;
* the replay's rows straight from global memory (the default) and through
  shared-memory stages (``replay_stages`` 2 and 8: TMA bulk copies);
* whole rows (``replay_split`` 0) and replay warps that take several regions
  (more recording blocks per SM than the replay's registers allow);
* recording and replay in one launch per launch pair (``replay_fused``);
* record regions far too small for the ensemble (``replay_mb``): many
  recording launches, members still running when their region fills (the
  plain warm-up and feature passes run them again);
* an event limit the observers reach (``max_event_count``): members the
  replay hands back to the plain feature pass;
* members whose span is empty (no step at all);
* the stochastic stepper (the noise replayed, RNG words as integrated);
* a continuation (``features(False)``) after a replayed run.
The oracle comparisons of the other GPU tests run through the replay too,
since it is the default.
"""
import numpy as np
import pytest

from clode_gb300 import clode_cpp_wrapper as W, rhs_path

pytestmark = pytest.mark.gpu


def _lorenz(n, seed=3):
    r = np.random.default_rng(seed)
    x0 = np.ones((n, 3)) + r.normal(0, 1e-3, (n, 3))
    pars = np.stack([r.uniform(10, 40, n), r.uniform(5, 15, n), np.full(n, 8 / 3)], axis=1)
    ts = np.stack([np.zeros(n), r.uniform(5.0, 30.0, n)], axis=1)
    return x0, pars, ts


def _sim(observer, stepper, single, replay, options=None, max_events=100000, model="lorenz", n_store=0):
    if model == "lorenz":
        pi = W.ProblemInfo(rhs_path("lorenz.cl"), ["x", "y", "z"], ["rho", "sigma", "beta"], ["fx"], 0)
        op = W.ObserverParams(e_var_ix=2, f_var_ix=0, max_event_count=max_events, max_event_timestamps=n_store,
                              nhood_radius=0.1, x_up_threshold=0.3, x_down_threshold=0.2)
    else:
        pi = W.ProblemInfo(rhs_path("lactotroph_noise.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk", "sig"],
                           ["ica"], 1)
        op = W.ObserverParams(e_var_ix=3, f_var_ix=0, max_event_count=max_events, nhood_radius=0.05,
                              x_up_threshold=0.3, x_down_threshold=0.2)
    sim = W.FeatureSimulatorBase(pi, stepper, observer, op, single, W.OpenCLResource(), "")
    sim.set_option("schedule", 1)
    sim.set_option("replay", replay)
    for k, v in (options or {}).items():
        sim.set_option(k, v)
    sim.build_cl()
    dt = 0.01 if model != "lorenz" else (2e-3 if stepper in ("euler", "heun", "rk4") else 1e-3)
    sim.set_solver_params(W.SolverParams(dt=dt, dtmax=1.0, abstol=1e-9, reltol=1e-6, max_steps=10000000))
    return sim


def _run(sim, x0, pars, ts, seed=7, reinit=True):
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan_per_member(ts.ravel())
    sim.seed_rng(seed)
    sim.features(reinit)
    return _outputs(sim)


def _outputs(sim):
    return {"F": np.asarray(sim.get_f()), "xf": np.asarray(sim.get_xf()), "tf": np.asarray(sim.get_tf()),
            "dt": np.asarray(sim.get_dt()), "rng": sim.get_rng_state(), "status": sim.get_status()}


def _equal(a, b):
    for k in a:
        x, y = a[k], b[k]
        same = (x == y) | (np.isnan(x) & np.isnan(y)) if x.dtype.kind == "f" else (x == y)
        assert same.all(), f"{k}: {np.size(same) - np.count_nonzero(same)} differ"


@pytest.mark.parametrize("observer", ["nhood2", "thresh2"])
@pytest.mark.parametrize("stepper", ["rk4", "dopri5", "bs23", "euler", "heun"])
@pytest.mark.parametrize("single", [True, False])
def test_replay_equals_integrated_feature_pass(observer, stepper, single):
    x0, pars, ts = _lorenz(2000)
    on = _sim(observer, stepper, single, 1)
    off = _sim(observer, stepper, single, 0)
    a, b = _run(on, x0, pars, ts), _run(off, x0, pars, ts)
    _equal(a, b)
    assert on.get_option("replay_chunks") >= 1
    assert on.get_option("replay_stages_used") == 0  # the default: rows from global memory
    # the counters: the replayed run integrates each member once (plus any fallback)
    assert on.get_stats()["rhs_evals"] < 0.75 * off.get_stats()["rhs_evals"]


@pytest.mark.parametrize("split", [1, 0])
def test_recording_and_replay_in_one_launch(split):
    x0, pars, ts = _lorenz(20000, seed=13)
    on = _sim("nhood2", "dopri5", True, 1, {"replay_fused": 1, "replay_split": split, "replay_mb": 200})
    off = _sim("nhood2", "dopri5", True, 0)
    _equal(_run(on, x0, pars, ts), _run(off, x0, pars, ts))
    assert on.get_option("replay_chunks") >= 1


@pytest.mark.parametrize("stages", [0, 2, 8])
def test_rows_from_global_memory_or_stages(stages):
    x0, pars, ts = _lorenz(3000, seed=11)
    on = _sim("nhood2", "dopri5", True, 1, {"replay_stages": stages})
    off = _sim("nhood2", "dopri5", True, 0)
    _equal(_run(on, x0, pars, ts), _run(off, x0, pars, ts))
    assert on.get_option("replay_stages_used") == stages


def test_replay_warps_take_several_regions():
    # 8 recording blocks of 128 threads per SM: the replay (its own register
    # cap) fits fewer, so each replay warp takes two or more regions; whole
    # rows (replay_split 0) with the replay running the whole update
    x0, pars, ts = _lorenz(160000, seed=12)
    ts[:, 1] = np.minimum(ts[:, 1], 8.0)
    on = _sim("nhood2", "dopri5", True, 1, {"blocks_per_sm": 8, "replay_split": 0})
    off = _sim("nhood2", "dopri5", True, 0)
    _equal(_run(on, x0, pars, ts), _run(off, x0, pars, ts))
    assert on.get_option("replay_regions_per_warp") >= 2


def test_small_regions_many_launches_and_overflow():
    # one 32-lane block per SM, so each lane holds several members in turn,
    # and regions of a few hundred rows per warp: members of a few thousand
    # steps do not fit and are run again by the plain passes
    x0, pars, ts = _lorenz(20000, seed=5)
    on = _sim("thresh2", "dopri5", True, 1, {"replay_mb": 60, "blocks_per_sm": 1, "block_size": 32})
    off = _sim("thresh2", "dopri5", True, 0)
    _equal(_run(on, x0, pars, ts), _run(off, x0, pars, ts))
    assert on.get_option("replay_chunks") > 1
    assert on.get_option("replay_rewarm") > 0
    # a second run: regions sized from the first run's step counts
    _equal(_run(on, x0, pars, ts, seed=9), _run(off, x0, pars, ts, seed=9))


def test_tiny_regions_every_member_falls_back():
    x0, pars, ts = _lorenz(500, seed=6)
    on = _sim("nhood2", "rk4", False, 1, {"replay_mb": 3})
    off = _sim("nhood2", "rk4", False, 0)
    _equal(_run(on, x0, pars, ts), _run(off, x0, pars, ts))
    assert on.get_option("replay_fallback") > 0
    assert on.get_option("replay_rewarm") > 0


@pytest.mark.parametrize("observer", ["nhood2", "thresh2"])
def test_event_limit_hands_members_back(observer):
    x0, pars, ts = _lorenz(1500, seed=8)
    on = _sim(observer, "dopri5", True, 1, max_events=4)
    off = _sim(observer, "dopri5", True, 0, max_events=4)
    a, b = _run(on, x0, pars, ts), _run(off, x0, pars, ts)
    _equal(a, b)
    assert on.get_option("replay_fallback") > 0
    assert (a["status"] & 8).any()  # members ended by the event limit


def test_members_without_steps():
    x0, pars, ts = _lorenz(700, seed=9)
    ts[::7, 1] = ts[::7, 0]        # empty spans: the feature pass still takes its t <= t1 step
    ts[3::11, 1] = ts[3::11, 0] - 1.0  # spans ending before they start: no step
    on = _sim("thresh2", "rk4", True, 1)
    off = _sim("thresh2", "rk4", True, 0)
    _equal(_run(on, x0, pars, ts), _run(off, x0, pars, ts))


def test_stochastic_stepper_replay():
    n = 512
    r = np.random.default_rng(4)
    pars = np.stack([r.uniform(0.5, 3.0, n), np.full(n, 3.0), r.uniform(0.0, 2.0, n), np.full(n, 2.0)], axis=1)
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
    ts = np.stack([np.zeros(n), r.uniform(200.0, 800.0, n)], axis=1)
    on = _sim("nhood2", "seuler", True, 1, model="lacto")
    off = _sim("nhood2", "seuler", True, 0, model="lacto")
    a, b = _run(on, x0, pars, ts), _run(off, x0, pars, ts)
    _equal(a, b)
    assert on.get_option("replay_fallback") == 0


def test_continuation_after_replay():
    x0, pars, ts = _lorenz(1000, seed=10)
    outs = []
    for replay in (1, 0):
        sim = _sim("nhood2", "dopri5", False, replay, n_store=2)
        first = _run(sim, x0, pars, ts)
        sim.shift_x0()
        sim.features(False)  # continue from the parked observer state
        outs.append((first, _outputs(sim)))
    _equal(outs[0][0], outs[1][0])
    _equal(outs[0][1], outs[1][1])
