"""Parity of the CUDA engine (called through the drop-in API and the C ABI)
with the CPU oracle on identical seeded inputs.

Tolerances:
  * fixed-step steppers (Euler, Heun, RK4) on models built from + - * /
    only: bitwise equality of final states, times, step sizes and every
    feature, in FP64 and FP32 (the engine reproduces the reference's
    operation order with contraction off);
  * anything that calls a transcendental function — the adaptive
    controller's pow, exp in the lactotroph model, log in the normal
    deviates — differs from the CPU's libm in the last bit now and then, so
    those runs are compared with a relative tolerance written in each test,
    event counts exactly for all but a stated fraction of members.
"""
import numpy as np
import pytest

from tests.parity import Scenario, assert_bitwise, mismatch_fraction, run_engine, run_oracle

pytestmark = pytest.mark.gpu

SEED = 20261203


def vdp_inputs(n, seed=SEED):
    rng = np.random.default_rng(seed)
    mu = rng.uniform(0.1, 5.0, n)
    x0 = rng.uniform(-2.0, 2.0, (n, 2))
    return x0, mu[:, None]


def lorenz_inputs(n, seed=SEED):
    rng = np.random.default_rng(seed)
    x0 = np.ones((n, 3)) + rng.normal(0.0, 1e-3, (n, 3))
    rho = rng.uniform(10, 60, n)
    sigma = rng.uniform(5, 15, n)
    return x0, np.stack([rho, sigma, np.full(n, 8.0 / 3.0)], axis=1)


def test_vdp_rk4_fp64_localmax_bitwise():
    x0, p = vdp_inputs(512)
    sc = Scenario("van_der_pol.cl", 2, 1, x0, p, stepper="rk4", observer="localmax", single=False,
                  sp=dict(dt=0.01, max_steps=10000000),
                  steps=[("transient", (0.0, 20.0)), ("shift_x0",), ("features", (20.0, 100.0))])
    eng, ora = run_engine(sc), run_oracle(sc)
    assert_bitwise(eng, ora)
    F = eng["F_list"][0]
    names = eng["feature_names"]
    assert len(names) == F.shape[1] == 18
    # every member oscillates: several local maxima, positive mean period
    assert (F[:, names.index("event count")] >= 3).all()
    assert (F[:, names.index("mean IMI")] > 0).all()


@pytest.mark.parametrize("stepper", ["euler", "heun", "rk4"])
@pytest.mark.parametrize("observer", ["basic", "basicall", "localmax", "nhood1", "nhood2", "thresh2"])
@pytest.mark.parametrize("single", [False, True])
def test_fixed_steppers_all_observers_bitwise(stepper, observer, single):
    x0, p = lorenz_inputs(256)
    sc = Scenario("lorenz.cl", 3, 3, x0, p, n_aux=1, stepper=stepper, observer=observer, single=single,
                  n_store_events=3 if observer in ("thresh2", "nhood2") else 0,
                  sp=dict(dt=0.005, max_steps=100000),
                  op=dict(e_var_ix=2, f_var_ix=2, max_event_count=10000, x_up_threshold=0.3,
                          x_down_threshold=0.2, nhood_radius=0.1),
                  steps=[("features", (0.0, 10.0)), ("shift_x0",), ("shift_tspan",), ("features", None)])
    eng, ora = run_engine(sc), run_oracle(sc)
    assert_bitwise(eng, ora)


@pytest.mark.parametrize("single", [False, True])
def test_fixed_steppers_trajectory_bitwise(single):
    x0, p = vdp_inputs(300)
    sc = Scenario("van_der_pol.cl", 2, 1, x0, p, stepper="rk4", single=single,
                  sp=dict(dt=0.01, max_store=500, nout=3),
                  steps=[("trajectory", (0.0, 20.0))])
    eng, ora = run_engine(sc), run_oracle(sc)
    assert_bitwise(eng, ora, keys=("xf", "tf", "dt", "t", "x", "dx", "n_stored"))
    # max_store bounds the rows: 500 stored rows stop the run at step 1500 (t = 15), before t = 20
    assert (eng["n_stored"] == 500).all()
    assert np.allclose(eng["tf"], 15.0, atol=1e-4)


@pytest.mark.parametrize("stepper", ["bs23", "dopri5"])
@pytest.mark.parametrize("single", [False, True])
def test_adaptive_thresh2_close(stepper, single):
    x0, p = vdp_inputs(256)
    sc = Scenario("van_der_pol.cl", 2, 1, x0, p, stepper=stepper, observer="thresh2", single=single,
                  sp=dict(dt=0.01, dtmax=0.5, abstol=1e-9 if not single else 1e-6, reltol=1e-6 if not single else 1e-4,
                          max_steps=1000000),
                  op=dict(e_var_ix=0, f_var_ix=0, max_event_count=10000, x_up_threshold=0.3, x_down_threshold=0.2),
                  steps=[("features", (0.0, 200.0))])
    eng, ora = run_engine(sc), run_oracle(sc)
    F, G = eng["F_list"][0], ora["F_list"][0]
    names = eng["feature_names"]
    # tolerance: pow() in the step-size controller may differ by an ulp between
    # CUDA and the host libm; the step sequences then drift apart and the
    # solutions agree to about 100x the integration tolerance
    rtol = 1e-4 if not single else 2e-2
    ev = names.index("event count")
    assert (np.abs(F[:, ev] - G[:, ev]) <= 1).all()
    assert np.mean(F[:, ev] == G[:, ev]) >= 0.98
    per = names.index("mean period")
    assert mismatch_fraction(F[:, per], G[:, per], rtol=rtol, atol=1e-6) <= 0.02
    assert mismatch_fraction(eng["xf"], ora["xf"], rtol=1e-3 if single else 1e-5, atol=1e-5) <= 0.05


def test_lactotroph_transient_published_state():
    # samples/test_outputs_cpp.md:10 of the reference: RK4 dt=0.1 over [0,1000],
    # FP32, x0 = 0, (gcal, gsk, gbk) = (1.5, 3, 1): -64.7058 0.022137 6.25581e-06 0.209086
    n = 32
    sc = Scenario("lactotroph.cl", 4, 3, np.zeros((n, 4)), np.tile([1.5, 3.0, 1.0], (n, 1)), n_aux=1,
                  stepper="rk4", single=True,
                  sp=dict(dt=0.1, dtmax=1.0, max_steps=10000000, nout=50),
                  steps=[("transient", (0.0, 1000.0)), ("transient", (0.0, 1000.0))])
    eng = run_engine(sc)
    xf = eng["xf"][0]
    np.testing.assert_allclose(xf, [-64.7058, 0.022137, 6.25581e-06, 0.209086], rtol=2e-5)
    ora = run_oracle(sc)
    # tolerance: expf differs between CUDA and the host libm in the last bit
    np.testing.assert_allclose(eng["xf"], ora["xf"], rtol=1e-4, atol=1e-9)


def test_ou_trajectory_seuler_fp32():
    # 16 parameter points x 16 realisations, Euler-Maruyama dt=1e-3, every 10th step stored
    th = np.linspace(0.1, 2.0, 4)
    sg = np.linspace(0.1, 1.0, 4)
    TH, SG = np.meshgrid(th, sg, indexing="ij")
    reps = 16
    pars = np.stack([np.repeat(TH.ravel(), reps), np.zeros(16 * reps), np.repeat(SG.ravel(), reps)], axis=1)
    n = pars.shape[0]
    sc = Scenario("ornstein_uhlenbeck.cl", 1, 3, np.zeros((n, 1)), pars, n_wiener=1, stepper="seuler", single=True,
                  sp=dict(dt=1e-3, max_steps=5000, max_store=502, nout=10), seed=7,
                  steps=[("trajectory", (0.0, 5.0))])
    eng, ora = run_engine(sc), run_oracle(sc)
    assert (eng["n_stored"] == ora["n_stored"]).all()
    assert (eng["n_stored"] == 500).all()
    np.testing.assert_array_equal(eng["t"], ora["t"])
    # tolerance: logf in the normal deviates may differ by an ulp from the host libm
    np.testing.assert_allclose(eng["x"], ora["x"], rtol=1e-3, atol=2e-5)


def test_lactotroph_nhood2_per_member_tspan():
    n = 512
    rng = np.random.default_rng(SEED)
    gcal = rng.uniform(0.5, 3.0, n)
    gbk = rng.uniform(0.0, 2.0, n)
    pars = np.stack([gcal, np.full(n, 3.0), gbk], axis=1)
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
    t1 = rng.uniform(1e3, 3e3, n)
    tspan = np.stack([np.zeros(n), t1], axis=1)
    sc = Scenario("lactotroph.cl", 4, 3, x0, pars, n_aux=1, stepper="dopri5", observer="nhood2", single=True,
                  sp=dict(dt=0.1, dtmax=100.0, abstol=1e-6, reltol=1e-6, max_steps=10000000),
                  op=dict(e_var_ix=3, f_var_ix=0, max_event_count=100000, nhood_radius=0.05,
                          x_down_threshold=0.2), tspan_pm=tspan,
                  steps=[("features",)])
    eng, ora = run_engine(sc), run_oracle(sc)
    F, G = eng["F_list"][0], ora["F_list"][0]
    names = eng["feature_names"]
    assert len(names) == 42
    np.testing.assert_allclose(eng["tf"], ora["tf"], rtol=1e-5)
    ev = names.index("event count")
    # tolerance: exp/pow ulp differences; spike counts exact for >= 97% of members
    assert np.mean(F[:, ev] == G[:, ev]) >= 0.97
    pk = names.index("mean peaks")
    assert np.mean(np.isclose(F[:, pk], G[:, pk], rtol=1e-3, atol=1e-3)) >= 0.95


@pytest.mark.parametrize("fuse", [0, 1])
def test_observer_initialisation_fused_or_separate(fuse):
    x0, p = lorenz_inputs(128)
    sc = Scenario("lorenz.cl", 3, 3, x0, p, n_aux=1, stepper="rk4", observer="thresh2", single=False,
                  sp=dict(dt=0.005, max_steps=100000),
                  op=dict(e_var_ix=2, f_var_ix=2, max_event_count=10000, x_up_threshold=0.3, x_down_threshold=0.2),
                  steps=[("features", (0.0, 10.0)), ("features", (0.0, 10.0), True), ("initialize_observer", None),
                         ("features", None)])
    eng, ora = run_engine(sc, options={"fuse_init": fuse}), run_oracle(sc)
    assert_bitwise(eng, ora)


# ------------------------------------------------------------ persistent schedule
PERSISTENT = {"schedule": 1}


@pytest.mark.parametrize("observer", ["localmax", "nhood2", "thresh2"])
@pytest.mark.parametrize("single", [False, True])
@pytest.mark.parametrize("fuse", [1, 0])
def test_persistent_schedule_bitwise(observer, single, fuse):
    # uneven members: per-member time spans over a factor of 20
    x0, p = lorenz_inputs(2000)
    rng = np.random.default_rng(3)
    tspan = np.stack([np.zeros(2000), rng.uniform(0.5, 10.0, 2000)], axis=1)
    sc = Scenario("lorenz.cl", 3, 3, x0, p, n_aux=1, stepper="rk4", observer=observer, single=single,
                  sp=dict(dt=0.005, max_steps=100000),
                  op=dict(e_var_ix=2, f_var_ix=2, max_event_count=10000, x_up_threshold=0.3, x_down_threshold=0.2,
                          nhood_radius=0.1),
                  tspan_pm=tspan, steps=[("features",), ("shift_x0",), ("features",), ("features", None, True)])
    eng, ora = run_engine(sc, options=dict(PERSISTENT, fuse_init=fuse)), run_oracle(sc)
    assert_bitwise(eng, ora)


@pytest.mark.parametrize("kind", ["transient", "trajectory"])
def test_persistent_transient_trajectory_bitwise(kind):
    x0, p = vdp_inputs(1500)
    rng = np.random.default_rng(4)
    tspan = np.stack([np.zeros(1500), rng.uniform(1.0, 8.0, 1500)], axis=1)
    steps = [("transient",), ("shift_x0",), ("transient",)] if kind == "transient" else [("trajectory",)]
    sc = Scenario("van_der_pol.cl", 2, 1, x0, p, stepper="heun", single=False, tspan_pm=tspan,
                  sp=dict(dt=0.01, max_store=1000, nout=2), steps=steps)
    eng, ora = run_engine(sc, options=PERSISTENT), run_oracle(sc)
    keys = ("xf", "tf", "dt") + (("t", "x", "dx", "n_stored") if kind == "trajectory" else ())
    assert_bitwise(eng, ora, keys=keys)


@pytest.mark.parametrize("stepper", ["bs23", "dopri5"])
@pytest.mark.parametrize("kind", ["features", "transient", "trajectory"])
def test_split_attempts_bitwise(stepper, kind):
    # adaptive steps with rejections: one attempt per loop iteration
    # (split_attempts 1) gives the same results as whole steps, on both
    # schedules, since each member's operations are unchanged (fmad off: with
    # contraction allowed the compiler may fuse differently in each kernel)
    x0, p = lorenz_inputs(1500)
    rng = np.random.default_rng(6)
    tspan = np.stack([np.zeros(1500), rng.uniform(2.0, 12.0, 1500)], axis=1)
    steps = {"features": [("features",), ("shift_x0",), ("features",)],
             "transient": [("transient",), ("shift_x0",), ("transient",)],
             "trajectory": [("trajectory",)]}[kind]
    sc = Scenario("lorenz.cl", 3, 3, x0, p, n_aux=1, stepper=stepper, observer="thresh2" if kind == "features" else None,
                  single=True, sp=dict(dt=0.05, dtmax=0.5, abstol=1e-7, reltol=1e-5, max_steps=200000,
                                      max_store=2000, nout=3),
                  op=dict(e_var_ix=2, f_var_ix=2, max_event_count=10000, x_up_threshold=0.3, x_down_threshold=0.2),
                  tspan_pm=tspan, steps=steps)
    assert sc.kind == kind
    ref = run_engine(sc, options={"schedule": 0, "fmad": 0})
    assert ref["stats"][0]["rejected"] > 0
    # the counters match where both runs integrate the same passes; the
    # replayed feature pass (last options) integrates the trajectory once
    for opts in ({"schedule": 1, "fmad": 0, "split_attempts": 0, "replay": 0},
                 {"schedule": 1, "fmad": 0, "split_attempts": 1, "replay": 0},
                 {"schedule": 1, "fmad": 0, "split_attempts": 1, "fuse_init": 0, "replay": 0},
                 {"schedule": 1, "fmad": 0, "split_attempts": 1, "fuse_init": 0, "replay": 1}):
        eng = run_engine(sc, options=opts)
        keys = ("xf", "tf", "dt") + (("t", "x", "dx", "n_stored") if kind == "trajectory" else ())
        assert_bitwise(eng, ref, keys=keys)  # and every features run
        if not (kind == "features" and opts["replay"]):
            assert eng["stats"][0]["rejected"] == ref["stats"][0]["rejected"]


@pytest.mark.parametrize("single", [False, True], ids=["fp64", "fp32"])
@pytest.mark.parametrize("schedule", [0, 1], ids=["grid", "persistent"])
def test_stochastic_bitwise_rng_state(single, schedule):
    # seuler on the OU process, two launches in a row: the RNG words the
    # engine stores after each launch must be the oracle's, whatever lanes
    # of a warp drew ahead of need (the look-ahead is undone before the
    # store), and in FP32 whichever conversion of the u64 words ran.  The
    # deviates use log, so the states are compared with a tolerance.
    n = 3000
    rng = np.random.default_rng(5)
    pars = np.stack([rng.uniform(0.1, 2, n), np.zeros(n), rng.uniform(0.1, 1, n)], axis=1)
    sc = Scenario("ornstein_uhlenbeck.cl", 1, 3, np.zeros((n, 1)), pars, n_wiener=1, stepper="seuler",
                  single=single, sp=dict(dt=1e-3, max_steps=3000), seed=99,
                  steps=[("transient", (0.0, 2.0)), ("shift_x0",), ("transient", (0.0, 1.5))])
    eng = run_engine(sc, options={"schedule": schedule})
    from oracle.runner import OracleSimulator
    s = OracleSimulator(sc.oracle_config())
    s.set_solver_params(dt=1e-3, dtmax=0.5, abstol=1e-6, reltol=1e-3, max_steps=3000, max_store=1, nout=1)
    s.set_problem_data(sc.x0, sc.pars)
    s.seed_rng(99)
    s.set_tspan((0.0, 2.0))
    s.transient()
    s.shift_x0()
    s.set_tspan((0.0, 1.5))
    s.transient()
    np.testing.assert_array_equal(eng["sim"].get_rng_state(), s.rng)
    # tolerance: log() of the polar method may differ by an ulp from the host libm
    if single:
        np.testing.assert_allclose(eng["xf"], s.get_xf(), rtol=1e-3, atol=2e-5)
    else:
        np.testing.assert_allclose(eng["xf"], s.get_xf(), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("fuse", [0, 1])
def test_longest_span_first_order_changes_nothing(fuse):
    # the persistent lanes take members in decreasing order of their time
    # span, and the feature pass in decreasing order of the warm-up steps,
    # by default; every member's results must equal those of the natural
    # order bit for bit
    n = 3000
    rng = np.random.default_rng(8)
    pars = np.stack([rng.uniform(0.5, 3.0, n), np.full(n, 3.0), rng.uniform(0.0, 2.0, n)], axis=1)
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
    tspan = np.stack([np.zeros(n), rng.uniform(200.0, 2000.0, n)], axis=1)
    sc = Scenario("lactotroph.cl", 4, 3, x0, pars, n_aux=1, stepper="dopri5", single=True,
                  observer="nhood2", op=dict(e_var_ix=3, f_var_ix=0), tspan_pm=tspan, steps=[("features", None, True)])
    # (span order, warm-up-steps order of the feature pass): neither, both, each alone
    runs = [run_engine(sc, options={"schedule": 1, "fuse_init": fuse, "order_by_span": o, "order_by_work": w})
            for o, w in ((0, 0), (1, 1), (1, 0), (0, 1))]
    for r in runs[1:]:
        for k in ("xf", "tf", "dt"):
            assert np.array_equal(runs[0][k], r[k], equal_nan=True), k
        assert np.array_equal(runs[0]["F_list"][0], r["F_list"][0], equal_nan=True)
        assert runs[0]["stats"] == r["stats"]


def test_all_zero_rng_state_is_rejected():
    # (0, 0) is xoroshiro128+'s fixed point: the polar method would reject
    # every candidate drawn from it, so such a state is refused on the host
    # and the stored state stays as it was
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path
    n = 16
    pi = W.ProblemInfo(rhs_path("ornstein_uhlenbeck.cl"), ["x"], ["theta", "mu", "sigma"], [], 1)
    sim = W.SimulatorBase(pi, "seuler", True, W.OpenCLResource(), "")
    sim.set_problem_data(np.zeros(n), np.tile([1.0, 0.0, 0.5], (n, 1)).flatten(order="F"))
    sim.seed_rng(3)
    before = sim.get_rng_state()
    st = before.copy()
    st[5] = st[n + 5] = 0
    with pytest.raises(W.ClodeValueError, match="fixed point"):
        sim.set_rng_state(st)
    assert np.array_equal(sim.get_rng_state(), before)
    st = before.copy()
    st[5] = 0  # one zero word is a valid state
    sim.set_rng_state(st)
    assert np.array_equal(sim.get_rng_state(), st)


def test_time_budget_marks_unprocessed_members():
    # a 50 us budget, far shorter than one member (5000 RK4 steps): lanes take
    # a member at the start, finish it, and take no other; the members never
    # taken are flagged, and every member taken completes normally
    x0, p = vdp_inputs(200000)
    sc = Scenario("van_der_pol.cl", 2, 1, x0, p, stepper="rk4", single=False,
                  sp=dict(dt=0.01, max_steps=1000000), steps=[("transient", (0.0, 50.0))])
    eng = run_engine(sc, options={"schedule": 1, "time_budget_ms": 0.05, "blocks_per_sm": 1, "block_size": 64})
    status = eng["status"][-1]
    done = (status & 16) == 0
    sim = eng["sim"]
    grid = int(sim.get_option("last_grid")) * int(sim.get_option("last_block"))
    assert 0 < done.sum() <= grid
    assert (status[~done] == 16).all()
    ora = run_oracle(sc)
    np.testing.assert_array_equal(eng["xf"][done], ora["xf"][done])


def test_xpp_style_float_literals_match_the_oracle():
    # literals with an `f` suffix (clODE's XPP translator) are float constants
    # promoted in FP64 arithmetic on both sides, so the FP64 RK4 run matches
    # the oracle bit for bit in the state (the aux feature uses exp: 1e-12)
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models", "xpp_style.cl")
    n = 512
    rng = np.random.default_rng(21)
    x0 = rng.uniform(-2.0, 2.0, (n, 2))
    pars = np.stack([rng.uniform(0.5, 0.9, n), rng.uniform(0.6, 0.9, n)], axis=1)
    sc = Scenario(path, 2, 2, x0, pars, n_aux=1, stepper="rk4", observer="localmax", single=False,
                  sp=dict(dt=0.01, max_steps=1000000), steps=[("features", (0.0, 60.0), True)])
    eng, ora = run_engine(sc), run_oracle(sc)
    assert_bitwise(eng, ora, keys=("xf", "tf", "dt"))
    np.testing.assert_allclose(eng["F_list"][0], ora["F_list"][0], rtol=1e-12, atol=1e-14)
