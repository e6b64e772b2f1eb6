"""The autotuner changes only how a run is scheduled and compiled (register
cap, block size, one attempt per iteration, separate observer
initialisation), never its results: with contraction off, a tuned simulator
gives the same bits as an untuned one, and the members it samples keep
their dt and RNG state.  With contraction on it also chooses between paired
and scalar stage sums; a fast build's rounding can then differ between the
kernels a member runs through (the replay's launch layout depends on the
simulator's history), so a tuned fast simulator is compared with an untuned
one built with the options it chose to rounding level: spike counts equal
for 99 % of the members and continuous features within a median relative
difference of 1e-5."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(n=6000, seed=12, options=None):
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path

    pi = W.ProblemInfo(rhs_path("lactotroph.cl"), ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"], 0)
    op = W.ObserverParams(e_var_ix=3, f_var_ix=0, max_event_count=100000, nhood_radius=0.05,
                          x_down_threshold=0.2)
    sim = W.FeatureSimulatorBase(pi, "dopri5", "nhood2", op, True, W.OpenCLResource(), "")
    for k, v in (options or {"fmad": 0}).items():
        sim.set_option(k, v)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=0.1, dtmax=1.0, abstol=1e-6, reltol=1e-6, max_steps=10000000))
    rng = np.random.default_rng(seed)
    pars = np.stack([rng.uniform(0.5, 3.0, n), np.full(n, 3.0), rng.uniform(0.0, 2.0, n)], axis=1)
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1))
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    ts = np.stack([np.zeros(n), rng.uniform(200.0, 1500.0, n)], axis=1)
    sim.set_tspan_per_member(ts.ravel())
    return sim


def test_autotuned_results_equal_untuned():
    a = _sim()
    a.features(True)
    Fa, xa, dta = np.asarray(a.get_f()), np.asarray(a.get_xf()), np.asarray(a.get_dt())

    b = _sim()
    rng_before = np.asarray(b.get_rng_state()).copy()
    dt_before = np.asarray(b.get_dt()).copy()
    tuned = b.autotune(2000)
    assert tuned["ms"] > 0 and int(b.get_option("schedule")) == 1
    assert tuned["maxrregcount"] in (0, 64, 80, 96, 128) and tuned["block_size"] in (64, 128)
    # the sampled members' state is restored
    np.testing.assert_array_equal(np.asarray(b.get_rng_state()), rng_before)
    np.testing.assert_array_equal(np.asarray(b.get_dt()), dt_before)
    b.features(True)
    np.testing.assert_array_equal(np.asarray(b.get_f()), Fa)
    np.testing.assert_array_equal(np.asarray(b.get_xf()), xa)
    np.testing.assert_array_equal(np.asarray(b.get_dt()), dta)


def test_autotuned_fast_build_matches_untuned_with_its_choices():
    fast = {"fmad": 1, "prec_div": 0, "ftz": 1}
    b = _sim(options=fast)
    tuned = b.autotune(2000)
    assert tuned["paired"] in (0, 1)
    b.features(True)
    chosen = dict(fast, schedule=1, **{k: tuned[k] for k in ("maxrregcount", "block_size", "split_attempts",
                                                             "paired", "fuse_init", "replay", "replay_split",
                                                             "replay_fused")})
    a = _sim(options=chosen)
    a.features(True)
    names = list(a.get_feature_names())
    n = 6000
    Fa = np.asarray(a.get_f()).reshape(-1, n).T
    Fb = np.asarray(b.get_f()).reshape(-1, n).T
    counts = [names.index(c) for c in ("event count", "max peaks", "min peaks", "mean peaks")]
    cont = [names.index(f"{s} {v}") for v in ("v", "n", "f", "c") for s in ("max", "min", "mean")]
    agree = np.all(Fa[:, counts] == Fb[:, counts], axis=1)
    rel = np.abs(Fa[agree][:, cont] - Fb[agree][:, cont]) / np.maximum(np.abs(Fb[agree][:, cont]), 1e-6)
    print(f"\ntuned {tuned}: {np.mean(np.all(Fa == Fb, axis=1)):.4f} of members bitwise equal, counts agree "
          f"{agree.mean():.4f}, median rel {np.median(rel):.2e}")
    assert agree.mean() >= 0.99
    assert np.median(rel) < 1e-5
