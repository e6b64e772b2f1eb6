"""Features with storage (clode_sim_features_store): one feature pass that
also stores the trajectory rows and the state at each observer event.

The reference's unified driver that this repairs (clode/cpp/odedriver.cl)
does not compile, so its parity is stated through the two kernels it
combines, each pinned to the oracle elsewhere: F, xf, dt, tf equal those of
features() bit for bit, the stored rows equal those of trajectory() bit for
bit, the event times equal the observer's own event-time features, and every
stored event state is a state of the nout = 1 trajectory.  FP arithmetic
without contraction (fmad off, the default), so separate builds agree
exactly."""
import numpy as np
import pytest

from clode_gb300 import clode_cpp_wrapper as W, rhs_path

pytestmark = pytest.mark.gpu

N = 256
VARS, PARS, AUX = ["v", "n", "f", "c"], ["gcal", "gsk", "gbk"], ["ica"]


def _problem(noise=False):
    if noise:
        return W.ProblemInfo(rhs_path("lactotroph_noise.cl"), VARS, PARS + ["sig"], AUX, 1)
    return W.ProblemInfo(rhs_path("lactotroph.cl"), VARS, PARS, AUX, 0)


def _data(noise=False):
    rng = np.random.default_rng(7)
    pars = np.stack([rng.uniform(0.5, 3.0, N), np.full(N, 3.0), rng.uniform(0.0, 2.0, N)], axis=1)
    if noise:
        pars = np.concatenate([pars, np.full((N, 1), 2.0)], axis=1)
    x0 = np.tile([-60.0, 0.0, 0.0, 0.1], (N, 1))
    return x0.flatten(order="F"), pars.flatten(order="F")


def _setup(sim, noise, max_store, nout, options):
    for k, v in options.items():
        sim.set_option(k, v)
    if noise:
        sim.set_solver_params(W.SolverParams(dt=0.01, max_steps=10000000, max_store=max_store, nout=nout))
        t1 = 500.0
    else:
        sim.set_solver_params(W.SolverParams(dt=0.1, dtmax=1.0, abstol=1e-6, reltol=1e-6, max_steps=10000000,
                                             max_store=max_store, nout=nout))
        t1 = 10000.0
    x0, pars = _data(noise)
    sim.set_problem_data(x0, pars)
    sim.set_tspan([0.0, t1])
    if noise:
        sim.seed_rng(99)


def _features_sim(noise, max_store, nout, options, nse=5, single=True):
    sim = W.FeatureSimulatorBase(_problem(noise), "seuler" if noise else "dopri5", "nhood2",
                                 W.ObserverParams(e_var_ix=3, f_var_ix=0, max_event_timestamps=nse,
                                                  nhood_radius=0.05, max_event_count=100000),
                                 single, W.OpenCLResource(), "")
    _setup(sim, noise, max_store, nout, options)
    return sim


def _trajectory_sim(noise, max_store, nout, options, single=True):
    sim = W.TrajectorySimulatorBase(_problem(noise), "seuler" if noise else "dopri5", single, W.OpenCLResource(), "")
    _setup(sim, noise, max_store, nout, {k: v for k, v in options.items() if k != "fuse_init"})
    return sim


def _same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


@pytest.mark.parametrize("noise", [False, True], ids=["dopri5", "seuler"])
@pytest.mark.parametrize("schedule,fuse", [(0, 0), (1, 0), (1, 1)])
def test_store_run_equals_features_and_trajectory(noise, schedule, fuse):
    options = {"schedule": schedule, "fuse_init": fuse}
    max_store, nout, ev_rows = 8000, 20, 8
    plain = _features_sim(noise, max_store, nout, options)
    plain.features(True)
    store = _features_sim(noise, max_store, nout, options)
    store.features_store(True, event_rows=ev_rows)
    for get in ("get_f", "get_xf", "get_tf", "get_dt"):
        assert _same(getattr(store, get)(), getattr(plain, get)()), get
    if noise:
        assert _same(store.get_rng_state(), plain.get_rng_state())

    traj = _trajectory_sim(noise, max_store, nout, options)
    traj.trajectory()
    ns = traj.get_n_stored()
    assert ns.max() < max_store  # the trajectory kernel was not cut short by its buffer
    assert _same(store.get_n_stored(), ns)
    for get in ("get_t", "get_x", "get_dx", "get_aux"):
        assert _same(getattr(store, get)(), getattr(traj, get)()), get

    # events: counts and times against the observer's own features
    names = store.get_feature_names()
    F = store.get_f().reshape(len(names), N)
    n_ev = store.get_n_events()
    assert _same(n_ev, F[names.index("event count")])
    if not noise:
        assert n_ev.max() > ev_rows  # some members fill the event store
    et = store.get_event_t().reshape(ev_rows, N)
    for k in range(5):
        have = n_ev > k
        assert _same(et[k, have], F[names.index(f"nhood event time {k}"), have]), k
        assert (et[k, ~have] == 0).all()


def test_store_run_fp64():
    options = {"schedule": 1}
    plain = _features_sim(False, 8000, 20, options, single=False)
    plain.features(True)
    store = _features_sim(False, 8000, 20, options, single=False)
    store.features_store(True, event_rows=4)
    assert _same(store.get_f(), plain.get_f()) and _same(store.get_xf(), plain.get_xf())
    traj = _trajectory_sim(False, 8000, 20, options, single=False)
    traj.trajectory()
    assert _same(store.get_n_stored(), traj.get_n_stored())
    for get in ("get_t", "get_x", "get_dx", "get_aux"):
        assert _same(getattr(store, get)(), getattr(traj, get)()), get
    by_member = store.get_trajectory_by_member(first=3, count=9)
    ns = traj.get_n_stored()[3:12]
    t_flat = traj.get_t().reshape(8000, N)[:, 3:12].T
    for i in range(9):
        assert _same(by_member["t"][i, :ns[i] + 1], t_flat[i, :ns[i] + 1])


def test_event_states_lie_on_the_trajectory():
    options = {"schedule": 1}
    ev_rows = 6
    store = _features_sim(False, 4000, 20, options)
    store.features_store(True, event_rows=ev_rows)
    n_ev = store.get_n_events()
    ev = {k: getattr(store, "get_event_" + k)() for k in ("t", "x", "dx", "aux")}
    traj = _trajectory_sim(False, 100000, 1, options)
    traj.trajectory()
    ns = traj.get_n_stored()
    assert ns.max() < 100000
    rows = traj.get_trajectory_by_member()
    ev_x = ev["x"].reshape(ev_rows, 4, N)
    ev_dx = ev["dx"].reshape(ev_rows, 4, N)
    ev_aux = ev["aux"].reshape(ev_rows, 1, N)
    ev_t = ev["t"].reshape(ev_rows, N)
    checked = 0
    for i in range(N):
        ti = rows["t"][i, :ns[i] + 1]
        for k in range(min(int(n_ev[i]), ev_rows)):
            r = np.flatnonzero(ti == ev_t[k, i])
            assert r.size == 1, (i, k)
            r = int(r[0])
            assert _same(rows["x"][i, r], ev_x[k, :, i])
            assert _same(rows["dx"][i, r], ev_dx[k, :, i])
            assert _same(rows["aux"][i, r], ev_aux[k, :, i])
            checked += 1
    assert checked > 32  # event states of the members that have events (63 with these inputs)


def test_store_subset():
    options = {"schedule": 1}
    full = _trajectory_sim(False, 4000, 20, options)
    full.trajectory()
    sub = _trajectory_sim(False, 4000, 20, options)
    sub.set_store_variables([3, 0], [])
    sub.trajectory()
    ms = 4000
    x_full = full.get_x().reshape(ms, 4, N)
    assert _same(sub.get_x().reshape(ms, 2, N), x_full[:, [3, 0], :])
    assert _same(sub.get_dx().reshape(ms, 2, N), full.get_dx().reshape(ms, 4, N)[:, [3, 0], :])
    assert _same(sub.get_t(), full.get_t())
    assert sub.get_aux().size == 1  # no stored auxiliary columns
    got = sub.get_trajectory_by_member(first=5, count=7)
    assert got["x"].shape[2] == 2 and "aux" not in got

    store = _features_sim(False, 4000, 20, options)
    store.set_store_variables([1], [0])
    store.features_store(True, event_rows=4)
    assert _same(store.get_x().reshape(ms, 1, N), x_full[:, [1], :])
    assert _same(store.get_aux(), full.get_aux())
    assert store.get_event_x().size == 4 * N and store.get_event_aux().size == 4 * N

    # back to all columns: the reference layout again.  Each run starts from
    # the step size the previous one ended with (CLODE.cpp writes dt back),
    # so both simulators run a second time.
    sub.set_store_variables(None, None)
    sub.trajectory()
    full.trajectory()
    ns = full.get_n_stored()
    assert _same(sub.get_n_stored(), ns)
    a, b = sub.get_trajectory_by_member(), full.get_trajectory_by_member()
    valid = np.arange(a["t"].shape[1])[None, :] <= ns[:, None]  # rows older runs left behind are not compared
    for k in ("t", "x", "dx", "aux"):
        assert a[k].shape == b[k].shape and _same(a[k][valid], b[k][valid]), k
    with pytest.raises(W.ClodeValueError):
        sub.set_store_variables([4], None)


def test_features_after_store_run_is_plain_features():
    options = {"schedule": 1}
    sim = _features_sim(False, 500, 20, options)
    sim.features_store(True, event_rows=2)
    sim.features(True)
    ref = _features_sim(False, 500, 20, options)
    ref.features(True)  # the first run leaves the same dt behind as the store run
    ref.features(True)
    assert _same(sim.get_f(), ref.get_f())
    with pytest.raises(Exception):
        sim.set_solver_params(W.SolverParams(dt=0.1, dtmax=1.0, abstol=1e-6, reltol=1e-6, max_steps=1000,
                                             max_store=10, nout=0))
        sim.features_store(True)


def test_noalloc_refuses_the_store_program():
    # the allocation-free entry point runs the plain features kernel only: after
    # a features_store run it asks for the plain program to be rebuilt first
    import ctypes as C
    from clode_gb300 import _native as Nt
    sim = _features_sim(False, 500, 20, {"schedule": 1})
    sim.features_store(True, event_rows=2)
    rc = Nt.lib.clode_sim_features_noalloc(sim._handle, 0, None, None, None, None, None, None, None, None, None, None)
    assert rc == 4  # CLODE_ERR_NOT_BUILT
    sim.build_cl()
    rc = Nt.lib.clode_sim_features_noalloc(sim._handle, 0, None, None, None, None, None, None, None, None, None, None)
    assert rc == 0  # n_pts = 0: nothing to launch


def test_events_by_member_match_the_flat_arrays():
    from oracle.trajectory_frontend import regroup_by_member
    ev_rows = 6
    store = _features_sim(False, 4000, 20, {"schedule": 1})
    store.features_store(True, event_rows=ev_rows)
    n_ev = store.get_n_events()
    got = store.get_events_by_member()
    rows = got["t"].shape[1]
    assert rows == min(ev_rows, int(n_ev.max()))
    assert np.array_equal(got["n_events"], n_ev)
    for k, w in (("t", 1), ("x", 4), ("dx", 4), ("aux", 1)):
        flat = getattr(store, "get_event_" + k)()
        want = regroup_by_member(flat, N, w, 0, N, rows)
        assert _same(got[k].reshape(N, rows, w), want), k
    part = store.get_events_by_member(first=100, count=20, rows=ev_rows)
    assert part["t"].shape == (20, ev_rows)
    assert _same(part["t"], regroup_by_member(store.get_event_t(), N, 1, 100, 20, ev_rows)[:, :, 0])


def test_store_run_equals_the_oracle_bitwise():
    # Lorenz (+ - * only), RK4 in FP64, thresh2: the engine's one-pass store
    # against the oracle's restatement of it, bit for bit
    from oracle.build import OracleConfig
    from oracle.runner import OracleSimulator
    n = 300
    rng = np.random.default_rng(4)
    x0 = np.ones((n, 3)) + rng.normal(0, 1e-3, (n, 3))
    pars = np.stack([rng.uniform(10, 60, n), rng.uniform(5, 15, n), np.full(n, 8 / 3)], axis=1)
    sp = dict(dt=1e-3, max_steps=100000, max_store=3000, nout=5)
    opk = dict(e_var_ix=2, f_var_ix=2, max_event_count=100000, x_up_threshold=0.3, x_down_threshold=0.2)
    pi = W.ProblemInfo(rhs_path("lorenz.cl"), ["x", "y", "z"], ["rho", "sigma", "beta"], ["fx"], 0)
    sim = W.FeatureSimulatorBase(pi, "rk4", "thresh2", W.ObserverParams(**opk), False, W.OpenCLResource(), "")
    sim.set_option("schedule", 1)
    sim.set_solver_params(W.SolverParams(dtmax=1.0, abstol=1e-6, reltol=1e-3, **sp))
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    sim.set_tspan([0.0, 10.0])
    sim.features_store(True, event_rows=8)
    cfg = OracleConfig(rhs_path("lorenz.cl"), n_var=3, n_par=3, n_aux=1, stepper="rk4", single_precision=False,
                       observer="thresh2", n_store_events=0)
    ora = OracleSimulator(cfg)
    ora.set_solver_params(**sp)
    ora.set_observer_params(**opk)
    ora.set_problem_data(x0, pars)
    ora.set_tspan((0.0, 10.0))
    ora.features_store(event_rows=8, reinitialize=True)
    ms = 3000
    assert np.array_equal(sim.get_f(), ora.F.astype(np.float64))
    assert np.array_equal(sim.get_n_stored(), ora.n_stored)
    assert np.array_equal(sim.get_t(), ora.t[: ms * n])
    assert np.array_equal(sim.get_x(), ora.x[: ms * n * 3])
    assert np.array_equal(sim.get_dx(), ora.dx[: ms * n * 3])
    assert np.array_equal(sim.get_n_events(), ora.n_events)
    for k in ("t", "x", "dx", "aux"):
        assert np.array_equal(getattr(sim, "get_event_" + k)(), getattr(ora, "ev_" + k)), k
