"""Chains of runs (transient -> shift_x0 -> features -> shift_x0), eager and
replayed as a CUDA graph, against the same calls made one by one through
the API: bit-for-bit equal (same kernels, same arguments)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(schedule, fuse=1):
    from clode_gb300 import clode_cpp_wrapper as W, rhs_path

    pi = W.ProblemInfo(rhs_path("van_der_pol.cl"), ["x", "y"], ["mu"], [], 0)
    op = W.ObserverParams(e_var_ix=0, f_var_ix=0, max_event_count=10000, x_up_threshold=0.3, x_down_threshold=0.2)
    sim = W.FeatureSimulatorBase(pi, "rk4", "thresh2", op, False, W.OpenCLResource(), "")
    sim.set_option("schedule", schedule)
    sim.set_option("fuse_init", fuse)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=0.01, max_steps=1000000))
    rng = np.random.default_rng(8)
    n = 3000
    x0 = rng.uniform(-2, 2, (n, 2))
    mu = rng.uniform(0.1, 5, (n, 1))
    sim.set_problem_data(x0.flatten(order="F"), mu.flatten(order="F"))
    sim.set_tspan([0.0, 20.0])
    return sim, n


@pytest.mark.parametrize("schedule,fuse", [(0, 1), (1, 1), (1, 0)])
def test_graph_chain_equals_api_calls(schedule, fuse):
    from clode_gb300 import _native as N

    a, n = _sim(schedule, fuse)
    for _ in range(3):
        a.transient()
        a.shift_x0()
        a.features()
        a.shift_x0()
    Fa, xa = np.asarray(a.get_f()), np.asarray(a.get_xf())

    for use_graph in (False, True):
        b, _ = _sim(schedule, fuse)
        launches = []
        for _ in range(3):
            before = N.lib.clode_launch_count()
            b.run_chain(["transient", "shift_x0", "features", "shift_x0"], use_graph=use_graph)
            launches.append(N.lib.clode_launch_count() - before)
        np.testing.assert_array_equal(np.asarray(b.get_f()), Fa)
        np.testing.assert_array_equal(np.asarray(b.get_xf()), xa)
        assert b.is_observer_initialized()
        # two ensemble kernels per chain, the first features launch initialising
        # the observer (or a separate initialisation launch before it)
        assert launches == ([2, 2, 2] if fuse else [3, 2, 2])
