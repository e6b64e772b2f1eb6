"""clode_sim_features_noalloc, the features entry point for callers that may
not allocate device memory (a device-memory budget fixed at start-up, a
pipeline that forbids allocation after initialisation, a plug-in whose host
application owns every allocation).  The test allocates the caller's buffers
itself (with torch), calls the entry point through the C ABI twice in a row,
and checks both results against the regular features() entry point: the same
kernel does the same arithmetic, so the comparison is exact.  One case uses the
simulator's tspan and the default stream, the other per-member time spans and
a stream of the caller's.  Around the second call (the first has looked up the
scratch array) the device's free memory must not change.  It also checks that
an ensemble too large for the fixed scratch array, and a missing parameter
buffer, are refused with nothing launched.

Collected last on purpose (file name), so a run stopped at the first failure
has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    # model, nVar, nPar, nAux, stepper, observer, single, tspan (None: per member), n, caller's stream
    "vdp_rk4_fp64_localmax": ("van_der_pol.cl", 2, 1, 0, "rk4", "localmax", False, (0.0, 30.0), 4096, False),
    "lactotroph_dopri5_fp32_nhood2": ("lactotroph.cl", 4, 3, 1, "dopri5", "nhood2", True, None, 2048, True),
}


def _inputs(name, n):
    rng = np.random.default_rng(11)
    if name.startswith("vdp"):
        return rng.uniform(-2, 2, (n, 2)), rng.uniform(0.1, 5.0, (n, 1))
    pars = np.stack([rng.uniform(0.5, 3.0, n), np.full(n, 3.0), rng.uniform(0.0, 2.0, n)], axis=1)
    return np.tile([-60.0, 0.0, 0.0, 0.1], (n, 1)), pars


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_features_matches_regular_entry_point(name):
    torch = pytest.importorskip("torch")
    from clode_gb300 import _native as N, clode_cpp_wrapper as W, rhs_path

    model, nv, np_, na, stepper, observer, single, tspan, n, own_stream = CASES[name]
    x0, pars = _inputs(name, n)
    ts_pm = None
    if tspan is None:  # per-member spans [0, T_i], T_i in [200, 600] ms
        ts_pm = np.stack([np.zeros(n), np.random.default_rng(3).uniform(200.0, 600.0, n)], axis=1).ravel()
    pi = W.ProblemInfo(rhs_path(model), [f"x{j}" for j in range(nv)], [f"p{j}" for j in range(np_)],
                       [f"a{j}" for j in range(na)], 0)
    op = W.ObserverParams(e_var_ix=nv - 1, f_var_ix=0, max_event_count=100000)
    sim = W.FeatureSimulatorBase(pi, stepper, observer, op, single, W.OpenCLResource(), "")
    sp = W.SolverParams(dt=0.01 if not single else 0.1, dtmax=1.0, abstol=1e-6, reltol=1e-6, max_steps=10000000)
    sim.build_cl()
    sim.set_solver_params(sp)
    sim.set_problem_data(x0.flatten(order="F"), pars.flatten(order="F"))
    if ts_pm is None:
        sim.set_tspan(list(tspan))
    else:
        sim.set_tspan_per_member(ts_pm)
    sim.seed_rng(5)
    rng0 = sim.get_rng_state()

    # the existing entry point
    sim.features(True)
    nf = sim.get_n_features()
    F_ref = np.asarray(sim.get_f())
    xf_ref, tf_ref = np.asarray(sim.get_xf()), np.asarray(sim.get_tf())

    # the caller's own device buffers (allocated here, by the caller)
    dev = torch.device("cuda:0")
    real = torch.float32 if single else torch.float64
    x0_d = torch.tensor(x0.flatten(order="F"), dtype=real, device=dev)
    pars_d = torch.tensor(pars.flatten(order="F"), dtype=real, device=dev)
    rng_d = torch.tensor(rng0.view(np.int64), dtype=torch.int64, device=dev)
    dt_d = torch.empty(n, dtype=real, device=dev)
    xf_d = torch.empty(n * nv, dtype=real, device=dev)
    tf_d = torch.empty(n, dtype=real, device=dev)
    F_d = torch.empty(n * nf, dtype=real, device=dev)
    st_d = torch.empty(n, dtype=torch.int32, device=dev)
    rng_init_d = rng_d.clone()
    ts_d = None if ts_pm is None else torch.tensor(ts_pm, dtype=real, device=dev)
    stream = torch.cuda.Stream(device=dev) if own_stream else None
    stream_h = C.c_void_p(stream.cuda_stream) if stream is not None else None

    def ptr(t):
        return C.c_void_p(t.data_ptr()) if t is not None else None

    for call in range(2):
        dt_d.fill_(sp.dt)  # dt is read and updated in place, as in the regular path
        rng_d.copy_(rng_init_d)
        F_d.fill_(float("nan"))
        torch.cuda.synchronize()
        launches = N.lib.clode_launch_count()
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = N.lib.clode_sim_features_noalloc(sim._handle, n, ptr(x0_d), ptr(pars_d), ptr(ts_d),
                                              C.cast(C.c_void_p(rng_d.data_ptr()), C.POINTER(C.c_ulonglong)),
                                              ptr(dt_d), ptr(xf_d), ptr(tf_d), ptr(F_d),
                                              C.cast(C.c_void_p(st_d.data_ptr()), C.POINTER(C.c_int)), stream_h)
        assert rc == 0, N.lib.clode_last_error()
        assert N.lib.clode_launch_count() == launches + 1
        if stream is not None:
            stream.synchronize()
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        if call == 1:  # the first call looked the scratch array up; nothing may allocate after it
            assert free_after == free_before, (free_before, free_after)
        assert torch.cuda.current_device() == 0
        F = F_d.double().cpu().numpy()
        np.testing.assert_array_equal(F, F_ref, err_msg=f"call {call}")
        np.testing.assert_array_equal(xf_d.double().cpu().numpy(), xf_ref, err_msg=f"call {call}")
        np.testing.assert_array_equal(tf_d.double().cpu().numpy(), tf_ref, err_msg=f"call {call}")
        assert (st_d.cpu().numpy() & 2 == 0).all()  # no non-finite member

    # an ensemble too large for the fixed scratch is refused, nothing launched
    launches = N.lib.clode_launch_count()
    rc = N.lib.clode_sim_features_noalloc(sim._handle, 1 << 29, ptr(x0_d), ptr(pars_d), None,
                                          C.cast(C.c_void_p(rng_d.data_ptr()), C.POINTER(C.c_ulonglong)),
                                          ptr(dt_d), ptr(xf_d), ptr(tf_d), ptr(F_d), None, None)
    assert rc == 1
    assert b"at most" in N.lib.clode_last_error()
    assert N.lib.clode_launch_count() == launches

    # a model with parameters needs the parameter buffer
    rc = N.lib.clode_sim_features_noalloc(sim._handle, n, ptr(x0_d), None, None,
                                          C.cast(C.c_void_p(rng_d.data_ptr()), C.POINTER(C.c_ulonglong)),
                                          ptr(dt_d), ptr(xf_d), ptr(tf_d), ptr(F_d), None, None)
    assert rc == 1
    assert b"pars" in N.lib.clode_last_error()
    assert N.lib.clode_launch_count() == launches
