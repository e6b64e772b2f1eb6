"""C ABI checks that need no GPU: the library loads, exports every entry
point include/clode_gb300.h declares, reports errors with the documented
codes, and cross-compiles ensemble programs for sm_103a with NVRTC."""
import ctypes as C
import os
import re

import pytest

from clode_gb300 import _native as N, rhs_path

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "clode_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?(?:unsigned\s+long\s+long|int|const char)\s*\*?\s*(clode_\w+)\s*\(",
                       text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_abi():
    names = declared_functions()
    assert len(names) >= 45
    for must in ("clode_sim_create", "clode_sim_features", "clode_sim_trajectory", "clode_sim_transient",
                 "clode_sim_get", "clode_last_error", "clode_device_query"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(N.library_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes binding covers the whole header
    assert set(declared_functions()) <= set(N.SIGNATURES)


def test_version_and_device_count_without_gpu():
    assert N.lib.clode_version() == 100
    n = C.c_int(-1)
    assert N.lib.clode_device_count(C.byref(n)) == 0
    assert n.value >= 0


def _problem(name="van_der_pol.cl", nv=2, np_=1, na=0, nw=0):
    src = open(rhs_path(name)).read().encode()
    keep = [src]
    return N.CProblem(src, name.encode(), nv, np_, na, nw, b"x\ny", b"mu", b""), keep


def test_create_rejects_unknown_stepper_and_observer():
    cp, keep = _problem()
    h = C.c_void_p()
    rc = N.lib.clode_sim_create(N.SIM_BASE, C.byref(cp), b"rk5", None, None, 0, 0, C.byref(h))
    assert rc == 1 and b"stepper" in N.lib.clode_last_error()
    op = N.CObserverParams(0, 0, 100, 0, 0, 0, 0.05, 0.2, 0.2, 0, 0, 0)
    rc = N.lib.clode_sim_create(N.SIM_FEATURES, C.byref(cp), b"rk4", b"nhood3", C.byref(op), 0, 0, C.byref(h))
    assert rc == 1 and b"observer" in N.lib.clode_last_error()


def test_runs_need_problem_data_and_report_state_errors():
    cp, keep = _problem()
    h = C.c_void_p()
    N.check(N.lib.clode_sim_create(N.SIM_BASE, C.byref(cp), b"rk4", None, None, 0, 0, C.byref(h)))
    try:
        assert N.lib.clode_sim_transient(h) == 7  # CLODE_ERR_STATE
        assert b"problem data" in N.lib.clode_last_error()
        assert N.lib.clode_sim_features(h, -1) == 7
        # setters that need nothing on the device
        sp = N.CSolverParams(0.05, 1.0, 1e-7, 1e-5, 1000, 10, 2)
        N.check(N.lib.clode_sim_set_solver_params(h, C.byref(sp)))
        back = N.CSolverParams()
        N.check(N.lib.clode_sim_get_solver_params(h, C.byref(back)))
        assert (back.dt, back.max_store, back.nout) == (0.05, 10, 2)
        # unknown option and an out-of-range one
        assert N.lib.clode_sim_set_option(h, b"no_such_option", 1.0) == 1
        assert N.lib.clode_sim_set_option(h, b"block_size", 7.0) == 1
    finally:
        N.lib.clode_sim_destroy(h)


def test_strings_available_steppers_and_observers():
    cp, keep = _problem("lorenz.cl", 3, 3, 1)
    op = N.CObserverParams(2, 2, 100, 2, 0, 0, 0.05, 0.3, 0.2, 0, 0, 0)
    h = C.c_void_p()
    N.check(N.lib.clode_sim_create(N.SIM_FEATURES, C.byref(cp), b"dopri5", b"thresh2", C.byref(op), 1, 0, C.byref(h)))

    def get(which):
        n = C.c_size_t()
        N.check(N.lib.clode_sim_get_string(h, which, None, 0, C.byref(n)))
        b = C.create_string_buffer(n.value + 1)
        N.check(N.lib.clode_sim_get_string(h, which, b, n.value + 1, C.byref(n)))
        return b.value.decode()

    try:
        # std::map order of clode/cpp/steppers.cl:26-43 and observers.cl:122-143
        assert get(N.STRING_AVAILABLE_STEPPERS).split("\n") == ["bs23", "dopri5", "euler", "heun", "rk4", "seuler"]
        assert get(N.STRING_AVAILABLE_OBSERVERS).split("\n") == ["basic", "basicall", "localmax", "nhood1",
                                                                  "nhood2", "thresh2"]
        names = get(N.STRING_FEATURE_NAMES).split("\n")
        # thresh2: 18 period stats + 5 per var + 3 per aux + 2 per stored event + 5 diagnostics
        assert len(names) == 18 + 15 + 3 + 4 + 5
        assert names[0] == "max period" and names[-1] == "mean dt"
        assert "up event time 1" in names and "down event time 0" in names
        assert get(N.STRING_OBSERVER_NAME) == "thresh2"
    finally:
        N.lib.clode_sim_destroy(h)


@pytest.mark.parametrize("stepper,observer,single", [
    ("euler", "basic", True), ("heun", "basicall", False), ("rk4", "localmax", True), ("bs23", "nhood1", False),
    ("dopri5", "nhood2", True), ("seuler", "thresh2", True), ("dopri5", "thresh2", False),
])
def test_nvrtc_builds_for_sm103a_without_spills(stepper, observer, single):
    cp, keep = _problem("lorenz.cl", 3, 3, 1, 1 if stepper == "seuler" else 0)
    op = N.CObserverParams(2, 0, 100, 1, 0, 0, 0.05, 0.3, 0.2, 0, 0, 0)
    h = C.c_void_p()
    N.check(N.lib.clode_sim_create(N.SIM_FEATURES, C.byref(cp), stepper.encode(), observer.encode(), C.byref(op),
                                   int(single), 0, C.byref(h)))
    try:
        N.check(N.lib.clode_sim_build(h))
        n = C.c_size_t()
        N.lib.clode_sim_get_string(h, N.STRING_BUILD_LOG, None, 0, C.byref(n))
        b = C.create_string_buffer(n.value + 1)
        N.lib.clode_sim_get_string(h, N.STRING_BUILD_LOG, b, n.value + 1, C.byref(n))
        log = b.value.decode()
        if log:  # empty when the program came from the on-disk cache of an earlier build without a log
            assert "sm_103a" in log
            for k in ("clode_features", "clode_init_observer", "clode_transient", "clode_trajectory"):
                assert f"entry function '{k}'" in log
            assert "bytes spill stores" in log
            # per kernel: its name, stack frame and spill stores.  The replay
            # kernels run on the recording launch's grid, so their register
            # cap is set by its residency, not by their own needs: they may
            # spill, within a bound; every other kernel spills nothing.
            per_kernel = re.findall(r"entry function '(\w+)'.*?(\d+) bytes stack frame, (\d+) bytes spill stores",
                                    log, flags=re.S)
            assert per_kernel
            for name, frame, spill in per_kernel:
                limit = 128 if name.startswith("clode_features_replay") else 0
                assert int(spill) <= limit and int(frame) <= limit, (name, frame, spill)
    finally:
        N.lib.clode_sim_destroy(h)


def _build_log(h):
    n = C.c_size_t()
    N.lib.clode_sim_get_string(h, N.STRING_BUILD_LOG, None, 0, C.byref(n))
    b = C.create_string_buffer(n.value + 1)
    N.lib.clode_sim_get_string(h, N.STRING_BUILD_LOG, b, n.value + 1, C.byref(n))
    return b.value.decode()


@pytest.mark.parametrize("paired", [1, 0])
@pytest.mark.parametrize("model,observer", [("lactotroph.cl", "nhood2"), ("lorenz.cl", "thresh2"),
                                            ("lorenz.cl", "nhood2")])
def test_fast_builds_compile_for_sm103a(model, observer, paired):
    """The benchmarked kind of build (contraction on, approximate division,
    denormals flushed): Dormand-Prince stage sums paired two variables per
    instruction (four variables: two pairs; three: a pair and a single) or
    scalar, and one division per step in the observer hooks.  ptxas runs
    here, so the paired PTX and the shared divisions are checked without a
    GPU; the spill rule is that of the exact builds above."""
    if model == "lactotroph.cl":
        cp, keep = _problem(model, 4, 3, 1, 0)
    else:
        cp, keep = _problem(model, 3, 3, 1, 0)
    op = N.CObserverParams(2, 0, 100, 1, 0, 0, 0.05, 0.3, 0.2, 0, 0, 0)
    h = C.c_void_p()
    N.check(N.lib.clode_sim_create(N.SIM_FEATURES, C.byref(cp), b"dopri5", observer.encode(), C.byref(op), 1, 0,
                                   C.byref(h)))
    try:
        for k, v in (("fmad", 1), ("prec_div", 0), ("ftz", 1), ("schedule", 1), ("paired", paired)):
            N.check(N.lib.clode_sim_set_option(h, k.encode(), C.c_double(v)))
        N.check(N.lib.clode_sim_build(h))
        log = _build_log(h)
        if log:  # empty when the program came from the on-disk cache of an earlier build without a log
            assert "sm_103a" in log
            per_kernel = re.findall(r"entry function '(\w+)'.*?(\d+) bytes stack frame, (\d+) bytes spill stores",
                                    log, flags=re.S)
            assert any(name == "clode_init_observer_record" for name, _, _ in per_kernel)
            for name, frame, spill in per_kernel:
                limit = 128 if name.startswith("clode_features_replay") else 0
                assert int(spill) <= limit and int(frame) <= limit, (name, frame, spill)
        v = C.c_double(-1)
        N.check(N.lib.clode_sim_get_option(h, b"paired", C.byref(v)))
        assert v.value == paired
    finally:
        N.lib.clode_sim_destroy(h)


def test_paired_option_leaves_the_exact_build_machine_code_unchanged(tmp_path):
    """With contraction off (the build that reproduces clODE bit for bit) the
    stage sums stay scalar: the compiled program is byte for byte the same
    with ``paired`` on and off, as is an FP64 build with contraction on.
    An FP32 build with contraction on differs (the paired stage sums are in
    it).  Compiled programs are compared as the on-disk
    cache stores them (a fresh cache directory per build)."""
    import hashlib

    def cubin(options, sub, single=1):
        d = tmp_path / sub
        d.mkdir()
        N.check(N.lib.clode_set_cache_dir(str(d).encode()))
        cp, keep = _problem("lactotroph.cl", 4, 3, 1, 0)
        op = N.CObserverParams(3, 0, 100, 1, 0, 0, 0.05, 0.3, 0.2, 0, 0, 0)
        h = C.c_void_p()
        N.check(N.lib.clode_sim_create(N.SIM_FEATURES, C.byref(cp), b"dopri5", b"nhood2", C.byref(op), single, 0,
                                       C.byref(h)))
        try:
            for k, v in options.items():
                N.check(N.lib.clode_sim_set_option(h, k.encode(), C.c_double(v)))
            N.check(N.lib.clode_sim_build(h))
        finally:
            N.lib.clode_sim_destroy(h)
        files = list(d.glob("*.cubin"))
        assert len(files) == 1
        return hashlib.sha256(files[0].read_bytes()).hexdigest()

    try:
        assert cubin({"paired": 1}, "exact1") == cubin({"paired": 0}, "exact0")
        fast = {"fmad": 1, "prec_div": 0, "ftz": 1}
        assert cubin(dict(fast, paired=1), "fast1") != cubin(dict(fast, paired=0), "fast0")
        # FP64 has no paired operations: the option changes nothing there either
        assert cubin(dict(fmad=1, paired=1), "fp64_1", single=0) == cubin(dict(fmad=1, paired=0), "fp64_0", single=0)
    finally:
        N.check(N.lib.clode_set_cache_dir(None))


def test_broken_model_source_reports_compile_error():
    src = b"void getRHS(const realtype t, const realtype x_[], const realtype p_[], realtype dx_[], " \
          b"realtype aux_[], const realtype w_[]) { dx_[0] = undefined_symbol * x_[0]; }"
    cp = N.CProblem(src, b"broken.cl", 1, 0, 0, 0, b"x", b"", b"")
    h = C.c_void_p()
    N.check(N.lib.clode_sim_create(N.SIM_BASE, C.byref(cp), b"rk4", None, None, 1, 0, C.byref(h)))
    try:
        rc = N.lib.clode_sim_build(h)
        assert rc == 3  # CLODE_ERR_COMPILE
        assert b"undefined_symbol" in N.lib.clode_last_error()
    finally:
        N.lib.clode_sim_destroy(h)


def test_log_levels_and_sink(capfd):
    from clode_gb300 import clode_cpp_wrapper as W

    lg = W.get_logger()
    lg.set_log_level(W.LogLevel.trace)
    assert lg.get_log_level() == W.LogLevel.trace
    W._log(W.LogLevel.info, "hello from the engine log")
    out = capfd.readouterr().out
    assert "hello from the engine log" in out and "[info]" in out
    lg.set_log_level(W.LogLevel.off)
    W._log(W.LogLevel.critical, "silent")
    out = capfd.readouterr()
    assert out.out == "" and out.err == ""
    lg.set_log_pattern("%l: %v")
    lg.set_log_level(W.LogLevel.warn)
    W._log(W.LogLevel.warn, "patterned")
    assert capfd.readouterr().out.strip() == "warning: patterned"
    lg.set_log_pattern("[%Y-%m-%d %H:%M:%S.%e] [%n] [%l] %v")


def test_storage_and_order_entry_points_validate_on_the_host():
    # the additions of the one-pass store, stored subsets, member orders and
    # member-major fetches check their arguments before touching a device
    cp, keep = _problem("lactotroph.cl", 4, 3, 1, 0)
    op = N.CObserverParams(3, 0, 100, 0, 0, 0, 0.05, 0.2, 0.2, 0, 0, 0)
    h = C.c_void_p()
    N.check(N.lib.clode_sim_create(N.SIM_FEATURES, C.byref(cp), b"dopri5", b"nhood2", C.byref(op), 1, 0,
                                   C.byref(h)))
    try:
        ix = (C.c_int * 2)(3, 0)
        bad = (C.c_int * 1)(4)
        N.check(N.lib.clode_sim_set_store_variables(h, ix, 2, None, 0))
        assert N.lib.clode_sim_set_store_variables(h, bad, 1, None, -1) == 1
        assert b"outside" in N.lib.clode_last_error()
        assert N.lib.clode_sim_set_store_variables(h, None, 1, None, -1) == 1
        N.check(N.lib.clode_sim_set_store_variables(h, None, -1, None, -1))
        # nothing stored yet: no rows, no events, fetches refused
        n = C.c_size_t(7)
        N.check(N.lib.clode_sim_get_n_events(h, None, 0, C.byref(n)))
        assert n.value == 0
        assert N.lib.clode_sim_get_trajectory_by_member(h, 0, 0, 0, None, None, None, None, None) == 1
        assert N.lib.clode_sim_get_events_by_member(h, 0, 0, 0, None, None, None, None, None) == 1
        assert N.lib.clode_sim_features_store(h, 1, 4) == 7  # no problem data yet
        for key in (b"order_by_span", b"order_by_work"):
            v = C.c_double(-1)
            N.check(N.lib.clode_sim_get_option(h, key, C.byref(v)))
            assert v.value == 1.0
            N.check(N.lib.clode_sim_set_option(h, key, 0.0))
            N.check(N.lib.clode_sim_get_option(h, key, C.byref(v)))
            assert v.value == 0.0
    finally:
        N.lib.clode_sim_destroy(h)


@pytest.mark.parametrize("single", [True, False], ids=["fp32", "fp64"])
def test_xpp_style_model_with_float_literals_builds(single):
    # decimal literals with an `f` suffix (what clODE's XPP translator emits)
    # compile in both precisions, as in OpenCL C
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models", "xpp_style.cl")
    src = open(path, "rb").read()
    cp = N.CProblem(src, b"xpp_style.cl", 2, 2, 1, 0, b"v\nr", b"a\nb", b"drive")
    op = N.CObserverParams(0, 0, 100, 0, 0, 0, 0.05, 0.2, 0.2, 0, 0, 0)
    h = C.c_void_p()
    N.check(N.lib.clode_sim_create(N.SIM_FEATURES, C.byref(cp), b"rk4", b"localmax", C.byref(op), int(single), 0,
                                   C.byref(h)))
    try:
        N.check(N.lib.clode_sim_build(h))
    finally:
        N.lib.clode_sim_destroy(h)
