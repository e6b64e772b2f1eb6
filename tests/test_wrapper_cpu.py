"""The drop-in module's Python surface, checked without a GPU against the
reference's stub (clode/cpp/clode_cpp_wrapper.pyi): names, enum values,
parameter defaults and representations, and the no-device behaviour."""
import pytest

from clode_gb300 import clode_cpp_wrapper as W

PYI_NAMES = ['CLDeviceType', 'CLVendor', 'DEVICE_TYPE_ACCELERATOR', 'DEVICE_TYPE_ALL', 'DEVICE_TYPE_CPU',
             'DEVICE_TYPE_CUSTOM', 'DEVICE_TYPE_DEFAULT', 'DEVICE_TYPE_GPU', 'DeviceInfo', 'FeatureSimulatorBase',
             'LogLevel', 'LoggerSingleton', 'ObserverParams', 'OpenCLResource', 'PlatformInfo', 'ProblemInfo',
             'SimulatorBase', 'SolverParams', 'TrajectorySimulatorBase', 'VENDOR_AMD', 'VENDOR_ANY',
             'VENDOR_INTEL', 'VENDOR_NVIDIA', 'critical', 'debug', 'err', 'get_logger', 'info', 'off',
             'query_opencl', 'trace', 'warn']


def test_module_exports_the_reference_names():
    for n in PYI_NAMES:
        assert hasattr(W, n), n
    assert callable(W._print_opencl)
    assert sorted(W.__all__) == sorted(PYI_NAMES)


def test_enum_values():
    assert int(W.DEVICE_TYPE_ALL) == -1 and int(W.DEVICE_TYPE_CPU) == 2 and int(W.DEVICE_TYPE_GPU) == 4
    assert int(W.DEVICE_TYPE_ACCELERATOR) == 8 and int(W.DEVICE_TYPE_DEFAULT) == 1 and int(W.DEVICE_TYPE_CUSTOM) == 16
    assert [int(v) for v in (W.VENDOR_ANY, W.VENDOR_NVIDIA, W.VENDOR_AMD, W.VENDOR_INTEL)] == [0, 1, 2, 3]
    assert [int(v) for v in (W.trace, W.debug, W.info, W.warn, W.err, W.critical, W.off)] == list(range(7))
    assert W.LogLevel.warn.name == "warn" and W.LogLevel(3) is W.LogLevel.warn
    assert set(W.CLDeviceType.__members__) == {"DEVICE_TYPE_ALL", "DEVICE_TYPE_CPU", "DEVICE_TYPE_GPU",
                                               "DEVICE_TYPE_ACCELERATOR", "DEVICE_TYPE_DEFAULT",
                                               "DEVICE_TYPE_CUSTOM"}


def test_parameter_defaults_and_repr():
    sp = W.SolverParams()
    assert (sp.dt, sp.dtmax, sp.abstol, sp.reltol, sp.max_steps, sp.max_store, sp.nout) == \
           (0.1, 0.5, 1e-6, 1e-3, 1000000, 1000000, 1)
    assert repr(sp).startswith("<solver_params(dt=0.100000, dtmax=0.500000")
    op = W.ObserverParams()
    assert (op.e_var_ix, op.f_var_ix, op.max_event_count, op.max_event_timestamps) == (0, 0, 100, 0)
    assert (op.min_amp, op.min_imi, op.nhood_radius, op.x_up_threshold, op.x_down_threshold) == \
           (0.0, 0.0, 0.05, 0.2, 0.2)
    assert "nhood_radius=0.050000" in repr(op)
    pi = W.ProblemInfo("m.cl", ["x", "y"], ["mu"], ["a"])
    assert (pi.num_var, pi.num_par, pi.num_aux, pi.num_noise) == (2, 1, 1, 1)
    assert repr(pi) == "<problem_info(src_file=m.cl, vars=[x, y, ], pars=[mu, ], aux=[a, ], num_noise=1)>"
    pi.vars = ["u"]
    assert pi.num_var == 1 and pi.vars == ["u"]
    empty = W.ProblemInfo()
    assert (empty.num_var, empty.num_par, empty.src_file) == (0, 0, "")


def test_cpu_device_requests_raise():
    with pytest.raises(RuntimeError):
        W.OpenCLResource(W.DEVICE_TYPE_CPU)
    with pytest.raises(RuntimeError):
        W.OpenCLResource(W.DEVICE_TYPE_GPU, W.VENDOR_AMD)


def test_no_gpu_means_no_device_here(gpu_available):
    if gpu_available:
        pytest.skip("a GPU is present")
    assert W.query_opencl() == []
    with pytest.raises(RuntimeError):
        W.OpenCLResource()
