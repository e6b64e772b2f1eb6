"""Drop-in replacement for clODE's native module ``clode.cpp.clode_cpp_wrapper``.

Same class, function, enum and argument names as the reference's pybind11
module (clode/cpp/CLODEpython.cpp:35-381, stub clode/cpp/clode_cpp_wrapper.pyi),
implemented over the C ABI of ``libclode_gb300.so`` (include/clode_gb300.h).
The reference's Python package (clode/solver.py, features.py, trajectory.py,
runtime.py) runs unchanged on top of it.

Behavioural notes, each mirroring the reference:
  * ``OpenCLResource`` selects a compute device.  Here the devices are CUDA
    GPUs on one platform ("NVIDIA CUDA"); asking for a CPU or a non-NVIDIA
    vendor finds no device and raises RuntimeError, as the reference does
    when OpenCL finds none (there is no CPU fallback).
  * Size mismatches in ``set_x0`` / ``set_pars`` / ``set_problem_data`` are
    logged at info level and leave the simulator unchanged
    (clode/cpp/CLODE.cpp:247-271, 309-349).
  * Getters of device arrays return float64 NumPy arrays (the reference
    returns Python lists; every use in the reference's Python package —
    ``np.array(...)``, slicing, ``reshape`` — accepts either).
  * Problems too large for the device raise ValueError (std::invalid_argument
    in the reference, clode/cpp/CLODE.cpp:179-182).
"""
from __future__ import annotations

import ctypes as C
import enum
import os
import sys
from typing import List, Optional

import numpy as np

from . import _native as N

__all__ = ["CLDeviceType", "CLVendor", "DEVICE_TYPE_ACCELERATOR", "DEVICE_TYPE_ALL", "DEVICE_TYPE_CPU",
           "DEVICE_TYPE_CUSTOM", "DEVICE_TYPE_DEFAULT", "DEVICE_TYPE_GPU", "DeviceInfo", "FeatureSimulatorBase",
           "LogLevel", "LoggerSingleton", "ObserverParams", "OpenCLResource", "PlatformInfo", "ProblemInfo",
           "SimulatorBase", "SolverParams", "TrajectorySimulatorBase", "VENDOR_AMD", "VENDOR_ANY", "VENDOR_INTEL",
           "VENDOR_NVIDIA", "critical", "debug", "err", "get_logger", "info", "off", "query_opencl", "trace", "warn"]


# ------------------------------------------------------------------ errors --
class ClodeValueError(N.ClodeError, ValueError):
    pass


def _check(rc: int) -> None:
    if rc == N.CLODE_OK:
        return
    msg = N.lib.clode_last_error().decode(errors="replace")
    if rc in (1, 6):  # invalid argument, out of memory
        raise ClodeValueError(rc, msg)
    raise N.ClodeError(rc, msg)


# ------------------------------------------------------------------- enums --
class LogLevel(enum.IntEnum):
    trace = 0
    debug = 1
    info = 2
    warn = 3
    err = 4
    critical = 5
    off = 6


trace, debug, info, warn, err, critical, off = (LogLevel.trace, LogLevel.debug, LogLevel.info, LogLevel.warn,
                                                 LogLevel.err, LogLevel.critical, LogLevel.off)


class CLVendor(enum.IntEnum):
    VENDOR_ANY = 0
    VENDOR_NVIDIA = 1
    VENDOR_AMD = 2
    VENDOR_INTEL = 3


VENDOR_ANY, VENDOR_NVIDIA, VENDOR_AMD, VENDOR_INTEL = (CLVendor.VENDOR_ANY, CLVendor.VENDOR_NVIDIA,
                                                       CLVendor.VENDOR_AMD, CLVendor.VENDOR_INTEL)


class CLDeviceType(enum.IntEnum):
    DEVICE_TYPE_ALL = -1
    DEVICE_TYPE_CPU = 2
    DEVICE_TYPE_GPU = 4
    DEVICE_TYPE_ACCELERATOR = 8
    DEVICE_TYPE_DEFAULT = 1
    DEVICE_TYPE_CUSTOM = 16


DEVICE_TYPE_ALL = CLDeviceType.DEVICE_TYPE_ALL
DEVICE_TYPE_CPU = CLDeviceType.DEVICE_TYPE_CPU
DEVICE_TYPE_GPU = CLDeviceType.DEVICE_TYPE_GPU
DEVICE_TYPE_ACCELERATOR = CLDeviceType.DEVICE_TYPE_ACCELERATOR
DEVICE_TYPE_DEFAULT = CLDeviceType.DEVICE_TYPE_DEFAULT
DEVICE_TYPE_CUSTOM = CLDeviceType.DEVICE_TYPE_CUSTOM


# ----------------------------------------------------------------- logging --
def _python_sink(level: int, message: bytes) -> None:
    # like the reference's PythonSink (clode/cpp/logging/PythonSink.hpp:21-38):
    # every message is printed through Python's own stdout
    sys.stdout.write(message.decode(errors="replace") + "\n")
    sys.stdout.flush()


_SINK = N.LOG_SINK(_python_sink)


class LoggerSingleton:
    """clODE's LoggerSingleton (clode/cpp/CLODEpython.cpp:53-86)."""

    _instance: Optional["LoggerSingleton"] = None

    def __init__(self):
        N.lib.clode_log_set_sink(_SINK)

    def set_log_level(self, level: LogLevel) -> None:
        _check(N.lib.clode_log_set_level(int(level)))

    def get_log_level(self) -> LogLevel:
        return LogLevel(N.lib.clode_log_get_level())

    def set_log_pattern(self, pattern: str) -> None:
        _check(N.lib.clode_log_set_pattern(pattern.encode()))


def get_logger() -> LoggerSingleton:
    """Get logger singleton instance"""
    if LoggerSingleton._instance is None:
        LoggerSingleton._instance = LoggerSingleton()
        # the reference's singleton starts at info (CLODEpython.cpp:60)
        LoggerSingleton._instance.set_log_level(LogLevel.info)
    return LoggerSingleton._instance


def _log(level: LogLevel, msg: str) -> None:
    get_logger()
    N.lib.clode_log_message(int(level), msg.encode())


# ----------------------------------------------------------------- devices --
class DeviceInfo:
    def __init__(self):
        self.name = ""
        self.vendor = ""
        self.version = ""
        self.device_type = int(CLDeviceType.DEVICE_TYPE_GPU)
        self.device_type_str = "GPU"
        self.compute_units = 0
        self.max_clock = 0
        self.max_work_group_size = 0
        self.device_memory_size = 0
        self.max_memory_alloc_size = 0
        self.extensions = ""
        self.double_support = True
        self.device_available = 1

    def __repr__(self) -> str:
        return (f"<device_info(name={self.name}, vendor={self.vendor}, version={self.version}, "
                f"device_type={self.device_type_str}, compute_units={self.compute_units}, "
                f"max_clock={self.max_clock}, max_work_group_size={self.max_work_group_size}, "
                f"device_memory_size={self.device_memory_size}, max_memory_alloc_size={self.max_memory_alloc_size}, "
                f"extensions={self.extensions}, double_support={int(self.double_support)}, "
                f"device_available={self.device_available})>")


class PlatformInfo:
    def __init__(self):
        self.name = ""
        self.vendor = ""
        self.version = ""
        self.device_info: List[DeviceInfo] = []
        self.device_count = 0

    def __repr__(self) -> str:
        return (f"<platform_info(name={self.name}, vendor={self.vendor}, version={self.version}, "
                f"device_count={self.device_count})>")


def _device_infos() -> List[DeviceInfo]:
    n = C.c_int(0)
    _check(N.lib.clode_device_count(C.byref(n)))
    out = []
    for k in range(n.value):
        ci = N.CDeviceInfo()
        _check(N.lib.clode_device_query(k, C.byref(ci)))
        d = DeviceInfo()
        d.name = ci.name.decode()
        d.vendor = ci.vendor.decode()
        d.version = ci.version.decode()
        d.compute_units = ci.compute_units
        d.max_clock = ci.max_clock_mhz
        d.max_work_group_size = ci.max_work_group_size
        d.device_memory_size = ci.device_memory_size
        d.max_memory_alloc_size = ci.max_memory_alloc_size
        d.extensions = f"sm_{ci.cc_major}{ci.cc_minor}"
        d.double_support = bool(ci.double_support)
        out.append(d)
    return out


def query_opencl() -> List[PlatformInfo]:
    """Query compute devices: one platform holding the CUDA GPUs (queryOpenCL, OpenCLResource.cpp:326)."""
    devs = _device_infos()
    if not devs:
        return []
    p = PlatformInfo()
    p.name = "NVIDIA CUDA"
    p.vendor = "NVIDIA Corporation"
    p.version = devs[0].version
    p.device_info = devs
    p.device_count = len(devs)
    return [p]


def _print_platforms(platforms: List[PlatformInfo]) -> None:
    _log(LogLevel.info, f"Number of platforms found: {len(platforms)}")
    for i, p in enumerate(platforms):
        _log(LogLevel.info, f"- Platform {i} ------------------------------")
        _log(LogLevel.info, f"Name:    {p.name} (OpenCL platform equivalent)")
        _log(LogLevel.info, f"Vendor:  {p.vendor}")
        _log(LogLevel.info, f"Version: {p.version}")
        for j, d in enumerate(p.device_info):
            _print_device(j, d)
    _log(LogLevel.info, "")


def _print_device(j: int, d: DeviceInfo) -> None:
    _log(LogLevel.info, f"- Device {j} ------------")
    _log(LogLevel.info, f"  Name:   {d.name}")
    _log(LogLevel.info, f"  Type:   {d.device_type_str}")
    _log(LogLevel.info, f"  Vendor: {d.vendor}")
    _log(LogLevel.info, f"  Version: {d.version}")
    _log(LogLevel.info, f"  Compute units (CUs): {d.compute_units}")
    _log(LogLevel.info, f"  Clock frequency:     {d.max_clock} MHz")
    _log(LogLevel.info, f"  Global memory size:  {d.device_memory_size // 1024 // 1024} MB")
    _log(LogLevel.info, f"  Max allocation size: {d.max_memory_alloc_size // 1024 // 1024} MB")
    _log(LogLevel.info, f"  Max work group/CU:   {d.max_work_group_size}")
    _log(LogLevel.info, f"  Double support:      {'true' if d.double_support else 'false'}")
    _log(LogLevel.info, f"  Device available:    {'true' if d.device_available else 'false'}")


def _print_opencl() -> None:
    """Print compute devices"""
    _log(LogLevel.info, "Querying OpenCL-equivalent (CUDA) platforms...")
    _print_platforms(query_opencl())


class OpenCLResource:
    """Device selection (OpenCLResource, clode/cpp/OpenCLResource.hpp:73-125).

    Accepted forms: (), (device_type), (vendor), (device_type, vendor),
    (platform_id, device_id), (platform_id, [device_ids]).  The first selected
    device runs every launch, as in the reference (OpenCLResource.hpp:110).
    """

    def __init__(self, *args):
        self.platform_id = 0
        self.device_ids: List[int] = [0]
        device_type = CLDeviceType.DEVICE_TYPE_DEFAULT
        vendor = CLVendor.VENDOR_ANY
        if len(args) == 1:
            a = args[0]
            if isinstance(a, CLVendor):
                vendor = a
            else:
                device_type = CLDeviceType(int(a))
        elif len(args) == 2:
            a, b = args
            if isinstance(b, (list, tuple)):
                self.platform_id, self.device_ids = int(a), [int(x) for x in b]
            elif isinstance(b, CLVendor):
                device_type, vendor = CLDeviceType(int(a)), b
            else:
                self.platform_id, self.device_ids = int(a), [int(b)]
        elif len(args) > 2:
            raise TypeError("OpenCLResource takes at most two arguments")
        devs = _device_infos()
        if device_type == CLDeviceType.DEVICE_TYPE_CPU or vendor in (CLVendor.VENDOR_AMD, CLVendor.VENDOR_INTEL):
            raise RuntimeError(f"no device of type {device_type.name} / vendor {vendor.name}: "
                               "this engine runs on NVIDIA CUDA GPUs only")
        if self.platform_id != 0:
            raise RuntimeError(f"platform {self.platform_id} does not exist (one platform: NVIDIA CUDA)")
        if not devs:
            raise RuntimeError("no CUDA device found")
        for d in self.device_ids:
            if d < 0 or d >= len(devs):
                raise RuntimeError(f"device {d} does not exist ({len(devs)} CUDA devices)")
        self._devices = devs

    @property
    def device(self) -> int:
        return self.device_ids[0]

    def get_double_support(self, device_id: int = 0) -> bool:
        """Get double support"""
        return bool(self._devices[self.device_ids[device_id]].double_support)

    def get_max_memory_alloc_size(self, device_id: int = 0) -> int:
        """Get max memory alloc size"""
        return int(self._devices[self.device_ids[device_id]].max_memory_alloc_size)

    def get_device_cl_version(self, device_id: int = 0) -> str:
        """Get device CL version"""
        return self._devices[self.device_ids[device_id]].version

    def print_devices(self) -> None:
        """Print device info to log"""
        _log(LogLevel.info, "Selected platform and device (OpenCL equivalents): ")
        _log(LogLevel.info, "Platform  --------------------")
        _log(LogLevel.info, "Name:    NVIDIA CUDA")
        for j, d in enumerate(self.device_ids):
            _print_device(j, self._devices[d])


# --------------------------------------------------------- parameter types --
class ProblemInfo:
    """clODE ProblemInfo (clode/cpp/CLODE.hpp:22-91)."""

    def __init__(self, src_file: str = "", vars: List[str] = None, pars: List[str] = None,
                 aux: List[str] = None, num_noise: int = 1):
        if vars is None and pars is None and src_file == "":
            num_noise = 0
        self.src_file = src_file
        self._vars = list(vars or [])
        self._pars = list(pars or [])
        self._aux = list(aux or [])
        self.num_var = len(self._vars)
        self.num_par = len(self._pars)
        self.num_aux = len(self._aux)
        self.num_noise = num_noise

    @property
    def vars(self) -> List[str]:
        return list(self._vars)

    @vars.setter
    def vars(self, v: List[str]) -> None:
        self._vars = list(v)
        self.num_var = len(self._vars)

    @property
    def pars(self) -> List[str]:
        return list(self._pars)

    @pars.setter
    def pars(self, v: List[str]) -> None:
        self._pars = list(v)
        self.num_par = len(self._pars)

    @property
    def aux(self) -> List[str]:
        return list(self._aux)

    @aux.setter
    def aux(self, v: List[str]) -> None:
        self._aux = list(v)
        self.num_aux = len(self._aux)

    def __repr__(self) -> str:
        def vec(v):
            return "[" + "".join(s + ", " for s in v) + "]"
        return (f"<problem_info(src_file={self.src_file}, vars={vec(self._vars)}, pars={vec(self._pars)}, "
                f"aux={vec(self._aux)}, num_noise={self.num_noise})>")


class SolverParams:
    """SolverParams<double> (clode/cpp/clODE_struct_defs.cl:11-20; defaults CLODEpython.cpp:219-225)."""

    def __init__(self, dt: float = 0.1, dtmax: float = 0.5, abstol: float = 1e-6, reltol: float = 1e-3,
                 max_steps: int = 1000000, max_store: int = 1000000, nout: int = 1):
        self.dt, self.dtmax, self.abstol, self.reltol = float(dt), float(dtmax), float(abstol), float(reltol)
        self.max_steps, self.max_store, self.nout = int(max_steps), int(max_store), int(nout)

    def _c(self) -> N.CSolverParams:
        return N.CSolverParams(self.dt, self.dtmax, self.abstol, self.reltol, self.max_steps, self.max_store,
                               self.nout)

    @classmethod
    def _from_c(cls, c: N.CSolverParams) -> "SolverParams":
        return cls(c.dt, c.dtmax, c.abstol, c.reltol, c.max_steps, c.max_store, c.nout)

    def __repr__(self) -> str:
        return (f"<solver_params(dt={self.dt:f}, dtmax={self.dtmax:f}, abstol={self.abstol:f}, "
                f"reltol={self.reltol:f}, max_steps={self.max_steps}, max_store={self.max_store}, nout={self.nout})>")


class ObserverParams:
    """ObserverParams<double> (clode/cpp/observers.cl:25-46; defaults CLODEpython.cpp:300-311)."""

    def __init__(self, e_var_ix: int = 0, f_var_ix: int = 0, max_event_count: int = 100,
                 max_event_timestamps: int = 0, min_amp: float = 0.0, min_imi: float = 0.0,
                 nhood_radius: float = 0.05, x_up_threshold: float = 0.2, x_down_threshold: float = 0.2,
                 dx_up_threshold: float = 0.0, dx_down_threshold: float = 0.0, eps_dx: float = 0.0):
        self.e_var_ix, self.f_var_ix = int(e_var_ix), int(f_var_ix)
        self.max_event_count, self.max_event_timestamps = int(max_event_count), int(max_event_timestamps)
        self.min_amp, self.min_imi, self.nhood_radius = float(min_amp), float(min_imi), float(nhood_radius)
        self.x_up_threshold, self.x_down_threshold = float(x_up_threshold), float(x_down_threshold)
        self.dx_up_threshold, self.dx_down_threshold = float(dx_up_threshold), float(dx_down_threshold)
        self.eps_dx = float(eps_dx)

    def _c(self) -> N.CObserverParams:
        return N.CObserverParams(self.e_var_ix, self.f_var_ix, self.max_event_count, self.max_event_timestamps,
                                 self.min_amp, self.min_imi, self.nhood_radius, self.x_up_threshold,
                                 self.x_down_threshold, self.dx_up_threshold, self.dx_down_threshold, self.eps_dx)

    @classmethod
    def _from_c(cls, c: N.CObserverParams) -> "ObserverParams":
        return cls(c.e_var_ix, c.f_var_ix, c.max_event_count, c.max_event_timestamps, c.min_x_amp, c.min_imi,
                   c.nhood_radius, c.x_up_thresh, c.x_down_thresh, c.dx_up_thresh, c.dx_down_thresh, c.eps_dx)

    def __repr__(self) -> str:
        return (f"<observer_params(e_var_ix={self.e_var_ix}, f_var_ix={self.f_var_ix}, "
                f"max_event_count={self.max_event_count}, max_event_timestamps={self.max_event_timestamps}, "
                f"min_amp={self.min_amp:f}, min_imi={self.min_imi:f}, nhood_radius={self.nhood_radius:f}, "
                f"x_up_threshold={self.x_up_threshold:f}, x_down_threshold={self.x_down_threshold:f}, "
                f"dx_up_threshold={self.dx_up_threshold:f}, dx_down_threshold={self.dx_down_threshold:f}, "
                f"eps_dx={self.eps_dx:f})>")


def _c_problem(pi: ProblemInfo):
    with open(pi.src_file, "r") as f:  # CLODE::setProblemInfo reads the file (CLODE.cpp:47)
        src = f.read()
    keep = [src.encode(), os.path.basename(pi.src_file).encode(), "\n".join(pi.vars).encode(),
            "\n".join(pi.pars).encode(), "\n".join(pi.aux).encode()]
    cp = N.CProblem(keep[0], keep[1], pi.num_var, pi.num_par, pi.num_aux, pi.num_noise, keep[2], keep[3], keep[4])
    return cp, keep


# -------------------------------------------------------------- simulators --
class SimulatorBase:
    """clODE's CLODE class (clode/cpp/CLODE.hpp:93-189) over libclode_gb300."""

    _kind = N.SIM_BASE

    def __init__(self, problem_info: ProblemInfo, stepper: str, cl_single_precision: bool,
                 opencl_resource: OpenCLResource, clode_root: str = ""):
        self._handle = C.c_void_p()
        self._pi = problem_info
        get_logger()
        self._init_handle(problem_info, stepper, cl_single_precision, opencl_resource)

    def _init_handle(self, pi, stepper, single, resource, observer=None, op=None):
        cp, keep = _c_problem(pi)
        self._resource = resource
        cop = op._c() if op is not None else None
        _check(N.lib.clode_sim_create(self._kind, C.byref(cp), str(stepper).encode(),
                                      observer.encode() if observer else None,
                                      C.byref(cop) if cop is not None else None, int(bool(single)),
                                      int(resource.device), C.byref(self._handle)))

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            N.lib.clode_sim_destroy(h)
            self._handle = C.c_void_p()

    # setters requiring a rebuild (CLODE.hpp:147-154)
    def set_problem_info(self, problem_info: ProblemInfo) -> None:
        cp, keep = _c_problem(problem_info)
        _check(N.lib.clode_sim_set_problem_info(self._handle, C.byref(cp)))
        self._pi = problem_info

    def set_stepper(self, stepper: str) -> None:
        _check(N.lib.clode_sim_set_stepper(self._handle, str(stepper).encode()))

    def set_precision(self, single_precision: bool) -> None:
        _check(N.lib.clode_sim_set_precision(self._handle, int(bool(single_precision))))

    def set_opencl(self, *args) -> None:
        res = args[0] if len(args) == 1 and isinstance(args[0], OpenCLResource) else OpenCLResource(*args)
        self._resource = res
        _check(N.lib.clode_sim_set_device(self._handle, int(res.device)))

    def build_cl(self) -> None:
        _check(N.lib.clode_sim_build(self._handle))

    # problem data (CLODE.cpp:245-402); size mismatches are logged and ignored
    def _size_checked(self, rc: int) -> None:
        if rc == 1:
            _log(LogLevel.info, N.lib.clode_last_error().decode(errors="replace"))
            _log(LogLevel.info, "...Problem data was not updated!")
            return
        _check(rc)

    def set_problem_data(self, x0, pars) -> None:
        a, b = N.as_f64(x0), N.as_f64(pars)
        self._size_checked(N.lib.clode_sim_set_problem_data(self._handle, N.dptr(a), a.size, N.dptr(b), b.size))

    def set_x0(self, x0) -> None:
        a = N.as_f64(x0)
        self._size_checked(N.lib.clode_sim_set_x0(self._handle, N.dptr(a), a.size))

    def set_pars(self, pars) -> None:
        a = N.as_f64(pars)
        self._size_checked(N.lib.clode_sim_set_pars(self._handle, N.dptr(a), a.size))

    def set_tspan(self, tspan) -> None:
        a = N.as_f64(tspan)
        if a.size < 2:
            raise ValueError("tspan needs two values [t0, t1]")
        _check(N.lib.clode_sim_set_tspan(self._handle, N.dptr(a)))

    def set_solver_params(self, sp: SolverParams) -> None:
        c = sp._c()
        _check(N.lib.clode_sim_set_solver_params(self._handle, C.byref(c)))

    def seed_rng(self, seed: Optional[int] = None) -> None:
        """Seed RNG"""
        if seed is None:
            _check(N.lib.clode_sim_seed_rng(self._handle, 0, 0))
        else:
            s = ((int(seed) + 2**31) % 2**32) - 2**31  # the reference takes a C int
            _check(N.lib.clode_sim_seed_rng(self._handle, 1, s))

    # runs
    def transient(self) -> None:
        _check(N.lib.clode_sim_transient(self._handle))

    def shift_tspan(self) -> None:
        _check(N.lib.clode_sim_shift_tspan(self._handle))

    def shift_x0(self) -> None:
        _check(N.lib.clode_sim_shift_x0(self._handle))

    # getters
    def _get(self, which: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        """The array `which` as float64; into `out` (a C-contiguous float64
        array of at least that many elements, e.g. in page-locked memory that
        a caller reuses between calls) when given, returning its leading part."""
        n = C.c_size_t(0)
        _check(N.lib.clode_sim_get(self._handle, which, None, 0, C.byref(n)))
        if out is None:
            out = np.empty(n.value, dtype=np.float64)
        else:
            if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or not out.flags["WRITEABLE"]:
                raise ValueError("out must be a writeable C-contiguous float64 array")
            if out.size < n.value:
                raise ValueError(f"out holds {out.size} values, {n.value} needed")
            out = out.reshape(-1)[:n.value]
        if n.value:
            _check(N.lib.clode_sim_get(self._handle, which, N.dptr(out), out.size, C.byref(n)))
        return out

    def _get_string(self, which: int) -> str:
        n = C.c_size_t(0)
        _check(N.lib.clode_sim_get_string(self._handle, which, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        _check(N.lib.clode_sim_get_string(self._handle, which, buf, n.value + 1, C.byref(n)))
        return buf.value.decode(errors="replace")

    def get_problem_info(self) -> ProblemInfo:
        return self._pi

    def get_tspan(self) -> List[float]:
        return self._get(N.ARRAY_TSPAN).tolist()

    def get_solver_params(self) -> SolverParams:
        c = N.CSolverParams()
        _check(N.lib.clode_sim_get_solver_params(self._handle, C.byref(c)))
        return SolverParams._from_c(c)

    def get_pars(self) -> np.ndarray:
        return self._get(N.ARRAY_PARS)

    def get_x0(self) -> np.ndarray:
        return self._get(N.ARRAY_X0)

    def get_xf(self) -> np.ndarray:
        return self._get(N.ARRAY_XF)

    def get_dt(self) -> np.ndarray:
        return self._get(N.ARRAY_DT)

    def get_tf(self) -> np.ndarray:
        return self._get(N.ARRAY_TF)

    def get_available_steppers(self) -> List[str]:
        return self._get_string(N.STRING_AVAILABLE_STEPPERS).split("\n")

    def get_program_string(self) -> str:
        return self._get_string(N.STRING_PROGRAM)

    def print_status(self) -> None:
        for line in self._get_string(N.STRING_STATUS_REPORT).rstrip("\n").split("\n"):
            _log(LogLevel.info, line)

    # ---------------------------------------------------- additions --
    def set_tspan_per_member(self, tspan) -> None:
        """Per-member time spans, array shaped (nPts, 2) (no reference counterpart)."""
        a = N.as_f64(tspan)
        _check(N.lib.clode_sim_set_tspan_per_member(self._handle, N.dptr(a), a.size))

    def get_status(self) -> np.ndarray:
        """Per-member status bits of the last run (CLODE_MEMBER_* of include/clode_gb300.h)."""
        n = C.c_size_t(0)
        _check(N.lib.clode_sim_get_status(self._handle, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.int32)
        if n.value:
            _check(N.lib.clode_sim_get_status(self._handle, out.ctypes.data_as(C.POINTER(C.c_int)), out.size,
                                              C.byref(n)))
        return out

    def get_rng_state(self) -> np.ndarray:
        """Raw RNG state, 2*nPts uint64 words laid out [j*nPts + i] (no reference counterpart)."""
        n = C.c_size_t(0)
        _check(N.lib.clode_sim_get_rng_state(self._handle, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.uint64)
        if n.value:
            _check(N.lib.clode_sim_get_rng_state(self._handle, out.ctypes.data_as(C.POINTER(C.c_ulonglong)),
                                                 out.size, C.byref(n)))
        return out

    def set_rng_state(self, state) -> None:
        """Set the raw RNG state (2*nPts uint64 words, layout [j*nPts + i])."""
        a = np.ascontiguousarray(np.asarray(state, dtype=np.uint64).ravel())
        _check(N.lib.clode_sim_set_rng_state(self._handle, a.ctypes.data_as(C.POINTER(C.c_ulonglong)), a.size))

    def get_stats(self) -> dict:
        """Launch-wide counters of the last run: steps, rejected, rhs_evals, events."""
        buf = (C.c_ulonglong * N.STAT_COUNT)()
        _check(N.lib.clode_sim_get_stats(self._handle, buf))
        return {"steps": buf[N.STAT_STEPS], "rejected": buf[N.STAT_REJECTED], "rhs_evals": buf[N.STAT_RHS_EVALS],
                "events": buf[N.STAT_EVENTS]}

    def last_kernel_ms(self) -> float:
        v = C.c_double(0.0)
        _check(N.lib.clode_sim_last_kernel_ms(self._handle, C.byref(v)))
        return v.value

    def set_option(self, key: str, value: float) -> None:
        _check(N.lib.clode_sim_set_option(self._handle, key.encode(), float(value)))

    def get_option(self, key: str) -> float:
        v = C.c_double(0.0)
        _check(N.lib.clode_sim_get_option(self._handle, key.encode(), C.byref(v)))
        return v.value

    CHAIN_OPS = {"transient": 0, "features": 1, "trajectory": 2, "shift_x0": 3}

    def run_chain(self, ops, use_graph: bool = True) -> None:
        """Run ops such as ["transient", "shift_x0", "features"] back to back,
        captured as a CUDA graph and replayed (no reference counterpart)."""
        codes = (C.c_int * len(ops))(*[self.CHAIN_OPS[o] for o in ops])
        _check(N.lib.clode_sim_chain(self._handle, codes, len(ops), int(bool(use_graph))))

    def autotune(self, sample: int = 0) -> dict:
        """Pick register cap, block size, (adaptive steppers) the stepping
        variant, (FP32 Dormand-Prince builds with contraction) paired or scalar
        stage sums and (two-pass observers) the replayed or integrated feature
        pass (and the replay's row and launch layout) and fused or separate
        observer initialisation, by timing the
        persistent kernels on a strided sample of ``sample`` members (no
        reference counterpart)."""
        ms = C.c_double(0.0)
        _check(N.lib.clode_sim_autotune(self._handle, int(sample), C.byref(ms)))
        return {"ms": ms.value, "maxrregcount": int(self.get_option("maxrregcount")),
                "block_size": int(self.get_option("block_size")),
                "split_attempts": int(self.get_option("split_attempts")),
                "paired": int(self.get_option("paired")),
                "fuse_init": int(self.get_option("fuse_init")), "replay": int(self.get_option("replay")),
                "replay_split": int(self.get_option("replay_split")),
                "replay_fused": int(self.get_option("replay_fused"))}

    def kernel_registers(self, kernel: str) -> int:
        r, t = C.c_int(0), C.c_int(0)
        _check(N.lib.clode_sim_kernel_info(self._handle, kernel.encode(), C.byref(r), C.byref(t)))
        return r.value

    def get_build_log(self) -> str:
        return self._get_string(N.STRING_BUILD_LOG)

    def set_store_variables(self, var_ix: Optional[List[int]] = None, aux_ix: Optional[List[int]] = None) -> None:
        """Store only these variables (and auxiliary variables) in trajectory
        rows and event states, in the given order; None keeps all of them.
        Addition (clode/cpp/trajectory.cl:3 leaves it as a TODO); the getters
        then return ``len(var_ix)`` (``len(aux_ix)``) columns per row."""
        def arr(ix):
            if ix is None:
                return None, -1
            a = (C.c_int * max(1, len(ix)))(*[int(v) for v in ix])
            return a, len(ix)
        v, nv = arr(var_ix)
        w, nw = arr(aux_ix)
        _check(N.lib.clode_sim_set_store_variables(self._handle, v, nv, w, nw))


class _StoredRows:
    """Getters of stored trajectory rows, shared by TrajectorySimulatorBase
    (clode/cpp/CLODEtrajectory.hpp:37-48) and the features-with-storage runs
    of FeatureSimulatorBase."""

    def get_t(self) -> np.ndarray:
        return self._get(N.ARRAY_T)

    def get_x(self) -> np.ndarray:
        return self._get(N.ARRAY_X)

    def get_dx(self) -> np.ndarray:
        return self._get(N.ARRAY_DX)

    def get_aux(self) -> np.ndarray:
        return self._get(N.ARRAY_AUX)

    def get_n_stored(self) -> np.ndarray:
        n = C.c_size_t(0)
        _check(N.lib.clode_sim_get_n_stored(self._handle, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.int32)
        if n.value:
            _check(N.lib.clode_sim_get_n_stored(self._handle, out.ctypes.data_as(C.POINTER(C.c_int)), out.size,
                                                C.byref(n)))
        return out

    def get_trajectory_by_member(self, first: int = 0, count: Optional[int] = None, rows: Optional[int] = None,
                                 which=("t", "x", "dx", "aux")) -> dict:
        """The last trajectory regrouped by member on the device (addition).

        Returns ``{"n_stored": (count,), "t": (count, rows), "x": (count, rows,
        nVar), "dx": (count, rows, nVar), "aux": (count, rows, nAux)}`` float64
        arrays for members ``first .. first + count - 1``: member i's rows
        are ``t[i, :n_stored[i] + 1]`` etc., the slices clODE's
        ``TrajectorySimulator.get_trajectory`` builds one member at a time
        (clode/trajectory.py:216-264).  ``rows`` defaults to the longest
        stored trajectory among those members; ``which`` selects the arrays
        to fetch ("aux" is omitted when the model has none).
        """
        return self._by_member(N.lib.clode_sim_get_trajectory_by_member, "n_stored", 1, first, count, rows, which,
                               lambda s: int(s.max_store))

    def _by_member(self, fn, counts_key: str, extra_row: int, first, count, rows, which, max_rows) -> dict:
        s = N.CSizes()
        _check(N.lib.clode_sim_get_sizes(self._handle, C.byref(s)))
        n_pts, n_var, n_aux = int(s.n_pts), int(s.n_store_var), int(s.n_store_aux)
        count = n_pts - first if count is None else int(count)
        ns = np.zeros(max(count, 0), dtype=np.int32)
        _check(fn(self._handle, first, count, 0, None, None, None, None, ns.ctypes.data_as(C.POINTER(C.c_int))))
        if rows is None:
            rows = min(max_rows(s), int(ns.max()) + extra_row) if count > 0 else 0
        out = {counts_key: ns}
        shapes = {"t": (count, rows), "x": (count, rows, n_var), "dx": (count, rows, n_var),
                  "aux": (count, rows, n_aux)}
        ptrs = []
        for k in ("t", "x", "dx", "aux"):
            if k in which and not (k == "aux" and n_aux == 0):
                out[k] = np.empty(shapes[k], dtype=np.float64)
                ptrs.append(N.dptr(out[k]))
            else:
                ptrs.append(None)
        _check(fn(self._handle, first, count, rows, *ptrs, None))
        return out


class FeatureSimulatorBase(SimulatorBase, _StoredRows):
    """clODE's CLODEfeatures class (clode/cpp/CLODEfeatures.hpp:23-76)."""

    _kind = N.SIM_FEATURES

    def __init__(self, problem_info: ProblemInfo, stepper: str, observer: str, observer_params: ObserverParams,
                 cl_single_precision: bool, opencl_resource: OpenCLResource, clode_root: str = ""):
        self._handle = C.c_void_p()
        self._pi = problem_info
        get_logger()
        self._init_handle(problem_info, stepper, cl_single_precision, opencl_resource,
                          observer=getattr(observer, "value", observer), op=observer_params)

    def __repr__(self) -> str:
        return f"<CLODEfeatures (observer={self.get_observer_name()}, n_features={self.get_n_features()})>"

    def set_observer_params(self, op: ObserverParams) -> None:
        c = op._c()
        _check(N.lib.clode_sim_set_observer_params(self._handle, C.byref(c)))

    def set_observer(self, observer) -> None:
        _check(N.lib.clode_sim_set_observer(self._handle, str(getattr(observer, "value", observer)).encode()))

    def initialize_observer(self) -> None:
        _check(N.lib.clode_sim_initialize_observer(self._handle))

    def is_observer_initialized(self) -> bool:
        v = C.c_int(0)
        _check(N.lib.clode_sim_is_observer_initialized(self._handle, C.byref(v)))
        return bool(v.value)

    def features(self, reinitialize_observer: Optional[bool] = None) -> None:
        flag = -1 if reinitialize_observer is None else int(bool(reinitialize_observer))
        _check(N.lib.clode_sim_features(self._handle, flag))

    def features_store(self, reinitialize_observer: Optional[bool] = None, event_rows: int = 0) -> None:
        """features() that also stores, in the same pass, the trajectory rows
        (as TrajectorySimulatorBase.trajectory: row 0 and every nout-th step,
        read with get_t/get_x/get_dx/get_aux/get_n_stored) and the state at
        each of the first ``event_rows`` observer events (get_event_t/x/dx/aux,
        get_n_events).  Addition: the design of the reference's unused unified
        driver (clode/cpp/odedriver.cl:10-162), repaired; F, xf, dt, tf and
        the RNG state come out as from features()."""
        flag = -1 if reinitialize_observer is None else int(bool(reinitialize_observer))
        _check(N.lib.clode_sim_features_store(self._handle, flag, int(event_rows)))

    def get_event_t(self) -> np.ndarray:
        return self._get(N.ARRAY_EVENT_T)

    def get_event_x(self) -> np.ndarray:
        return self._get(N.ARRAY_EVENT_X)

    def get_event_dx(self) -> np.ndarray:
        return self._get(N.ARRAY_EVENT_DX)

    def get_event_aux(self) -> np.ndarray:
        return self._get(N.ARRAY_EVENT_AUX)

    def get_events_by_member(self, first: int = 0, count: Optional[int] = None, rows: Optional[int] = None,
                             which=("t", "x", "dx", "aux")) -> dict:
        """The event states of the last ``features_store`` regrouped by member
        (addition): ``{"n_events": (count,), "t": (count, rows), "x": (count,
        rows, nVar), ...}``; member i's events are ``t[i, :min(n_events[i],
        rows)]``.  ``rows`` defaults to the most events any of these members
        stored."""
        return self._by_member(N.lib.clode_sim_get_events_by_member, "n_events", 0, first, count, rows, which,
                               lambda s: int(s.event_rows))

    def get_n_events(self) -> np.ndarray:
        n = C.c_size_t(0)
        _check(N.lib.clode_sim_get_n_events(self._handle, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.int32)
        if n.value:
            _check(N.lib.clode_sim_get_n_events(self._handle, out.ctypes.data_as(C.POINTER(C.c_int)), out.size,
                                                C.byref(n)))
        return out

    def get_observer_params(self) -> ObserverParams:
        c = N.CObserverParams()
        _check(N.lib.clode_sim_get_observer_params(self._handle, C.byref(c)))
        return ObserverParams._from_c(c)

    def get_observer_name(self) -> str:
        return self._get_string(N.STRING_OBSERVER_NAME)

    def get_f(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Features, [k * nPts + i] (clode/cpp/CLODEfeatures.hpp getF); `out`:
        optional destination (see SimulatorBase._get; no reference
        counterpart)."""
        return self._get(N.ARRAY_F, out)

    def get_n_features(self) -> int:
        s = N.CSizes()
        _check(N.lib.clode_sim_get_sizes(self._handle, C.byref(s)))
        return int(s.n_features)

    def get_feature_names(self) -> List[str]:
        s = self._get_string(N.STRING_FEATURE_NAMES)
        return s.split("\n") if s else []

    def get_available_observers(self) -> List[str]:
        return self._get_string(N.STRING_AVAILABLE_OBSERVERS).split("\n")


class TrajectorySimulatorBase(SimulatorBase, _StoredRows):
    """clODE's CLODEtrajectory class (clode/cpp/CLODEtrajectory.hpp:21-52)."""

    _kind = N.SIM_TRAJECTORY

    def __init__(self, problem_info: ProblemInfo, stepper: str, cl_single_precision: bool,
                 opencl_resource: OpenCLResource, clode_root: str = ""):
        self._handle = C.c_void_p()
        self._pi = problem_info
        get_logger()
        self._init_handle(problem_info, stepper, cl_single_precision, opencl_resource)

    def trajectory(self) -> None:
        _check(N.lib.clode_sim_trajectory(self._handle))
