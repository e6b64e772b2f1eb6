"""The OpenCL-C builtins a clODE model may call (the set the reference's
Python converter emits, clode/function_converter.py:54-124) through this
package's NVRTC shim: the probe model compiles for sm_103a on the CPU, and on
the GPU every builtin's value matches Python's math library at the inputs of
clODE's builtin test (test/test_opencl_builtins.py:81-171)."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from clode_gb300 import _native as N

HERE = os.path.dirname(os.path.abspath(__file__))
MODEL = os.path.join(HERE, "models", "builtins.cl")
N_AUX = 58
X = (0.3, 1.5, 2.5)
P = (2.8, 4.55)


def expected(t, real=np.float64):
    """The probe model's aux values at time t, computed with Python's math on
    inputs rounded to the working precision."""
    r = lambda v: float(real(v))  # noqa: E731
    x0, x1 = r(r(X[0]) * r(t)), r(r(X[1]) * r(t))
    p0, p1 = int(P[0]), int(P[1])
    pi = math.pi
    v = [math.acos(x0), math.acosh(x0 + 1), math.acos(x0) / pi, math.asin(x0), math.asinh(x0 + 1),
         math.asin(x0) / pi, math.atan(x0), math.atan2(x0, x1), math.atan2(x0, x1) / pi, math.atanh(x0 / 100),
         math.atan(x0) / pi, math.copysign(abs(x0) ** (1 / 3), x0), math.ceil(x0), math.copysign(x0, x1),
         math.cos(x0), math.cosh(x0), math.cos(pi * x0), math.erf(x0), math.erfc(x0), math.exp(x0), 2.0 ** x0,
         10.0 ** x0, math.expm1(x0), abs(x0), max(x0 - x1, 0.0), math.floor(x1), max(x0, x1),
         math.fmod(x0, x1 + 1), 1.0 if t - 0.5 >= 0 else 0.0, math.gamma(x0 + 1), math.hypot(x0, x1),
         float(math.frexp(x0 + 1)[1] - 1), math.ldexp(x0, int(x1)), math.lgamma(x0 + 1), math.log(x0 + 1),
         math.log1p(x0 + 1), math.log2(x0 + 1), math.log10(x0 + 1), min(x0, x1), math.sin(x0) + math.cos(x0),
         math.sinh(x0) - math.tanh(x0), math.nextafter(x0, x1) if real is np.float64 else
         float(np.nextafter(np.float32(x0), np.float32(x1))), x0 ** x1, x0 ** p0, (x0 + 0.5) ** (x1 + 0.2),
         math.remainder(x0, x1 + 1), float(round(x0)), x0 ** (1 / p1), 1 / math.sqrt(x0 + 1), math.sin(x0),
         math.sinh(x0), math.sin(pi * x0), math.sqrt(x0), math.tan(x0), math.tanh(x0), math.tan(pi * x0),
         float(math.trunc(x0)), float(math.floor(x0 + 0.2 + 0.5))]
    assert len(v) == N_AUX
    return np.array(v)


def _problem(src):
    names = [f"a{k}" for k in range(N_AUX)]
    return N.CProblem(src, b"builtins.cl", 3, 2, N_AUX, 0, b"x\ny\nz", b"p0\np1", "\n".join(names).encode())


@pytest.mark.parametrize("single", [True, False])
def test_every_builtin_compiles_for_sm103a(single):
    src = open(MODEL, "rb").read()
    cp = _problem(src)
    h = C.c_void_p()
    N.check(N.lib.clode_sim_create(N.SIM_TRAJECTORY, C.byref(cp), b"euler", None, None, int(single), 0,
                                   C.byref(h)))
    try:
        N.check(N.lib.clode_sim_build(h))
    finally:
        N.lib.clode_sim_destroy(h)


def test_expected_values_are_finite():
    for t in (0.0, 0.5, 1.0):
        assert np.isfinite(expected(t)).all()


@pytest.mark.gpu
@pytest.mark.parametrize("single", [False, True])
def test_builtin_values_match_python_math(single):
    from clode_gb300 import clode_cpp_wrapper as W

    pi = W.ProblemInfo(MODEL, ["x", "y", "z"], ["p0", "p1"], [f"a{k}" for k in range(N_AUX)], 0)
    sim = W.TrajectorySimulatorBase(pi, "euler", single, W.OpenCLResource(), "")
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=0.5, max_steps=3, max_store=3, nout=1))
    sim.set_problem_data(list(X), list(P))
    sim.set_tspan([0.0, 1.0])
    sim.trajectory()
    aux = np.asarray(sim.get_aux()).reshape(3, N_AUX)  # rows t = 0, 0.5, 1 of the single member
    t = np.asarray(sim.get_t())
    np.testing.assert_array_equal(t, [0.0, 0.5, 1.0])
    real = np.float32 if single else np.float64
    for row, tt in enumerate((0.0, 0.5, 1.0)):
        ref = expected(tt, real)
        # tolerance: CUDA's math functions are within a few ulp of the
        # correctly rounded value (FP64), FP32 results are compared at FP32
        # resolution; the reference's own test uses atol 1e-7
        rtol, atol = (2e-6, 1e-6) if single else (1e-13, 1e-15)
        np.testing.assert_allclose(aux[row], ref, rtol=rtol, atol=atol, err_msg=f"t={tt}")
