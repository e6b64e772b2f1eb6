"""The engine's optional FP32 exp (simulator option fast_exp) against the
correctly rounded value and against CUDA's expf, over the whole normal range
and the special values."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models", "exp_probe.cl")


def _exp_on_gpu(x, fast):
    from clode_gb300 import clode_cpp_wrapper as W

    pi = W.ProblemInfo(MODEL, ["x"], [], ["e"], 0)
    sim = W.TrajectorySimulatorBase(pi, "euler", True, W.OpenCLResource(), "")
    sim.set_option("fast_exp", fast)
    sim.set_option("ftz", 1)
    sim.build_cl()
    sim.set_solver_params(W.SolverParams(dt=1.0, max_steps=1, max_store=1, nout=1))
    sim.set_problem_data(np.asarray(x, dtype=np.float64), [])
    sim.set_tspan([0.0, 0.0])
    sim.trajectory()
    return np.asarray(sim.get_aux(), dtype=np.float64)[: len(x)].astype(np.float32)


def _ulp_error(got, x):
    ref = np.exp(x.astype(np.float64))
    spacing = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    return np.abs(got.astype(np.float64) - ref) / spacing


def test_fast_exp_within_a_few_ulp():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-87.0, 88.0, 400000), rng.uniform(-1.0, 1.0, 100000),
                        np.linspace(-0.01, 0.01, 20001)]).astype(np.float32)
    fast = _exp_on_gpu(x, 1)
    cuda = _exp_on_gpu(x, 0)
    err_fast, err_cuda = _ulp_error(fast, x), _ulp_error(cuda, x)
    print(f"max ulp: fast_exp {err_fast.max():.2f}, CUDA expf {err_cuda.max():.2f}; "
          f"mean {err_fast.mean():.3f} / {err_cuda.mean():.3f}")
    # tolerance: the hardware exp2 approximation (about 2 ulp) plus one
    # rounding of the correction; CUDA's expf is documented at 2 ulp
    assert err_fast.max() <= 4.0
    assert err_cuda.max() <= 2.0


def test_fast_exp_special_values():
    x = np.array([0.0, -0.0, 89.0, 1e30, -104.0, -1e30, np.inf, -np.inf, np.nan], dtype=np.float32)
    got = _exp_on_gpu(x, 1)
    assert got[0] == 1.0 and got[1] == 1.0
    assert np.isinf(got[2]) and np.isinf(got[3]) and np.isinf(got[6])
    assert got[4] == 0.0 and got[5] == 0.0 and got[7] == 0.0  # below the normal range (flushed)
    assert np.isnan(got[8])
