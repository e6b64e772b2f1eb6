"""Regenerate ``lorenz_grid_fp64.npz``: the FP64 reference solution of a
seeded sample of the Lorenz parameter grid.

Grid (member i -> (iy, ix) = divmod(i, 1024)): sigma = linspace(5, 15, 1024)[ix],
rho = linspace(10, 60, 1024)[iy], beta = 8/3; initial state (1, 1, 1) plus
N(0, 1e-3^2) per component; tspan [0, 500]; the threshold observer on z
(x_up 0.3, x_down 0.2, up to 1e5 events).  2048 members are drawn without
replacement (numpy default_rng(20261203)).

Stored: the sample's indices, inputs, and the features of three runs of
clODE's own kernels compiled as C (``oracle/build.py build_reference``;
needs the clODE source tree) in FP64 with Dormand-Prince at
rtol = 1e-10, atol = 1e-13: at the inputs (``F``, every feature) and with
the initial state scaled by 1 + 1e-9 and 1 - 1e-9 (``F_up``, ``F_down``:
the mean period, the extrema and means of x, y, z and their slopes, and
the event count).  The perturbed runs tell which members amplify a 1e-9
change of their initial state (chaotic members).
Usage: ``python -m tests.golden.make_lorenz_grid``.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.build import reference_available  # noqa: E402
from tests.parity import Scenario, run_oracle  # noqa: E402

G = 1024
N = 2048
SEED = 20261203
TOL = 1e-10
PERTURBATION = 1e-9
# columns kept from the perturbed runs: mean period, then x/y/z max, min,
# mean, slope max, slope min, then the event count
PERTURBED_COLUMNS = (2,) + tuple(range(18, 33)) + (36,)


def sample():
    rng = np.random.default_rng(SEED)
    idx = np.sort(rng.choice(G * G, N, replace=False))
    iy, ix = np.divmod(idx, G)
    sigma, rho = np.linspace(5.0, 15.0, G), np.linspace(10.0, 60.0, G)
    pars = np.stack([rho[iy], sigma[ix], np.full(N, 8.0 / 3.0)], axis=1)
    x0 = np.ones((N, 3)) + rng.normal(0.0, 1e-3, (N, 3))
    return idx, x0, pars


def scenario(x0, pars, single, tol):
    return Scenario("lorenz.cl", 3, 3, x0, pars, n_aux=1, stepper="dopri5", observer="thresh2", single=single,
                    sp=dict(dt=1e-3, dtmax=1.0, abstol=tol * 1e-3, reltol=tol, max_steps=10000000),
                    op=dict(e_var_ix=2, f_var_ix=2, max_event_count=100000, x_up_threshold=0.3,
                            x_down_threshold=0.2),
                    steps=[("features", (0.0, 500.0))], seed=None)


def main():
    if not reference_available():
        sys.exit("clODE sources not found: cannot regenerate the fixture")
    idx, x0, pars = sample()
    F = run_oracle(scenario(x0, pars, False, TOL), reference=True)["F_list"][0]
    up = run_oracle(scenario(x0 * (1 + PERTURBATION), pars, False, TOL), reference=True)["F_list"][0]
    down = run_oracle(scenario(x0 * (1 - PERTURBATION), pars, False, TOL), reference=True)["F_list"][0]
    cols = list(PERTURBED_COLUMNS)
    meta = {"source": "clODE kernels compiled as C (oracle/_ref), FP64", "rtol": TOL, "atol": TOL * 1e-3,
            "perturbation": PERTURBATION, "perturbed_columns": cols}
    np.savez_compressed(os.path.join(HERE, "lorenz_grid_fp64.npz"), meta=json.dumps(meta), idx=idx, x0=x0,
                        pars=pars, F=F, F_up=up[:, cols], F_down=down[:, cols])
    print("lorenz_grid_fp64", F.shape)


if __name__ == "__main__":
    main()
