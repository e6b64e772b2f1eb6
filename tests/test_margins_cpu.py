"""The re-evaluation of nhood2 decisions in ``tests/margins.py`` against the
oracle itself: from the oracle's stored steps it must reproduce the
oracle's event count and its maximum and minimum peaks per event interval,
member by member, so the margins it reports describe the decisions the
observer actually took."""
import os

import numpy as np

import bench
from tests.margins import nhood2_counts, nhood2_margins


def test_reevaluation_reproduces_oracle_counts():
    from clode_gb300 import rhs_path
    from oracle.build import OracleConfig
    from oracle.runner import OracleSimulator

    x0, pars, tspan = bench.make_workload(2048, 20261203, 1e3, 1e4)
    # 96 members from the band of the map where the counts are sensitive
    # (gcal 0.80-0.86) and 32 from elsewhere, 3000 ms each
    rng = np.random.default_rng(5)
    band = np.where((pars[:, 0] > 0.80) & (pars[:, 0] < 0.86))[0]
    idx = np.concatenate([rng.choice(band, 96, replace=False), rng.choice(pars.shape[0], 32, replace=False)])
    ts = np.stack([np.zeros(idx.size), np.full(idx.size, 3000.0)], axis=1)
    full_ts = np.zeros_like(tspan)
    full_ts[idx] = ts
    F, _, _ = bench.run_cpu(x0, pars, full_ts, idx, os.cpu_count(), prefer_reference=False)
    steps = F[:, -4]  # "step count"
    cfg = OracleConfig(rhs_path("lactotroph.cl"), n_var=4, n_par=3, n_aux=1, stepper="dopri5", single_precision=True)
    s = OracleSimulator(cfg)
    sp = dict(bench.SOLVER)
    sp.update(max_store=int(steps.max()) + 8, nout=1)
    s.set_solver_params(**sp)
    s.set_problem_data(x0[idx], pars[idx])
    s.set_tspan(ts)
    s.trajectory()
    n = idx.size
    T, X, D = s.t.reshape(-1, n), s.x.reshape(-1, 4, n), s.dx.reshape(-1, 4, n)
    e, f = bench.OBSERVER["e_var_ix"], bench.OBSERVER["f_var_ix"]
    radius, x_down = np.float32(bench.OBSERVER["nhood_radius"]), bench.OBSERVER["x_down_threshold"]
    with_events = 0
    for j in range(n):
        k = s.n_stored[j] + 1
        assert k - 1 == steps[j]
        r = nhood2_counts(T[:k, j], X[:k, :, j], D[:k, :, j], np.float32(3000.0), e, f, radius, x_down)
        assert r["event_steps"].size == F[j, -5]  # "event count"
        if r["peaks"]:
            with_events += 1
            assert max(r["peaks"]) == F[j, 3] and min(r["peaks"]) == F[j, 4]  # max / min peaks
        m = nhood2_margins(T[:k, j], X[:k, :, j], D[:k, :, j], np.float32(3000.0), e, f, radius, x_down)
        assert m["margin"] >= 0
    assert with_events >= 10  # the sample exercises the event and peak logic
