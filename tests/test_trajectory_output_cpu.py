"""Per-member trajectory assembly (clode_gb300.trajectory_output) against the
restatement of clODE's per-member loop (oracle/trajectory_frontend.py,
clode/trajectory.py:216-264), on a fake integrator that holds SoA arrays
and regroups them by the layout contract of
clode_sim_get_trajectory_by_member.  The device regrouping itself is
checked in tests/test_gpu_trajectory_output.py."""
import numpy as np
import pytest

from clode_gb300.trajectory_output import TrajectoryOutput, get_trajectory
from clode_gb300.clode_cpp_wrapper import ProblemInfo
from oracle.trajectory_frontend import reference_get_trajectory, regroup_by_member


class FakeIntegrator:
    def __init__(self, n_pts, n_var, n_aux, max_store, seed=3):
        rng = np.random.default_rng(seed)
        self.n_pts, self.n_var, self.n_aux, self.max_store = n_pts, n_var, n_aux, max_store
        self.t = rng.standard_normal(max_store * n_pts)
        self.x = rng.standard_normal(max_store * n_var * n_pts)
        self.dx = rng.standard_normal(max_store * n_var * n_pts)
        self.aux = rng.standard_normal(max_store * n_aux * n_pts) if n_aux else np.zeros(1)
        # ragged lengths, including the reference's n_stored == max_store
        self.ns = rng.integers(0, max_store, n_pts).astype(np.int32)
        self.ns[0] = max_store
        self.ns[-1] = 0
        self.pi = ProblemInfo("m.cl", [f"v{j}" for j in range(n_var)], ["p"], [f"a{k}" for k in range(n_aux)])

    def get_problem_info(self):
        return self.pi

    def get_n_stored(self):
        return self.ns.copy()

    def get_t(self):
        return self.t.copy()

    def get_x(self):
        return self.x.copy()

    def get_dx(self):
        return self.dx.copy()

    def get_aux(self):
        return self.aux.copy()

    def get_trajectory_by_member(self, first=0, count=None, rows=None, which=("t", "x", "dx", "aux")):
        count = self.n_pts - first if count is None else count
        ns = self.ns[first:first + count]
        if rows is None:
            rows = min(self.max_store, int(ns.max()) + 1)
        out = {"n_stored": ns.copy(),
               "t": regroup_by_member(self.t, self.n_pts, 1, first, count, rows)[:, :, 0],
               "x": regroup_by_member(self.x, self.n_pts, self.n_var, first, count, rows),
               "dx": regroup_by_member(self.dx, self.n_pts, self.n_var, first, count, rows)}
        if self.n_aux:
            out["aux"] = regroup_by_member(self.aux, self.n_pts, self.n_aux, first, count, rows)
        return out


class FakeFrontEnd:
    """The attributes of clODE's TrajectorySimulator that get_trajectory reads."""

    def __init__(self, integ):
        self._integrator = integ
        self.variable_names = integ.pi.vars
        self.aux_names = integ.pi.aux
        self._ensemble_size = integ.n_pts


def _assert_same(ours, ref, has_aux):
    assert len(ours) == len(ref)
    for o, r in zip(ours, ref):
        assert np.array_equal(o.t, r["t"])
        assert o.x.dtype == r["x"].dtype and np.array_equal(o.x, r["x"])
        assert np.array_equal(o.dx, r["dx"])
        assert hasattr(o, "aux") == has_aux
        if has_aux:
            assert o.aux.dtype == r["aux"].dtype and np.array_equal(o.aux, r["aux"])
            assert np.array_equal(o.to_ndarray("aux"), rfn_un(r["aux"]))
        assert np.array_equal(o.to_ndarray("x"), rfn_un(r["x"]))


def rfn_un(a):
    from numpy.lib import recfunctions as rfn
    return rfn.structured_to_unstructured(a)


@pytest.mark.parametrize("n_var,n_aux", [(1, 0), (3, 2), (4, 1)])
def test_matches_reference_loop(n_var, n_aux):
    integ = FakeIntegrator(37, n_var, n_aux, 11)
    ref = reference_get_trajectory(integ, integ.pi.vars, integ.pi.aux, integ.n_pts, integ.max_store)
    _assert_same(get_trajectory(integ), ref, n_aux > 0)
    _assert_same(get_trajectory(FakeFrontEnd(integ)), ref, n_aux > 0)


def test_member_range():
    integ = FakeIntegrator(50, 2, 1, 9)
    ref = reference_get_trajectory(integ, integ.pi.vars, integ.pi.aux, integ.n_pts, integ.max_store)
    _assert_same(get_trajectory(integ, first=13, count=20), ref[13:33], True)


def test_single_member_returns_the_output():
    integ = FakeIntegrator(1, 2, 0, 5)
    out = get_trajectory(integ)
    assert isinstance(out, TrajectoryOutput)
    assert repr(out).startswith("TrajectoryOutput( length: ")


def test_constructor_matches_reference_semantics():
    t = np.arange(4.0)
    x = np.arange(8.0).reshape(4, 2)
    out = TrajectoryOutput(t, x, -x, np.zeros((4, 0)), ["a", "b"], [])
    assert out.x["b"].tolist() == [1.0, 3.0, 5.0, 7.0]
    assert out.dx["a"].tolist() == [-0.0, -2.0, -4.0, -6.0]
    assert not hasattr(out, "aux")
    assert np.array_equal(out.to_ndarray("x"), x)


def test_views_share_memory():
    integ = FakeIntegrator(8, 2, 1, 6)
    outs = get_trajectory(integ)
    assert outs[1].x.base is not None and np.shares_memory(outs[1].x, outs[2].x.base)


def test_trajectory_chunks_call_sequence():
    from clode_gb300.trajectory_output import trajectory_chunks

    class Sim:
        def __init__(self):
            self.calls = []

        def set_tspan(self, ts):
            self.calls.append(("tspan", tuple(ts)))

        def trajectory(self):
            self.calls.append(("trajectory",))

        def get_trajectory_by_member(self):
            self.calls.append(("get",))
            return {"n_stored": np.zeros(1, dtype=np.int32)}

        def shift_x0(self):
            self.calls.append(("shift_x0",))

    s = Sim()
    chunks = list(trajectory_chunks(s, (1.0, 4.0), 3))
    assert [c[:2] for c in chunks] == [(1.0, 2.0), (2.0, 3.0), (3.0, 4.0)]
    assert s.calls == [("tspan", (1.0, 2.0)), ("trajectory",), ("get",), ("shift_x0",),
                       ("tspan", (2.0, 3.0)), ("trajectory",), ("get",), ("shift_x0",),
                       ("tspan", (3.0, 4.0)), ("trajectory",), ("get",), ("shift_x0",)]
    s2 = Sim()
    list(trajectory_chunks(s2, (0.0, 1.0), 1, update_x0=False))
    assert ("shift_x0",) not in s2.calls
    with pytest.raises(ValueError):
        list(trajectory_chunks(Sim(), (0.0, 1.0), 0))
