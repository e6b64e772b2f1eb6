"""Per-member trajectory outputs without a per-member host loop.

clODE's ``TrajectorySimulator.get_trajectory`` (clode/trajectory.py:204-266)
copies the four stored arrays to the host, reshapes them, and then builds one
``TrajectoryOutput`` per member, each converting its slices into structured
arrays by copy (:250-264).  Here the regrouping runs on the device
(``TrajectorySimulatorBase.get_trajectory_by_member``: one transpose per
stored array, one device-to-host copy each, rows landing member-major), and
every member's output is a view into those arrays with the attributes of
clODE's ``TrajectoryOutput`` (clode/trajectory.py:18-56): ``t`` of shape
(n,), and ``x``, ``dx`` (and ``aux`` when the model has auxiliary variables)
as structured arrays of shape (n,) with one float64 field per name, where
n = n_stored + 1 rows of that member.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np
from numpy.lib import recfunctions as rfn


def _fields(names: Sequence[str]) -> np.dtype:
    return np.dtype({"names": list(names), "formats": [np.float64] * len(names)})


class TrajectoryOutput:
    """clODE's ``TrajectoryOutput`` (clode/trajectory.py:18-56), same
    constructor, attributes, ``to_ndarray`` and ``repr``."""

    def __init__(self, t: np.ndarray, x: np.ndarray, dx: np.ndarray, aux: np.ndarray,
                 variable_names: List[str], aux_names: List[str]) -> None:
        self.t = t
        x_dtype = _fields(variable_names)
        self.x = rfn.unstructured_to_structured(x, dtype=x_dtype)
        self.dx = rfn.unstructured_to_structured(dx, dtype=x_dtype)
        if len(aux_names) > 0:
            self.aux = rfn.unstructured_to_structured(aux, dtype=_fields(aux_names))
        self._variable_names = variable_names
        self._aux_names = aux_names

    @classmethod
    def _view(cls, t, x, dx, aux, variable_names, aux_names) -> "TrajectoryOutput":
        """An output over already-structured views (no copy)."""
        out = cls.__new__(cls)
        out.t, out.x, out.dx = t, x, dx
        if len(aux_names) > 0:
            out.aux = aux
        out._variable_names = variable_names
        out._aux_names = aux_names
        return out

    def __repr__(self) -> str:
        return (f"TrajectoryOutput( length: {len(self.t)}, variable names: {self._variable_names}, "
                f"aux variable names: {self._aux_names} )")

    def to_ndarray(self, slot: str, **kwargs):
        if slot == "x":
            return rfn.structured_to_unstructured(self.x, **kwargs)
        elif slot == "dx":
            return rfn.structured_to_unstructured(self.dx, **kwargs)
        elif slot == "aux":
            return rfn.structured_to_unstructured(self.aux, **kwargs)


def _structured(a: np.ndarray, names: Sequence[str]) -> np.ndarray:
    """(members, rows, k) float64 -> (members, rows) structured view, one field per name."""
    return a.view(_fields(names)).reshape(a.shape[:2])


def get_trajectory(sim, variable_names: Optional[List[str]] = None, aux_names: Optional[List[str]] = None,
                   first: int = 0, count: Optional[int] = None):
    """The last trajectory as clODE's list of per-member ``TrajectoryOutput``.

    ``sim`` is either this package's ``TrajectorySimulatorBase`` (names are
    then taken from its ``ProblemInfo`` unless given) or clODE's
    ``TrajectorySimulator`` front-end, whose ``get_trajectory`` this
    replaces with the same return value: a list with one output per member,
    or the output itself when the ensemble has one member
    (clode/trajectory.py:266).  ``first``/``count`` restrict the members.
    """
    integrator = getattr(sim, "_integrator", sim)
    if variable_names is None:
        variable_names = list(getattr(sim, "variable_names", None) or integrator.get_problem_info().vars)
    if aux_names is None:
        names = getattr(sim, "aux_names", None)
        aux_names = list(names if names is not None else integrator.get_problem_info().aux)
    parts = integrator.get_trajectory_by_member(first=first, count=count)
    ns = parts["n_stored"]
    t = parts["t"]
    x = _structured(parts["x"], variable_names)
    dx = _structured(parts["dx"], variable_names)
    aux = _structured(parts["aux"], aux_names) if len(aux_names) > 0 else None
    results = [
        TrajectoryOutput._view(t[i, :n], x[i, :n], dx[i, :n], None if aux is None else aux[i, :n],
                               variable_names, aux_names)
        for i, n in enumerate((ns + 1).tolist())
    ]
    return results[0] if len(results) == 1 else results


def trajectory_chunks(sim, t_span, n_chunks: int, update_x0: bool = True):
    """A long trajectory as ``n_chunks`` consecutive runs over equal parts of
    ``t_span``, so the stored rows of one part at a time fill the device
    buffers (max_store rows per part).  clODE leaves this as a TODO
    (clode/trajectory.py:166: "chunk time - keep max_store to a reasonable
    level, loop solve/get until t_span is covered").

    Each chunk is exactly what a clODE user gets from
    ``TrajectorySimulator.trajectory(t_span=part, update_x0=True)``: the
    trajectory kernel over the part, then ``shift_x0`` so the next part
    starts from the final state (the step size and the RNG stream continue;
    the cached second normal deviate is dropped at every launch, as in the
    reference).  Yields, per chunk, ``(t0, t1, rows)`` with ``rows`` the
    member-major arrays of ``get_trajectory_by_member``.
    """
    a, b = float(t_span[0]), float(t_span[1])
    if n_chunks < 1:
        raise ValueError("n_chunks must be at least 1")
    edges = [a + (b - a) * k / n_chunks for k in range(n_chunks)] + [b]
    for k in range(n_chunks):
        sim.set_tspan([edges[k], edges[k + 1]])
        sim.trajectory()
        rows = sim.get_trajectory_by_member()
        if update_x0:
            sim.shift_x0()
        yield edges[k], edges[k + 1], rows
