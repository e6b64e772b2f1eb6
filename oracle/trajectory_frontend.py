"""Test infrastructure (the oracle), not product code.

Restatement of clODE's host-side trajectory assembly,
``TrajectorySimulator.get_trajectory`` (clode/trajectory.py:204-266): the
four flat getters (getT/getX/getDx/getAux, SoA ``[r * nPts * w + j * nPts
+ i]`` with ``max_store`` rows), reshaped column-major to (nPts, w,
max_store) (:227-246), then one loop iteration per member that slices its
``n_stored + 1`` rows and converts them to structured arrays (:250-264,
``TrajectoryOutput.__init__`` :19-42).  It is the per-member loop the
device regrouping replaces, kept here as the checker of that replacement
and as the host baseline it is timed against.
"""
from __future__ import annotations

from typing import List

import numpy as np
from numpy.lib import recfunctions as rfn


def _fields(names):
    return np.dtype({"names": list(names), "formats": [np.float64] * len(names)})


def reference_get_trajectory(integrator, variable_names: List[str], aux_names: List[str], ensemble_size: int,
                             max_store: int):
    """One dict per member: {"t": (n,), "x": structured (n,), "dx": ..., "aux": ... (when aux_names)}.

    Follows clode/trajectory.py:216-264 step by step, including the
    column-major reshapes of the flat device arrays and ``ni = n_stored + 1``.
    """
    n_stored = integrator.get_n_stored()
    t = np.array(integrator.get_t(), dtype=np.float64)
    x = np.array(integrator.get_x(), dtype=np.float64)
    dx = np.array(integrator.get_dx(), dtype=np.float64)
    aux = np.array(integrator.get_aux(), dtype=np.float64)
    t_shape = (ensemble_size, max_store)
    t = t[: np.prod(t_shape)].reshape(t_shape, order="F")
    data_shape = (ensemble_size, len(variable_names), max_store)
    x = x[: np.prod(data_shape)].reshape(data_shape, order="F")
    dx = dx[: np.prod(data_shape)].reshape(data_shape, order="F")
    aux_shape = (ensemble_size, len(aux_names), max_store)
    aux = aux[: np.prod(aux_shape)].reshape(aux_shape, order="F")
    x_dtype = _fields(variable_names)
    out = []
    for i in range(ensemble_size):
        ni = n_stored[i] + 1
        member = {
            "t": t[i, :ni].transpose(),
            "x": rfn.unstructured_to_structured(x[i, :, :ni].transpose(), dtype=x_dtype),
            "dx": rfn.unstructured_to_structured(dx[i, :, :ni].transpose(), dtype=x_dtype),
        }
        if len(aux_names) > 0:
            member["aux"] = rfn.unstructured_to_structured(aux[i, :, :ni].transpose(), dtype=_fields(aux_names))
        out.append(member)
    return out


def regroup_by_member(flat: np.ndarray, n_pts: int, width: int, first: int, count: int, rows: int) -> np.ndarray:
    """The layout contract of clode_sim_get_trajectory_by_member on a flat SoA
    array: out[i - first, r, j] = flat[(r * width + j) * n_pts + i]."""
    a = np.asarray(flat, dtype=np.float64)[: rows * width * n_pts].reshape(rows, width, n_pts)
    return np.ascontiguousarray(a[:, :, first:first + count].transpose(2, 0, 1))
