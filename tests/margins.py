"""Decision margins of the neighbourhood observer (nhood2), read from a
member's stored trajectory.

nhood2 (clode/cpp/observers/observer_neighborhood_2.clh) turns a continuous
trajectory into counts through three threshold decisions:

* the centre: the first downward crossing of the event variable through
  ``x_thresh = min + xDownThresh * range`` (range from the warm-up pass),
  at step 2 or later (``:150-154``, ``:258-266``);
* events: exits of the trajectory from the ball of radius ``nHoodRadius``
  around the centre, distances normalised by each variable's range
  (``:157-175``);
* peaks: sign changes of the feature variable's slope from >= 0 to < 0
  after the centre is set (``:250-255``).

``nhood2_counts`` re-evaluates those decisions from the rows of a trajectory
run that stores every step (the same steps as the feature pass: same start,
same stepper, the same ``t <= t1`` loop), and ``nhood2_margins`` measures how
close each decision quantity comes to its threshold without crossing it, or
how little it crosses: a count can change under a small change of the
trajectory only through such a near-tangency.

* ``m_ball``: over the local extrema of the normalised distance d after the
  centre, min |d - r| / r;
* ``m_peak``: over the local extrema of the feature variable's slope after
  the centre, min |slope| / max |slope|;
* ``m_center``: over the local minima of the event variable up to 50 steps
  past the centre (all of them when no centre is found), min |x - x_thresh|
  / range.
"""
from __future__ import annotations

import numpy as np


def _local_extrema(s: np.ndarray) -> np.ndarray:
    if s.size < 3:
        return np.zeros(0, dtype=np.int64)
    mid = s[1:-1]
    up = (mid > s[:-2]) & (mid >= s[2:])
    down = (mid < s[:-2]) & (mid <= s[2:])
    return np.where(up | down)[0] + 1


def nhood2_counts(t, x, dx, t1, e_var, f_var, radius, x_down):
    """Re-evaluate nhood2 on one member's rows (row 0 = the initial state).

    ``t`` (K+1,), ``x``/``dx`` (K+1, nVar) in the run's precision.  Returns
    a dict: ``warm`` (warm-up steps: those taken while t < t1), ``x_thresh``,
    ``range``, ``center_step`` (None when no centre), ``event_steps``,
    ``peak_steps`` and ``peaks`` (peaks between consecutive events, as the
    observer counts them)."""
    real = x.dtype.type
    K = t.size - 1
    warm = 0
    while warm < K and t[warm] < t1:
        warm += 1
    xw = x[1:warm + 1]
    rng = (xw.max(0) - xw.min(0)).astype(x.dtype)
    thr = real(xw.min(0)[e_var] + real(x_down) * rng[e_var])
    kc = None
    for k in range(2, K + 1):
        if x[k - 1, e_var] > thr and x[k, e_var] < thr:
            kc = k
            break
    out = dict(warm=warm, x_thresh=thr, range=rng, center_step=kc, event_steps=np.zeros(0, np.int64),
               peak_steps=np.zeros(0, np.int64), peaks=[])
    if kc is None:
        return out
    c = x[kc]
    d = np.sqrt(np.sum(((x[kc:] - c) / rng) ** 2, axis=1))  # rows kc..K
    inside = d < real(radius)
    ev = np.where(inside[:-1] & ~inside[1:])[0] + 1 + kc
    pk = np.where((dx[kc:K, f_var] >= 0) & (dx[kc + 1:K + 1, f_var] < 0))[0] + kc + 1
    out.update(event_steps=ev, peak_steps=pk, distance=d)
    if ev.size > 1:
        out["peaks"] = [int(np.sum((pk > ev[j]) & (pk <= ev[j + 1]))) for j in range(ev.size - 1)]
    return out


def nhood2_margins(t, x, dx, t1, e_var, f_var, radius, x_down) -> dict:
    """The three decision margins of one member (module docstring)."""
    r = nhood2_counts(t, x, dx, t1, e_var, f_var, radius, x_down)
    kc = r["center_step"]
    m = dict(m_ball=np.inf, m_peak=np.inf, m_center=np.inf)
    if kc is not None:
        d = r["distance"][1:]
        ext = _local_extrema(d)
        if ext.size:
            m["m_ball"] = float(np.min(np.abs(d[ext] - radius)) / radius)
        s = dx[kc:, f_var].astype(np.float64)
        ext = _local_extrema(s)
        scale = np.max(np.abs(s))
        if ext.size and scale > 0:
            m["m_peak"] = float(np.min(np.abs(s[ext])) / scale)
    xe = x[2:, e_var].astype(np.float64)
    lo = np.where((xe[1:-1] < xe[:-2]) & (xe[1:-1] <= xe[2:]))[0] + 1
    if kc is not None:
        lo = lo[lo <= kc - 2 + 50]
    span = float(r["range"][e_var])
    if lo.size and span > 0:
        m["m_center"] = float(np.min(np.abs(xe[lo] - float(r["x_thresh"]))) / span)
    m["margin"] = min(m["m_ball"], m["m_peak"], m["m_center"])
    return m
