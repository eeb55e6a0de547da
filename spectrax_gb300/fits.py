"""Damping / growth-rate fits of the field energy (host side).

* Landau: gamma = slope/2 of a line fit of log E at the local maxima of E[:n]
  (Examples/1D_Landau_damping_dr_curve.py:106-110: find_peaks, polyfit, /2).
* Two-stream: gamma = slope/2 of a line fit of log E over samples [start:]
  (Examples/1D_two_stream_gr_curve.py:101-104).
* ``window_slope``: least-squares slope of log E over t in [ta, tb].
"""
from __future__ import annotations

import numpy as np


def peaks(x):
    """Indices of strict local maxima; a flat top counts once, at its middle sample."""
    x = np.asarray(x, dtype=np.float64)
    out = []
    i, n = 1, len(x)
    while i < n - 1:
        if x[i - 1] < x[i]:
            j = i
            while j + 1 < n and x[j + 1] == x[i]:
                j += 1
            if j + 1 < n and x[j + 1] < x[i]:
                out.append((i + j) // 2)
                i = j
        i += 1
    return np.array(out, dtype=np.int64)


def landau_damping_rate(t, E, nsamples=100):
    t = np.asarray(t, np.float64)
    E = np.asarray(E, np.float64)
    pk = peaks(E[:nsamples])
    if len(pk) < 2:
        return float("nan")
    return 0.5 * float(np.polyfit(t[pk], np.log(E[pk]), 1)[0])


def two_stream_growth_rate(t, E, start=300):
    t = np.asarray(t, np.float64)
    E = np.asarray(E, np.float64)
    return 0.5 * float(np.polyfit(t[start:], np.log(E[start:]), 1)[0])


def window_slope(t, E, ta, tb):
    t = np.asarray(t, np.float64)
    sel = (t >= ta) & (t <= tb)
    tt, ll = t[sel], np.log(np.asarray(E, np.float64)[sel])
    tm, lm = tt.mean(), ll.mean()
    return float(np.sum((tt - tm) * (ll - lm)) / np.sum((tt - tm) ** 2))
