"""Damping / growth-rate fits of the field energy (test infrastructure only).

* Landau: gamma = slope/2 of a line fit of log E at the local maxima of E[:100]
  (Examples/1D_Landau_damping_dr_curve.py:106-110; ``scipy.signal.find_peaks``
  with default arguments = strict local maxima, plateaus by their middle sample).
* Two-stream: gamma = slope/2 of a line fit of log E over samples [300:]
  (Examples/1D_two_stream_gr_curve.py:101-104).
* Windowed least-squares slope of log E over t in [t_a, t_b] (the differentiable
  loss of the adjoint workload): slope = sum (t-tm)(l-lm) / sum (t-tm)^2.
"""
from __future__ import annotations

import numpy as np


def local_maxima(x):
    """Indices of strict local maxima (find_peaks default semantics incl. flat tops)."""
    x = np.asarray(x, dtype=np.float64)
    peaks = []
    i = 1
    n = len(x)
    while i < n - 1:
        if x[i - 1] < x[i]:
            j = i
            while j + 1 < n and x[j + 1] == x[i]:
                j += 1
            if j + 1 < n and x[j + 1] < x[i]:
                peaks.append((i + j) // 2)
                i = j
        i += 1
    return np.array(peaks, dtype=np.int64)


def landau_rate(t, E, nsamples=100):
    pk = local_maxima(E[:nsamples])
    slope = np.polyfit(np.asarray(t)[pk], np.log(np.asarray(E)[pk]), 1)[0]
    return 0.5 * slope


def growth_rate(t, E, start=300):
    slope = np.polyfit(np.asarray(t)[start:], np.log(np.asarray(E)[start:]), 1)[0]
    return 0.5 * slope


def window_slope(t, E, ta, tb):
    t = np.asarray(t, np.float64)
    sel = (t >= ta) & (t <= tb)
    tt, ll = t[sel], np.log(np.asarray(E, np.float64)[sel])
    tm, lm = tt.mean(), ll.mean()
    return float(np.sum((tt - tm) * (ll - lm)) / np.sum((tt - tm) ** 2))
