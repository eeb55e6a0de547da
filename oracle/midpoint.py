"""Implicit midpoint step with Newton iterations (test infrastructure only).

Restates spectrax/midpoint_solver.py:37-98: y1 solves
    F(y1) = y1 - y0 - dt f((y0 + y1)/2) = 0,
starting from the explicit-Euler guess y0 + dt f(y0); each Newton iteration
measures norm = ||F(y1) / (atol + rtol max(|y0|, |y1|))||_2 (a 2-norm, as in
the reference) and stops once norm < 1 (max 300 iterations).  The reference
solves each Newton system with GMRES through jax.linearize; for the small
oracle cases the Jacobian of the quadratic right-hand side is assembled exactly
(central differences of a quadratic map are exact) and solved densely, so the
oracle lands on the same root with a tighter linear solve.  The error estimate
returned is y1 - (y0 + dt f(y0)) (midpoint_solver.py:51).
"""
from __future__ import annotations

import numpy as np


def jacobian(f, y):
    n = len(y)
    J = np.empty((n, n), np.complex128)
    for j in range(n):
        e = np.zeros(n, np.complex128)
        e[j] = 1.0
        J[:, j] = 0.5 * (f(y + e) - f(y - e))
    return J


def step(f, y0, dt, rtol=1e-10, atol=1e-10, max_iters=300):
    f0 = f(y0)
    y1_init = y0 + dt * f0
    y1 = y1_init.copy()
    iters = 0
    for i in range(max_iters):
        ymid = 0.5 * (y0 + y1)
        res = y1 - y0 - dt * f(ymid)
        scale = atol + rtol * np.maximum(np.abs(y0), np.abs(y1))
        norm = np.linalg.norm(res / scale)
        if norm < 1.0:
            break
        JF = np.eye(len(y0)) - 0.5 * dt * jacobian(f, ymid)
        y1 = y1 + np.linalg.solve(JF, -res)
        iters += 1
    return y1, y1 - y1_init, iters
