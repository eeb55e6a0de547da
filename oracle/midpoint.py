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


def jvp_quadratic(f, y, v):
    """J(y) v of a right-hand side that is affine plus quadratic in y (this one is:
    every term is linear in Ck or bilinear in (Fk, Ck)): the central difference
    (f(y + v) - f(y - v)) / 2 is then exact up to rounding, for any size of v."""
    return 0.5 * (f(y + v) - f(y - v))


def gmres(matvec, b, restart=30, tol=1e-10, maxiter=20):
    """Restarted GMRES(restart) for A x = b from x = 0, stopping when the residual
    is below tol * ||b||; Gram-Schmidt with one re-orthogonalisation pass and
    Givens rotations.  Returns (x, relative residual, matrix-vector products)."""
    n = len(b)
    x = np.zeros(n, np.complex128)
    bnorm = np.linalg.norm(b)
    if bnorm == 0.0:
        return x, 0.0, 0
    r = b.copy()
    beta = bnorm
    its = 0
    for _ in range(maxiter):
        V = np.empty((restart + 1, n), np.complex128)
        V[0] = r / beta
        H = np.zeros((restart + 1, restart), np.complex128)
        g = np.zeros(restart + 1, np.complex128)
        g[0] = beta
        cs = np.zeros(restart, np.complex128)
        sn = np.zeros(restart, np.complex128)
        k = 0
        for j in range(restart):
            w = matvec(V[j])
            its += 1
            for _pass in range(2):
                for i in range(j + 1):
                    hij = np.vdot(V[i], w)
                    H[i, j] += hij
                    w = w - hij * V[i]
            hn = np.linalg.norm(w)
            H[j + 1, j] = hn
            for i in range(j):
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -np.conj(sn[i]) * H[i, j] + np.conj(cs[i]) * H[i + 1, j]
                H[i, j] = t
            a, bb = H[j, j], H[j + 1, j]
            den = np.hypot(abs(a), abs(bb))
            if den == 0.0:
                cs[j], sn[j] = 1.0, 0.0
            elif abs(a) > 0:
                cs[j], sn[j] = abs(a) / den, (a / abs(a)) * np.conj(bb) / den
            else:
                cs[j], sn[j] = 0.0, np.conj(bb) / den
            H[j, j] = cs[j] * a + sn[j] * bb
            H[j + 1, j] = 0.0
            g[j + 1] = -np.conj(sn[j]) * g[j]
            g[j] = cs[j] * g[j]
            k = j + 1
            if hn > 0.0:
                V[j + 1] = w / hn
            if abs(g[j + 1]) <= tol * bnorm or hn == 0.0:
                break
        yk = np.linalg.solve(np.triu(H[:k, :k]), g[:k])
        x = x + yk @ V[:k]
        r = b - matvec(x)
        its += 1
        beta = np.linalg.norm(r)
        if beta <= tol * bnorm:
            break
    return x, beta / bnorm, its


def step_newton_gmres(f, y0, dt, rtol=1e-10, atol=1e-10, max_iters=300, restart=30, gmres_tol=1e-10,
                      gmres_maxiter=20):
    """Matrix-free implicit midpoint step for large states.

    The Newton loop of spectrax/midpoint_solver.py:56-98 (residual F(y1) =
    y1 - y0 - dt f((y0 + y1)/2); a scaled 2-norm below 1 stops; the Newton
    system (I - dt/2 J(y_mid)) delta = -F linearised at the current iterate)
    with each system solved by restarted GMRES(restart) to the relative
    tolerance gmres_tol (restart 30 / tol 1e-10 by default, a deliberate
    difference from the reference's Eisenstat-Walker tolerance); J v from
    ``jvp_quadratic``.  Returns (y1, y_error, Newton iterations, products)."""
    f0 = f(y0)
    y1_init = y0 + dt * f0
    y1 = y1_init.copy()
    newton = mv = 0
    for _ in range(max_iters):
        ymid = 0.5 * (y0 + y1)
        res = y1 - y0 - dt * f(ymid)
        scale = atol + rtol * np.maximum(np.abs(y0), np.abs(y1))
        if np.linalg.norm(res / scale) < 1.0:
            break
        delta, _rel, its = gmres(lambda v: v - 0.5 * dt * jvp_quadratic(f, ymid, v), -res, restart, gmres_tol,
                                 gmres_maxiter)
        y1 = y1 + delta
        newton += 1
        mv += its
    return y1, y1 - y1_init, newton, mv


def controller_factor(errnorm, accepted, order=2.0):
    """Diffrax PIDController defaults with error order `order` (2 for this solver)."""
    if errnorm == 0.0:
        f = 10.0
    elif not np.isfinite(errnorm):
        f = 0.2
    else:
        f = 0.9 * errnorm ** (-1.0 / order)
    return min(max(f, 1.0 if accepted else 0.2), 10.0)


def solve(f, t1, y0, dt0, ts, rtol=1e-10, atol=1e-10, ctrl_rtol=1e-6, ctrl_atol=1e-6, adaptive=True,
          step_fn=None, max_steps=100000):
    """Implicit midpoint from 0 to t1 as spectrax/_simulation.py:164-180 runs it.

    adaptive: Diffrax's PIDController (ctrl_rtol, ctrl_atol) on the RMS of
    y_error / (ctrl_atol + ctrl_rtol max(|y0|, |y1|)) with y_error = y1 - y1_init
    (spectrax/midpoint_solver.py:51) and error order 2; steps end only on t1 and a
    save time inside an accepted step gets the linear interpolation of the step's
    end points (LocalLinearInterpolation, midpoint_solver.py:24).  Otherwise steps
    of dt0 that land on every save time.  step_fn(f, y, h) -> (y1, y_error) defaults
    to the dense-Newton ``step``.  Returns dict(ys, accepted, rejected, t)."""
    step_fn = step_fn or (lambda ff, y, h: step(ff, y, h, rtol, atol)[:2])
    ts = np.asarray(ts, np.float64)
    y = np.array(y0, np.complex128)
    t, h_prop = 0.0, float(dt0)
    isave, saved, acc, rej = 0, [], 0, 0
    while isave < len(ts) and ts[isave] <= t:
        saved.append(y.copy())
        isave += 1
    while t < t1 * (1 - 1e-15):
        if acc + rej >= max_steps:
            raise RuntimeError("max_steps reached")
        t_stop = t1 if adaptive else (min(ts[isave], t1) if isave < len(ts) else t1)
        h, landed = h_prop, False
        if t + h * (1 + 1e-9) >= t_stop:
            h, landed = t_stop - t, True
        y1, yerr = step_fn(f, y, h)
        if adaptive:
            scale = ctrl_atol + ctrl_rtol * np.maximum(np.abs(y), np.abs(y1))
            r = yerr / scale
            en = float(np.sqrt(np.mean(r.real ** 2 + r.imag ** 2)))
            accepted = en < 1.0
            h_next = h * controller_factor(en, accepted)
        else:
            accepted, h_next = True, h_prop
        if not accepted:
            rej += 1
            h_prop = h_next
            continue
        t_new = t_stop if landed else t + h
        while isave < len(ts) and ts[isave] <= t_new:
            if adaptive and ts[isave] != t_new:
                w = (ts[isave] - t) / h
                saved.append(y + w * (y1 - y))
            else:
                saved.append(y1.copy())
            isave += 1
        y, t = y1, t_new
        acc += 1
        h_prop = h_next if adaptive else h_prop
    return dict(ys=np.stack(saved), accepted=acc, rejected=rej, t=t, y=y)
