"""Implicit midpoint stepper with Newton-GMRES on the device (spectrax/midpoint_solver.py).

Each step solves F(y1) = y1 - y0 - dt f((y0 + y1)/2) = 0 by Newton iterations
from the explicit-Euler guess; every Newton system (I - dt/2 J(y_mid)) delta = -F
is solved matrix-free by restarted GMRES whose matrix-vector product is the
hand-written linearised right-hand side (``spx_linearize`` once per Newton
system, then ``spx_jvp_lin`` per product).  The Newton stopping rule is
the reference's (scaled 2-norm < 1, at most 300 iterations,
spectrax/midpoint_solver.py:56-98); the inner solve uses restart 30 and, by
default, a fixed relative tolerance of 1e-10 (parity on the converged root), or
with gmres_tol=None the reference's Eisenstat-Walker tolerance min(0.1, norm/2)
with absolute tolerance atol, at most 20 restarts.

Krylov vectors live in one (restart+1, n) complex128 block on the device; the
orthogonalisation is classical Gram-Schmidt with one re-orthogonalisation pass
against the rows built so far (``spx_krylov_cgs2``: four streaming passes, the
projections and the norm come back in one copy); the small Hessenberg
least-squares problem is solved on the host with Givens rotations.
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

import ctypes as C

from . import _lib
from .params import ImplicitMidpoint
from .vector_field import Plan, _stream_ptr, plan_for_params


class NewtonGMRES:
    def __init__(self, plan: Plan, restart=30, gmres_tol=1e-10, gmres_maxiter=20):
        self.plan = plan
        self.m = int(restart)
        if not 1 <= self.m < _lib.KRYLOV_MAX_ROWS:
            raise ValueError(f"restart must be in [1, {_lib.KRYLOV_MAX_ROWS - 1}]")
        # None: the reference's Eisenstat-Walker rule, set per Newton system by step()
        self.tol = None if gmres_tol is None else float(gmres_tol)
        self.maxiter = int(gmres_maxiter)
        n = plan.state_len
        dev = plan.device
        self.n = n
        self.V = torch.empty((self.m + 1, n), dtype=torch.complex128, device=dev)
        self.w = torch.empty(n, dtype=torch.complex128, device=dev)
        self.jv = torch.empty(n, dtype=torch.complex128, device=dev)
        self.hout = torch.empty(self.m + 2, dtype=torch.complex128, device=dev)
        self.kws = torch.empty(int(_lib.lib().spx_krylov_ws_bytes(n)), dtype=torch.uint8, device=dev)
        # J(ymid) linearised once per Newton system (jax.linearize,
        # spectrax/midpoint_solver.py:75), reused by every GMRES product
        self.lin = torch.empty(plan.linearize_bytes, dtype=torch.uint8, device=dev)
        self.matvecs = 0

    def _A(self, ymid, v, out, c):
        """out = v - c * J(ymid) v, with J(ymid) from the last ``linearize``."""
        self.plan.jvp_lin_into(self.lin, v, self.jv)
        torch.add(v, self.jv, alpha=-c, out=out)
        self.matvecs += 1
        return out

    def _cgs2(self, k):
        """Orthogonalise w against V[:k]; returns (projections h (k,), ||w||)."""
        _lib.check(_lib.lib().spx_krylov_cgs2(C.c_void_p(self.V.data_ptr()), C.c_int64(self.n), C.c_int32(k),
                                              C.c_void_p(self.w.data_ptr()), C.c_void_p(self.hout.data_ptr()),
                                              C.c_void_p(self.kws.data_ptr()), C.c_size_t(self.kws.numel()),
                                              _stream_ptr(None)), "spx_krylov_cgs2")
        hv = self.hout[: k + 1].cpu().numpy()
        return hv[:k], float(hv[k].real)

    def _axpy(self, k, coef, x):
        """x += sum_{i<k} coef[i] V[i] (coef: device complex128)."""
        _lib.check(_lib.lib().spx_krylov_axpy(C.c_void_p(self.V.data_ptr()), C.c_int64(self.n), C.c_int32(k),
                                              C.c_void_p(coef.data_ptr()), C.c_void_p(x.data_ptr()),
                                              _stream_ptr(None)), "spx_krylov_axpy")

    def solve(self, ymid, b, c, atol=0.0, tol=None, deadline=None):
        """Solve (I - c J(ymid)) x = b to ||r|| <= max(tol ||b||, atol) (tol: this
        call's relative tolerance, default the solver's); returns (x, relative
        residual, iterations).  deadline (time.perf_counter() value): stop the
        Arnoldi process there and return the current iterate."""
        V, w, m = self.V, self.w, self.m
        tol = self.tol if tol is None else tol
        self.plan.linearize(ymid, self.lin)
        x = torch.zeros_like(b)
        bnorm = torch.linalg.vector_norm(b).item()
        if bnorm == 0.0:
            return x, 0.0, 0
        target = max(tol * bnorm, atol)
        r = b.clone()
        beta = bnorm
        its = 0
        rel = 1.0
        for _cycle in range(self.maxiter):
            torch.div(r, beta, out=V[0])
            H = np.zeros((m + 1, m), np.complex128)
            cs = np.zeros(m, np.complex128)
            sn = np.zeros(m, np.complex128)
            g = np.zeros(m + 1, np.complex128)
            g[0] = beta
            k_done = 0
            for j in range(m):
                self._A(ymid, V[j], w, c)
                its += 1
                hh, hn = self._cgs2(j + 1)          # classical Gram-Schmidt, twice
                H[: j + 1, j] = hh
                H[j + 1, j] = hn
                # apply previous rotations, then a new one
                for i in range(j):
                    t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                    H[i + 1, j] = -np.conj(sn[i]) * H[i, j] + np.conj(cs[i]) * H[i + 1, j]
                    H[i, j] = t
                a, bb = H[j, j], H[j + 1, j]
                den = math.sqrt(abs(a) ** 2 + abs(bb) ** 2)
                if den == 0.0:
                    cs[j], sn[j] = 1.0, 0.0
                else:
                    cs[j] = a / den
                    sn[j] = bb / den
                    if abs(a) > 0:
                        cs[j] = abs(a) / den
                        sn[j] = (a / abs(a)) * np.conj(bb) / den
                H[j, j] = cs[j] * a + sn[j] * bb
                H[j + 1, j] = 0.0
                g[j + 1] = -np.conj(sn[j]) * g[j]
                g[j] = cs[j] * g[j]
                k_done = j + 1
                res = abs(g[j + 1])
                if hn > 0.0 and j + 1 < m + 1:
                    torch.div(w, hn, out=V[j + 1])
                if res <= target or hn == 0.0:
                    break
                if deadline is not None and time.perf_counter() > deadline:
                    break
            # back substitution and update
            k = k_done
            yk = np.zeros(k, np.complex128)
            for i in reversed(range(k)):
                yk[i] = (g[i] - np.dot(H[i, i + 1:k], yk[i + 1:k])) / H[i, i]
            if k > 0:
                self._axpy(k, torch.from_numpy(yk).to(V.device), x)
            # true residual for the restart
            self._A(ymid, x, w, c)
            r = b - w
            beta = torch.linalg.vector_norm(r).item()
            rel = beta / bnorm
            if beta <= target or (deadline is not None and time.perf_counter() > deadline):
                break
        return x, rel, its


class _Glue:
    """Device buffers of one step (y_mid, f(y_mid), residual, the two reduced sums)."""

    def __init__(self, plan: Plan, ws):
        self.plan, self.ws = plan, ws
        self.ymid = torch.empty(plan.state_len, dtype=torch.complex128, device=plan.device)
        self.fmid = torch.empty_like(self.ymid)
        self.res = torch.empty_like(self.ymid)
        self.sums = torch.empty(2, dtype=torch.float64, device=plan.device)

    def residual(self, y0, y1, f, dt, rtol, atol, store=True):
        """Scaled squared 2-norm of y1 - y0 - dt f (and the residual in self.res when store);
        one 16-byte device-to-host read."""
        _lib.check(_lib.lib().spx_midpoint_residual(
            self.plan.state_len, C.c_void_p(y0.data_ptr()), C.c_void_p(y1.data_ptr()), C.c_void_p(f.data_ptr()),
            float(dt), float(rtol), float(atol), C.c_void_p(self.res.data_ptr()) if store else None,
            C.c_void_p(self.sums.data_ptr()), C.c_void_p(self.ws.data_ptr()), C.c_size_t(self.ws.numel()),
            _stream_ptr(None)), "spx_midpoint_residual")
        sq, bad = self.sums.tolist()
        if bad != 0.0:
            raise FloatingPointError("implicit midpoint: non-finite residual")
        return sq

    def update(self, y0, y1, delta=None, sign=1.0):
        """y1 += sign delta; y_mid = (y0 + y1) / 2."""
        _lib.check(_lib.lib().spx_midpoint_update(
            self.plan.state_len, C.c_void_p(y0.data_ptr()), C.c_void_p(y1.data_ptr()),
            C.c_void_p(delta.data_ptr()) if delta is not None else None, float(sign),
            C.c_void_p(self.ymid.data_ptr()), _stream_ptr(None)), "spx_midpoint_update")


def step(plan: Plan, y0, dt, rtol, atol, max_iters=300, solver: NewtonGMRES | None = None, stats=None,
         glue: _Glue | None = None, f0=None, want_error=True, deadline=None):
    """One implicit midpoint step; returns (y1, y_error, f0) with y_error = y1 - (y0 + dt f(y0))
    (spectrax/midpoint_solver.py:37-53; None unless want_error).  Per Newton iteration: one right-hand side at
    y_mid, one fused residual + scaled-norm pass with a single scalar read, the GMRES
    solve, and one fused update of y1 and y_mid."""
    solver = solver or NewtonGMRES(plan)
    glue = glue or _Glue(plan, solver.kws)
    f0 = plan.rhs(y0) if f0 is None else f0
    y1 = torch.add(y0, f0, alpha=dt)               # the explicit-Euler guess y1_init
    glue.update(y0, y1)
    newton = 0
    for _ in range(max_iters):
        plan.rhs_into(glue.ymid, glue.fmid)
        norm = math.sqrt(glue.residual(y0, y1, glue.fmid, dt, rtol, atol))
        if norm < 1.0:
            break
        # (I - dt/2 J(y_mid)) delta = -res: solve with +res and subtract.  A solver
        # without its own tolerance takes the reference's Eisenstat-Walker rule:
        # relative min(0.1, norm / 2), absolute atol (spectrax/midpoint_solver.py:80-89)
        if solver.tol is None:
            delta, _rel, _its = solver.solve(glue.ymid, glue.res, 0.5 * dt, atol=atol, tol=min(0.1, 0.5 * norm),
                                             deadline=deadline)
        else:
            delta, _rel, _its = solver.solve(glue.ymid, glue.res, 0.5 * dt, atol=0.0, deadline=deadline)
        glue.update(y0, y1, delta, -1.0)
        newton += 1
        if deadline is not None and time.perf_counter() > deadline:
            # a caller's wall-clock limit (benchmarks): the step is left unconverged
            if stats is not None:
                stats["deadline"] = True
            break
    if stats is not None:
        stats["newton"] = stats.get("newton", 0) + newton
        stats["rhs"] = stats.get("rhs", 0) + newton + 2
    return y1, (y1 - y0 - dt * f0) if want_error else None, f0


def energies(plan: Plan, y: torch.Tensor, masses):
    """EM and kinetic energies of one state (spectrax/_diagnostics.py:191-219), real parts."""
    pb = plan.problem
    Ny, Nx, Nz, Nn, Nm, Np, Ns = pb.Ny, pb.Nx, pb.Nz, pb.Nn, pb.Nm, pb.Np, pb.Ns
    plane = Nx * Ny * Nz
    nc = Ns * Nn * Nm * Np * plane
    F = y[nc:]
    em = 0.5 * float(pb.Omega_cs[0]) ** 2 * torch.sum(F.real ** 2 + F.imag ** 2).item()
    kc = ((Ny // 2) * Nx + Nx // 2) * Nz + Nz // 2
    Hs = Nn * Nm * Np
    offs = [0, 1, Nn, Nn * Nm, 2, 2 * Nn, 2 * Nn * Nm]
    idx = [(s * Hs + o) * plane + kc for s in range(Ns) for o in offs]
    vals = y[torch.tensor([min(i, nc - 1) for i in idx], device=y.device)].real.cpu().numpy().reshape(Ns, 7)
    ke = []
    for s in range(Ns):
        c = [vals[s, k] if offs[k] < Hs else 0.0 for k in range(7)]
        a0, a1, a2 = (float(pb.alpha_s[3 * s + d]) for d in range(3))
        u0, u1, u2 = (float(pb.u_s[3 * s + d]) for d in range(3))
        pref = 0.5 * masses[s] * a0 * a1 * a2
        t0 = 0.5 * (a0 * a0 + a1 * a1 + a2 * a2) + (u0 * u0 + u1 * u1 + u2 * u2)
        t1 = math.sqrt(2.0) * (a0 * u0 * c[1] + a1 * u1 * c[2] + a2 * u2 * c[3])
        t2 = (a0 * a0 * c[4] + a1 * a1 * c[5] + a2 * a2 * c[6]) / math.sqrt(2.0)
        ke.append(pref * (t0 * c[0] + t1 + t2))
    return em, sum(ke), ke


# Diffrax PIDController defaults (the Dopri8 stepper's), with the error order of this
# order-2 solver: the next step is h clip(0.9 err^(-1/2), 1 if kept else 0.2, 10)
_SAFETY, _FACTORMIN, _FACTORMAX, _ORDER = 0.9, 0.2, 10.0, 2.0


def controller_factor(en: float, accepted: bool) -> float:
    if en == 0.0:
        f = _FACTORMAX
    elif not math.isfinite(en):
        f = _FACTORMIN
    else:
        f = _SAFETY * en ** (-1.0 / _ORDER)
    return min(max(f, 1.0 if accepted else _FACTORMIN), _FACTORMAX)


def solve(plan: Plan, y0, t_max, dt, ts, solver: ImplicitMidpoint, masses, save_states=True, adaptive=False,
          ctrl_rtol=None, ctrl_atol=None, max_steps=1_000_000):
    """Implicit midpoint from 0 to t_max, saving at ts.

    adaptive=False: steps of dt, landing exactly on each save time.
    adaptive=True (the reference's default, spectrax/_simulation.py:164-180): steps
    end only on t_max; the step size follows Diffrax's PIDController on the RMS of
    y_error / (ctrl_atol + ctrl_rtol max(|y0|, |y1|)), error order 2; a save time
    inside an accepted step gets the linear interpolation of its end points (the
    solver's LocalLinearInterpolation, spectrax/midpoint_solver.py:24).
    Returns (saved states or None, energies (len(ts), 2 + Ns), info)."""
    ts = np.asarray(ts, np.float64)
    ng = NewtonGMRES(plan, restart=solver.restart, gmres_tol=solver.gmres_tol)
    glue = _Glue(plan, ng.kws)
    y = torch.as_tensor(y0).to(plan.device, torch.complex128).contiguous().clone()
    n = plan.state_len
    t = 0.0
    isave = 0
    ys, en = [], []
    info = {"steps": 0, "rejected": 0}

    def save(yy):
        if save_states:
            ys.append(yy.clone())
        e, k, ks = energies(plan, yy, masses)
        en.append([e, k] + list(ks))

    while isave < len(ts) and ts[isave] <= t:
        save(y)
        isave += 1
    h_prop = float(dt)
    f0 = None
    while t < t_max * (1 - 1e-15):
        if info["steps"] + info["rejected"] >= max_steps:
            raise RuntimeError("implicit midpoint: max_steps reached")
        t_stop = t_max if adaptive else (min(ts[isave], t_max) if isave < len(ts) else t_max)
        h, landed = h_prop, False
        if t + h * (1 + 1e-9) >= t_stop:
            h, landed = t_stop - t, True
        y1, _, f0 = step(plan, y, h, solver.rtol, solver.atol, solver.max_iters, ng, info, glue, f0,
                         want_error=False)
        if adaptive:
            sq = glue.residual(y, y1, f0, h, ctrl_rtol, ctrl_atol, store=False)
            e = math.sqrt(sq / n)
            accept = e < 1.0
            h_next = h * controller_factor(e, accept)
        else:
            accept, h_next = True, h_prop
        if not accept:
            info["rejected"] += 1
            h_prop = h_next
            continue
        t_new = t_stop if landed else t + h
        while isave < len(ts) and ts[isave] <= t_new:
            if adaptive and ts[isave] != t_new:
                w = (ts[isave] - t) / h
                save(torch.lerp(y, y1, w))
            else:
                save(y1)
            isave += 1
        y, t = y1, t_new
        f0 = None                                    # f(y) of the new state next step
        info["steps"] += 1
        h_prop = h_next if adaptive else h_prop
    info["matvecs"] = ng.matvecs
    info["t"] = t
    info["y"] = y                                    # the final state (device)
    ys_np = torch.stack(ys).cpu().numpy() if save_states and ys else None
    return ys_np, np.array(en), info


def midpoint_solve(p, time, solver: ImplicitMidpoint, mask_mode=None, adaptive=False):
    """Driver used by ``simulation(..., solver=ImplicitMidpoint(...))``."""
    from .dopri8 import species_masses
    from .params import initial_state
    plan = plan_for_params(p, mask_mode)
    tol = float(p.get("ode_tolerance", 1e-12))
    ys, en, info = solve(plan, initial_state(p), float(p["t_max"]), float(p["dt"]), time, solver,
                         species_masses(p), adaptive=adaptive, ctrl_rtol=tol, ctrl_atol=tol)
    return ys, en, info
