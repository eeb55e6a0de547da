"""Device Dopri8 solver and the ``simulation`` driver (spectrax/_simulation.py:113-194).

``Dopri8Solver`` wraps ``spx_dopri8_*``: stage buffers, a CUDA graph of step
attempts, and an on-device controller (Diffrax PIDController defaults or a
constant step).  ``simulation`` mirrors the reference driver: it builds the
merged parameters, integrates from 0 to t_max saving at
``linspace(0, t_max, timesteps)``, and returns the same output dictionary
(Ck, Fk, time, dCk, the parameters and the energy diagnostics).

Save times follow Diffrax's ``SaveAt(ts)`` by default (``saveat="interpolate"``):
steps are shortened only to end on t_max, and a save time inside an accepted
step gets that step's dense output (``tableau.DENSE``: a degree-8 continuous
extension of the 13 stages, order 4 for every problem and order 8 on linear
ones).  ``saveat="land"`` instead shortens steps to end exactly on every save
time.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .params import Dopri8, ImplicitMidpoint, initial_state, initialize_simulation_parameters
from .vector_field import Plan, _stream_ptr, plan_for_params


def species_masses(params):
    """spectrax/_diagnostics.py:44-68: (1, mi_me) for two species, else ``ms``/ones."""
    Ns = int(params["Ns"])
    if "ms" in params:
        return np.asarray(params["ms"], np.float64)
    if "masses" in params:
        return np.asarray(params["masses"], np.float64)
    if Ns == 2 and "mi_me" in params:
        return np.array([1.0, float(params["mi_me"])])
    return np.ones(Ns)


_SAVEAT_MODES = {"interpolate": 0, "land": 1}


def _saveat_code(saveat: str) -> int:
    if saveat not in _SAVEAT_MODES:
        raise ValueError("saveat must be 'interpolate' (Diffrax SaveAt(ts)) or 'land'")
    return _SAVEAT_MODES[saveat]


class DeviceWaitTimeout(RuntimeError):
    """A bounded device-side wait gave up (status SPX_ST_WAIT_TIMEOUT); the solve
    stopped and its state is not a valid trajectory point."""


def _check_wait(status: int) -> int:
    if status == _lib.SPX_ST_WAIT_TIMEOUT:
        raise DeviceWaitTimeout("Dopri8 solve stopped: a bounded device-side wait timed out")
    return status


class Dopri8Solver:
    def __init__(self, plan: Plan, t0: float, t1: float, dt0: float, ts=None, adaptive=True,
                 rtol=1e-10, atol=1e-12, max_steps=1_000_000, save_states=True, masses=None,
                 hermitian=True, persistent=False, saveat="interpolate"):
        L = _lib.lib()
        self.plan = plan
        self.ts = np.ascontiguousarray(np.asarray([] if ts is None else ts, np.float64))
        self.nsave = len(self.ts)
        self.Ns = plan.problem.Ns
        self._masses = np.ascontiguousarray(np.ones(self.Ns) if masses is None else np.asarray(masses, np.float64))
        o = _lib.spx_dopri8_opts()
        o.t0, o.t1, o.dt0, o.rtol, o.atol = float(t0), float(t1), float(dt0), float(rtol), float(atol)
        o.adaptive = 1 if adaptive else 0
        o.nsave = self.nsave
        o.save_ts = self.ts.ctypes.data_as(C.POINTER(C.c_double)) if self.nsave else None
        o.max_steps = int(max_steps)
        o.save_states = 1 if save_states else 0
        o.masses = self._masses.ctypes.data_as(C.POINTER(C.c_double))
        # detect an exactly Hermitian y0 at reset (odd Nx, fused 1D1V path) and use
        # packed real transforms for it
        o.hermitian = 1 if hermitian else 0
        # optional: one cooperative launch per replay, stages chained by per-CTA
        # completion counters (same results bit for bit; not faster on the
        # two-stream workload, where the stages are FP64-issue bound); land mode only
        o.persistent = 1 if persistent else 0
        o.saveat = _saveat_code(saveat)
        self.saveat = saveat
        self.save_states = bool(save_states)
        h = C.c_void_p()
        with torch.cuda.device(plan.device):
            _lib.check(L.spx_dopri8_create(plan.handle, C.byref(o), C.byref(h)), "spx_dopri8_create")
        self.handle = h

    def reset(self, y0, stream=None):
        """Start a new solve from y0 (stream-ordered; a page-locked complex128 host
        tensor is copied straight from host memory and must not change until the
        stream has consumed it)."""
        t = torch.as_tensor(y0)
        if t.device.type == "cpu" and t.is_pinned() and t.dtype == torch.complex128 and t.is_contiguous():
            if t.numel() != self.plan.state_len:
                raise ValueError(f"y0 must have {self.plan.state_len} entries")
        else:
            t = t.to(self.plan.device, torch.complex128).contiguous()
            self.plan.check_state(t, "y0")
        self._y0 = t                     # alive until the copy has run (next reset at the earliest)
        _lib.check(_lib.lib().spx_dopri8_reset(self.handle, C.c_void_p(t.data_ptr()), _stream_ptr(stream)),
                   "spx_dopri8_reset")
        return self

    def advance(self, attempts: int, stream=None) -> int:
        st = C.c_int32()
        _lib.check(_lib.lib().spx_dopri8_advance(self.handle, int(attempts), _stream_ptr(stream), C.byref(st)),
                   "spx_dopri8_advance")
        return _check_wait(int(st.value))

    def enqueue(self, attempts: int, stream=None):
        """Queue exactly `attempts` step attempts without synchronising."""
        _lib.check(_lib.lib().spx_dopri8_enqueue(self.handle, int(attempts), _stream_ptr(stream)),
                   "spx_dopri8_enqueue")

    def run(self, stream=None) -> int:
        st = C.c_int32()
        _lib.check(_lib.lib().spx_dopri8_run(self.handle, _stream_ptr(stream), C.byref(st)), "spx_dopri8_run")
        return _check_wait(int(st.value))

    def set_wait_test(self, polls: int = 0, unreachable: bool = False):
        """Fault-handling test hook (spx_dopri8_set_wait_test): the persistent
        kernel's counter waits give up after `polls` polls (0: default); with
        `unreachable` they wait for a count no CTA publishes.  From the next reset."""
        _lib.check(_lib.lib().spx_dopri8_set_wait_test(self.handle, int(polls), 1 if unreachable else 0),
                   "spx_dopri8_set_wait_test")

    def stats(self, stream=None) -> dict:
        s = _lib.spx_dopri8_stats()
        _lib.check(_lib.lib().spx_dopri8_stats_get(self.handle, C.byref(s), _stream_ptr(stream)), "stats")
        return dict(t=s.t, dt=s.dt, accepted=s.accepted, rejected=s.rejected, rhs_evals=s.rhs_evals,
                    status=s.status, status_name=_lib.STATUS_NAMES.get(s.status, "?"), saved=s.saved,
                    hermitian=bool(s.hermitian), persistent=bool(s.persistent))

    def _copy(self, what, out):
        _lib.check(_lib.lib().spx_dopri8_copy(self.handle, what, C.c_void_p(out.data_ptr()),
                                              out.numel() * out.element_size(), _stream_ptr()), "copy")
        return out

    def state(self) -> torch.Tensor:
        return self._copy(0, torch.empty(self.plan.state_len, dtype=torch.complex128, device=self.plan.device))

    def saved_states(self) -> torch.Tensor:
        out = torch.empty((self.nsave, self.plan.state_len), dtype=torch.complex128, device=self.plan.device)
        return self._copy(1, out) if self.nsave else out

    def energies(self) -> torch.Tensor:
        out = torch.empty((self.nsave, 2 + self.Ns), dtype=torch.float64, device=self.plan.device)
        return self._copy(2, out) if self.nsave else out

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            try:
                _lib._lib.spx_dopri8_destroy(h)
            except Exception:
                pass
            self.handle = None


# Diffrax PIDController defaults, the same as the device controller (csrc/spx_tableau.cuh)
_SAFETY, _FACTORMIN, _FACTORMAX, _EXPONENT, _SNAP = 0.9, 0.2, 10.0, -1.0 / 8.0, 1e-9


def _controller_factor(en: float, accepted: bool) -> float:
    if en == 0.0:
        f = _FACTORMAX
    elif not np.isfinite(en):
        f = _FACTORMIN
    else:
        f = _SAFETY * en ** _EXPONENT
    return min(max(f, 1.0 if accepted else _FACTORMIN), _FACTORMAX)


def host_dopri8_solve(plan: Plan, y0, t1: float, dt0: float, ts=None, adaptive=True, rtol=1e-10,
                      atol=1e-12, max_steps=1_000_000, stream=None, saveat="interpolate"):
    """Dopri8 driven from the host around the plain right-hand side ``plan.rhs_into``.

    This is how an external solver uses the drop-in vector field (the role
    Diffrax plays for spectrax/_simulation.py:164-180): one RHS launch per
    stage, the stage combinations as separate device operations, and the
    step-size decision on the host after each attempt (one device-to-host read
    per step).  Same tableau, controller and save-time rule as the device
    solver.  Returns (final state, saved states (len(ts), n), stats dict)."""
    from .tableau import A, B, DENSE, E, dense_weights
    interp = _saveat_code(saveat) == 0
    y = torch.as_tensor(y0).to(plan.device, torch.complex128).contiguous().clone()
    plan.check_state(y, "y0")
    ts = np.asarray([] if ts is None else ts, np.float64)
    K = [torch.empty_like(y) for _ in range(13)]
    S = torch.empty_like(y)
    ynew = torch.empty_like(y)
    err = torch.empty_like(y)
    saved = torch.empty((len(ts), y.numel()), dtype=torch.complex128, device=y.device)
    t, dt = 0.0, float(dt0)
    isave = 0
    while isave < len(ts) and ts[isave] <= t:
        saved[isave].copy_(y)
        isave += 1
    acc = rej = evals = 0
    k1_valid = False
    status = "DONE" if t >= t1 else "RUNNING"
    while status == "RUNNING":
        t_stop = min(ts[isave], t1) if (isave < len(ts) and not interp) else t1
        h, landed = dt, False
        if t + h * (1.0 + _SNAP) >= t_stop:
            h, landed = t_stop - t, True
        if h <= 0.0 or t + h == t:
            status = "DT_UNDERFLOW"
            break
        if acc + rej >= max_steps:
            status = "MAX_STEPS"
            break
        for i in range(13):
            if i == 0:
                if not k1_valid:
                    plan.rhs_into(y, K[0], stream)
                continue
            S.copy_(y)
            for j, a in A[i].items():
                S.add_(K[j], alpha=h * a)
            plan.rhs_into(S, K[i], stream)
        ynew.copy_(y)
        err.zero_()
        for j in range(13):
            if B[j] != 0.0:
                ynew.add_(K[j], alpha=h * B[j])
            if E[j] != 0.0:
                err.add_(K[j], alpha=h * E[j])
        evals += 12 if k1_valid else 13
        nonfinite = False
        if adaptive:
            # one device-to-host read per attempt: the error norm and the finiteness of y_new
            sc = atol + rtol * torch.maximum(y.abs(), ynew.abs())
            en_t = torch.sqrt(torch.mean((err.abs() / sc) ** 2))
            bad = (~torch.isfinite(torch.view_as_real(ynew)).all()).to(torch.float64)
            en, nf = torch.stack([en_t, bad]).tolist()
            nonfinite = nf != 0.0
            accept = en < 1.0
            dt_next = h * _controller_factor(en, accept)
            if accept and landed and dt_next < dt:
                dt_next = dt
        else:
            accept, dt_next = True, dt
        if accept:
            t_old = t
            t = t_stop if landed else t + h
            y, ynew = ynew, y
            acc += 1
            k1_valid = False
            while isave < len(ts) and ts[isave] <= t:
                if interp and ts[isave] != t:
                    # dense output of the step just taken (ynew now holds its start)
                    w = dense_weights((ts[isave] - t_old) / h)
                    saved[isave].copy_(ynew)
                    for j in range(13):
                        if any(DENSE[j]):
                            saved[isave].add_(K[j], alpha=h * w[j])
                else:
                    saved[isave].copy_(y)
                isave += 1
            if nonfinite:
                status = "NONFINITE"
            elif t >= t1:
                status = "DONE"
        else:
            rej += 1
            k1_valid = True
        dt = dt_next
    return y, saved, dict(t=t, dt=dt, accepted=acc, rejected=rej, rhs_evals=evals, status_name=status)


def solve(params, y0=None, t_max=None, dt=None, ts=None, adaptive=True, rtol=None, atol=None,
          max_steps=1_000_000, save_states=True, mask_mode=None, saveat="interpolate"):
    """Integrate one instance; returns (solver, status)."""
    plan = plan_for_params(params, mask_mode)
    y0 = initial_state(params) if y0 is None else y0
    t_max = float(params["t_max"] if t_max is None else t_max)
    dt = float(params["dt"] if dt is None else dt)
    tol = float(params.get("ode_tolerance", 1e-12))
    s = Dopri8Solver(plan, 0.0, t_max, dt, ts=ts, adaptive=adaptive,
                     rtol=tol if rtol is None else rtol, atol=tol if atol is None else atol,
                     max_steps=max_steps, save_states=save_states, masses=species_masses(params),
                     saveat=saveat)
    s.reset(torch.as_tensor(np.asarray(y0, np.complex128)))
    status = s.run()
    return s, status


def simulation(input_parameters=None, Nx=33, Ny=1, Nz=1, Nn=20, Nm=1, Np=1, Ns=2, timesteps=200,
               dt=0.01, solver=None, adaptive_time_step=True, mask_mode=None, max_steps=1_000_000,
               saveat="interpolate"):
    """Mirror of spectrax/_simulation.py:113-194 running on the GPU.

    ``saveat``: "interpolate" (the reference's Diffrax ``SaveAt(ts)``: dense
    output at the save times) or "land" (steps end on every save time)."""
    solver = Dopri8() if solver is None else solver
    p = initialize_simulation_parameters(input_parameters or {}, Nx, Ny, Nz, Nn, Nm, Np, Ns, timesteps, dt)
    time = np.linspace(0, p["t_max"], timesteps)
    if isinstance(solver, ImplicitMidpoint):
        from .midpoint import midpoint_solve
        ys, en, info = midpoint_solve(p, time, solver, mask_mode=mask_mode, adaptive=adaptive_time_step)
    elif plan_for_params(p, mask_mode).path == 2:
        # planes too large for the device stepper's shared memory: the same
        # tableau, controller and save rule driven from the host around spx_rhs
        plan = plan_for_params(p, mask_mode)
        from .midpoint import energies
        tol = float(p.get("ode_tolerance", 1e-12))
        _, saved, info = host_dopri8_solve(plan, initial_state(p), float(time[-1]), dt, ts=time,
                                           adaptive=adaptive_time_step, rtol=tol, atol=tol, max_steps=max_steps,
                                           saveat=saveat)
        if info["status_name"] != "DONE":
            raise RuntimeError(f"Dopri8 solve ended with status {info['status_name']}")
        masses = species_masses(p)
        en = np.array([[e, k] + list(ks) for e, k, ks in (energies(plan, y, masses) for y in saved)])
        ys = saved.cpu().numpy()
    else:
        s, status = solve(p, ts=time, adaptive=adaptive_time_step, dt=dt, max_steps=max_steps,
                          mask_mode=mask_mode, saveat=saveat)
        if status not in (1,):
            raise RuntimeError(f"Dopri8 solve ended with status {_lib.STATUS_NAMES.get(status, status)}")
        ys = s.saved_states().cpu().numpy()
        en = s.energies().cpu().numpy()
        info = s.stats()
    NF = 6 * Nx * Ny * Nz
    Ck = ys[:, :-NF].reshape(len(time), Ns * Nn * Nm * Np, Ny, Nx, Nz)
    Fk = ys[:, -NF:].reshape(len(time), 6, Ny, Nx, Nz)
    dCk = Ck.copy()
    c = (int((Ny - 1) / 2), int((Nx - 1) / 2), int((Nz - 1) / 2))
    dCk[:, 0, c[0], c[1], c[2]] = 0
    dCk[:, Nn * Nm * Np, c[0], c[1], c[2]] = 0
    out = {"Ck": Ck, "Fk": Fk, "time": time, "dCk": dCk, **p}
    out.update(diagnostics_from_energies(p, en))
    out["solver_stats"] = info
    return out


def diagnostics_from_energies(p, en):
    """Keys added by spectrax/_diagnostics.py:221-233 from the device energies."""
    Ns = int(p["Ns"])
    alpha_s = np.asarray(p["alpha_s"], np.float64)
    if Ns == 2 and "mi_me" in p:
        lam = np.sqrt(1.0 / (2.0 * (1.0 / alpha_s[0] ** 2 + 1.0 / (p["mi_me"] * alpha_s[3] ** 2))))
    else:
        ax = alpha_s.reshape(Ns, 3)[:, 0]
        lam = np.sqrt(1.0 / (2.0 * np.sum(1.0 / ax ** 2)))
    d = {"Ns": Ns, "lambda_D": lam, "k_norm": np.sqrt(2.0) * np.pi * alpha_s[0] / p["Lx"],
         "EM_energy": en[:, 0], "kinetic_energy": en[:, 1], "kinetic_energy_species": en[:, 2:],
         "total_energy": en[:, 0] + en[:, 1]}
    for s in range(Ns):
        d[f"kinetic_energy_species{s + 1}"] = en[:, 2 + s]
    return d

