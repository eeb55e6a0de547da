"""Hand-written discrete adjoint of fixed-step Dopri8, with sqrt(N) checkpointing.

The reference has no adjoint code: gradients would come from ``jax.grad``
through ``diffeqsolve``.  Here the gradient of a scalar loss of the field-energy
history is computed exactly for the discrete solution:

* forward: the fused device stepper (``Dopri8Solver``), keeping every
  m-th state (m = ceil(sqrt(N))) and the field energy of every step;
* backward, segment by segment in reverse: recompute the segment's steps with
  ``spx_rk_step_store_ex`` (keeping the 13 stage inputs of each step), then sweep
  back through the steps with the Runge-Kutta adjoint recursion
      gk_j = h b_j lam + sum_{i>j} h a_ij gY_i ,   gY_j = J(Y_j)^H gk_j ,
      lam_n = lam_{n+1} + sum_j gY_j ,
  using ``spx_vjp_param_ex`` (plain transpose, plus the parameter sums) on
  conjugated adjoints:
  conj(J^H lam) = J^T conj(lam), so every adjoint vector is stored conjugated;
* parameter gradients accumulate Re sum conj(gk_j) . df/dtheta(Y_j) on the device
  (in the same launch) for theta = (nu, k, u_x per species), plus the
  initial-state terms for k and the perturbation amplitude;
* an exactly Hermitian trajectory (odd Nx, the spectrum of real fields) runs all
  three on packed real transforms (``hermitian=True``, the default);
* 2-D / 3-D layouts: the same recursion for the state gradient, the steps
  recomputed with ``spx_rhs`` and device linear combinations, the sweep on
  ``spx_vjp`` (no parameter sums).

``TwoStreamLoss`` puts this behind ``torch.autograd.Function`` for the adjoint
workload (1D1V two-stream, loss = LSQ slope of log E over t in [10, 40] plus
the final field energy; parameters k, nu, u, amplitude).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from .dopri8 import Dopri8Solver
from .params import initialize_simulation_parameters
from .vector_field import Plan, _stream_ptr, plan_for_params

from .tableau import A as _A, B as _B, S


def _ptr(t: torch.Tensor):
    return C.c_void_p(t.data_ptr())


def lincomb(out: torch.Tensor, terms):
    """out = sum c_i v_i on the device (terms: list of (coef, tensor), <= 16)."""
    terms = [(float(c), v) for c, v in terms if c != 0.0]
    n = len(terms)
    vecs = (C.c_void_p * max(1, n))(*[v.data_ptr() for _, v in terms])
    coefs = (C.c_double * max(1, n))(*[c for c, _ in terms])
    _lib.check(_lib.lib().spx_lincomb(out.numel(), n, vecs, coefs, _ptr(out), _stream_ptr()), "spx_lincomb")
    return out


class Dopri8Adjoint:
    """Fixed-step Dopri8 trajectory with its discrete adjoint."""

    def __init__(self, plan: Plan, dt: float, nsteps: int, ckpt_every: int | None = None, masses=None,
                 hermitian=True):
        pb = plan.problem
        # 2-D / 3-D layouts: the state gradient only (no parameter sums), with
        # the steps recomputed through spx_rhs and the sweep through spx_vjp
        self.general = not (pb.Ny == 1 and pb.Nz == 1 and pb.Nm == 1 and pb.Np == 1)
        self.plan, self.dt, self.N = plan, float(dt), int(nsteps)
        # exactly Hermitian trajectories (the spectra of real fields) run the
        # forward, the recomputation and the adjoint sweep on packed transforms;
        # the adjoint of a Hermitian state stays exactly Hermitian
        self.hermitian = bool(hermitian) and not self.general
        self.herm = False
        self.m = int(ckpt_every or math.ceil(math.sqrt(self.N)))
        self.masses = masses
        self.n = plan.state_len
        self.nc = self.n - 6 * pb.Nx * pb.Ny * pb.Nz
        self.O0 = float(plan.problem.Omega_cs[0])
        dev = plan.device
        self.ts = np.arange(self.N + 1) * self.dt

    # ------------------------------------------------------------------ forward
    def forward(self, y0: torch.Tensor):
        # the stage kernels the recomputation uses too: packed real transforms when
        # y0 is exactly Hermitian (odd Nx), general complex transforms otherwise
        s = Dopri8Solver(self.plan, 0.0, self.ts[-1], self.dt, ts=self.ts, adaptive=False,
                         save_states=False, masses=self.masses, max_steps=self.N + 10,
                         hermitian=self.hermitian)
        s.reset(y0)
        ckpts = [y0.clone()]
        done = 0
        while done < self.N:
            k = min(self.m, self.N - done)
            s.advance(k)
            done += k
            ckpts.append(s.state())
        st = s.stats()
        if st["status"] != 1 or st["accepted"] != self.N:
            raise RuntimeError(f"forward solve failed: {st}")
        E = s.energies()[:, 0].clone()
        self.ckpts = ckpts
        self.herm = bool(st["hermitian"])
        return E, ckpts[-1]

    # ------------------------------------------------------------------ backward
    def _buffers(self):
        if getattr(self, "_buf", None) is None:
            dev, n, m = self.plan.device, self.n, self.m
            self._buf = dict(
                Ys=torch.empty((m + 1, S, n), dtype=torch.complex128, device=dev),
                Kb=torch.empty((S, n), dtype=torch.complex128, device=dev),
                gY=torch.empty((S, n), dtype=torch.complex128, device=dev),
                gk=torch.empty(n, dtype=torch.complex128, device=dev),
                mu=torch.empty(n, dtype=torch.complex128, device=dev),
                acc=torch.zeros(2 + self.plan.problem.Ns, dtype=torch.float64, device=dev),
                coef=torch.zeros(m + 1, dtype=torch.float64, device=dev),
            )
            self._graphs = {}
        return self._buf

    def _recompute(self, steps):
        """Recompute `steps` steps from Ys[0, 0], keeping the stage inputs Ys[q]."""
        B = self._buffers()
        L = _lib.lib()
        if self.general:
            # stage inputs Y_j = y + h sum_{i<j} a_ji K_i, K_j = f(Y_j); y' = y + h sum_j b_j K_j
            h, Kb = self.dt, B["Kb"]
            for q in range(steps):
                Yq, y = B["Ys"][q], B["Ys"][q, 0]
                for j in range(S):
                    if j > 0:
                        lincomb(Yq[j], [(1.0, y)] + [(h * _A.get(j, {}).get(i, 0.0), Kb[i]) for i in range(j)])
                    self.plan.rhs_into(Yq[j], Kb[j])
                lincomb(B["Ys"][q + 1, 0], [(1.0, y)] + [(h * _B[j], Kb[j]) for j in range(S)])
            return
        for q in range(steps):
            _lib.check(L.spx_rk_step_store_ex(self.plan.handle, _ptr(B["Ys"][q, 0]), C.c_double(self.dt),
                                              _ptr(B["Ys"][q]), _ptr(B["Kb"]), _ptr(B["Ys"][q + 1, 0]),
                                              int(self.herm), _stream_ptr()), "spx_rk_step_store_ex")

    def _sweep(self, steps):
        """Adjoint sweep back over `steps` steps (stage inputs in Ys), seeding the
        field-energy gradient coef[q] * Omega0^2 conj(F(y_q)) after each step."""
        B = self._buffers()
        L = _lib.lib()
        ws, wsb = self.plan.ws_ptr()
        h, nc, c2 = self.dt, self.nc, self.O0 ** 2
        mu, gY, gk, acc = B["mu"], B["gY"], B["gk"], B["acc"]
        accp = C.cast(C.c_void_p(acc.data_ptr()), C.POINTER(C.c_double))
        for q in reversed(range(steps)):
            Yq = B["Ys"][q]
            for j in reversed(range(S)):
                terms = [(h * _B[j], mu)]
                for i in range(j + 1, S):
                    aij = _A.get(i, {}).get(j, 0.0)
                    if aij != 0.0:
                        terms.append((h * aij, gY[i]))
                lincomb(gk, terms)
                if self.general:
                    self.plan.vjp_into(Yq[j], gk, gY[j])
                    continue
                _lib.check(L.spx_vjp_param_ex(self.plan.handle, _ptr(Yq[j]), _ptr(gk), _ptr(gY[j]), accp, ws, wsb,
                                              int(self.herm), _stream_ptr()), "spx_vjp_param_ex")
            lincomb(mu, [(1.0, mu)] + [(1.0, gY[j]) for j in range(S)])
            mu[nc:].add_((B["coef"][q] * c2) * Yq[0, nc:].conj())

    def _run(self, kind, steps, use_graphs):
        fn = self._recompute if kind == "recompute" else self._sweep
        if not use_graphs:
            fn(steps)
            return
        key = (kind, steps)
        g = self._graphs.get(key)
        if g is None:
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self.plan.workspace()
                fn(steps) if kind == "recompute" else None     # warm-up outside capture (recompute is idempotent)
            torch.cuda.current_stream().wait_stream(s)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                fn(steps)
            self._graphs[key] = g
        g.replay()

    def backward(self, dLdE: torch.Tensor, mu_final=None, use_graphs=True):
        """dLdE: (N+1,) field-energy sensitivities.  Returns (conj of dL/dy0, param dots
        (2 + Ns): [nu, k d/dk, u_x per species]); the param dots are None on the
        2-D / 3-D layouts."""
        B = self._buffers()
        dev = self.plan.device
        dLdE = dLdE.to(dev, torch.float64)
        mu, acc = B["mu"], B["acc"]
        if mu_final is None:
            mu.zero_()
        else:
            mu.copy_(mu_final)
        acc.zero_()
        c2 = self.O0 ** 2
        mu[self.nc:].add_((dLdE[self.N] * c2) * self.ckpts[-1][self.nc:].conj())
        m = self.m
        starts = list(range(0, self.N, m))
        for g in reversed(range(len(starts))):
            a = starts[g]
            b = min(a + m, self.N)
            B["Ys"][0, 0].copy_(self.ckpts[g])
            B["coef"][: b - a].copy_(dLdE[a:b])
            self._run("recompute", b - a, use_graphs)
            self._run("sweep", b - a, use_graphs)
        st = C.c_int32()
        _lib.check(_lib.lib().spx_rk_status(C.byref(st), _stream_ptr()), "spx_rk_status")
        if st.value != 0:
            raise RuntimeError(f"step recomputation failed: status {_lib.STATUS_NAMES.get(st.value, st.value)}")
        return mu.clone(), (None if self.general else acc.clone())


# ----------------------------------------------------------------- two-stream workload
def two_stream_setup(k=0.2, nu=1.0, u=0.5, amp=1e-3, Nx=65, Nn=128, alpha=0.5, mi_me=1836.0, seed=0):
    """Parameters and initial state of the adjoint workload.

    Three species: beams at +-u (half density each, thermal alpha) and ions;
    perturbation of amplitude `amp` with seeded random phases on modes 1..8,
    the field from Gauss's law (i K E_x = rho / Omega_0).
    Returns (params, bg, delta, ddelta_dk) with y0 = bg + amp * delta.
    """
    ai = alpha * np.sqrt(1.0 / mi_me)
    user = dict(Lx=2 * np.pi / k, nu=nu, D=0.0, qs=[-1.0, -1.0, 1.0], alpha_s=[alpha] * 6 + [ai] * 3,
                u_s=[u, 0, 0, -u, 0, 0, 0, 0, 0], Omega_cs=[1.0, 1.0, 1.0 / mi_me], mi_me=mi_me,
                ms=[1.0, 1.0, mi_me])
    p = initialize_simulation_parameters(user, Nx, 1, 1, Nn, 1, 1, 3, 2, 0.05)
    rng = np.random.default_rng(seed)
    c0 = Nx // 2
    Ns = 3
    dens = [0.5, 0.5, 1.0]
    a = np.asarray(p["alpha_s"]).reshape(Ns, 3)
    bg = np.zeros((Ns, Nn, Nx), np.complex128)
    dC = np.zeros((Ns, Nn, Nx), np.complex128)
    for s in range(Ns):
        bg[s, 0, c0] = dens[s] / a[s, 0] ** 3
    for j in range(1, min(8, (Nx - 1) // 2) + 1):
        ph = np.exp(2j * np.pi * rng.random())
        for s in (0, 1):
            dC[s, 0, c0 + j] = 0.5 * bg[s, 0, c0] * ph
            dC[s, 0, c0 - j] = np.conj(dC[s, 0, c0 + j])
    rho = sum(p["qs"][s] * a[s].prod() * dC[s, 0] for s in range(Ns))
    K = p["kx_grid"][0, :, 0] / p["Lx"]
    nz = np.abs(K) > 0
    dF = np.zeros((6, Nx), np.complex128)
    dF[0, nz] = -1j * rho[nz] / (K[nz] * p["Omega_cs"][0])
    dFdk = np.zeros_like(dF)
    dFdk[0] = -dF[0] / k                      # K = j k  =>  E ~ 1/k
    bgv = np.concatenate([bg.ravel(), np.zeros(6 * Nx, np.complex128)])
    delta = np.concatenate([dC.ravel(), dF.ravel()])
    ddk = np.concatenate([np.zeros(dC.size, np.complex128), dFdk.ravel()])
    return p, bgv, delta, ddk


def window_weights(ts, ta=10.0, tb=40.0):
    """w with slope = sum w_i log E_i for the least-squares line over [ta, tb]."""
    ts = np.asarray(ts, np.float64)
    sel = (ts >= ta - 1e-12) & (ts <= tb + 1e-12)
    tt = ts[sel]
    w = np.zeros_like(ts)
    w[sel] = (tt - tt.mean()) / np.sum((tt - tt.mean()) ** 2)
    return w


def loss_from_energy(E, w):
    E = np.asarray(E, np.float64)
    return float(np.sum(w * np.log(E)) + E[-1])


class TwoStreamProblem:
    """Forward loss and adjoint gradients of the two-stream adjoint workload."""

    def __init__(self, Nx=65, Nn=128, dt=0.05, nsteps=2000, seed=0, ckpt_every=None, window=(10.0, 40.0),
                 hermitian=True):
        self.Nx, self.Nn, self.dt, self.N, self.seed = Nx, Nn, dt, nsteps, seed
        self.hermitian = hermitian
        self.ckpt_every = ckpt_every
        self.window = window

    def _build(self, k, nu, u, amp):
        p, bg, delta, ddk = two_stream_setup(k, nu, u, amp, self.Nx, self.Nn, seed=self.seed)
        plan = plan_for_params(p, "divide")
        adj = Dopri8Adjoint(plan, self.dt, self.N, self.ckpt_every, masses=[1.0, 1.0, 1836.0],
                            hermitian=self.hermitian)
        y0 = torch.from_numpy(bg + amp * delta).to(plan.device)
        return p, plan, adj, y0, delta, ddk

    def loss(self, k, nu, u, amp):
        p, plan, adj, y0, _, _ = self._build(k, nu, u, amp)
        E, _ = adj.forward(y0)
        w = window_weights(adj.ts, *self.window)
        return loss_from_energy(E.cpu().numpy(), w)

    def loss_and_grad(self, k, nu, u, amp):
        p, plan, adj, y0, delta, ddk = self._build(k, nu, u, amp)
        E, _ = adj.forward(y0)
        En = E.cpu().numpy()
        w = window_weights(adj.ts, *self.window)
        L = loss_from_energy(En, w)
        dLdE = w / En
        dLdE[-1] += 1.0
        mu0, acc = adj.backward(torch.from_numpy(dLdE))
        mu0 = mu0.cpu().numpy()
        acc = acc.cpu().numpy()
        # mu0 = conj(dL/dy0): Re sum mu0 * dy0/dtheta is the directional derivative
        g_amp = float(np.real(np.sum(mu0 * delta)))
        g_k = float(acc[1] / k + np.real(np.sum(mu0 * amp * ddk)))
        g_nu = float(acc[0])
        g_u = float(acc[2] - acc[3])           # beams at +u and -u
        return L, dict(k=g_k, nu=g_nu, u=g_u, amp=g_amp)


class TwoStreamLoss(torch.autograd.Function):
    """loss(k, nu, u, amp) with the hand-written discrete adjoint as its backward."""

    @staticmethod
    def forward(ctx, k, nu, u, amp, problem: TwoStreamProblem):
        vals = [float(x) for x in (k, nu, u, amp)]
        L, g = problem.loss_and_grad(*vals)
        ctx.save_for_backward(torch.tensor([g["k"], g["nu"], g["u"], g["amp"]], dtype=torch.float64))
        return torch.tensor(L, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        g = g * gout
        return g[0], g[1], g[2], g[3], None
