"""Torch-facing right-hand side: the drop-in for ``spectrax._simulation.ode_system``.

``ode_system(Nx, Ny, Nz, Nn, Nm, Np, Ns, t, Ck_Fk, args)`` has the reference's
signature and flat complex128 layout (spectrax/_simulation.py:55-111).  It runs
the hand-written sm_103a kernels of ``libspectrax_gb300.so``; there is no CPU
path.  A CUDA tensor in gives a CUDA tensor out on the current torch stream; a
NumPy array in is copied to the GPU and the result copied back.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np
import torch

from . import _lib
from .params import get_mask_mode, problem_from_args, problem_from_params

_cache_lock = threading.Lock()
_plan_cache: dict = {}


def _stream_ptr(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return C.c_void_p(s.cuda_stream)


class Plan:
    """Owns one ``spx_plan`` (device tables) plus a cached workspace."""

    def __init__(self, problem: _lib.spx_problem, device=None, tile=0, threads=0):
        L = _lib.lib()
        self.problem = problem
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        with torch.cuda.device(self.device):
            h = C.c_void_p()
            _lib.check(L.spx_plan_create_ex(C.byref(problem), int(tile), int(threads), C.byref(h)),
                       "spx_plan_create_ex")
        self.handle = h
        self.state_len = int(L.spx_state_len(C.byref(problem)))
        self.ws_bytes = int(L.spx_rhs_workspace_bytes(h))
        self._ws = None
        t, nt, th, path = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        _lib.check(L.spx_plan_info(h, C.byref(t), C.byref(nt), C.byref(th), C.byref(path)), "spx_plan_info")
        self.tile, self.ntiles, self.threads, self.path = t.value, nt.value, th.value, path.value
        self.product_grid = int(L.spx_plan_product_grid(h))
        rads = (C.c_int32 * 16)()
        nr = int(L.spx_plan_product_radices(h, rads, 16))
        self.product_radices = tuple(int(rads[i]) for i in range(min(max(nr, 0), 16)))

    @property
    def shape(self):
        p = self.problem
        return (p.Nx, p.Ny, p.Nz, p.Nn, p.Nm, p.Np, p.Ns)

    def workspace(self):
        if self.ws_bytes and self._ws is None:
            self._ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
        return self._ws

    def ws_ptr(self):
        ws = self.workspace()
        return (C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel())) if ws is not None else (None, 0)

    def check_state(self, y: torch.Tensor, name="y"):
        if not isinstance(y, torch.Tensor) or not y.is_cuda:
            raise TypeError(f"{name} must be a CUDA tensor")
        if y.dtype != torch.complex128:
            raise TypeError(f"{name} must be complex128, got {y.dtype}")
        if y.numel() != self.state_len or not y.is_contiguous():
            raise ValueError(f"{name} must be contiguous with {self.state_len} entries")
        if y.device != self.device:
            raise ValueError(f"{name} is on {y.device}, plan on {self.device}")

    def rhs_into(self, y: torch.Tensor, dy: torch.Tensor, stream=None):
        self.check_state(y)
        self.check_state(dy, "dy")
        ws, nb = self.ws_ptr()
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().spx_rhs(self.handle, C.c_void_p(y.data_ptr()), C.c_void_p(dy.data_ptr()),
                                          ws, nb, _stream_ptr(stream)), "spx_rhs")
        return dy

    def rhs(self, y: torch.Tensor, stream=None):
        dy = torch.empty_like(y)
        return self.rhs_into(y, dy, stream)

    def jvp_into(self, y, v, out, stream=None):
        for t, nm in ((y, "y"), (v, "v"), (out, "out")):
            self.check_state(t, nm)
        ws, nb = self.ws_ptr()
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().spx_jvp(self.handle, C.c_void_p(y.data_ptr()), C.c_void_p(v.data_ptr()),
                                          C.c_void_p(out.data_ptr()), ws, nb, _stream_ptr(stream)), "spx_jvp")
        return out

    def linearize(self, y, lin=None, stream=None):
        """What J(y) v needs from y, computed once (jax.linearize,
        spectrax/midpoint_solver.py:75); reuse it with ``jvp_lin_into``.
        ``lin`` (uint8, ``linearize_bytes``) is reused when given."""
        self.check_state(y)
        nb = self.linearize_bytes
        if lin is None:
            lin = torch.empty(nb, dtype=torch.uint8, device=self.device)
        if lin.dtype != torch.uint8 or lin.numel() < nb or not lin.is_cuda or lin.device != self.device:
            raise ValueError(f"lin must be a uint8 CUDA tensor of {nb} bytes on {self.device}")
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().spx_linearize(self.handle, C.c_void_p(y.data_ptr()), C.c_void_p(lin.data_ptr()),
                                                C.c_size_t(lin.numel()), _stream_ptr(stream)), "spx_linearize")
        return lin

    @property
    def linearize_bytes(self) -> int:
        return int(_lib.lib().spx_linearize_bytes(self.handle))

    def jvp_lin_into(self, lin, v, out, stream=None):
        """J(y) v for the y given to ``linearize`` (same bits as ``jvp_into(y, v)``)."""
        for t, nm in ((v, "v"), (out, "out")):
            self.check_state(t, nm)
        if lin.numel() < self.linearize_bytes:
            raise ValueError("lin is too small for this plan")
        ws, nb = self.ws_ptr()
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().spx_jvp_lin(self.handle, C.c_void_p(lin.data_ptr()), C.c_void_p(v.data_ptr()),
                                              C.c_void_p(out.data_ptr()), ws, nb, _stream_ptr(stream)),
                       "spx_jvp_lin")
        return out

    def vjp_into(self, y, w, out, stream=None):
        for t, nm in ((y, "y"), (w, "w"), (out, "out")):
            self.check_state(t, nm)
        ws, nb = self.ws_ptr()
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().spx_vjp(self.handle, C.c_void_p(y.data_ptr()), C.c_void_p(w.data_ptr()),
                                          C.c_void_p(out.data_ptr()), ws, nb, _stream_ptr(stream)), "spx_vjp")
        return out

    def vjp_noalloc_into(self, y, w, out, stream=None):
        """J(y)^T w through spx_vjp_noalloc: no workspace, nothing allocated.

        For callers that may not allocate device memory at this point (inside a
        stream capture, real-time loops, host frameworks that own all device
        memory).  The scratch is a fixed 1 MiB device array shared by all calls;
        calls that overlap on the GPU race."""
        for t, nm in ((y, "y"), (w, "w"), (out, "out")):
            self.check_state(t, nm)
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().spx_vjp_noalloc(self.handle, C.c_void_p(y.data_ptr()), C.c_void_p(w.data_ptr()),
                                                  C.c_void_p(out.data_ptr()), _stream_ptr(stream)),
                       "spx_vjp_noalloc")
        return out

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            try:
                _lib._lib.spx_plan_destroy(h)
            except Exception:
                pass
            self.handle = None


_product_grid = "auto"


_GRID_MODES = {"auto": 0, "nx": 1, "fp64": 2}


def set_product_grid(mode: str) -> None:
    """Grid of the nonlinear products in the 1D1V stepper kernels for plans made
    from now on (spx_set_product_grid): "auto" (an Nx with a prime factor >= 5
    takes the 2^a 3^b length M >= 3K + 1 of least modeled time in radix-4/3/2
    stages, e.g. 129 -> 144), "nx" (always Nx points) or "fp64" (the least FP64
    count).  Results agree to rounding."""
    global _product_grid
    if mode not in _GRID_MODES:
        raise ValueError("mode must be one of " + ", ".join(_GRID_MODES))
    _lib.check(_lib.lib().spx_set_product_grid(_GRID_MODES[mode]), "spx_set_product_grid")
    _product_grid = mode


def get_product_grid() -> str:
    return _product_grid


def get_plan(problem: _lib.spx_problem, device=None, tile=0, threads=0) -> Plan:
    dev = torch.cuda.current_device() if device is None else device
    key = (bytes(problem), dev, int(tile), int(threads), _product_grid)
    with _cache_lock:
        pl = _plan_cache.get(key)
        if pl is None:
            pl = Plan(problem, dev, tile, threads)
            _plan_cache[key] = pl
        return pl


_tuned: dict = {}


def autotune(problem: _lib.spx_problem, device=None, reps=20, verbose=False, target="rhs", sample=None):
    """Pick (tile, threads) for a problem by timing over a candidate grid; returns
    the tuned Plan (cached per problem and target).

    target "rhs" times the plain right-hand side; "dopri8" times fixed-step
    Dopri8 attempts (13 staged stage kernels), whose kernels
    balance shared memory and latency differently.  `sample` is the state to
    time with (an exactly Hermitian one selects the packed-transform stages);
    default: small random values."""
    if target not in ("rhs", "dopri8"):
        raise ValueError("target must be 'rhs' or 'dopri8'")
    dev = torch.cuda.current_device() if device is None else device
    key = (bytes(problem), dev, target, sample is not None, _product_grid)
    if key in _tuned:
        return _tuned[key]
    base = get_plan(problem, dev)
    if base.path != 0:
        cands = [(0, t) for t in (128, 256)]
    else:
        Nn = problem.Nn
        tiles = sorted({t for t in (1, 2, 3, 4, 5, 6, 8, 12, 16) if t <= max(1, Nn)} | {base.tile})
        cands = [(t, th) for t in tiles for th in (128, 256)]
    if sample is not None:
        y = torch.as_tensor(sample).to(base.device, torch.complex128).contiguous()
        base.check_state(y, "sample")
    else:
        y = torch.randn(base.state_len, dtype=torch.complex128, device=base.device) * 1e-3
    best, table = None, []
    for t, th in cands:
        try:
            pl = get_plan(problem, dev, t, th)
        except _lib.SpectraxError:
            continue
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if target == "rhs":
            dy = torch.empty_like(y)
            for _ in range(3):
                pl.rhs_into(y, dy)
            e0.record()
            for _ in range(reps):
                pl.rhs_into(y, dy)
            e1.record()
        else:
            from .dopri8 import Dopri8Solver
            sv = Dopri8Solver(pl, 0.0, 1e30, 1e-6, adaptive=False, max_steps=1 << 40, save_states=False)
            sv.reset(y)
            sv.enqueue(3)
            e0.record()
            sv.enqueue(reps)
            e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        table.append((pl.tile, th, ms))
        if verbose:
            print(f"autotune tile={pl.tile} threads={th}: {ms * 1e3:.1f} us", flush=True)
        if best is None or ms < best[2]:
            best = (pl, th, ms)
    best[0].tuning = table
    _tuned[key] = best[0]
    return best[0]


def plan_for_params(params, mask_mode=None, device=None, tuned=False, tune_for="rhs", sample=None) -> Plan:
    pb = problem_from_params(params, mask_mode or get_mask_mode())
    return autotune(pb, device, target=tune_for, sample=sample) if tuned else get_plan(pb, device)


class RHSFunction(torch.autograd.Function):
    """dy/dt = f(y) as a torch autograd node, for ``RHSFunction.apply(y, plan)``.

    f is holomorphic in y (spectrax/_model.py uses no conjugation), so with
    torch's convention for complex gradients the reverse mode is
    grad_y = J^H g = conj(J^T conj(g)) (``spx_vjp`` computes the plain
    transpose J^T) and the forward mode is J v (``spx_jvp``).  The backward is
    not itself differentiable."""

    @staticmethod
    def forward(ctx, y, plan):
        ctx.plan = plan
        ctx.save_for_backward(y)
        ctx.save_for_forward(y)
        return plan.rhs(y.detach().contiguous())

    @staticmethod
    @torch.autograd.function.once_differentiable
    def backward(ctx, g):
        (y,) = ctx.saved_tensors
        out = torch.empty_like(y)
        ctx.plan.vjp_into(y.contiguous(), torch.conj_physical(g).contiguous(), out)
        return torch.conj_physical(out), None

    @staticmethod
    def jvp(ctx, y_t, plan_t):
        (y,) = ctx.saved_tensors
        out = torch.empty_like(y)
        return ctx.plan.jvp_into(y.contiguous(), y_t.contiguous(), out)


def _apply_rhs(plan, y):
    if y.requires_grad and torch.is_grad_enabled():
        return RHSFunction.apply(y, plan)
    return plan.rhs(y)


def _as_cuda_state(y, dev):
    if isinstance(y, torch.Tensor):
        return (y if y.is_cuda else y.to(dev)).to(torch.complex128).contiguous(), "torch_cpu" if not y.is_cuda else "torch"
    arr = np.ascontiguousarray(np.asarray(y, dtype=np.complex128))
    return torch.from_numpy(arr).to(dev), "numpy"


def ode_system(Nx, Ny, Nz, Nn, Nm, Np, Ns, t, Ck_Fk, args, mask_mode=None):
    """Drop-in for spectrax/_simulation.py:55-111 (same signature and layout).
    A torch state that requires grad goes through ``RHSFunction`` (reverse and
    forward mode on the GPU)."""
    del t
    pb = problem_from_args(Nx, Ny, Nz, Nn, Nm, Np, Ns, args, mask_mode or get_mask_mode())
    plan = get_plan(pb)
    y, kind = _as_cuda_state(Ck_Fk, plan.device)
    dy = _apply_rhs(plan, y)
    if kind == "numpy":
        return dy.cpu().numpy()
    if kind == "torch_cpu":
        return dy.cpu()
    return dy


def rhs(t, y, params, mask_mode=None):
    """dy/dt for a merged parameter dict (``initialize_simulation_parameters`` output)."""
    del t
    plan = plan_for_params(params, mask_mode)
    yy, kind = _as_cuda_state(y, plan.device)
    dy = _apply_rhs(plan, yy)
    if kind == "numpy":
        return dy.cpu().numpy()
    if kind == "torch_cpu":
        return dy.cpu()
    return dy
