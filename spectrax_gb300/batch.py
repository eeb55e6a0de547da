"""Batched solves of many uneven 1D1V instances in one persistent launch.

The reference's damping-rate scan (Examples/1D_Landau_damping_dr_curve.py:88-110)
calls ``simulation`` once per wavenumber, serially.  ``BatchSolver`` packs all
instances (different k, Nn, Nx, nu, ...) into one graph-captured persistent
kernel (``spx_batch_*``): each thread-block cluster integrates one instance at a
time with its own adaptive step, taking instances largest-first from a device
work queue.  ``autotune`` picks the cluster size and the Hermite tile by timing
short runs of the actual instances.  ``serial_solve`` is the one-instance-at-a-
time baseline on the plain GPU right-hand side.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import tempfile
import time

import numpy as np
import torch

from . import _lib
from .params import initialize_simulation_parameters, make_problem
from .vector_field import _stream_ptr, get_plan


# ----------------------------------------------------------------- workload
def landau_scan(n=256, seed=0, amplitude=0.01, mask_mode="divide"):
    """The 256-instance damping-rate scan: k ~ U[0.1, 0.6], Nn ~ U{32,64,128,256},
    Nx ~ U{17,33,65}, nu ~ U[0.5, 4]; electrons (alpha = sqrt2 vth, vth = 1) and
    ions (mi/me = 1836); perturbation amplitude 0.01 on mode 1
    (initial state as in Examples/1D_Landau_damping.py:40-54)."""
    rng = np.random.default_rng(seed)
    ks = rng.uniform(0.1, 0.6, n)
    Nns = rng.choice([32, 64, 128, 256], n)
    Nxs = rng.choice([17, 33, 65], n)
    nus = rng.uniform(0.5, 4.0, n)
    mi_me = 1836.0
    ae = np.sqrt(2.0)
    ai = ae * np.sqrt(1.0 / mi_me)
    insts = []
    for i in range(n):
        k, Nn, Nx, nu = float(ks[i]), int(Nns[i]), int(Nxs[i]), float(nus[i])
        L = 2 * np.pi / k
        qs, Om = [-1.0, 1.0], [1.0, 1.0 / mi_me]
        alpha = [ae] * 3 + [ai] * 3
        u = [0.0] * 6
        pb = make_problem(Nx, 1, 1, Nn, 1, 1, 2, qs, nu, 0.0, Om, alpha, u, L, 1.0, 1.0, mask_mode)
        c0 = (Nx - 1) // 2
        Ck = np.zeros((2, Nn, Nx), np.complex128)
        Ck[0, 0, c0 - 1] = 1j * amplitude / (2 * ae ** 3)
        Ck[0, 0, c0] = 1.0 / ae ** 3
        Ck[0, 0, c0 + 1] = -1j * amplitude / (2 * ae ** 3)
        Ck[1, 0, c0] = 1.0 / ai ** 3
        Fk = np.zeros((6, Nx), np.complex128)
        Fk[0, c0 - 1] = Fk[0, c0 + 1] = amplitude * L / (4 * np.pi * 1 * Om[0])
        y0 = np.concatenate([Ck.ravel(), Fk.ravel()])
        insts.append(dict(problem=pb, y0=y0, k=k, Nn=Nn, Nx=Nx, nu=nu, L=L, masses=[1.0, mi_me],
                          shape=(Nx, 1, 1, Nn, 1, 1, 2)))
    return insts


# ----------------------------------------------------------------- solver
class BatchSolver:
    def __init__(self, problems, t1, dt0=0.01, rtol=1e-8, atol=1e-8, save_ts=None, adaptive=True,
                 max_steps=10_000_000, cluster=2, tile=8, masses=None, device=None, hermitian=True,
                 saveat="interpolate", costs=None):
        from .dopri8 import _saveat_code
        L = _lib.lib()
        self.n = len(problems)
        self.problems = list(problems)
        arr = (_lib.spx_problem * self.n)(*self.problems)
        self.ts = np.ascontiguousarray(np.asarray([] if save_ts is None else save_ts, np.float64))
        self.nsave = len(self.ts)
        m = np.ones((self.n, _lib.MAX_SPECIES))
        if masses is not None:
            for i, mm in enumerate(masses):
                m[i, :len(mm)] = mm
        self._masses = np.ascontiguousarray(m)
        o = _lib.spx_batch_opts()
        o.t1, o.dt0, o.rtol, o.atol = float(t1), float(dt0), float(rtol), float(atol)
        o.max_steps = int(max_steps)
        o.adaptive = 1 if adaptive else 0
        o.nsave = self.nsave
        o.save_ts = self.ts.ctypes.data_as(C.POINTER(C.c_double)) if self.nsave else None
        o.cluster = int(cluster)
        o.tile = int(tile)
        o.masses = self._masses.ctypes.data_as(C.POINTER(C.c_double))
        # instances with odd Nx and an exactly Hermitian y0 use packed real transforms
        o.hermitian = 1 if hermitian else 0
        # save times: dense output inside a step (Diffrax SaveAt(ts)) or steps landing on them
        o.saveat = _saveat_code(saveat)
        self.saveat = saveat
        # queue order: the caller's relative costs (largest first), else the built-in estimate
        self._costs = None if costs is None else np.ascontiguousarray(np.asarray(costs, np.float64))
        if self._costs is not None:
            if self._costs.shape != (self.n,):
                raise ValueError("costs must hold one value per instance")
            o.costs = self._costs.ctypes.data_as(C.POINTER(C.c_double))
        self.cluster, self.tile = int(cluster), int(tile)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(L.spx_batch_create(self.n, arr, C.byref(o), C.byref(h)), "spx_batch_create")
        self.handle = h
        self.offsets = [int(L.spx_batch_offset(h, i)) for i in range(self.n + 1)]
        self.en_offsets = [int(L.spx_batch_energy_offset(h, i)) for i in range(self.n)]
        self.grid = int(L.spx_batch_grid(h))
        self.total_len = self.offsets[-1]

    def pack(self, states):
        out = np.empty(self.total_len, np.complex128)
        for i, y in enumerate(states):
            out[self.offsets[i]:self.offsets[i + 1]] = y
        return torch.from_numpy(out).to(self.device)

    def unpack(self, packed):
        p = packed.cpu().numpy() if isinstance(packed, torch.Tensor) else packed
        return [p[self.offsets[i]:self.offsets[i + 1]] for i in range(self.n)]

    def run(self, y0_packed, y_out=None, stream=None):
        """Asynchronous: copy states in, replay the graph, copy final states out."""
        if y_out is None:
            y_out = torch.empty(self.total_len, dtype=torch.complex128, device=self.device)
        _lib.check(_lib.lib().spx_batch_run(self.handle, C.c_void_p(y0_packed.data_ptr()),
                                            C.c_void_p(y_out.data_ptr()), _stream_ptr(stream)), "spx_batch_run")
        return y_out

    def results(self):
        st = (_lib.spx_batch_stats * self.n)()
        en_len = (self.en_offsets[-1] + max(1, self.nsave) * (2 + self.problems[-1].Ns)) if self.n else 0
        en = np.zeros(en_len, np.float64)
        _lib.check(_lib.lib().spx_batch_results(self.handle, st, en.ctypes.data_as(C.POINTER(C.c_double)),
                                                _stream_ptr()), "spx_batch_results")
        torch.cuda.current_stream().synchronize()
        stats = [dict(t=s.t, dt=s.dt, accepted=s.accepted, rejected=s.rejected, rhs_evals=s.rhs_evals,
                      status=s.status, saved=s.saved, hermitian=bool(s.hermitian),
                      start_s=s.start_s, end_s=s.end_s) for s in st]
        energies = []
        for i in range(self.n):
            w = 2 + self.problems[i].Ns
            o = self.en_offsets[i]
            energies.append(en[o:o + max(1, self.nsave) * w].reshape(max(1, self.nsave), w)[:self.nsave])
        return stats, energies

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            try:
                _lib._lib.spx_batch_destroy(h)
            except Exception:
                pass
            self.handle = None


# ----------------------------------------------------------------- autotuner
def _cache_path():
    base = os.environ.get("SPECTRAX_GB300_CACHE") or os.path.join(tempfile.gettempdir(), "spectrax_gb300")
    os.makedirs(base, exist_ok=True)
    return os.path.join(base, "batch_autotune.json")


def _signature(problems, t1, rtol):
    shapes = sorted((p.Nx, p.Nn, p.Ns) for p in problems)
    name = torch.cuda.get_device_name()
    return f"{name}|{len(problems)}|{hash(tuple(shapes)) & 0xffffffff}|{rtol}"


def autotune(problems, y0s, t1_probe=0.5, rtol=1e-8, atol=1e-8, dt0=0.01, masses=None,
             clusters=(1, 2, 4, 8, 16), tiles=(4, 8, 16, 32, -1), use_cache=True, verbose=False,
             refine=3, t1_refine=2.0):
    """Time a short horizon of the real instances for every (cluster, tile), then
    the `refine` fastest again over t1_refine (the short probe ranks close
    candidates by the start-up transient of the step sizes), and return the
    fastest as dict(cluster=, tile=, ms=, table=[...], refined=[...]).  tile -1:
    each instance's tile height chosen to fill whole rounds of the cluster's CTAs."""
    sig = _signature(problems, t1_probe, rtol) + f"|refine{refine}@{t1_refine:g}"
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except Exception:
            cache = {}
        if sig in cache:
            return cache[sig]
    def timed(c, t, t1):
        try:
            s = BatchSolver(problems, t1, dt0=dt0, rtol=rtol, atol=atol, save_ts=np.array([t1]), cluster=c,
                            tile=t, masses=masses)
        except _lib.SpectraxError:
            return None
        y0 = s.pack(y0s)
        s.run(y0)                         # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        s.run(y0)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    table = []
    for c in clusters:
        for t in tiles:
            ms = timed(c, t, t1_probe)
            if ms is None:
                continue
            table.append(dict(cluster=c, tile=t, ms=ms))
            if verbose:
                print(f"autotune cluster={c} tile={t}: {ms:.2f} ms", flush=True)
    if not table:
        raise _lib.SpectraxError("batch autotune: no (cluster, tile) candidate could be created")
    ranked = sorted(table, key=lambda r: r["ms"])
    refined = []
    if refine and refine > 1 and t1_refine > t1_probe:
        for r in ranked[:refine]:
            ms = timed(r["cluster"], r["tile"], t1_refine)
            if ms is not None:
                refined.append(dict(cluster=r["cluster"], tile=r["tile"], ms=ms))
                if verbose:
                    print(f"autotune refine cluster={r['cluster']} tile={r['tile']}: {ms:.2f} ms", flush=True)
    best = min(refined, key=lambda r: r["ms"]) if refined else ranked[0]
    best = dict(best, table=table, refined=refined)
    cache[sig] = best
    try:
        json.dump(cache, open(path, "w"))
    except OSError:
        pass
    return best


# ----------------------------------------------------------------- serial baseline
def serial_solve(insts, t1, dt0=0.01, rtol=1e-8, atol=1e-8, save_ts=None, hermitian=True, saveat="interpolate"):
    """Solve the instances one after another with the single-instance device
    Dopri8 (graph-captured stage kernels).  Returns (final states, stats,
    energies, seconds); the plans and solvers (device buffers, captured graphs)
    are built before the clock starts, so the seconds cover only the solves.
    hermitian=True (as the batch) runs packed real transforms for exactly
    Hermitian instances, on the same product grids: the batched kernel's
    arithmetic; False forces the general complex-transform stages."""
    from .dopri8 import Dopri8Solver
    solvers = []
    for it in insts:
        plan = get_plan(it["problem"])
        solvers.append(Dopri8Solver(plan, 0.0, t1, dt0, ts=save_ts, adaptive=True, rtol=rtol, atol=atol,
                                    save_states=False, masses=it.get("masses"), hermitian=hermitian,
                                    saveat=saveat))
    y0s = [torch.from_numpy(it["y0"]).to(solvers[0].plan.device) for it in insts]
    finals, stats, ens = [], [], []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s, y0 in zip(solvers, y0s):
        s.reset(y0)
        s.run()
        finals.append(s.state())
        stats.append(s.stats())
        ens.append(s.energies())
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    return [f.cpu().numpy() for f in finals], stats, [e.cpu().numpy() for e in ens], sec
