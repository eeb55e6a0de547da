"""Oracle fixtures for the full-size workloads (run once on a CPU; minutes each).

The GPU tests rebuild the same seeded inputs with the package's own builders and
compare the device results with what this script stores:

* two_stream_nx129_nn256.npz -- the two-stream workload (Nx = 129, Nn = 256,
  3 species), adaptive Dopri8 (rtol 1e-10, atol 1e-12, first step 0.2) from t = 0 to 100 with
  201 save times (Diffrax SaveAt(ts): dense output): the saved energies, the
  step counts and the final field lines and Hermite-plane norms;
* adjoint_two_stream_nx65_nn128.npz -- the adjoint workload's loss (2000 fixed
  Dopri8 steps of dt = 0.05; LSQ slope of log E over t in [10, 40] plus the
  final E) and its field-energy history;
* orszag_tang_64x64_8cubed.npz -- the 2D3V Orszag-Tang-like state (64 x 64,
  8^3 Hermite modes, 2 species): one right-hand side, one Jacobian-vector
  product along a seeded direction and one implicit-midpoint step (dt = 0.1,
  Newton-GMRES with restart 30 and tolerance 1e-10), each reduced to its norm,
  its per-plane norms and 4096 entries at seeded positions.

Everything is computed by the NumPy oracle (``oracle/``); only the inputs come
from the package (``bench.two_stream_params``, ``adjoint.two_stream_setup``,
``maxwellian.orszag_tang_state``), as in the tests.

    python tests/golden/make_workload_fixtures.py [two_stream|adjoint|orszag_tang ...] [--workers N]
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import diag as odiag  # noqa: E402
from oracle import dopri8 as od  # noqa: E402
from oracle import midpoint as om  # noqa: E402
from oracle import rhs as orhs  # noqa: E402

SAMPLES = 4096


def reduce_state(y, nplanes, plane, idx):
    """(norm, per-plane norms of the Hermite planes then the 6 field planes, y[idx])."""
    nc = nplanes * plane
    pn = np.concatenate([np.linalg.norm(y[:nc].reshape(nplanes, plane), axis=1),
                         np.linalg.norm(y[nc:].reshape(6, plane), axis=1)])
    return np.linalg.norm(y), pn, y[idx]


def sample_indices(n, seed=123):
    return np.sort(np.random.default_rng(seed).choice(n, SAMPLES, replace=False))


def two_stream():
    import bench
    p, y0 = bench.two_stream_params(seed=0)
    Nx, Nn, Ns = 129, 256, 3
    ts = np.linspace(0.0, 100.0, 201)
    en = np.zeros((len(ts), 2 + Ns))

    def on_save(i, y):
        e = odiag.energies(y[None], Nx, 1, 1, Nn, 1, 1, Ns, p["alpha_s"], p["u_s"], p["Omega_cs"],
                           ms=[1.0, 1.0, 1836.0])
        en[i, 0] = e["EM_energy"][0]
        en[i, 1] = e["kinetic_energy"][0].real
        en[i, 2:] = e["kinetic_energy_species"][0].real

    t0 = time.time()
    # first step 0.2 (the bench's); later steps follow the rounding noise of the ion
    # Hermite-1 plane's error estimate, so the GPU test compares step counts with a margin
    out = od.solve(lambda t, y: orhs.rhs(p, y, "divide"), 0.0, 100.0, y0, 0.2, ts=ts, adaptive=True,
                   rtol=1e-10, atol=1e-12, on_save=on_save, saveat="interpolate")
    print(f"two_stream: {out['accepted']} accepted, {out['rejected']} rejected, {time.time() - t0:.0f} s")
    yf = out["y"]
    np.savez(os.path.join(HERE, "two_stream_nx129_nn256.npz"), ts=ts, energies=en, accepted=out["accepted"],
             rejected=out["rejected"], rhs_evals=out["rhs_evals"], status=out["status"],
             final_fields=yf[Ns * Nn * Nx:],
             final_plane_norms=np.linalg.norm(yf[:Ns * Nn * Nx].reshape(Ns * Nn, Nx), axis=1))


def adjoint():
    from spectrax_gb300.adjoint import loss_from_energy, two_stream_setup, window_weights
    k, nu, u, amp = 0.2, 1.0, 0.5, 1e-3
    p, bg, delta, _ = two_stream_setup(k, nu, u, amp, 65, 128, seed=0)
    y0 = bg + amp * delta
    N, dt = 2000, 0.05
    ts = np.arange(N + 1) * dt
    E = np.zeros(N + 1)
    Nx, Nn, Ns = 65, 128, 3

    def on_save(i, y):
        E[i] = 0.5 * p["Omega_cs"][0] ** 2 * np.sum(np.abs(y[Ns * Nn * Nx:]) ** 2)

    t0 = time.time()
    out = od.solve(lambda t, y: orhs.rhs(p, y, "divide"), 0.0, ts[-1], y0, dt, ts=ts, adaptive=False,
                   on_save=on_save, saveat="interpolate")
    L = loss_from_energy(E, window_weights(ts, 10.0, 40.0))
    print(f"adjoint: loss {L!r}, {out['accepted']} steps, {time.time() - t0:.0f} s")
    np.savez(os.path.join(HERE, "adjoint_two_stream_nx65_nn128.npz"), params=np.array([k, nu, u, amp]),
             loss=L, field_energy=E, accepted=out["accepted"])


def orszag_tang():
    from spectrax_gb300.maxwellian import orszag_tang_state
    p, y0 = orszag_tang_state()
    n = len(y0)
    nplanes, plane = 2 * 8 * 8 * 8, 64 * 64
    idx = sample_indices(n)

    def f(y):
        return orhs.rhs(p, y, "divide")

    t0 = time.time()
    dy = f(y0)
    v = np.random.default_rng(5).standard_normal(n) + 1j * np.random.default_rng(6).standard_normal(n)
    jv = om.jvp_quadratic(f, y0, v)
    print(f"orszag_tang: rhs + jvp {time.time() - t0:.0f} s")
    t0 = time.time()
    y1, _, newton, mv = om.step_newton_gmres(f, y0, 0.1, rtol=1e-10, atol=1e-10, restart=30, gmres_tol=1e-10)
    print(f"orszag_tang: implicit step {newton} Newton iterations, {mv} products, {time.time() - t0:.0f} s")
    out = {}
    for name, vec in (("rhs", dy), ("jvp", jv), ("step", y1)):
        nrm, pn, smp = reduce_state(vec, nplanes, plane, idx)
        out[f"{name}_norm"], out[f"{name}_plane_norms"], out[f"{name}_samples"] = nrm, pn, smp
    np.savez(os.path.join(HERE, "orszag_tang_64x64_8cubed.npz"), idx=idx, newton=newton, matvecs=mv,
             y0_norm=np.linalg.norm(y0), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", nargs="*", default=["two_stream", "adjoint", "orszag_tang"])
    ap.add_argument("--workers", type=int, default=os.cpu_count())
    a = ap.parse_args()
    orhs.set_fft_workers(a.workers)
    jobs = {"two_stream": two_stream, "adjoint": adjoint, "orszag_tang": orszag_tang}
    for w in a.which:
        jobs[w]()


if __name__ == "__main__":
    main()
