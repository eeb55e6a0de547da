"""GPU: the full-size workloads against oracle fixtures (tests/golden/make_workload_fixtures.py).

* two-stream, Nx = 129, Nn = 256, 3 species, adaptive Dopri8 (rtol 1e-10,
  atol 1e-12) to t = 100 with 201 dense-output saves: field and kinetic
  energies within 1e-9 relative at every save and the final field lines within
  1e-9, on both the packed (Hermitian) and the general stages; the accepted
  step count within 3 % of the oracle's.  On this workload the error estimate is set by rounding: 99.99 %
  of the scaled error norm comes from the ion Hermite-1 plane, whose right-hand
  side E_x * C_0 multiplies the field by the ion density mode C_0(k=0) =
  1/alpha_i^3 ~ 6.3e5, so its transform carries ~1e-13 of rounding noise
  against an absolute tolerance of 1e-12.  Each FFT ordering takes its own,
  equally valid, step sequence (on the 129-point grid the general stages ended
  within one step of the oracle and the packed stages, which pair the ion line
  with its neighbour in one complex transform, took ~2 % more steps) while the
  energies agree to ~1e-10;
* adjoint workload (Nx = 65, Nn = 128, 2000 steps of dt = 0.05): the loss within
  1e-9 of the oracle's, and the adjoint gradient of each of (k, nu, u, amplitude)
  within 1e-6 of central differences of the device loss (h = 1e-6 relative; a
  fourth-order quotient at h = 1e-3 for nu and the amplitude, see the test);
* Orszag-Tang-like 2D3V state (64 x 64, 8^3 Hermite modes, 2 species, 4.2 M
  coefficients): one right-hand side and one Jacobian-vector product within
  1e-12 (norm, per-plane norms and 4096 sampled entries, relative to the
  vector's norm), and one implicit-midpoint step (Newton-GMRES, restart 30,
  tolerance 1e-10) within 1e-10.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _fixture(name):
    path = os.path.join(GOLD, name)
    if not os.path.exists(path):
        pytest.fail(f"missing fixture {name}: run tests/golden/make_workload_fixtures.py")
    return np.load(path)


@pytest.mark.gpu
@pytest.mark.parametrize("hermitian", [True, False], ids=["packed", "general"])
def test_two_stream_to_t100_matches_oracle(hermitian):
    import torch

    import bench
    from spectrax_gb300.dopri8 import Dopri8Solver
    from spectrax_gb300.vector_field import plan_for_params
    ref = _fixture("two_stream_nx129_nn256.npz")
    p, y0 = bench.two_stream_params(seed=0)
    plan = plan_for_params(p, "divide")
    s = Dopri8Solver(plan, 0.0, 100.0, 0.2, ts=ref["ts"], adaptive=True, rtol=1e-10, atol=1e-12,
                     masses=[1.0, 1.0, 1836.0], save_states=False, max_steps=1 << 30, hermitian=hermitian)
    s.reset(torch.from_numpy(y0))
    assert s.run() == 1
    st = s.stats()
    assert st["hermitian"] == hermitian
    acc, rej = int(ref["accepted"]), int(ref["rejected"])
    # the step sequence follows the rounding noise of the ion Hermite-1 plane (module docstring)
    assert abs(st["accepted"] - acc) <= 0.03 * acc, (st, acc, rej)
    en = s.energies().cpu().numpy()
    np.testing.assert_allclose(en[:, 0], ref["energies"][:, 0], rtol=1e-9)    # field energy
    np.testing.assert_allclose(en[:, 1:], ref["energies"][:, 1:], rtol=1e-9)  # kinetic, total and per species
    yf = s.state().cpu().numpy()
    nc = 3 * 256 * 129
    fields = yf[nc:]
    assert np.linalg.norm(fields - ref["final_fields"]) <= 1e-9 * np.linalg.norm(ref["final_fields"])
    pn = np.linalg.norm(yf[:nc].reshape(3 * 256, 129), axis=1)
    assert np.max(np.abs(pn - ref["final_plane_norms"])) <= 1e-9 * np.max(ref["final_plane_norms"])


@pytest.mark.gpu
def test_adjoint_workload_loss_and_gradients():
    from spectrax_gb300.adjoint import TwoStreamProblem
    ref = _fixture("adjoint_two_stream_nx65_nn128.npz")
    theta = [float(v) for v in ref["params"]]             # k, nu, u, amplitude
    prob = TwoStreamProblem(Nx=65, Nn=128, dt=0.05, nsteps=2000, seed=0)
    L, g = prob.loss_and_grad(*theta)
    assert abs(L - float(ref["loss"])) <= 1e-9 * abs(float(ref["loss"]))
    # central differences: h = 1e-6 relative for k and u (second order); for nu
    # and the amplitude, whose logarithmic sensitivities theta dL/dtheta are 6e-7
    # and 3e-6 (~1e-3 |L|), the loss's ~1e-16 of rounding from its 2000 steps
    # would limit a second-order quotient at h = 1e-4 to ~1e-6 relative, so those
    # take the fourth-order quotient at h = 1e-3 relative (rounding ~2e-7 relative,
    # truncation O(h^4))
    def loss_at(i, d):
        th = list(theta)
        th[i] += d
        return prob.loss(*th)

    for i, name in enumerate(("k", "nu", "u", "amp")):
        if name in ("nu", "amp"):
            h = 1e-3 * abs(theta[i])
            fd = (8.0 * (loss_at(i, h) - loss_at(i, -h)) - (loss_at(i, 2 * h) - loss_at(i, -2 * h))) / (12 * h)
        else:
            h = 1e-6 * abs(theta[i])
            fd = (loss_at(i, h) - loss_at(i, -h)) / (2 * h)
        assert abs(g[name] - fd) <= 1e-6 * abs(fd), (name, g[name], fd)


def _reduced(v, nplanes, plane, idx):
    nc = nplanes * plane
    pn = np.concatenate([np.linalg.norm(v[:nc].reshape(nplanes, plane), axis=1),
                         np.linalg.norm(v[nc:].reshape(6, plane), axis=1)])
    return np.linalg.norm(v), pn, v[idx]


def _check(vec, ref, name, tol):
    nplanes, plane = 2 * 8 * 8 * 8, 64 * 64
    nrm, pn, smp = _reduced(vec, nplanes, plane, ref["idx"])
    rn = float(ref[f"{name}_norm"])
    assert abs(nrm - rn) <= tol * rn, (name, nrm, rn)
    assert np.max(np.abs(pn - ref[f"{name}_plane_norms"])) <= tol * rn, name
    assert np.max(np.abs(smp - ref[f"{name}_samples"])) <= tol * rn, name


@pytest.mark.gpu
def test_orszag_tang_rhs_jvp_and_implicit_step():
    import torch

    from spectrax_gb300 import midpoint
    from spectrax_gb300.maxwellian import orszag_tang_state
    from spectrax_gb300.vector_field import plan_for_params
    ref = _fixture("orszag_tang_64x64_8cubed.npz")
    p, y0 = orszag_tang_state()
    n = len(y0)
    assert abs(np.linalg.norm(y0) - float(ref["y0_norm"])) <= 1e-14 * float(ref["y0_norm"])
    plan = plan_for_params(p, "divide")
    y = torch.from_numpy(y0).cuda()
    _check(plan.rhs(y).cpu().numpy(), ref, "rhs", 1e-12)
    v = np.random.default_rng(5).standard_normal(n) + 1j * np.random.default_rng(6).standard_normal(n)
    out = torch.empty_like(y)
    _check(plan.jvp_into(y, torch.from_numpy(v).cuda(), out).cpu().numpy(), ref, "jvp", 1e-12)
    ng = midpoint.NewtonGMRES(plan, restart=30, gmres_tol=1e-10)
    stats = {}
    y1, _, _ = midpoint.step(plan, y, 0.1, 1e-10, 1e-10, solver=ng, stats=stats)
    _check(y1.cpu().numpy(), ref, "step", 1e-10)
