"""GPU: implicit midpoint with Newton-GMRES (JVP kernel) against the oracle's dense Newton."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import midpoint as omid
from oracle import rhs as orhs
from oracle import tables as otab


def _params(shape, seed=0):
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    user = dict(Lx=50.0, Ly=50.0, nu=0.5, qs=[-1.0, 1.0][:Ns],
                alpha_s=([0.25] * 3 + [0.05] * 3)[:3 * Ns], u_s=list(rng.uniform(-0.1, 0.1, 3 * Ns)),
                Omega_cs=[0.5, 0.02][:Ns])
    return otab.initialize_simulation_parameters(user, *shape, 5, 0.1)


def _state(shape, seed=1):
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    plane = Nx * Ny * Nz
    n = Ns * Nn * Nm * Np * plane + 6 * plane
    rng = np.random.default_rng(seed)
    y = 1e-3 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    kc = ((Ny // 2) * Nx + Nx // 2) * Nz + Nz // 2
    for s in range(Ns):
        y[s * Nn * Nm * Np * plane + kc] += 1.0
    y[Ns * Nn * Nm * Np * plane + 5 * plane + kc] += 1.0     # background B_z
    return y


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(4, 5, 1, 2, 2, 2, 1), (9, 1, 1, 12, 1, 1, 2), (6, 4, 1, 2, 2, 1, 2)],
                         ids=lambda s: "x".join(map(str, s)))
def test_midpoint_step_matches_oracle(shape):
    import torch
    from spectrax_gb300 import midpoint, vector_field
    p = _params(shape)
    y0 = _state(shape)
    f = lambda y: orhs.rhs(p, y)
    ref, ref_err, _ = omid.step(f, y0, 0.1, rtol=1e-10, atol=1e-10)
    plan = vector_field.plan_for_params(p, "divide")
    ng = midpoint.NewtonGMRES(plan, restart=30, gmres_tol=1e-12)
    y1, err = midpoint.step(plan, torch.from_numpy(y0).cuda(), 0.1, 1e-10, 1e-10, solver=ng)
    assert rel_err(y1.cpu().numpy(), ref) < 1e-9
    assert rel_err(err.cpu().numpy(), ref_err) < 1e-6


@pytest.mark.gpu
def test_gmres_solves_linear_system():
    import torch
    from spectrax_gb300 import midpoint, vector_field
    shape = (8, 8, 1, 2, 2, 2, 1)
    p = _params(shape, 2)
    plan = vector_field.plan_for_params(p, "divide")
    ym = torch.from_numpy(_state(shape, 3)).cuda()
    rng = np.random.default_rng(4)
    b = torch.from_numpy(rng.standard_normal(plan.state_len) + 1j * rng.standard_normal(plan.state_len)).cuda()
    ng = midpoint.NewtonGMRES(plan, restart=3, gmres_tol=1e-11, gmres_maxiter=50)
    x, rel, its = ng.solve(ym, b, 0.05)
    Ax = torch.empty_like(x)
    ng._A(ym, x, Ax, 0.05)
    assert (torch.linalg.vector_norm(Ax - b) / torch.linalg.vector_norm(b)).item() < 1e-10
    assert its > 3           # restarted GMRES(3) needed more than one cycle


@pytest.mark.gpu
def test_simulation_with_implicit_midpoint():
    import spectrax_gb300 as sg
    from spectrax_gb300.dopri8 import simulation
    out = simulation({"t_max": 0.3, "ode_tolerance": 1e-10}, Nx=9, Nn=8, timesteps=4, dt=0.1,
                     solver=sg.ImplicitMidpoint(rtol=1e-10, atol=1e-10))
    assert out["Ck"].shape == (4, 16, 1, 9, 1)
    assert out["solver_stats"]["steps"] == 3
    assert np.all(np.isfinite(out["EM_energy"]))
