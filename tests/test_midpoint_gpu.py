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
    y1, err, _ = midpoint.step(plan, torch.from_numpy(y0).cuda(), 0.1, 1e-10, 1e-10, solver=ng)
    assert rel_err(y1.cpu().numpy(), ref) < 1e-9
    assert rel_err(err.cpu().numpy(), ref_err) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(4, 5, 1, 2, 2, 2, 1), (9, 1, 1, 12, 1, 1, 2)], ids=lambda s: "x".join(map(str, s)))
def test_midpoint_step_eisenstat_walker(shape):
    # the reference's inner tolerance min(0.1, norm / 2) (gmres_tol=None): Newton stops
    # on the same scaled-norm rule, so the step agrees with the tight solve to ~rtol
    import torch
    from spectrax_gb300 import midpoint, vector_field
    p = _params(shape)
    y0 = _state(shape)
    ref, _, _ = omid.step(lambda y: orhs.rhs(p, y), y0, 0.1, rtol=1e-10, atol=1e-10)
    plan = vector_field.plan_for_params(p, "divide")
    ng = midpoint.NewtonGMRES(plan, restart=30, gmres_tol=None)
    st = {}
    y1, _, _ = midpoint.step(plan, torch.from_numpy(y0).cuda(), 0.1, 1e-10, 1e-10, solver=ng, stats=st)
    assert st["newton"] >= 1
    assert rel_err(y1.cpu().numpy(), ref) < 1e-8


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
                     solver=sg.ImplicitMidpoint(rtol=1e-10, atol=1e-10), adaptive_time_step=False)
    assert out["Ck"].shape == (4, 16, 1, 9, 1)
    assert out["solver_stats"]["steps"] == 3
    assert np.all(np.isfinite(out["EM_energy"]))
    # the reference's default: the step size follows the PID controller on y_error
    out = simulation({"t_max": 0.3, "ode_tolerance": 1e-7}, Nx=9, Nn=8, timesteps=4, dt=0.1,
                     solver=sg.ImplicitMidpoint(rtol=1e-10, atol=1e-10))
    assert out["Ck"].shape == (4, 16, 1, 9, 1)
    st = out["solver_stats"]
    assert st["steps"] > 10 and st["rejected"] > 0          # the oracle takes 27 + 3
    assert np.all(np.isfinite(out["EM_energy"]))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(4, 5, 1, 2, 2, 2, 1), (9, 1, 1, 12, 1, 1, 2)],
                         ids=lambda s: "x".join(map(str, s)))
def test_adaptive_midpoint_matches_oracle(shape):
    # PID controller on y_error = y1 - y1_init (order 2), steps ending only on t1,
    # linear interpolation at the save times (spectrax/midpoint_solver.py:24,51):
    # the same accepted / rejected steps as the oracle and saved states within 1e-9.
    # The Newton tolerance (1e-12) is far below the controller's (1e-6), so the
    # controller sees the same error estimate on both sides.
    import torch
    import spectrax_gb300 as sg
    from spectrax_gb300 import midpoint, vector_field
    p = _params(shape)
    y0 = _state(shape)
    ts = np.linspace(0.0, 0.5, 7)
    ref = omid.solve(lambda y: orhs.rhs(p, y), 0.5, y0, 0.05, ts, rtol=1e-12, atol=1e-12, ctrl_rtol=1e-6,
                     ctrl_atol=1e-6)
    plan = vector_field.plan_for_params(p, "divide")
    solver = sg.ImplicitMidpoint(rtol=1e-12, atol=1e-12, restart=30, gmres_tol=1e-13)
    ys, en, info = midpoint.solve(plan, torch.from_numpy(y0), 0.5, 0.05, ts, solver, [1.0, 1.0][:shape[6]],
                                  adaptive=True, ctrl_rtol=1e-6, ctrl_atol=1e-6)
    assert (info["steps"], info["rejected"]) == (ref["accepted"], ref["rejected"]), (info, ref)
    assert ref["rejected"] + ref["accepted"] > 5
    assert rel_err(ys, ref["ys"]) < 1e-9


@pytest.mark.gpu
def test_midpoint_residual_kernel():
    # the fused residual / scaled norm against NumPy, with and without storing r
    import torch
    from spectrax_gb300 import midpoint, vector_field
    shape = (8, 8, 1, 2, 2, 2, 1)
    plan = vector_field.plan_for_params(_params(shape, 2), "divide")
    n = plan.state_len
    rng = np.random.default_rng(9)
    y0, y1, f = (rng.standard_normal(n) + 1j * rng.standard_normal(n) for _ in range(3))
    g = midpoint._Glue(plan, midpoint.NewtonGMRES(plan, restart=2).kws)
    t = [torch.from_numpy(a).cuda() for a in (y0, y1, f)]
    sq = g.residual(*t, 0.03, 1e-3, 1e-4)
    r = y1 - y0 - 0.03 * f
    ref = np.sum(np.abs(r / (1e-4 + 1e-3 * np.maximum(np.abs(y0), np.abs(y1)))) ** 2)
    assert abs(sq - ref) <= 1e-12 * ref
    assert rel_err(g.res.cpu().numpy(), r) < 1e-15
    assert abs(g.residual(*t, 0.03, 1e-3, 1e-4, store=False) - sq) == 0.0
    g.update(t[0], t[1], t[2], -0.5)
    assert rel_err(t[1].cpu().numpy(), y1 - 0.5 * f) < 1e-15
    assert rel_err(g.ymid.cpu().numpy(), 0.5 * (y0 + y1 - 0.5 * f)) < 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("n,k", [(1000, 1), (777, 9), (300001, 31), (200, 64), (5, 3)])
def test_krylov_cgs2_and_axpy(n, k):
    # the native Gram-Schmidt pass against the same two passes in numpy
    import ctypes as C
    import torch
    from spectrax_gb300 import _lib
    rng = np.random.default_rng(n + k)
    V = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    w = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    h = V.conj() @ w
    w1 = w - V.T @ h
    h2 = V.conj() @ w1
    w2 = w1 - V.T @ h2
    Vt = torch.from_numpy(V).cuda().contiguous()
    wt = torch.from_numpy(w).cuda()
    out = torch.empty(k + 1, dtype=torch.complex128, device="cuda")
    ws = torch.empty(int(_lib.lib().spx_krylov_ws_bytes(n)), dtype=torch.uint8, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(_lib.lib().spx_krylov_cgs2(C.c_void_p(Vt.data_ptr()), n, k, C.c_void_p(wt.data_ptr()),
                                          C.c_void_p(out.data_ptr()), C.c_void_p(ws.data_ptr()), ws.numel(), st),
               "spx_krylov_cgs2")
    o = out.cpu().numpy()
    assert rel_err(o[:k], h + h2) < 1e-12
    assert abs(o[k].real - np.linalg.norm(w2)) <= 1e-12 * np.linalg.norm(w2)
    assert o[k].imag == 0.0
    assert rel_err(wt.cpu().numpy(), w2) < 1e-12
    c = rng.standard_normal(k) + 1j * rng.standard_normal(k)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    xt = torch.from_numpy(x).cuda()
    _lib.check(_lib.lib().spx_krylov_axpy(C.c_void_p(Vt.data_ptr()), n, k,
                                          C.c_void_p(torch.from_numpy(c).cuda().data_ptr()),
                                          C.c_void_p(xt.data_ptr()), st), "spx_krylov_axpy")
    assert rel_err(xt.cpu().numpy(), x + V.T @ c) < 1e-12


@pytest.mark.gpu
def test_krylov_rejects_bad_arguments():
    import ctypes as C
    import torch
    from spectrax_gb300 import _lib
    V = torch.zeros((2, 8), dtype=torch.complex128, device="cuda")
    w = torch.zeros(8, dtype=torch.complex128, device="cuda")
    out = torch.zeros(80, dtype=torch.complex128, device="cuda")
    ws = torch.empty(int(_lib.lib().spx_krylov_ws_bytes(8)), dtype=torch.uint8, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for k in (0, 65):
        rc = _lib.lib().spx_krylov_cgs2(C.c_void_p(V.data_ptr()), 8, k, C.c_void_p(w.data_ptr()),
                                        C.c_void_p(out.data_ptr()), C.c_void_p(ws.data_ptr()), ws.numel(), st)
        assert rc == _lib.SPX_E_ARG
    rc = _lib.lib().spx_krylov_cgs2(C.c_void_p(V.data_ptr()), 8, 2, C.c_void_p(w.data_ptr()),
                                    C.c_void_p(out.data_ptr()), C.c_void_p(ws.data_ptr()), 8, st)
    assert rc == _lib.SPX_E_WORKSPACE
