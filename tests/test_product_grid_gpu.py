"""GPU: the 1D1V stepper's nonlinear products on a cheaper grid (M >= 3K + 1
points instead of Nx, plus the one term the Nx-point grid folds onto |k| = K
when Nx = 3K) against the Nx-point products and against the oracle."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import dopri8 as od
from oracle import rhs as orhs
from oracle import tables as otab


def _params(Nx, Nn, Ns, seed):
    rng = np.random.default_rng(seed)
    user = dict(Lx=float(rng.uniform(6, 30)), nu=float(rng.uniform(0.2, 2)), D=0.0,
                qs=list(rng.choice([-1.0, 1.0], Ns)), alpha_s=list(rng.uniform(0.4, 1.2, 3 * Ns)),
                u_s=list(rng.uniform(-0.8, 0.8, 3 * Ns)), Omega_cs=list(rng.uniform(0.5, 1.5, Ns)))
    return otab.initialize_simulation_parameters(user, Nx, 1, 1, Nn, 1, 1, Ns, 5, 0.01)


def _state(Nx, Nn, Ns, hermitian, seed):
    rng = np.random.default_rng(seed)
    n = Ns * Nn * Nx + 6 * Nx
    y = 1e-2 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    if hermitian:
        L = y.reshape(-1, Nx)
        y = (0.5 * (L + np.conj(L[:, ::-1]))).reshape(-1)
    return y


def _run(p, y0, mode, mask, steps=6, dt=0.02):
    import torch
    from spectrax_gb300 import dopri8, vector_field
    vector_field.set_product_grid(mode)
    try:
        plan = vector_field.plan_for_params(p, mask)
        ts = np.arange(steps + 1) * dt
        s = dopri8.Dopri8Solver(plan, 0.0, ts[-1], dt, ts=ts, adaptive=False, max_steps=steps + 5,
                                masses=[1.0] * p["Ns"])
        s.reset(torch.from_numpy(y0))
        assert s.run() == 1
        return plan.product_grid, s.saved_states().cpu().numpy(), bool(s.stats()["hermitian"])
    finally:
        vector_field.set_product_grid("auto")


CASES = [  # Nx, mask, grid mode, expected product grid, Nn, Ns, Hermitian state
    (129, "divide", "fp64", 136, 10, 2, False),   # Nx = 3K: the folded term is added back
    (129, "divide", "fp64", 136, 10, 2, True),    # same, packed real transforms
    (65, "divide", "fp64", 64, 12, 2, True),
    (97, "divide", "auto", 108, 6, 2, False),     # prime Nx
    (129, "divide", "auto", 144, 6, 2, True),     # the benchmark's grid: 4*4*3*3, Nx = 3K
    (129, "divide", "auto", 144, 7, 3, False),
    (33, "divide", "auto", 36, 9, 2, True),       # Nx = 3K, Ns * tiles > 1
    (17, "divide", "auto", 16, 7, 3, False),
    (33, "divide", "fp64", 33, 9, 2, True),       # no cheaper grid by the FP64 count: unchanged
    (17, "divide", "fp64", 17, 7, 3, False),
]


@pytest.mark.gpu
@pytest.mark.parametrize("Nx,mask,mode,M,Nn,Ns,herm", CASES,
                         ids=[f"{c[0]}-{c[2]}-{'herm' if c[6] else 'gen'}" for c in CASES])
def test_product_grid_matches_nx_grid_and_oracle(Nx, mask, mode, M, Nn, Ns, herm):
    p = _params(Nx, Nn, Ns, Nx + Nn)
    y0 = _state(Nx, Nn, Ns, herm, Nx * 3 + Nn)
    m_auto, ys_auto, h_auto = _run(p, y0, mode, mask)
    m_nx, ys_nx, h_nx = _run(p, y0, "nx", mask)
    assert m_auto == M and m_nx == Nx
    assert h_auto == h_nx == herm
    assert rel_err(ys_auto, ys_nx) <= 1e-12
    ref = od.solve(lambda t, y: orhs.rhs(p, y, mask), 0.0, 0.12, y0, 0.02, ts=np.arange(7) * 0.02,
                   adaptive=False)
    assert rel_err(ys_auto, ref["ys"]) <= 1e-11


@pytest.mark.gpu
def test_persistent_request_falls_back_on_a_product_grid():
    # the persistent kernel is compiled for Nx-point products only: a plan with
    # its own grid runs per-stage launches, with the same results
    import torch
    from spectrax_gb300 import dopri8, vector_field
    p = _params(97, 6, 2, 5)
    y0 = _state(97, 6, 2, True, 6)
    try:
        vector_field.set_product_grid("auto")
        plan = vector_field.plan_for_params(p, "divide")
        assert plan.product_grid == 108
        out = []
        for persistent in (True, False):
            s = dopri8.Dopri8Solver(plan, 0.0, 0.1, 0.02, ts=np.linspace(0, 0.1, 3), adaptive=False,
                                    max_steps=20, masses=[1.0, 1.0], persistent=persistent,
                                    saveat="land")
            s.reset(torch.from_numpy(y0))
            assert s.run() == 1
            assert not s.stats()["persistent"]
            out.append(s.saved_states().cpu().numpy())
        assert np.array_equal(out[0], out[1])
    finally:
        vector_field.set_product_grid("auto")


@pytest.mark.gpu
def test_adjoint_recomputation_on_a_product_grid():
    # the adjoint's staged recomputation on a plan with its own product grid
    # (65 -> 64 points) gives the gradient of the Nx-grid plan to rounding
    import torch
    from spectrax_gb300 import vector_field
    from spectrax_gb300.adjoint import Dopri8Adjoint, two_stream_setup, window_weights
    p, bg, delta, _ = two_stream_setup(0.3, 1.0, 0.5, 1e-3, 65, 12, seed=2)
    y0 = torch.from_numpy(bg + 1e-3 * delta).cuda()
    res = {}
    try:
        for mode in ("fp64", "nx"):
            vector_field.set_product_grid(mode)
            plan = vector_field.plan_for_params(p, "divide")
            adj = Dopri8Adjoint(plan, 0.05, 12, 4)
            E, _ = adj.forward(y0)
            w = window_weights(adj.ts, 0.1, 0.5)
            dLdE = torch.from_numpy(w / E.cpu().numpy())
            mu, dots = adj.backward(dLdE)
            res[mode] = (plan.product_grid, E.cpu().numpy(), mu.cpu().numpy(), dots.cpu().numpy())
    finally:
        vector_field.set_product_grid("auto")
    assert res["fp64"][0] == 64 and res["nx"][0] == 65
    for i in (1, 2, 3):
        assert rel_err(res["fp64"][i], res["nx"][i]) <= 1e-10, i


@pytest.mark.gpu
@pytest.mark.parametrize("Nx,herm", [(65, True), (65, False), (17, True), (97, False)])
def test_vjp_param_on_the_product_grid(Nx, herm):
    # the adjoint sweep's kernel on a plan with its own product grid (no folded
    # |k| = K term): the same g and parameter sums as on the Nx-point grid
    import ctypes as C

    import torch
    from spectrax_gb300 import _lib, vector_field
    from spectrax_gb300.vector_field import _stream_ptr
    Nn, Ns = 12, 2
    p = _params(Nx, Nn, Ns, Nx)
    y = torch.from_numpy(_state(Nx, Nn, Ns, herm, 11)).cuda()
    w = torch.from_numpy(_state(Nx, Nn, Ns, herm, 12)).cuda()
    out = {}
    for mode in ("auto", "nx"):
        vector_field.set_product_grid(mode)
        try:
            plan = vector_field.plan_for_params(p, "divide")
        finally:
            vector_field.set_product_grid("auto")
        g = torch.empty_like(y)
        acc = torch.zeros(2 + _lib.MAX_SPECIES, dtype=torch.float64, device=y.device)
        ws, wsb = plan.ws_ptr()
        _lib.check(_lib.lib().spx_vjp_param_ex(plan.handle, C.c_void_p(y.data_ptr()), C.c_void_p(w.data_ptr()),
                                                C.c_void_p(g.data_ptr()),
                                                C.cast(C.c_void_p(acc.data_ptr()), C.POINTER(C.c_double)),
                                                ws, wsb, int(herm), _stream_ptr()), "spx_vjp_param_ex")
        torch.cuda.synchronize()
        out[mode] = (plan.product_grid, g.cpu().numpy(), acc.cpu().numpy())
    assert out["auto"][0] != Nx and out["nx"][0] == Nx
    assert rel_err(out["auto"][1], out["nx"][1]) <= 1e-12
    a, b = out["auto"][2][:2 + Ns], out["nx"][2][:2 + Ns]
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
