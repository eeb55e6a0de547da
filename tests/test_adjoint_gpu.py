"""GPU: the discrete adjoint of fixed-step Dopri8 against central finite differences (h = 1e-6)."""
import numpy as np
import pytest

FD_H = 1e-6


def _problem(nsteps=60, ckpt=None):
    from spectrax_gb300.adjoint import TwoStreamProblem
    # a small two-stream case; loss window shrunk to the short horizon
    return TwoStreamProblem(Nx=17, Nn=16, dt=0.05, nsteps=nsteps, seed=3, ckpt_every=ckpt, window=(0.5, 2.0))


@pytest.mark.gpu
@pytest.mark.parametrize("ckpt", [None, 7, 1000])
def test_parameter_gradients_match_central_differences(ckpt):
    prob = _problem(ckpt=ckpt)
    theta = dict(k=0.35, nu=1.0, u=0.5, amp=1e-3)
    L, g = prob.loss_and_grad(**theta)
    for name in ("k", "nu", "u", "amp"):
        tp, tm = dict(theta), dict(theta)
        tp[name] += FD_H
        tm[name] -= FD_H
        fd = (prob.loss(**tp) - prob.loss(**tm)) / (2 * FD_H)
        assert abs(g[name] - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(L)), (name, g[name], fd)


@pytest.mark.gpu
def test_initial_state_gradient_direction():
    import torch
    from spectrax_gb300.adjoint import Dopri8Adjoint, two_stream_setup, window_weights, loss_from_energy
    from spectrax_gb300.vector_field import plan_for_params
    p, bg, delta, _ = two_stream_setup(0.3, 1.0, 0.5, 1e-3, 9, 10, seed=1)
    plan = plan_for_params(p, "divide")
    adj = Dopri8Adjoint(plan, 0.05, 30, 5)
    y0 = bg + 1e-3 * delta
    w = window_weights(adj.ts, 0.3, 1.2)

    def loss(y):
        E, _ = adj.forward(torch.from_numpy(y).cuda())
        return loss_from_energy(E.cpu().numpy(), w)

    E, _ = adj.forward(torch.from_numpy(y0).cuda())
    En = E.cpu().numpy()
    dLdE = w / En
    dLdE[-1] += 1.0
    mu0, _ = adj.backward(torch.from_numpy(dLdE))
    mu0 = mu0.cpu().numpy()
    rng = np.random.default_rng(0)
    for _ in range(2):
        v = 1e-3 * (rng.standard_normal(len(y0)) + 1j * rng.standard_normal(len(y0)))
        fd = (loss(y0 + FD_H * v) - loss(y0 - FD_H * v)) / (2 * FD_H)
        ad = float(np.real(np.sum(mu0 * v)))
        assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-12, (ad, fd)


@pytest.mark.gpu
def test_autograd_function_wiring():
    import torch
    from spectrax_gb300.adjoint import TwoStreamLoss
    prob = _problem(nsteps=20)
    k = torch.tensor(0.35, dtype=torch.float64, requires_grad=True)
    nu = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    u = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    amp = torch.tensor(1e-3, dtype=torch.float64, requires_grad=True)
    L = TwoStreamLoss.apply(k, nu, u, amp, prob)
    L.backward()
    _, g = prob.loss_and_grad(0.35, 1.0, 0.5, 1e-3)
    assert abs(k.grad.item() - g["k"]) <= 1e-12 * abs(g["k"])
    assert abs(amp.grad.item() - g["amp"]) <= 1e-12 * abs(g["amp"])


@pytest.mark.gpu
def test_fused_vjp_param_matches_separate_kernels():
    import ctypes as C
    import torch
    from spectrax_gb300 import _lib
    from spectrax_gb300.adjoint import two_stream_setup
    from spectrax_gb300.vector_field import plan_for_params
    p, bg, delta, _ = two_stream_setup(0.3, 1.2, 0.5, 1e-3, 17, 24, seed=2)
    plan = plan_for_params(p, "divide")
    n = plan.state_len
    rng = np.random.default_rng(5)
    y = torch.from_numpy(bg + 1e-2 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))).cuda()
    w = torch.from_numpy(rng.standard_normal(n) + 1j * rng.standard_normal(n)).cuda()
    g1, g2 = torch.empty_like(y), torch.empty_like(y)
    a1 = torch.zeros(2 + 3, dtype=torch.float64, device="cuda")
    a2 = torch.full((2 + 3,), 0.25, dtype=torch.float64, device="cuda")     # accumulates onto its input
    L = _lib.lib()
    ws, wsb = plan.ws_ptr()
    ptr = lambda t: C.c_void_p(t.data_ptr())
    dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
    _lib.check(L.spx_vjp(plan.handle, ptr(y), ptr(w), ptr(g1), ws, wsb, None), "spx_vjp")
    _lib.check(L.spx_param_dots(plan.handle, ptr(y), ptr(w), dp(a1), None), "spx_param_dots")
    for _ in range(2):                                  # the ticket resets itself
        _lib.check(L.spx_vjp_param(plan.handle, ptr(y), ptr(w), ptr(g2), dp(a2), ws, wsb, None), "spx_vjp_param")
    torch.cuda.synchronize()
    # same algebra; the fused kernel forms the forward transform of w as conj(inverse(conj w))
    assert (torch.linalg.vector_norm(g1 - g2) / torch.linalg.vector_norm(g1)).item() < 1e-13
    np.testing.assert_allclose((a2.cpu().numpy() - 0.25) / 2, a1.cpu().numpy(), rtol=1e-12, atol=1e-300)


def _hermitian(v, N):
    L = v.reshape(-1, N).copy()
    c0 = N // 2
    L[:, c0] = L[:, c0].real
    L[:, :c0] = np.conj(L[:, ::-1][:, :c0])
    return L.ravel()


@pytest.mark.gpu
@pytest.mark.parametrize("Nx,Nn", [(17, 24), (65, 40), (9, 5)])
def test_packed_vjp_param_matches_general(Nx, Nn):
    # exactly Hermitian y and w: the packed-transform VJP agrees with the general
    # one to rounding, writes an exactly Hermitian g, and the parameter sums agree
    import ctypes as C
    import torch
    from spectrax_gb300 import _lib
    from spectrax_gb300.adjoint import two_stream_setup
    from spectrax_gb300.vector_field import plan_for_params
    p, bg, delta, _ = two_stream_setup(0.3, 1.2, 0.5, 1e-3, Nx, Nn, seed=2)
    plan = plan_for_params(p, "divide")
    n = plan.state_len
    rng = np.random.default_rng(7)
    y = torch.from_numpy(_hermitian(bg + 1e-2 * (rng.standard_normal(n) + 1j * rng.standard_normal(n)), Nx)).cuda()
    w = torch.from_numpy(_hermitian(rng.standard_normal(n) + 1j * rng.standard_normal(n), Nx)).cuda()
    g1, g2 = torch.empty_like(y), torch.empty_like(y)
    a1 = torch.zeros(5, dtype=torch.float64, device="cuda")
    a2 = torch.zeros(5, dtype=torch.float64, device="cuda")
    L = _lib.lib()
    ws, wsb = plan.ws_ptr()
    ptr = lambda t: C.c_void_p(t.data_ptr())
    dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
    _lib.check(L.spx_vjp_param_ex(plan.handle, ptr(y), ptr(w), ptr(g1), dp(a1), ws, wsb, 0, None), "general")
    _lib.check(L.spx_vjp_param_ex(plan.handle, ptr(y), ptr(w), ptr(g2), dp(a2), ws, wsb, 1, None), "packed")
    torch.cuda.synchronize()
    G2 = g2.cpu().numpy().reshape(-1, Nx)
    assert np.array_equal(G2, np.conj(G2[:, ::-1]))
    assert (torch.linalg.vector_norm(g1 - g2) / torch.linalg.vector_norm(g1)).item() < 1e-13
    np.testing.assert_allclose(a2.cpu().numpy(), a1.cpu().numpy(), rtol=1e-12, atol=1e-14 * float(a1.abs().max()))


@pytest.mark.gpu
def test_packed_entry_points_reject_even_nx():
    import ctypes as C
    import torch
    from spectrax_gb300 import _lib
    from spectrax_gb300.adjoint import two_stream_setup
    from spectrax_gb300.vector_field import plan_for_params
    p, bg, _, _ = two_stream_setup(0.3, 1.2, 0.5, 1e-3, 16, 8, seed=2)
    plan = plan_for_params(p, "divide")
    y = torch.from_numpy(bg).cuda()
    Ys = torch.empty((13, plan.state_len), dtype=torch.complex128, device="cuda")
    K = torch.empty_like(Ys)
    yn = torch.empty_like(y)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    rc = _lib.lib().spx_rk_step_store_ex(plan.handle, ptr(y), C.c_double(0.05), ptr(Ys), ptr(K), ptr(yn), 1, None)
    assert rc == _lib.SPX_E_ARG
    acc = torch.zeros(5, dtype=torch.float64, device="cuda")
    ws, wsb = plan.ws_ptr()
    rc = _lib.lib().spx_vjp_param_ex(plan.handle, ptr(y), ptr(y), ptr(yn),
                                     C.cast(C.c_void_p(acc.data_ptr()), C.POINTER(C.c_double)), ws, wsb, 1, None)
    assert rc == _lib.SPX_E_ARG


@pytest.mark.gpu
def test_adjoint_runs_packed_transforms_for_hermitian_states():
    prob = _problem(nsteps=20)
    p, plan, adj, y0, _, _ = prob._build(0.35, 1.0, 0.5, 1e-3)
    adj.forward(y0)
    assert adj.herm


def _general_params(shape, seed):
    from oracle import tables as otab
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    user = dict(Lx=float(rng.uniform(6, 12)), Ly=float(rng.uniform(6, 12)), Lz=float(rng.uniform(6, 12)),
                nu=float(rng.uniform(0.2, 1)), D=float(rng.uniform(0, 0.05)),
                qs=list(rng.choice([-1.0, 1.0], Ns)), alpha_s=list(rng.uniform(0.5, 1.2, 3 * Ns)),
                u_s=list(rng.uniform(-0.5, 0.5, 3 * Ns)), Omega_cs=list(rng.uniform(0.5, 1.5, Ns)))
    return otab.initialize_simulation_parameters(user, *shape, 5, 0.01)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,ckpt", [((6, 5, 1, 3, 2, 2, 1), 3), ((5, 4, 3, 2, 2, 2, 2), None)],
                         ids=["2d", "3d-two-species"])
def test_initial_state_gradient_general_layout(shape, ckpt):
    # 2-D / 3-D layouts: the adjoint recursion through spx_rhs and spx_vjp
    import torch
    from spectrax_gb300.adjoint import Dopri8Adjoint
    from spectrax_gb300.vector_field import plan_for_params
    p = _general_params(shape, 11)
    plan = plan_for_params(p, "divide")
    assert plan.path == 1
    nsteps = 8
    adj = Dopri8Adjoint(plan, 0.02, nsteps, ckpt, masses=[1.0] * shape[-1])
    rng = np.random.default_rng(12)
    n = plan.state_len
    y0 = 1e-2 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    w = rng.uniform(0.5, 1.5, nsteps + 1)

    def loss(y):
        E, _ = adj.forward(torch.from_numpy(y).cuda())
        return float(np.sum(w * E.cpu().numpy()))

    loss(y0)
    mu0, dots = adj.backward(torch.from_numpy(w))
    assert dots is None
    mu0 = mu0.cpu().numpy()
    mu1, _ = adj.backward(torch.from_numpy(w), use_graphs=False)
    assert np.array_equal(mu0, mu1.cpu().numpy())
    for _ in range(2):
        v = 1e-2 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
        fd = (loss(y0 + FD_H * v) - loss(y0 - FD_H * v)) / (2 * FD_H)
        ad = float(np.real(np.sum(mu0 * v)))
        assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-12, (ad, fd)
