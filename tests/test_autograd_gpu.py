"""GPU: torch autograd through the right-hand side (``RHSFunction``): reverse mode
through spx_vjp (J^H g, torch's convention for complex gradients) and forward
mode through spx_jvp, against the oracle Jacobian assembled column by column
(exact: the right-hand side is affine plus bilinear)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import rhs as orhs
from oracle import tables as otab

SHAPES = [(9, 1, 1, 6, 1, 1, 2), (6, 5, 1, 2, 2, 2, 1), (5, 1, 4, 2, 2, 2, 1)]


def _params(shape, seed):
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    user = dict(Lx=float(rng.uniform(3, 12)), Ly=float(rng.uniform(3, 12)), Lz=float(rng.uniform(3, 12)),
                nu=float(rng.uniform(0.2, 2)), D=float(rng.uniform(0, 0.05)),
                qs=list(rng.choice([-1.0, 1.0], Ns)), alpha_s=list(rng.uniform(0.3, 1.4, 3 * Ns)),
                u_s=list(rng.uniform(-0.8, 0.8, 3 * Ns)), Omega_cs=list(rng.uniform(0.2, 1.5, Ns)))
    return otab.initialize_simulation_parameters(user, *shape, 5, 0.01)


def _jacobian(p, y):
    n = y.size
    J = np.empty((n, n), np.complex128)
    for j in range(n):
        e = np.zeros(n, np.complex128)
        e[j] = 1.0
        J[:, j] = 0.5 * (orhs.rhs(p, y + e) - orhs.rhs(p, y - e))
    return J


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_reverse_and_forward_mode_match_oracle_jacobian(shape):
    import torch
    import torch.autograd.forward_ad as fwAD
    from spectrax_gb300.vector_field import RHSFunction, plan_for_params
    p = _params(shape, 2)
    plan = plan_for_params(p, "divide")
    n = plan.state_len
    rng = np.random.default_rng(3)
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    c = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    J = _jacobian(p, y)
    # reverse: L = Re sum conj(c) f(y)  ->  grad = J^H c
    yt = torch.from_numpy(y).cuda().requires_grad_()
    f = RHSFunction.apply(yt, plan)
    assert rel_err(f.detach().cpu().numpy(), orhs.rhs(p, y)) <= 1e-12
    L = (torch.from_numpy(c).cuda().conj() * f).sum().real
    L.backward()
    assert rel_err(yt.grad.cpu().numpy(), J.conj().T @ c) <= 1e-12
    # forward: tangent J v
    with fwAD.dual_level():
        yd = fwAD.make_dual(torch.from_numpy(y).cuda(), torch.from_numpy(v).cuda())
        tangent = fwAD.unpack_dual(RHSFunction.apply(yd, plan)).tangent
    assert rel_err(tangent.cpu().numpy(), J @ v) <= 1e-12


@pytest.mark.gpu
def test_gradcheck_and_drop_in_entry_point():
    import torch
    from spectrax_gb300 import vector_field
    p = _params((6, 5, 1, 2, 2, 2, 1), 4)
    plan = vector_field.plan_for_params(p, "divide")
    g = torch.Generator().manual_seed(0)
    y = torch.randn(plan.state_len, dtype=torch.complex128, generator=g).cuda().requires_grad_()
    assert torch.autograd.gradcheck(lambda t: vector_field.RHSFunction.apply(t, plan), (y,), eps=1e-6,
                                    atol=1e-6, rtol=1e-6, fast_mode=True, check_forward_ad=True)
    # vector_field.rhs(t, y, params) takes the autograd path for a state that requires grad
    out = vector_field.rhs(0.0, y, p, "divide")
    out.abs().pow(2).sum().backward()
    g1 = y.grad.clone()
    y.grad = None
    vector_field.RHSFunction.apply(y, plan).abs().pow(2).sum().backward()
    assert torch.equal(g1, y.grad)
