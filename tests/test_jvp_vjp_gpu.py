"""GPU: linearised right-hand side (JVP) and its transpose (VJP) against the oracle.

The right-hand side is affine plus bilinear, so the oracle JVP is the exact
central difference (f(y+v) - f(y-v)) / 2, and the oracle VJP is the transpose of
the Jacobian assembled column by column from it (1D1V and the general 2-D / 3-D
layout)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import rhs as orhs
from oracle import tables as otab

TOL = 1e-12


def _params(shape, seed=0):
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    user = dict(Lx=float(rng.uniform(3, 12)), Ly=float(rng.uniform(3, 12)), Lz=float(rng.uniform(3, 12)),
                nu=float(rng.uniform(0.2, 2)), D=float(rng.uniform(0, 0.05)),
                qs=list(rng.choice([-1.0, 1.0], Ns)), alpha_s=list(rng.uniform(0.3, 1.4, 3 * Ns)),
                u_s=list(rng.uniform(-0.8, 0.8, 3 * Ns)), Omega_cs=list(rng.uniform(0.2, 1.5, Ns)))
    return otab.initialize_simulation_parameters(user, *shape, 5, 0.01)


def _n(shape):
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    return Ns * Nn * Nm * Np * Nx * Ny * Nz + 6 * Nx * Ny * Nz


def _rand(n, rng):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def _plan(p):
    from spectrax_gb300 import vector_field
    return vector_field.plan_for_params(p, "divide")


JVP_SHAPES = [(17, 1, 1, 20, 1, 1, 2), (33, 1, 1, 7, 1, 1, 3), (64, 1, 1, 5, 1, 1, 1),
              (6, 5, 1, 2, 3, 2, 2), (5, 1, 4, 3, 2, 2, 1), (8, 8, 1, 2, 2, 2, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", JVP_SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_jvp_matches_central_difference(shape):
    import torch
    p = _params(shape, 1)
    rng = np.random.default_rng(2)
    n = _n(shape)
    y, v = _rand(n, rng), _rand(n, rng)
    ref = 0.5 * (orhs.rhs(p, y + v) - orhs.rhs(p, y - v))
    plan = _plan(p)
    yt, vt = torch.from_numpy(y).cuda(), torch.from_numpy(v).cuda()
    out = torch.empty_like(yt)
    plan.jvp_into(yt, vt, out)
    assert rel_err(out.cpu().numpy(), ref) <= TOL


LIN_SHAPES = JVP_SHAPES + [(5, 6, 1, 2, 3, 2, 2), (64, 64, 1, 2, 2, 2, 1), (16, 16, 1, 3, 3, 3, 2)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", LIN_SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_linearized_jvp_is_bit_identical(shape):
    # spx_linearize once, then spx_jvp_lin for several v: the same bits as spx_jvp,
    # and y may change after spx_linearize without affecting later products
    import torch
    p = _params(shape, 5)
    rng = np.random.default_rng(6)
    n = _n(shape)
    plan = _plan(p)
    yt = torch.from_numpy(_rand(n, rng)).cuda()
    y_keep = yt.clone()
    lin = plan.linearize(yt)
    yt.mul_(3.0)
    a, b = torch.empty_like(yt), torch.empty_like(yt)
    for _ in range(3):
        vt = torch.from_numpy(_rand(n, rng)).cuda()
        plan.jvp_lin_into(lin, vt, a)
        plan.jvp_into(y_keep, vt, b)
        assert torch.equal(a, b)
    if n <= 20000:
        ref = 0.5 * (orhs.rhs(p, y_keep.cpu().numpy() + vt.cpu().numpy()) -
                     orhs.rhs(p, y_keep.cpu().numpy() - vt.cpu().numpy()))
        assert rel_err(a.cpu().numpy(), ref) <= TOL


VJP_SHAPES = [(9, 1, 1, 6, 1, 1, 2), (16, 1, 1, 5, 1, 1, 3), (17, 1, 1, 40, 1, 1, 2)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", VJP_SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_vjp_is_transpose(shape):
    import torch
    p = _params(shape, 3)
    rng = np.random.default_rng(4)
    n = _n(shape)
    y, w = _rand(n, rng), _rand(n, rng)
    plan = _plan(p)
    yt, wt = torch.from_numpy(y).cuda(), torch.from_numpy(w).cuda()
    g = torch.empty_like(yt)
    plan.vjp_into(yt, wt, g)
    g = g.cpu().numpy()
    if n <= 400:
        # assemble J column by column (exact for a quadratic map)
        Jm = np.empty((n, n), np.complex128)
        for j in range(n):
            e = np.zeros(n, np.complex128)
            e[j] = 1.0
            Jm[:, j] = 0.5 * (orhs.rhs(p, y + e) - orhs.rhs(p, y - e))
        assert rel_err(g, Jm.T @ w) <= TOL
    # bilinear adjoint identity <w, J v> = <J^T w, v> for random v
    v = _rand(n, rng)
    Jv = 0.5 * (orhs.rhs(p, y + v) - orhs.rhs(p, y - v))
    lhs, rhs = np.sum(w * Jv), np.sum(g * v)
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)


VJP_GEN_SHAPES = [(6, 5, 1, 2, 2, 2, 1), (5, 1, 4, 3, 2, 2, 1), (4, 3, 2, 2, 3, 2, 2), (6, 6, 1, 3, 3, 1, 2),
                  (9, 7, 1, 4, 3, 1, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", VJP_GEN_SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_vjp_general_layout_is_transpose(shape):
    # 2-D / 3-D layouts: J^T w against the oracle Jacobian assembled column by column
    import torch
    p = _params(shape, 3)
    rng = np.random.default_rng(4)
    n = _n(shape)
    y, w = _rand(n, rng), _rand(n, rng)
    plan = _plan(p)
    assert plan.path == 1
    yt, wt = torch.from_numpy(y).cuda(), torch.from_numpy(w).cuda()
    g = torch.empty_like(yt)
    plan.vjp_into(yt, wt, g)
    g = g.cpu().numpy()
    Jm = np.empty((n, n), np.complex128)
    for j in range(n):
        e = np.zeros(n, np.complex128)
        e[j] = 1.0
        Jm[:, j] = 0.5 * (orhs.rhs(p, y + e) - orhs.rhs(p, y - e))
    assert rel_err(g, Jm.T @ w) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(16, 16, 1, 3, 3, 3, 2), (8, 8, 8, 2, 2, 2, 1), (33, 32, 1, 4, 4, 1, 2),
                                   (16, 16, 1, 5, 5, 5, 2)],   # 125 planes per species: two partial field sums
                         ids=lambda s: "x".join(map(str, s)))
def test_vjp_general_layout_adjoint_identity(shape):
    # <w, J v> = <J^T w, v> with J v from the oracle (exact central difference),
    # and J^T w independent of the output buffer's previous contents
    import torch
    p = _params(shape, 7)
    rng = np.random.default_rng(8)
    n = _n(shape)
    y, w, v = _rand(n, rng), _rand(n, rng), _rand(n, rng)
    plan = _plan(p)
    yt, wt = torch.from_numpy(y).cuda(), torch.from_numpy(w).cuda()
    g = torch.full_like(yt, float("nan"))
    plan.vjp_into(yt, wt, g)
    g2 = torch.empty_like(yt)
    plan.vjp_into(yt, wt, g2)
    assert torch.equal(g, g2)
    g = g.cpu().numpy()
    Jv = 0.5 * (orhs.rhs(p, y + v) - orhs.rhs(p, y - v))
    lhs, rhs = np.sum(w * Jv), np.sum(g * v)
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)
    # against the GPU JVP too: <w, J v> from spx_jvp
    Jv_gpu = torch.empty_like(yt)
    plan.jvp_into(yt, torch.from_numpy(v).cuda(), Jv_gpu)
    lhs2 = np.sum(w * Jv_gpu.cpu().numpy())
    assert abs(lhs2 - rhs) <= 1e-11 * abs(lhs2)
