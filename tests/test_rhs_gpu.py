"""GPU parity: the CUDA right-hand side against the FP64 oracle (tolerance 1e-12 relative).

Every call goes through the C ABI (ctypes) of libspectrax_gb300.so."""
import numpy as np
import pytest

from conftest import golden_cases, golden_params, rel_err
from oracle import rhs as orhs
from oracle import tables

TOL = 1e-12
G, NAMES = golden_cases()


def _gpu_rhs(p, y, mask_mode="divide"):
    import torch
    from spectrax_gb300 import vector_field
    plan = vector_field.plan_for_params(p, mask_mode)
    yy = torch.from_numpy(np.ascontiguousarray(y)).cuda()
    out = plan.rhs(yy)
    torch.cuda.synchronize()
    return out.cpu().numpy(), plan


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_rhs_golden(name):
    p = golden_params(G, name)
    dy, _ = _gpu_rhs(p, G[name + "/y"])
    assert rel_err(dy, G[name + "/dy"]) <= TOL


def _random_params(rng, shape, drift=True):
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    user = dict(Lx=float(rng.uniform(2, 20)), Ly=float(rng.uniform(2, 20)), Lz=float(rng.uniform(2, 20)),
                nu=float(rng.uniform(0, 3)), D=float(rng.uniform(0, 0.1)),
                qs=list(rng.choice([-1.0, 1.0], Ns)),
                alpha_s=list(rng.uniform(0.2, 1.5, 3 * Ns)),
                u_s=list(rng.uniform(-1, 1, 3 * Ns) if drift else np.zeros(3 * Ns)),
                Omega_cs=list(rng.uniform(0.1, 2.0, Ns)))
    return tables.initialize_simulation_parameters(user, Nx, Ny, Nz, Nn, Nm, Np, Ns, 10, 0.01)


SHAPES = [
    # 1D1V fused path: odd/even/prime/composite lengths, many Hermite tiles
    (1, 1, 1, 1, 1, 1, 1), (2, 1, 1, 3, 1, 1, 1), (3, 1, 1, 5, 1, 1, 2), (17, 1, 1, 32, 1, 1, 2),
    (33, 1, 1, 64, 1, 1, 2), (64, 1, 1, 9, 1, 1, 3), (65, 1, 1, 40, 1, 1, 2), (129, 1, 1, 37, 1, 1, 3),
    (96, 1, 1, 4, 1, 1, 1), (151, 1, 1, 3, 1, 1, 2), (256, 1, 1, 2, 1, 1, 1), (255, 1, 1, 2, 1, 1, 1),
    # general path
    (8, 1, 1, 3, 3, 4, 2), (5, 6, 1, 2, 3, 2, 2), (5, 4, 3, 3, 2, 2, 1), (16, 16, 1, 3, 3, 3, 2),
    (7, 1, 1, 4, 1, 1, 2), (1, 9, 1, 5, 2, 1, 1), (4, 1, 6, 2, 1, 3, 1), (64, 64, 1, 2, 2, 2, 1),
]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_rhs_random_shapes(shape):
    rng = np.random.default_rng(hash(shape) % (2 ** 32))
    p = _random_params(rng, shape)
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    N = Ns * Nn * Nm * Np * Nx * Ny * Nz + 6 * Nx * Ny * Nz
    y = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    ref = orhs.rhs(p, y)
    dy, plan = _gpu_rhs(p, y)
    assert rel_err(dy, ref) <= TOL, (plan.shape, rel_err(dy, ref))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["divide", "multiply"])
def test_rhs_mask_modes_n33(mode):
    rng = np.random.default_rng(33)
    shape = (33, 1, 1, 12, 1, 1, 2)
    p = _random_params(rng, shape)
    N = 2 * 12 * 33 + 6 * 33
    y = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    ref = orhs.rhs(p, y, mode)
    dy, _ = _gpu_rhs(p, y, mode)
    assert rel_err(dy, ref) <= TOL
    other = orhs.rhs(p, y, "multiply" if mode == "divide" else "divide")
    assert rel_err(dy, other) > 1e-6   # the two conventions really differ at N=33


@pytest.mark.gpu
def test_rhs_zero_and_constant_states():
    rng = np.random.default_rng(5)
    shape = (33, 1, 1, 16, 1, 1, 2)
    p = _random_params(rng, shape)
    N = 2 * 16 * 33 + 6 * 33
    dy, _ = _gpu_rhs(p, np.zeros(N, np.complex128))
    assert np.all(dy == 0)
    y = np.full(N, 1e-300 + 1e-300j)   # tiny values stay finite
    dy, _ = _gpu_rhs(p, y)
    assert np.all(np.isfinite(dy))


@pytest.mark.gpu
def test_drop_in_ode_system_signature():
    import torch
    import spectrax_gb300 as sg
    name = "1d1v_n33_landau"
    p = golden_params(G, name)
    args = sg.make_args(p)
    Nx, Ny, Nz, Nn, Nm, Np, Ns = (int(v) for v in G[name + "/shape"])
    y = torch.from_numpy(G[name + "/y"]).cuda()
    dy = sg.ode_system(Nx, Ny, Nz, Nn, Nm, Np, Ns, 0.0, y, args)
    assert dy.is_cuda and dy.dtype == torch.complex128
    assert rel_err(dy.cpu().numpy(), G[name + "/dy"]) <= TOL
    dy_np = sg.ode_system(Nx, Ny, Nz, Nn, Nm, Np, Ns, 0.0, G[name + "/y"], args)
    assert isinstance(dy_np, np.ndarray) and rel_err(dy_np, G[name + "/dy"]) <= TOL


@pytest.mark.gpu
def test_rhs_rejects_bad_inputs():
    import torch
    import spectrax_gb300 as sg
    from spectrax_gb300 import vector_field
    p = golden_params(G, "1d1v_n9")
    plan = vector_field.plan_for_params(p)
    with pytest.raises(TypeError):
        plan.rhs(torch.zeros(plan.state_len, dtype=torch.complex64, device="cuda"))
    with pytest.raises(ValueError):
        plan.rhs(torch.zeros(plan.state_len + 1, dtype=torch.complex128, device="cuda"))
    with pytest.raises(ValueError):
        sg.make_problem(300, 1, 1, 2, 1, 1, 1, [-1], 1, 0, [1], [1, 1, 1], [0, 0, 0], 1, 1, 1)


@pytest.mark.gpu
def test_oversized_planes_take_the_multipass_path():
    # a general-path plane whose two shared-memory buffers exceed a CTA's
    # shared memory gets plan path 2 (spx_rhs through the multi-pass kernels);
    # the entry points that hold whole planes refuse it before any launch
    import torch
    import spectrax_gb300 as sg
    from spectrax_gb300 import SpectraxError, vector_field
    pb = sg.make_problem(64, 64, 8, 2, 2, 1, 1, [-1], 1, 0, [1], [1, 1, 1], [0, 0, 0], 1, 1, 1)
    plan = vector_field.get_plan(pb)
    assert plan.path == 2
    z = torch.zeros(plan.state_len, dtype=torch.complex128, device="cuda")
    with pytest.raises(SpectraxError):
        plan.jvp_into(z, z.clone(), torch.empty_like(z))


@pytest.mark.gpu
def test_maxwellian_builder_refuses_a_masked_plan():
    import ctypes as C
    import torch
    import spectrax_gb300 as sg
    from spectrax_gb300 import _lib, vector_field
    pb = sg.make_problem(9, 1, 1, 3, 1, 1, 1, [-1], 1, 0, [1], [1, 1, 1], [0, 0, 0], 1, 1, 1)   # 2/3 mask on
    plan = vector_field.get_plan(pb)
    Us = torch.zeros(3 * 9, dtype=torch.float64, device="cuda")
    out = torch.empty(3 * 9, dtype=torch.complex128, device="cuda")
    rc = _lib.lib().spx_maxwellian(plan.handle, C.c_void_p(Us.data_ptr()), None, 0, C.c_void_p(out.data_ptr()),
                                   None)
    assert rc == _lib.SPX_E_ARG
