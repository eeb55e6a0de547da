"""GPU: the allocation-free VJP entry point (spx_vjp_noalloc) against spx_vjp.

spx_vjp_noalloc serves callers that may not allocate device memory where they
need the vector-Jacobian product (inside a CUDA stream capture, in real-time
loops, under a host framework that owns all device memory).  Its scratch lives
in a fixed 1 MiB device array shared by every call.  This file is collected
last so that a run stopping at the first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

TOL = 1e-12


def _plan(shape, seed=0):
    from oracle import tables as otab
    from spectrax_gb300 import vector_field
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    user = dict(Lx=float(rng.uniform(3, 12)), nu=float(rng.uniform(0.2, 2)), D=0.01,
                qs=list(rng.choice([-1.0, 1.0], Ns)), alpha_s=list(rng.uniform(0.3, 1.4, 3 * Ns)),
                u_s=list(rng.uniform(-0.8, 0.8, 3 * Ns)), Omega_cs=list(rng.uniform(0.2, 1.5, Ns)))
    p = otab.initialize_simulation_parameters(user, *shape, 5, 0.01)
    return vector_field.plan_for_params(p, "divide")


@pytest.mark.gpu
def test_vjp_noalloc_matches_vjp_twice():
    import torch
    plan = _plan((65, 1, 1, 128, 1, 1, 3), seed=1)
    n = plan.state_len
    g = torch.Generator(device="cpu").manual_seed(7)

    def rand():
        re = torch.randn(n, dtype=torch.float64, generator=g)
        im = torch.randn(n, dtype=torch.float64, generator=g)
        return torch.complex(re, im).cuda()

    y = rand()
    for _ in range(2):                      # two calls in a row share the scratch array
        w = rand()
        ref = torch.empty_like(y)
        plan.vjp_into(y, w, ref)
        out = torch.full_like(y, complex(np.nan, np.nan))
        plan.vjp_noalloc_into(y, w, out)
        torch.cuda.synchronize()
        err = (torch.linalg.vector_norm(out - ref) / torch.linalg.vector_norm(ref)).item()
        assert err <= TOL, err


@pytest.mark.gpu
def test_vjp_noalloc_rejects_oversized_problem():
    import torch
    from spectrax_gb300 import _lib
    plan = _plan((256, 1, 1, 4000, 1, 1, 8), seed=2)
    L = _lib.lib()
    buf = [torch.zeros(16, dtype=torch.complex128, device="cuda") for _ in range(3)]
    rc = L.spx_vjp_noalloc(plan.handle, C.c_void_p(buf[0].data_ptr()), C.c_void_p(buf[1].data_ptr()),
                           C.c_void_p(buf[2].data_ptr()), None)
    assert rc == _lib.SPX_E_UNSUPPORTED
    assert b"fixed maximum" in L.spx_last_error()
