"""GPU: Dopri8 with packed real transforms for exactly Hermitian states (odd Nx).

The stages of an exactly Hermitian state (C(-k) == conj C(k) bit for bit) use
two-for-one real transforms; the result must match the oracle like the general
path does (1e-10 on saved states, 1e-9 on the field energy), keep the symmetry
exactly, and the solver must fall back to the general stages whenever the
symmetry does not hold."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import diag as odiag
from oracle import dopri8 as od
from oracle import rhs as orhs
from oracle import tables as otab


def _params(Nx, Nn, Ns, **kw):
    user = dict(Lx=4 * np.pi, nu=2.0, qs=[-1.0, -1.0, 1.0][:Ns],
                alpha_s=([0.5] * 6 + [0.0117] * 3)[:3 * Ns],
                u_s=([1.0, 0.1, -0.2, -1.0, 0.0, 0.05, 0.0, 0.0, 0.0])[:3 * Ns],
                Omega_cs=[1.0, 1.0, 1 / 1836.0][:Ns], mi_me=1836.0)
    user.update(kw)
    return otab.initialize_simulation_parameters(user, Nx, 1, 1, Nn, 1, 1, Ns, 5, 0.05)


def _hermitian_state(Nx, Nn, Ns, seed=3, amp=1e-2):
    """Random state with C(-k) = conj C(k) on every line (Hermite planes and fields)."""
    rng = np.random.default_rng(seed)
    nlines = Ns * Nn + 6
    y = amp * (rng.standard_normal((nlines, Nx)) + 1j * rng.standard_normal((nlines, Nx)))
    c0 = Nx // 2
    y[:, c0] = y[:, c0].real
    y[:, :c0] = np.conj(y[:, ::-1][:, :c0])          # mirror of the upper half
    for s in range(Ns):
        y[s * Nn, c0] += 1.0
    return y.ravel()


def _is_hermitian(y, Nx):
    L = np.asarray(y).reshape(-1, Nx)
    return bool(np.all(L == np.conj(L[:, ::-1])))


def _solve(p, y0, t1, dt, ts, adaptive, hermitian):
    import torch
    from spectrax_gb300 import dopri8, vector_field
    plan = vector_field.plan_for_params(p, "divide")
    s = dopri8.Dopri8Solver(plan, 0.0, t1, dt, ts=ts, adaptive=adaptive, rtol=1e-10, atol=1e-12,
                            max_steps=100000, masses=dopri8.species_masses(p), hermitian=hermitian)
    s.reset(torch.from_numpy(y0))
    assert s.run() == 1
    return s


CASES = [
    ("fixed_33", 33, 16, 3, False, 0.05, 1.0),
    ("adaptive_65", 65, 24, 2, True, 0.01, 1.5),
    ("fixed_17_tile1", 17, 5, 2, False, 0.05, 0.5),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,Nx,Nn,Ns,adaptive,dt,t1", CASES, ids=[c[0] for c in CASES])
def test_hermitian_stages_match_oracle(name, Nx, Nn, Ns, adaptive, dt, t1):
    p = _params(Nx, Nn, Ns)
    y0 = _hermitian_state(Nx, Nn, Ns)
    assert _is_hermitian(y0, Nx)
    ts = np.linspace(0.0, t1, 5)
    ref = od.solve(lambda t, y: orhs.rhs(p, y, "divide"), 0.0, t1, y0, dt, ts=ts, adaptive=adaptive,
                   rtol=1e-10, atol=1e-12)
    s = _solve(p, y0, t1, dt, ts, adaptive, hermitian=True)
    info = s.stats()
    assert info["hermitian"]
    assert info["accepted"] == ref["accepted"] and info["rejected"] == ref["rejected"], (info, ref)
    ys = s.saved_states().cpu().numpy()
    assert rel_err(ys, ref["ys"]) < 1e-10
    for y in ys:
        assert _is_hermitian(y, Nx)                      # kept exactly, step after step
    e_ref = odiag.energies(ref["ys"], Nx, 1, 1, Nn, 1, 1, Ns, p["alpha_s"], p["u_s"], p["Omega_cs"],
                           mi_me=p["mi_me"])
    np.testing.assert_allclose(s.energies().cpu().numpy()[:, 0], e_ref["EM_energy"], rtol=1e-9)
    # the general stages on the same input agree to rounding
    g = _solve(p, y0, t1, dt, ts, adaptive, hermitian=False)
    assert not g.stats()["hermitian"]
    assert rel_err(ys, g.saved_states().cpu().numpy()) < 1e-12


@pytest.mark.gpu
def test_falls_back_when_not_hermitian():
    p = _params(33, 8, 2)
    y0 = _hermitian_state(33, 8, 2)
    y0[5] += 1e-13j                                     # one entry breaks the symmetry
    ts = np.linspace(0.0, 0.4, 3)
    s = _solve(p, y0, 0.4, 0.05, ts, False, hermitian=True)
    assert not s.stats()["hermitian"]
    ref = od.solve(lambda t, y: orhs.rhs(p, y, "divide"), 0.0, 0.4, y0, 0.05, ts=ts, adaptive=False)
    assert rel_err(s.saved_states().cpu().numpy(), ref["ys"]) < 1e-10


@pytest.mark.gpu
def test_even_nx_never_uses_packed_transforms():
    # even Nx: the wavenumber grid is not antisymmetric (spectrax/_initialization.py:114-117)
    p = _params(32, 8, 2)
    rng = np.random.default_rng(0)
    y0 = 1e-2 * (rng.standard_normal((2 * 8 + 6, 32)) + 1j * rng.standard_normal((2 * 8 + 6, 32)))
    s = _solve(p, y0.ravel(), 0.2, 0.05, np.linspace(0.0, 0.2, 2), False, hermitian=True)
    assert not s.stats()["hermitian"]


@pytest.mark.gpu
@pytest.mark.parametrize("tile,threads", [(6, 256), (3, 128), (3, 256), (0, 0)])
def test_benchmark_configuration_matches_oracle(tile, threads):
    # the exact two-stream workload of the benchmark (Nx=129, Nn=256, Ns=3), with
    # the tile shapes the autotuner chooses between: a few adaptive steps against
    # the oracle stepper (same tableau, same controller)
    import os
    import sys
    import torch
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from spectrax_gb300 import dopri8, vector_field
    p, y0 = bench.two_stream_params(seed=0)
    ts = np.array([0.0, 0.05, 0.1])
    ref = od.solve(lambda t, y: orhs.rhs(p, y, "divide"), 0.0, 0.1, y0, 0.02, ts=ts, adaptive=True,
                   rtol=1e-10, atol=1e-12)
    plan = vector_field.get_plan(vector_field.problem_from_params(p, "divide"), None, tile, threads)
    s = dopri8.Dopri8Solver(plan, 0.0, 0.1, 0.02, ts=ts, adaptive=True, rtol=1e-10, atol=1e-12,
                            masses=[1.0, 1.0, 1836.0])
    s.reset(torch.from_numpy(y0))
    assert s.run() == 1
    info = s.stats()
    assert info["hermitian"]
    assert info["accepted"] == ref["accepted"] and info["rejected"] == ref["rejected"], (info, ref)
    assert rel_err(s.saved_states().cpu().numpy(), ref["ys"]) < 1e-11
