"""GPU: the persistent cooperative Dopri8 kernel against the per-stage launches.

Both run the same stage body (staged_stage_1v) in the same order, so saved
states, energies and step counts must agree bit for bit; the persistent one
chains stages through per-CTA completion counters inside one launch."""
import numpy as np
import pytest

from oracle import tables as otab


def _params(Nx, Nn, Ns):
    user = dict(Lx=4 * np.pi, nu=2.0, qs=[-1.0, -1.0, 1.0][:Ns],
                alpha_s=([0.5] * 6 + [0.0117] * 3)[:3 * Ns],
                u_s=([1.0, 0.1, -0.2, -1.0, 0.0, 0.05, 0.0, 0.0, 0.0])[:3 * Ns],
                Omega_cs=[1.0, 1.0, 1 / 1836.0][:Ns], mi_me=1836.0)
    return otab.initialize_simulation_parameters(user, Nx, 1, 1, Nn, 1, 1, Ns, 5, 0.05)


def _state(Nx, Nn, Ns, hermitian, seed=5, amp=1e-2):
    rng = np.random.default_rng(seed)
    y = amp * (rng.standard_normal((Ns * Nn + 6, Nx)) + 1j * rng.standard_normal((Ns * Nn + 6, Nx)))
    if hermitian:
        c0 = Nx // 2
        y[:, c0] = y[:, c0].real
        y[:, :c0] = np.conj(y[:, ::-1][:, :c0])
    for s in range(Ns):
        y[s * Nn, Nx // 2] += 1.0
    return y.ravel()


def _run(plan, p, y0, t1, dt, ts, adaptive, persistent, max_steps=100000):
    import torch
    from spectrax_gb300 import dopri8
    s = dopri8.Dopri8Solver(plan, 0.0, t1, dt, ts=ts, adaptive=adaptive, rtol=1e-10, atol=1e-12,
                            max_steps=max_steps, masses=dopri8.species_masses(p), persistent=persistent,
                            saveat="land")
    s.reset(torch.from_numpy(y0))
    status = s.run()
    return s, status


def _nx_plan(p, tile):
    # the persistent kernel is compiled for Nx-point products: plans on the Nx grid
    from spectrax_gb300 import vector_field
    vector_field.set_product_grid("nx")
    try:
        return vector_field.get_plan(vector_field.problem_from_params(p, "divide"), None, tile, 256)
    finally:
        vector_field.set_product_grid("auto")


CASES = [
    # name, Nx, Nn, Ns, hermitian, adaptive, dt0, t1, tile
    ("herm_adaptive_65", 65, 40, 3, True, True, 0.2, 2.0, 0),
    ("general_fixed_33", 33, 16, 2, False, False, 0.05, 1.0, 0),
    ("herm_fixed_17_tile1", 17, 6, 2, True, False, 0.05, 0.6, 1),
    ("general_adaptive_tile2", 33, 9, 2, False, True, 0.5, 1.0, 2),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,Nx,Nn,Ns,herm,adaptive,dt,t1,tile", CASES, ids=[c[0] for c in CASES])
def test_persistent_matches_stage_launches(name, Nx, Nn, Ns, herm, adaptive, dt, t1, tile):
    p = _params(Nx, Nn, Ns)
    plan = _nx_plan(p, tile)
    y0 = _state(Nx, Nn, Ns, herm)
    ts = np.linspace(0.0, t1, 7)
    a, sa = _run(plan, p, y0, t1, dt, ts, adaptive, persistent=True)
    b, sb = _run(plan, p, y0, t1, dt, ts, adaptive, persistent=False)
    ia, ib = a.stats(), b.stats()
    assert ia["persistent"] and not ib["persistent"]
    assert sa == sb == 1
    assert ia["hermitian"] == ib["hermitian"] == herm
    for k in ("accepted", "rejected", "rhs_evals", "saved", "t"):
        assert ia[k] == ib[k], (k, ia, ib)
    if adaptive:
        assert ia["rejected"] > 0                          # the rebuilt first stage input is covered
    assert np.array_equal(a.saved_states().cpu().numpy(), b.saved_states().cpu().numpy())
    assert np.array_equal(a.energies().cpu().numpy(), b.energies().cpu().numpy())
    assert np.array_equal(a.state().cpu().numpy(), b.state().cpu().numpy())


@pytest.mark.gpu
def test_persistent_stops_at_max_steps():
    p = _params(33, 8, 2)
    plan = _nx_plan(p, 0)
    y0 = _state(33, 8, 2, True)
    a, sa = _run(plan, p, y0, 10.0, 0.05, None, False, persistent=True, max_steps=13)
    b, sb = _run(plan, p, y0, 10.0, 0.05, None, False, persistent=False, max_steps=13)
    assert sa == sb == 2                                   # SPX_ST_MAX_STEPS
    assert a.stats()["accepted"] == b.stats()["accepted"] == 13
    assert np.array_equal(a.state().cpu().numpy(), b.state().cpu().numpy())


@pytest.mark.gpu
def test_bounded_counter_wait_times_out_and_the_context_stays_usable():
    # the persistent kernel's counter waits are made to run out (a target no CTA
    # publishes, 1000 polls): the solve must stop with SPX_ST_WAIT_TIMEOUT, the
    # wrapper must raise, and the same solver must then run normally again
    import torch
    from spectrax_gb300 import _lib, dopri8
    p = _params(33, 16, 2)
    plan = _nx_plan(p, 0)
    y0 = _state(33, 16, 2, True)
    s = dopri8.Dopri8Solver(plan, 0.0, 1.0, 0.05, ts=np.linspace(0, 1.0, 5), adaptive=False,
                            masses=dopri8.species_masses(p), persistent=True, saveat="land")
    s.set_wait_test(polls=1000, unreachable=True)
    s.reset(torch.from_numpy(y0))
    with pytest.raises(dopri8.DeviceWaitTimeout):
        s.run()
    torch.cuda.synchronize()                               # the context is intact
    st = s.stats()
    assert st["persistent"] and st["status"] == _lib.SPX_ST_WAIT_TIMEOUT
    s.set_wait_test()                                      # back to the default limit
    s.reset(torch.from_numpy(y0))
    assert s.run() == 1
    ref, sref = _run(plan, p, y0, 1.0, 0.05, np.linspace(0, 1.0, 5), False, persistent=False)
    assert sref == 1
    assert np.array_equal(s.state().cpu().numpy(), ref.state().cpu().numpy())
