"""GPU: the device Dopri8 solver against the oracle stepper (same tableau, same controller).

Trajectory tolerance: 1e-10 relative on saved states, 1e-9 relative on the field energy."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import diag as odiag
from oracle import dopri8 as od
from oracle import rhs as orhs
from oracle import tables as otab


def _params(shape, **kw):
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    user = dict(Lx=4 * np.pi, Ly=5.0, Lz=3.0, nu=2.0, qs=[-1.0, 1.0, -1.0][:Ns],
                alpha_s=([1.41, 1.2, 1.1] + [0.033] * 3 + [0.9] * 3)[:3 * Ns],
                u_s=([0.0, 0.1, -0.1, 0.0, 0.0, 0.05, 0.5, 0.0, 0.0])[:3 * Ns],
                Omega_cs=[1.0, 1 / 1836.0, 1.0][:Ns], mi_me=1836.0)
    user.update(kw)
    return otab.initialize_simulation_parameters(user, *shape, 5, 0.05)


def _y0(shape, seed=1, amp=0.01):
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    n = Ns * Nn * Nm * Np * Nx * Ny * Nz + 6 * Nx * Ny * Nz
    rng = np.random.default_rng(seed)
    y = amp * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    # a background Maxwellian (n=0, k=0) per species keeps the problem physical
    plane = Nx * Ny * Nz
    kc = ((Ny // 2) * Nx + Nx // 2) * Nz + Nz // 2
    for s in range(Ns):
        y[s * Nn * Nm * Np * plane + kc] += 1.0
    return y


def _run_gpu(p, y0, t1, dt, ts, adaptive, rtol=1e-10, atol=1e-12, max_steps=100000, saveat="interpolate"):
    import torch
    from spectrax_gb300 import dopri8, vector_field
    plan = vector_field.plan_for_params(p, "divide")
    s = dopri8.Dopri8Solver(plan, 0.0, t1, dt, ts=ts, adaptive=adaptive, rtol=rtol, atol=atol,
                            max_steps=max_steps, masses=dopri8.species_masses(p), saveat=saveat)
    s.reset(torch.from_numpy(y0))
    st = s.run()
    return s, st


CASES = [
    ("1v_fixed", (17, 1, 1, 12, 1, 1, 2), False, 0.05, 1.0, 6),
    ("1v_adaptive", (33, 1, 1, 16, 1, 1, 3), True, 0.01, 1.5, 6),
    ("1v_dense_saves", (33, 1, 1, 16, 1, 1, 3), True, 0.01, 1.5, 61),   # several saves inside one step
    ("1v_fixed_off_grid", (17, 1, 1, 12, 1, 1, 2), False, 0.07, 1.0, 9),
    ("gen_fixed", (6, 5, 1, 2, 2, 2, 2), False, 0.02, 0.2, 6),
    ("gen_adaptive", (5, 1, 4, 3, 2, 2, 1), True, 0.05, 0.3, 6),
    ("gen_dense_saves", (5, 1, 4, 3, 2, 2, 1), True, 0.05, 0.3, 31),
    ("gen_adaptive_reject", (5, 1, 4, 3, 2, 2, 1), True, 0.1, 0.3, 31),
    ("gen2d_adaptive", (6, 5, 1, 2, 2, 2, 2), True, 0.1, 0.2, 21),
]
# First steps are chosen so that every error estimate is well above rounding
# (scaled error norm >= 1e-3): a norm of ~1e-7 is rounding noise of the stage
# combination, GPU and oracle then propose different next steps, and with a
# few coarse steps the interpolated saves differ by the interpolation error.


@pytest.mark.gpu
@pytest.mark.parametrize("saveat", ["interpolate", "land"])
@pytest.mark.parametrize("name,shape,adaptive,dt,t1,nts", CASES, ids=[c[0] for c in CASES])
def test_dopri8_matches_oracle(name, shape, adaptive, dt, t1, nts, saveat):
    # identical step sequences (accepted, rejected, RHS evaluations) in both save
    # modes; saved states (interpolated or landed on) within 1e-10
    p = _params(shape)
    y0 = _y0(shape)
    ts = np.linspace(0.0, t1, nts)
    f = lambda t, y: orhs.rhs(p, y, "divide")
    ref = od.solve(f, 0.0, t1, y0, dt, ts=ts, adaptive=adaptive, rtol=1e-10, atol=1e-12, saveat=saveat)
    s, st = _run_gpu(p, y0, t1, dt, ts, adaptive, saveat=saveat)
    assert st == 1
    info = s.stats()
    assert info["accepted"] == ref["accepted"] and info["rejected"] == ref["rejected"], (info, ref)
    assert info["rhs_evals"] == ref["rhs_evals"]
    assert info["saved"] == nts
    ys = s.saved_states().cpu().numpy()
    assert rel_err(ys, ref["ys"]) < 1e-10
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    e_ref = odiag.energies(ref["ys"], Nx, Ny, Nz, Nn, Nm, Np, Ns, p["alpha_s"], p["u_s"], p["Omega_cs"],
                           mi_me=p["mi_me"])
    en = s.energies().cpu().numpy()
    np.testing.assert_allclose(en[:, 0], e_ref["EM_energy"], rtol=1e-9)
    np.testing.assert_allclose(en[:, 1], e_ref["kinetic_energy"].real, rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(en[:, 2:], e_ref["kinetic_energy_species"].real, rtol=1e-9, atol=1e-300)


@pytest.mark.gpu
def test_dopri8_rejections_reuse_stage_one():
    # a deliberately too-large first step must be rejected and retried with 12 new stages
    shape = (17, 1, 1, 24, 1, 1, 2)
    p = _params(shape, nu=0.5)
    y0 = _y0(shape, amp=0.05)
    f = lambda t, y: orhs.rhs(p, y, "divide")
    ref = od.solve(f, 0.0, 0.6, y0, 0.5, ts=np.array([0.6]), adaptive=True, rtol=1e-10, atol=1e-12)
    assert ref["rejected"] > 0
    s, st = _run_gpu(p, y0, 0.6, 0.5, np.array([0.6]), True)
    info = s.stats()
    assert st == 1 and info["rejected"] == ref["rejected"] and info["rhs_evals"] == ref["rhs_evals"]
    assert rel_err(s.state().cpu().numpy(), ref["ys"][-1]) < 1e-10


@pytest.mark.gpu
def test_dopri8_status_words():
    shape = (9, 1, 1, 6, 1, 1, 2)
    p = _params(shape)
    y0 = _y0(shape)
    s, st = _run_gpu(p, y0, 1.0, 0.01, None, False, max_steps=5)
    assert st == 2 and s.stats()["accepted"] == 5                       # MAX_STEPS
    bad = y0.copy()
    bad[3] = np.nan
    s, st = _run_gpu(p, bad, 1.0, 0.1, None, False)
    assert st == 4                                                      # NONFINITE
    s, st = _run_gpu(p, bad, 1.0, 0.1, None, True)
    assert st == 3                                                      # DT_UNDERFLOW (rejected forever)
    s, st = _run_gpu(p, y0, 0.0, 0.1, np.array([0.0]), True)
    assert st == 1 and s.stats()["saved"] == 1                          # empty interval


@pytest.mark.gpu
def test_simulation_driver_defaults():
    # the reference's default run (two-stream defaults), shortened
    import spectrax_gb300.dopri8 as d8
    out = d8.simulation({"t_max": 2.0, "ode_tolerance": 1e-10}, Nx=33, Nn=20, timesteps=11)
    assert set(["Ck", "Fk", "time", "dCk", "EM_energy", "total_energy"]) <= set(out)
    assert not np.all(out["Fk"] == 0)
    assert out["Ck"].shape == (11, 40, 1, 33, 1)


@pytest.mark.gpu
@pytest.mark.parametrize("saveat", ["interpolate", "land"])
def test_host_driven_dopri8_matches_oracle(saveat):
    # the plain RHS driven from the host (external-solver use of the drop-in)
    import torch
    from spectrax_gb300 import dopri8, vector_field
    shape = (33, 1, 1, 16, 1, 1, 3)
    p = _params(shape)
    y0 = _y0(shape)
    ts = np.linspace(0.0, 1.0, 23)
    ref = od.solve(lambda t, y: orhs.rhs(p, y, "divide"), 0.0, 1.0, y0, 0.01, ts=ts, adaptive=True,
                   rtol=1e-10, atol=1e-12, saveat=saveat)
    plan = vector_field.plan_for_params(p, "divide")
    y, ys, st = dopri8.host_dopri8_solve(plan, torch.from_numpy(y0), 1.0, 0.01, ts=ts, rtol=1e-10, atol=1e-12,
                                         saveat=saveat)
    assert st["status_name"] == "DONE"
    assert st["accepted"] == ref["accepted"] and st["rejected"] == ref["rejected"], (st, ref)
    assert rel_err(ys.cpu().numpy(), ref["ys"]) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(17, 1, 1, 12, 1, 1, 2), (6, 5, 1, 2, 2, 2, 2)], ids=["1v", "general"])
def test_reset_and_export_through_host_memory(shape):
    # reset from page-locked host memory, from a device tensor and from a NumPy
    # array give the same solve; the state read back into page-locked, pageable
    # and device memory is the same (no host round trip for the buffer index)
    import torch
    from spectrax_gb300 import dopri8, vector_field
    p = _params(shape)
    y0 = _y0(shape)
    plan = vector_field.plan_for_params(p, "divide")
    outs = []
    for src in ("pinned", "device", "numpy"):
        s = dopri8.Dopri8Solver(plan, 0.0, 1e9, 0.01, adaptive=True, max_steps=1 << 30, save_states=False)
        y = {"pinned": torch.from_numpy(y0).pin_memory(), "device": torch.from_numpy(y0).cuda(), "numpy": y0}[src]
        for _ in range(2):                          # a second reset starts over
            s.reset(y)
            s.enqueue(5)
        pinned = torch.empty(plan.state_len, dtype=torch.complex128).pin_memory()
        pageable = torch.empty(plan.state_len, dtype=torch.complex128)
        s._copy(0, pinned)
        s._copy(0, pageable)
        dev = s.state()
        torch.cuda.synchronize()
        assert torch.equal(pinned, pageable) and torch.equal(pinned, dev.cpu())
        outs.append(pinned.numpy().copy())
        assert s.stats()["accepted"] + s.stats()["rejected"] == 5
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
