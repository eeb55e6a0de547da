"""Physics runs end to end: the Landau damping workload (Nx=33, Nn=64, k=0.5, nu=2,
Dopri8 dt=0.05 to t=40) on the GPU against the oracle run, and the initial-state
builder on the host."""
import os

import numpy as np
import pytest

from oracle import diag as odiag
from oracle import dopri8 as od
from oracle import rhs as orhs
from oracle import tables as otab


def _user(Lx=4 * np.pi, nu=2.0, mi_me=1836.0):
    ae = np.sqrt(2.0)
    return dict(Lx=Lx, nu=nu, D=0.0, qs=[-1.0, 1.0], alpha_s=[ae] * 3 + [ae * np.sqrt(1 / mi_me)] * 3,
                u_s=[0.0] * 6, Omega_cs=[1.0, 1.0 / mi_me], mi_me=mi_me)


def test_landau_initial_state_is_hermitian():
    from spectrax_gb300.params import initialize_simulation_parameters, landau_initial_state
    p = initialize_simulation_parameters(_user(), 33, 1, 1, 64, 1, 1, 2, 5, 0.05)
    y = landau_initial_state(p, 0.01)
    L = y.reshape(-1, 33)
    assert np.all(L == np.conj(L[:, ::-1]))
    assert L[0, 16] == 1 / np.sqrt(2) ** 3 and L[0, 15] == 0.005j / np.sqrt(2) ** 3
    assert L[2 * 64, 15] == L[2 * 64, 17] == pytest.approx(0.01 * 4 * np.pi / (4 * np.pi))


@pytest.mark.gpu
def test_landau_run_matches_oracle():
    import torch
    from spectrax_gb300.dopri8 import Dopri8Solver, species_masses
    from spectrax_gb300.fits import landau_damping_rate
    from spectrax_gb300.params import initialize_simulation_parameters, landau_initial_state
    from spectrax_gb300.vector_field import plan_for_params
    Nx, Nn, Ns = 33, 64, 2
    p = initialize_simulation_parameters(_user(), Nx, 1, 1, Nn, 1, 1, Ns, 401, 0.05)
    po = otab.initialize_simulation_parameters(_user(), Nx, 1, 1, Nn, 1, 1, Ns, 401, 0.05)
    y0 = landau_initial_state(p, 0.01)
    ts = np.linspace(0.0, 40.0, 401)
    s = Dopri8Solver(plan_for_params(p, "divide"), 0.0, 40.0, 0.05, ts=ts, adaptive=False,
                     masses=species_masses(p), max_steps=10000)
    s.reset(torch.from_numpy(y0))
    assert s.run() == 1
    assert s.stats()["hermitian"] and s.stats()["accepted"] == 800
    Eg = s.energies().cpu().numpy()[:, 0]
    ref = od.solve(lambda t, y: orhs.rhs(po, y, "divide"), 0.0, 40.0, y0, 0.05, ts=ts, adaptive=False)
    Eo = odiag.energies(ref["ys"], Nx, 1, 1, Nn, 1, 1, Ns, po["alpha_s"], po["u_s"], po["Omega_cs"],
                        mi_me=1836.0)["EM_energy"]
    np.testing.assert_allclose(Eg, Eo, rtol=1e-9)
    gg, go = landau_damping_rate(ts, Eg, len(ts)), landau_damping_rate(ts, Eo, len(ts))
    assert gg < 0 and abs(gg - go) <= 1e-6 * abs(go)
    # loose physics pin: the reference's damping-rate curve for mi/me = 1836
    # (Examples/damping_rate_1836.csv, copied by tests/golden/make_physics_golden.py)
    curve = np.load(os.path.join(os.path.dirname(__file__), "golden", "physics_curves.npz"))
    g_ref = float(np.interp(0.5, curve["damping_k"], curve["damping_rate"]))
    assert abs(gg - g_ref) <= 0.03 * abs(g_ref), (gg, g_ref)


@pytest.mark.gpu
@pytest.mark.parametrize("kx", [0.3, 0.5])
def test_two_stream_growth_rate_matches_reference_curve(kx, tmp_path):
    # the reference's growth-rate scan (Examples/1D_two_stream_gr_curve.py:55-104)
    # through the drop-in simulation(): its input file, its initial state and box
    # length for the target k v_th / omega_pe, adaptive Dopri8 to t = 80 and the fit
    # log E ~ 2 gamma t over t[300:]; against the reference's tabulated curve
    # (Examples/growth_rate.csv, copied by tests/golden/make_physics_golden.py)
    from example_configs import configs, write_toml
    from spectrax_gb300.dopri8 import simulation
    from spectrax_gb300.params import load_parameters
    path = tmp_path / "gr.toml"
    write_toml(configs()["input_1D_two_stream_gr_curve.toml"], path)
    inp, sol = load_parameters(str(path))
    a0, a3, dn1, dn2, nx = inp["alpha_s"][0], inp["alpha_s"][3], inp["dn1"], inp["dn2"], inp["nx"]
    Nx, Nn = sol["Nx"], sol["Nn"]
    idx = [int((Nx - 1) / 2 - nx), int((Nx - 1) / 2), int((Nx - 1) / 2 + nx)]
    Ck0 = np.zeros((2 * Nn, 1, Nx, 1), np.complex128)
    Ck0[0, 0, idx, 0] = [1j * dn1 / (2 * a0 ** 3), 1 / a0 ** 3, -1j * dn1 / (2 * a0 ** 3)]
    Ck0[Nn, 0, idx, 0] = [1j * dn2 / (2 * a3 ** 3), 1 / a3 ** 3, -1j * dn2 / (2 * a3 ** 3)]
    Lx = np.sqrt(2) * np.pi * a0 / kx
    Fk0 = np.zeros((6, 1, Nx, 1), np.complex128)
    Fk0[0, 0, [idx[0], idx[2]], 0] = (dn1 + dn2) * Lx / (4 * np.pi * nx * inp["Omega_cs"][0])
    inp.update(Ck_0=Ck0, Fk_0=Fk0, Lx=Lx)
    out = simulation(inp, **sol)
    t, E = out["time"], out["EM_energy"]
    gamma = np.polyfit(t[300:], np.log(E[300:]), 1)[0] / 2
    curve = np.load(os.path.join(os.path.dirname(__file__), "golden", "physics_curves.npz"))
    g_ref = float(np.interp(kx, curve["growth_k"], curve["growth_rate"]))
    assert gamma > 0 and abs(gamma - g_ref) <= 0.03 * g_ref, (gamma, g_ref)
