"""CPU: the oracle against fixtures generated from the reference's own source."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, golden_params, rel_err
from oracle import diag, fits, rhs, tables


G, NAMES = golden_cases()


@pytest.mark.parametrize("name", NAMES)
def test_rhs_matches_reference_source(name):
    p = golden_params(G, name)
    dy = rhs.rhs(p, G[name + "/y"])
    assert rel_err(dy, G[name + "/dy"]) <= 1e-13


def test_tables_match_reference_source():
    t = np.load(os.path.join(GOLDEN, "tables.npz"))
    for name in NAMES:
        if name == "defaults":
            continue
        p = golden_params(G, name)
        for k in ("kx_grid", "ky_grid", "kz_grid", "k2_grid", "nabla", "collision_matrix",
                  "sqrt_n_plus", "sqrt_m_minus", "sqrt_p_plus"):
            np.testing.assert_allclose(p[k], t[f"{name}/{k}"], rtol=0, atol=0)
        Nx, Ny, Nz = (int(v) for v in G[name + "/shape"][:3])
        np.testing.assert_array_equal(rhs.twothirds_mask(Ny, Nx, Nz), t[f"{name}/mask"])
    p = tables.initialize_simulation_parameters({}, 33, 1, 1, 20, 1, 1, 2, 10, 0.01)
    assert p["vte"] == t["defaults/vte"] and p["vti"] == t["defaults/vti"]
    np.testing.assert_array_equal(tables.initial_state(p), G["defaults/y"])


def test_energies_match_reference_source():
    g = np.load(os.path.join(GOLDEN, "diag.npz"))
    for name in sorted({k.split("/")[0] for k in g.files}):
        Nx, Ny, Nz, Nn, Nm, Np, Ns = (int(v) for v in g[name + "/shape"])
        e = diag.energies(g[name + "/ys"], Nx, Ny, Nz, Nn, Nm, Np, Ns, g[name + "/alpha_s"],
                          g[name + "/u_s"], g[name + "/Omega_cs"], mi_me=float(g[name + "/mi_me"]))
        for k in ("EM_energy", "kinetic_energy", "total_energy", "kinetic_energy_species"):
            np.testing.assert_allclose(e[k], g[f"{name}/{k}"], rtol=1e-14, atol=0)


def test_mask_edge_rounding():
    # N=33: JAX's divide form keeps |k| <= 11 (23 modes); the multiply form 21 modes
    assert rhs.centered_cutoff(33, "divide") == 11
    assert rhs.centered_cutoff(33, "multiply") == 10
    for n in (17, 64, 65, 129):
        assert rhs.centered_cutoff(n, "divide") == rhs.centered_cutoff(n, "multiply") == n // 3
    assert rhs.twothirds_mask(1, 33, 1, "divide").sum() == 23
    assert rhs.twothirds_mask(1, 33, 1, "multiply").sum() == 21


def test_hermite_neighbor_direction():
    # shift_multi(C, dn=+1) reads C_{n+1} (spectrax/_model.py:79-97)
    C = np.arange(2 * 1 * 1 * 4, dtype=np.complex128).reshape(2, 1, 1, 4, 1, 1, 1)
    up = rhs.hermite_neighbor(C, 1, 0, 0)
    dn = rhs.hermite_neighbor(C, -1, 0, 0)
    assert up[0, 0, 0, 0, 0, 0, 0] == C[0, 0, 0, 1, 0, 0, 0] and up[0, 0, 0, 3, 0, 0, 0] == 0
    assert dn[0, 0, 0, 1, 0, 0, 0] == C[0, 0, 0, 0, 0, 0, 0] and dn[0, 0, 0, 0, 0, 0, 0] == 0


def test_rhs_is_affine_plus_bilinear():
    # f(y) = L y + N(F, C): check the bilinear identity on the golden 2D3V case
    name = "2d3v_6x5"
    p = golden_params(G, name)
    rng = np.random.default_rng(3)
    n = len(G[name + "/y"])
    a = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    f = lambda y: rhs.rhs(p, y)
    # s -> f(a + s b) is a quadratic polynomial: its third difference vanishes
    third = f(a + 3 * b) - 3 * f(a + 2 * b) + 3 * f(a + b) - f(a)
    assert np.linalg.norm(third) <= 1e-12 * np.linalg.norm(f(a + 3 * b))
    # and the map is not affine (the nonlinear term is really there)
    second = f(a + 2 * b) - 2 * f(a + b) + f(a)
    assert np.linalg.norm(second) > 1e-3 * np.linalg.norm(f(a))


def test_fits_on_synthetic_signals():
    t = np.linspace(0, 40, 801)
    E = np.exp(2 * -0.15 * t) * (1.1 + np.cos(2.8 * t))
    assert abs(fits.landau_rate(t, E, 100) - (-0.15)) < 5e-3
    E2 = 1e-8 * np.exp(2 * 0.2 * t)
    assert abs(fits.growth_rate(t, E2, 300) - 0.2) < 1e-10
    assert abs(fits.window_slope(t, E2, 10, 40) - 0.4) < 1e-10


def test_physics_curve_fixture():
    # the copied reference curves: damping at k = 0.5 (the Landau workload) and
    # a positive two-stream growth rate somewhere on the curve
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "physics_curves.npz"))
    assert d["damping_k"].shape == d["damping_rate"].shape == (200,)
    g = float(np.interp(0.5, d["damping_k"], d["damping_rate"]))
    assert -0.16 < g < -0.15
    assert np.max(d["growth_rate"]) > 0


def test_oracle_two_stream_growth_rate_on_reference_curve(tmp_path):
    # the oracle stepping the reference's growth-rate example (input file, initial
    # state and box length of Examples/1D_two_stream_gr_curve.py:55-104 at
    # k v_th / omega_pe = 0.5, adaptive Dopri8 to t = 80, fit over t[300:]):
    # within 1 % of the tabulated curve (Examples/growth_rate.csv)
    import os
    from example_configs import configs, write_toml
    from oracle import diag as odiag
    from oracle import dopri8 as od
    from oracle import rhs as orhs
    from oracle import tables as otab
    from spectrax_gb300.params import load_parameters
    path = tmp_path / "gr.toml"
    write_toml(configs()["input_1D_two_stream_gr_curve.toml"], path)
    inp, sol = load_parameters(str(path))
    kx = 0.5
    a0, a3, dn1, dn2, nx = inp["alpha_s"][0], inp["alpha_s"][3], inp["dn1"], inp["dn2"], inp["nx"]
    Nx, Nn, Ns = sol["Nx"], sol["Nn"], sol["Ns"]
    idx = [int((Nx - 1) / 2 - nx), int((Nx - 1) / 2), int((Nx - 1) / 2 + nx)]
    Ck0 = np.zeros((2 * Nn, 1, Nx, 1), np.complex128)
    Ck0[0, 0, idx, 0] = [1j * dn1 / (2 * a0 ** 3), 1 / a0 ** 3, -1j * dn1 / (2 * a0 ** 3)]
    Ck0[Nn, 0, idx, 0] = [1j * dn2 / (2 * a3 ** 3), 1 / a3 ** 3, -1j * dn2 / (2 * a3 ** 3)]
    Lx = np.sqrt(2) * np.pi * a0 / kx
    Fk0 = np.zeros((6, 1, Nx, 1), np.complex128)
    Fk0[0, 0, [idx[0], idx[2]], 0] = (dn1 + dn2) * Lx / (4 * np.pi * nx * inp["Omega_cs"][0])
    user = dict(inp)
    user.update(Ck_0=Ck0, Fk_0=Fk0, Lx=Lx)
    p = otab.initialize_simulation_parameters(user, Nx, 1, 1, Nn, 1, 1, Ns, sol["timesteps"], sol["dt"])
    ts = np.linspace(0.0, p["t_max"], sol["timesteps"])
    tol = inp["ode_tolerance"]
    out = od.solve(lambda t, y: orhs.rhs(p, y, "divide"), 0.0, ts[-1], np.concatenate([Ck0.ravel(), Fk0.ravel()]),
                   sol["dt"], ts=ts, adaptive=True, rtol=tol, atol=tol)
    E = odiag.energies(out["ys"], Nx, 1, 1, Nn, 1, 1, Ns, p["alpha_s"], p["u_s"], p["Omega_cs"], mi_me=1.0)["EM_energy"]
    gamma = np.polyfit(ts[300:], np.log(E[300:]), 1)[0] / 2
    curve = np.load(os.path.join(os.path.dirname(__file__), "golden", "physics_curves.npz"))
    g_ref = float(np.interp(kx, curve["growth_k"], curve["growth_rate"]))
    assert abs(gamma - g_ref) <= 0.01 * g_ref, (gamma, g_ref)
