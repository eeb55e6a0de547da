"""GPU: general-layout planes larger than one CTA's shared memory (plan path 2):
the multi-pass right-hand side against the oracle, the entry points that refuse
such plans, and the reference's 2-D Orszag-Tang example (151 x 151 plane) run
end to end from its input file."""
import numpy as np
import pytest

from conftest import rel_err
from example_configs import SIZES, configs, write_toml
from oracle import rhs as orhs
from oracle import tables as otab


def _params(shape, seed):
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    user = dict(Lx=float(rng.uniform(3, 12)), Ly=float(rng.uniform(3, 12)), Lz=float(rng.uniform(3, 12)),
                nu=float(rng.uniform(0.2, 2)), D=float(rng.uniform(0, 0.05)),
                qs=list(rng.choice([-1.0, 1.0], Ns)), alpha_s=list(rng.uniform(0.3, 1.4, 3 * Ns)),
                u_s=list(rng.uniform(-0.8, 0.8, 3 * Ns)), Omega_cs=list(rng.uniform(0.2, 1.5, Ns)))
    return otab.initialize_simulation_parameters(user, *shape, 5, 0.01)


SHAPES = [(96, 96, 1, 2, 2, 2, 1), (151, 151, 1, 2, 2, 1, 2), (24, 24, 20, 2, 1, 2, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("mask", ["divide", "multiply"])
def test_multipass_rhs_matches_oracle(shape, mask):
    import torch
    from spectrax_gb300 import vector_field
    p = _params(shape, 3)
    plan = vector_field.plan_for_params(p, mask)
    assert plan.path == 2
    rng = np.random.default_rng(4)
    n = plan.state_len
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    got = plan.rhs(torch.from_numpy(y).cuda()).cpu().numpy()
    assert rel_err(got, orhs.rhs(p, y, mask)) <= 1e-12


@pytest.mark.gpu
def test_entry_points_that_hold_whole_planes_refuse():
    import torch
    from spectrax_gb300 import SpectraxError, dopri8, vector_field
    p = _params((96, 96, 1, 2, 2, 2, 1), 5)
    plan = vector_field.plan_for_params(p, "divide")
    z = torch.zeros(plan.state_len, dtype=torch.complex128, device="cuda")
    out = torch.empty_like(z)
    for call in (lambda: plan.jvp_into(z, z.clone(), out), lambda: plan.vjp_into(z, z.clone(), out),
                 lambda: plan.linearize(z)):
        with pytest.raises(SpectraxError):
            call()
    with pytest.raises(SpectraxError):
        dopri8.Dopri8Solver(plan, 0.0, 0.1, 0.01)


@pytest.mark.gpu
def test_orszag_tang_example_runs_end_to_end(tmp_path):
    # Examples/input_2D_orszag_tang.toml with the example's own initial state
    # (drifting Maxwellians of the Orszag-Tang flow, as Examples/2D_orszag_tang.py
    # builds it), horizon shortened to three saves
    from spectrax_gb300.dopri8 import simulation
    from spectrax_gb300.maxwellian import orszag_tang_state
    from spectrax_gb300.params import load_parameters
    path = tmp_path / "ot.toml"
    write_toml(configs()["input_2D_orszag_tang.toml"], path)
    inp, sol = load_parameters(str(path))
    Nx, Ny, Nz, Nn, Nm, Np, Ns = (sol[k] for k in SIZES[:7])
    _, y0 = orszag_tang_state(Nx=Nx, Ny=Ny, Nz=Nz, Nn=Nn, Nm=Nm, Np=Np, L=inp["Lx"], alpha_e=inp["alpha_s"][0],
                              mi_me=inp["mi_me"], Omega_ce=inp["Omega_cs"][0])
    nc = Ns * Nn * Nm * Np * Nx * Ny * Nz
    inp["Ck_0"] = y0[:nc].reshape(Ns * Np * Nm * Nn, Ny, Nx, Nz)
    inp["Fk_0"] = y0[nc:].reshape(6, Ny, Nx, Nz)
    inp["t_max"] = 3 * sol["dt"]
    out = simulation(inp, Nx=Nx, Ny=Ny, Nz=Nz, Nn=Nn, Nm=Nm, Np=Np, Ns=Ns, timesteps=sol["timesteps"],
                     dt=sol["dt"], solver=sol["solver"], adaptive_time_step=sol["adaptive_time_step"])
    assert out["Ck"].shape == (3, Ns * Nn * Nm * Np, Ny, Nx, Nz)
    assert np.all(np.isfinite(out["Ck"])) and np.all(np.isfinite(out["Fk"]))
    tot = out["total_energy"]
    assert np.all(np.isfinite(tot)) and abs(tot[-1] - tot[0]) <= 1e-6 * abs(tot[0])
    assert out["solver_stats"]["status_name"] == "DONE"


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in sorted(configs()) if n.startswith("input_1D")])
def test_1d_examples_run_end_to_end(name, tmp_path):
    from spectrax_gb300.dopri8 import simulation
    from spectrax_gb300.params import load_parameters
    path = tmp_path / name
    write_toml(configs()[name], path)
    inp, sol = load_parameters(str(path))
    inp["t_max"] = 1.0
    out = simulation(inp, **{k: sol[k] for k in SIZES}, solver=sol["solver"],
                     adaptive_time_step=sol["adaptive_time_step"])
    assert np.all(np.isfinite(out["EM_energy"])) and out["Ck"].shape[0] == sol["timesteps"]
