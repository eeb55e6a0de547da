"""Generate the golden fixtures in this folder from the reference's own source.

Run once in a container that has the SPECTRAX source tree (read-only is fine):

    python tests/golden/make_golden.py <path to the SPECTRAX source tree>

JAX, Diffrax and orthax are not installable in that container, so this script
installs a small NumPy stand-in for ``jax`` / ``jax.numpy`` / ``diffrax`` in
``sys.modules`` and then imports the reference modules ``spectrax._simulation``,
``spectrax._model``, ``spectrax._initialization`` and ``spectrax._diagnostics``
from the source tree WITHOUT modification.  ``jit`` becomes the identity,
``jnp`` functions are NumPy's, and ``jnp.fft.fftfreq`` follows JAX's definition
(integer bins divided by n).  The outputs therefore pin the reference's
operator algebra, index conventions, tables and energies; they do not exercise
XLA's own FFT rounding.

Outputs: ``rhs_cases.npz`` (RHS in/out for several shapes),
``tables.npz`` (grids and tables), ``diag.npz`` (energies of a short trajectory).
Nothing on the test path reads the reference: only these fixtures travel.
"""
from __future__ import annotations

import importlib
import os
import sys
import types
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# ----------------------------------------------------------------- the stand-in
class _AtIndex:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def set(self, v):
        out = np.array(self.arr, copy=True).view(_JArray)
        out[self.idx] = v
        return out


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self.arr, idx)


class _JArray(np.ndarray):
    """ndarray with JAX's functional ``.at[idx].set(v)``."""

    @property
    def at(self):
        return _At(self)


def _wrap(fn):
    def inner(*a, **k):
        r = fn(*a, **k)
        return r.view(_JArray) if isinstance(r, np.ndarray) else r
    return inner


def _jax_fftfreq(n, d=1.0, dtype=None):
    # JAX's definition: integer bins, then a division by d*n.
    k = np.zeros(n)
    if n % 2 == 0:
        k[: n // 2] = np.arange(0, n // 2)
        k[n // 2:] = np.arange(-n // 2, 0)
    else:
        k[: (n - 1) // 2 + 1] = np.arange(0, (n - 1) // 2 + 1)
        k[(n - 1) // 2 + 1:] = np.arange(-((n - 1) // 2), 0)
    return k / np.array(d * n, dtype=np.float64)


def install_standin():
    jax = types.ModuleType("jax")
    jnp = types.ModuleType("jax.numpy")
    for name in dir(np):
        if not name.startswith("__"):
            setattr(jnp, name, getattr(np, name))
    for name in ("array", "zeros", "zeros_like", "ones", "asarray", "concatenate", "stack"):
        setattr(jnp, name, _wrap(getattr(np, name)))
    fft = types.ModuleType("jax.numpy.fft")
    for name in ("fftn", "ifftn", "fftshift", "ifftshift", "fft", "ifft"):
        setattr(fft, name, getattr(np.fft, name))
    fft.fftfreq = _jax_fftfreq
    jnp.fft = fft

    def jit(f=None, **kw):
        if f is None:
            return lambda g: g
        return f

    class _Config:
        def update(self, *a, **k):
            pass

    jax.jit = jit
    jax.config = _Config()
    jax.numpy = jnp
    jax.block_until_ready = lambda x: x
    lax = types.ModuleType("jax.lax")
    jax.lax = lax
    scipy = types.ModuleType("jax.scipy")
    sparse = types.ModuleType("jax.scipy.sparse")
    linalg = types.ModuleType("jax.scipy.sparse.linalg")
    linalg.gmres = None
    special = types.ModuleType("jax.scipy.special")
    import scipy.special as _ss
    special.factorial = _ss.factorial
    scipy.sparse, sparse.linalg, scipy.special = sparse, linalg, special
    jax.scipy = scipy

    diffrax = types.ModuleType("diffrax")
    for name in ("diffeqsolve", "Dopri8", "ODETerm", "SaveAt", "PIDController",
                 "TqdmProgressMeter", "NoProgressMeter", "ConstantStepSize",
                 "LocalLinearInterpolation", "RESULTS"):
        setattr(diffrax, name, type(name, (), {}))
    diffrax.AbstractSolver = type("AbstractSolver", (), {})

    mods = {"jax": jax, "jax.numpy": jnp, "jax.numpy.fft": fft, "jax.lax": lax,
            "jax.scipy": scipy, "jax.scipy.sparse": sparse, "jax.scipy.sparse.linalg": linalg,
            "jax.scipy.special": special, "diffrax": diffrax}
    sys.modules.update(mods)


def import_reference(ref_root):
    pkg = types.ModuleType("spectrax")
    pkg.__path__ = [os.path.join(ref_root, "spectrax")]
    sys.modules["spectrax"] = pkg
    sim = importlib.import_module("spectrax._simulation")
    init = importlib.import_module("spectrax._initialization")
    diag = importlib.import_module("spectrax._diagnostics")
    return sim, init, diag


# ----------------------------------------------------------------- the cases
CASES = [
    # name, shape (Nx, Ny, Nz, Nn, Nm, Np, Ns), user parameter overrides
    ("1d1v_n9", (9, 1, 1, 6, 1, 1, 2), dict(Lx=7.0, nu=2.0, mi_me=1836.0,
        qs=[-1.0, 1.0], alpha_s=[1.41, 1.3, 1.2, 0.033, 0.031, 0.03],
        u_s=[0.2, -0.3, 0.4, 0.0, 0.1, -0.05], Omega_cs=[1.0, 1.0 / 1836.0], D=0.1)),
    ("1d1v_n33_landau", (33, 1, 1, 16, 1, 1, 2), dict(Lx=4 * np.pi, nu=2.0, mi_me=1836.0,
        qs=[-1.0, 1.0], alpha_s=[1.4142135623730951] * 3 + [1.4142135623730951 / np.sqrt(1836.0)] * 3,
        u_s=[0.0] * 6, Omega_cs=[1.0, 1.0 / 1836.0])),
    ("1d1v_n16_even", (16, 1, 1, 7, 1, 1, 3), dict(Lx=10 * np.pi, nu=1.0,
        qs=[-1.0, -1.0, 1.0], alpha_s=[0.5] * 6 + [0.0117] * 3,
        u_s=[1.0, 0.0, 0.0, -1.0, 0.0, 0.0, 0.0, 0.0, 0.0], Omega_cs=[1.0, 1.0, 1.0 / 1836.0])),
    ("1d3v_n8", (8, 1, 1, 3, 3, 4, 2), dict(Lx=5.0, Ly=3.0, Lz=2.0, nu=0.7, D=0.05,
        qs=[-1.0, 1.0], alpha_s=[0.9, 0.7, 1.1, 0.3, 0.25, 0.2],
        u_s=[0.1, 0.2, -0.3, 0.05, -0.07, 0.02], Omega_cs=[0.5, 0.02])),
    ("2d3v_6x5", (5, 6, 1, 2, 3, 2, 2), dict(Lx=6.0, Ly=4.0, nu=0.5,
        qs=[-1.0, 1.0], alpha_s=[0.25, 0.3, 0.35, 0.05, 0.06, 0.07],
        u_s=[0.3, -0.2, 0.1, -0.1, 0.05, 0.2], Omega_cs=[0.5, 0.02])),
    ("3d3v_4x5x3", (5, 4, 3, 3, 2, 2, 1), dict(Lx=3.0, Ly=2.0, Lz=1.5, nu=1.5, D=0.01,
        qs=[-1.0], alpha_s=[0.8, 0.9, 1.0], u_s=[0.1, 0.2, 0.3], Omega_cs=[1.3])),
    ("2d2v_n64x4", (4, 64, 1, 2, 2, 1, 1), dict(Lx=2.0, Ly=9.0, nu=0.2,
        qs=[-1.0], alpha_s=[0.6, 0.5, 0.4], u_s=[0.0, 0.3, -0.2], Omega_cs=[1.0])),
]


def random_state(rng, shape):
    Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
    n = Ns * Np * Nm * Nn * Ny * Nx * Nz + 6 * Ny * Nx * Nz
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def main(ref_root):
    warnings.simplefilter("ignore")
    install_standin()
    sim, init, diag = import_reference(ref_root)
    rng = np.random.default_rng(20261203)

    rhs = {}
    tables = {}
    for name, shape, user in CASES:
        Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
        p = init.initialize_simulation_parameters(dict(user), Nx, Ny, Nz, Nn, Nm, Np, Ns, 10, 0.01)
        args = (Nx, Ny, Nz, Nn, Nm, Np, Ns, p["qs"], p["nu"], p["D"], p["Omega_cs"], p["alpha_s"],
                p["u_s"], p["Lx"], p["Ly"], p["Lz"], p["kx_grid"], p["ky_grid"], p["kz_grid"],
                p["k2_grid"], p["nabla"], p["collision_matrix"], p["sqrt_n_plus"],
                p["sqrt_n_minus"], p["sqrt_m_plus"], p["sqrt_m_minus"], p["sqrt_p_plus"],
                p["sqrt_p_minus"])
        y = random_state(rng, shape)
        dy = np.asarray(sim.ode_system(Nx, Ny, Nz, Nn, Nm, Np, Ns, 0.0, y, args))
        rhs[f"{name}/shape"] = np.array(shape)
        rhs[f"{name}/y"] = y
        rhs[f"{name}/dy"] = dy
        for k in ("qs", "alpha_s", "u_s", "Omega_cs"):
            rhs[f"{name}/{k}"] = np.asarray(p[k], dtype=np.float64)
        for k in ("nu", "D", "Lx", "Ly", "Lz"):
            rhs[f"{name}/{k}"] = np.float64(p[k])
        for k in ("kx_grid", "ky_grid", "kz_grid", "k2_grid", "nabla", "collision_matrix",
                  "sqrt_n_plus", "sqrt_m_minus", "sqrt_p_plus"):
            tables[f"{name}/{k}"] = np.asarray(p[k], dtype=np.float64)
        tables[f"{name}/mask"] = np.asarray(sim._twothirds_mask(Ny, Nx, Nz))

    # defaults: the reference's own two-stream state (spectrax/_initialization.py:75-94)
    p = init.initialize_simulation_parameters({}, 33, 1, 1, 20, 1, 1, 2, 10, 0.01)
    args = (33, 1, 1, 20, 1, 1, 2, p["qs"], p["nu"], p["D"], p["Omega_cs"], p["alpha_s"],
            p["u_s"], p["Lx"], p["Ly"], p["Lz"], p["kx_grid"], p["ky_grid"], p["kz_grid"],
            p["k2_grid"], p["nabla"], p["collision_matrix"], p["sqrt_n_plus"],
            p["sqrt_n_minus"], p["sqrt_m_plus"], p["sqrt_m_minus"], p["sqrt_p_plus"],
            p["sqrt_p_minus"])
    y0 = np.concatenate([np.asarray(p["Ck_0"]).ravel(), np.asarray(p["Fk_0"]).ravel()])
    rhs["defaults/shape"] = np.array((33, 1, 1, 20, 1, 1, 2))
    rhs["defaults/y"] = y0
    rhs["defaults/dy"] = np.asarray(sim.ode_system(33, 1, 1, 20, 1, 1, 2, 0.0, y0, args))
    for k in ("qs", "alpha_s", "u_s", "Omega_cs"):
        rhs[f"defaults/{k}"] = np.asarray(p[k], dtype=np.float64)
    for k in ("nu", "D", "Lx", "Ly", "Lz"):
        rhs[f"defaults/{k}"] = np.float64(p[k])
    for k in ("vte", "vti"):
        tables[f"defaults/{k}"] = np.float64(p[k])

    # energies of a short synthetic trajectory (spectrax/_diagnostics.py:71-233)
    dg = {}
    for name, shape, user in (CASES[0], CASES[3], CASES[4]):
        Nx, Ny, Nz, Nn, Nm, Np, Ns = shape
        p = init.initialize_simulation_parameters(dict(user), Nx, Ny, Nz, Nn, Nm, Np, Ns, 3, 0.01)
        Nt = 3
        NC = Ns * Np * Nm * Nn * Ny * Nx * Nz
        ys = np.stack([random_state(rng, shape) for _ in range(Nt)])
        out = {"Ck": ys[:, :NC].reshape(Nt, Ns * Nn * Nm * Np, Ny, Nx, Nz),
               "Fk": ys[:, NC:].reshape(Nt, 6, Ny, Nx, Nz)}
        out.update({k: p[k] for k in ("alpha_s", "u_s", "Omega_cs", "Lx", "Nn", "Nm", "Np",
                                      "mi_me")})
        diag.diagnostics(out)
        dg[f"{name}/shape"] = np.array(shape)
        dg[f"{name}/ys"] = ys
        for k in ("alpha_s", "u_s", "Omega_cs"):
            dg[f"{name}/{k}"] = np.asarray(p[k], dtype=np.float64)
        dg[f"{name}/mi_me"] = np.float64(p["mi_me"])
        dg[f"{name}/Lx"] = np.float64(p["Lx"])
        for k in ("EM_energy", "kinetic_energy", "total_energy", "kinetic_energy_species",
                  "lambda_D", "k_norm"):
            dg[f"{name}/{k}"] = np.asarray(out[k])

    np.savez_compressed(os.path.join(HERE, "rhs_cases.npz"), **rhs)
    np.savez_compressed(os.path.join(HERE, "tables.npz"), **tables)
    np.savez_compressed(os.path.join(HERE, "diag.npz"), **dg)
    print("wrote", sorted({k.split("/")[0] for k in rhs}))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_golden.py <path to the SPECTRAX source tree>")
    main(sys.argv[1])
