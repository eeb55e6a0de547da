"""FP64 restatement of SPECTRAX's parameter set-up (test infrastructure only).

Follows spectrax/_initialization.py:14-156 (``initialize_simulation_parameters``):
defaults with derived lambdas (:47-72), the default two-stream initial state
(:75-94), the user merge and lambda evaluation (:104-113), k-grids (:114-119),
the hypercollision table (:121-130) and the Hermite ladder tables (:132-144);
and spectrax/_simulation.py:154-161 for the 28-entry ``args`` tuple.
"""
from __future__ import annotations

import numpy as np


def _default_parameters():
    return {
        "Lx": 4 * np.pi, "Ly": 1.0, "Lz": 1.0,
        "mi_me": 1.0, "Ti_Te": 1.0,
        "qs": np.array([-1, -1]),
        "alpha_e": np.array([0.707107, 0.707107, 0.707107]),
        "alpha_s": lambda p: np.concatenate([p["alpha_e"],
                                             p["alpha_e"] * np.sqrt(p["Ti_Te"] / p["mi_me"])]),
        "u_s": np.array([1.0, 0.0, 0.0, -1.0, 0.0, 0.0]),
        "Omega_cs": lambda p: np.array([1.0, 1.0 / p["mi_me"]]),
        "nu": 3.0, "D": 0.0, "t_max": 50.0,
        "nx": 1, "ny": 0, "nz": 0,
        "dn1": 0.001, "dn2": 0.001,
        "ode_tolerance": 1e-12,
        "vte": lambda p: p["alpha_s"][0] / np.sqrt(2),
        "vti": lambda p: p["vte"] * np.sqrt(1 / p["mi_me"]),
    }


def collision_table(Nn, Nm, Np):
    """col[p, m, n] = c(Nn, n) + c(Nm, m) + c(Np, p); spectrax/_initialization.py:121-130.

    c(N, i) = i(i-1)(i-2) / ((N-1)(N-2)(N-3)) for N > 3, else 0.
    """
    def c(N, i):
        i = np.asarray(i, dtype=np.float64)
        if N > 3:
            return i * (i - 1) * (i - 2) / float((N - 1) * (N - 2) * (N - 3))
        return np.zeros_like(i)
    p = np.arange(Np)[:, None, None]
    m = np.arange(Nm)[None, :, None]
    n = np.arange(Nn)[None, None, :]
    return c(Nn, n) + c(Nm, m) + c(Np, p)


def k_axis(N):
    """2*pi*j with j = arange(-N//2, N//2) + 1; spectrax/_initialization.py:114-116.

    For even N this runs -N/2+1 .. N/2 while the fftshift ordering of the data runs
    -N/2 .. N/2-1; the reference pairs them index by index and so does this code.
    """
    return (np.arange(-N // 2, N // 2) + 1) * 2 * np.pi


def _scatter_x(arr, row, xs, vals):
    """arr[row, 0, x, 0] = v with JAX ``.at[].set`` index rules: negative indices
    count from the end, indices past the end are dropped, later writes win."""
    N = arr.shape[2]
    for x, v in zip(xs, vals):
        x = x + N if x < 0 else x
        if 0 <= x < N:
            arr[row, 0, x, 0] = v


def initialize_simulation_parameters(user_parameters=None, Nx=33, Ny=1, Nz=1, Nn=50, Nm=1,
                                     Np=1, Ns=2, timesteps=500, dt=0.01):
    """Merged parameter dict with grids and tables; spectrax/_initialization.py:14-156."""
    user_parameters = {} if user_parameters is None else dict(user_parameters)
    d = _default_parameters()

    # default two-stream initial state, built from the defaults (:75-94)
    nx = d["nx"]
    c0 = int((Nx - 1) / 2)
    Omega0 = d["Omega_cs"](d)[0]
    val = (d["dn1"] + d["dn2"]) * d["Lx"] / (4 * np.pi * nx * Omega0)
    Fk_0 = np.zeros((6, 1, Nx, 1), dtype=np.complex128)
    _scatter_x(Fk_0, 0, [c0 - nx, c0 + nx], [val, val])
    ae = d["alpha_e"][0]
    def triple(dn):
        return np.array([1j * (1 / (2 * ae ** 3)) * dn, 1 / ae ** 3 + 0j, -1j * (1 / (2 * ae ** 3)) * dn])
    Ck_0 = np.zeros((2 * Nn, 1, Nx, 1), dtype=np.complex128)
    _scatter_x(Ck_0, 0, [c0 - nx, c0, c0 + nx], triple(d["dn1"]))
    _scatter_x(Ck_0, Nn, [c0 - nx, c0, c0 + nx], triple(d["dn2"]))
    d.update({"Ck_0": Ck_0, "Fk_0": Fk_0, "Ns": Ns, "timesteps": timesteps, "dt": dt,
              "Nx": Nx, "Ny": Ny, "Nz": Nz, "Nn": Nn, "Nm": Nm, "Np": Np})

    p = {**d, **user_parameters}
    Lx, Ly, Lz = p["Lx"], p["Ly"], p["Lz"]
    for key in list(p.keys()):
        v = p[key]
        if callable(v):
            p[key] = v(p)
        if isinstance(v, list):
            p[key] = np.array(v)

    kx, ky, kz = k_axis(Nx), k_axis(Ny), k_axis(Nz)
    kx_grid, ky_grid, kz_grid = np.meshgrid(kx, ky, kz, indexing="xy")
    k2_grid = kx_grid ** 2 + ky_grid ** 2 + kz_grid ** 2
    nabla = np.array([kx_grid / Lx, ky_grid / Ly, kz_grid / Lz])

    pp = np.arange(Np)[None, :, None, None, None, None, None]
    mm = np.arange(Nm)[None, None, :, None, None, None, None]
    nn = np.arange(Nn)[None, None, None, :, None, None, None]
    p.update({
        "kx_grid": kx_grid, "ky_grid": ky_grid, "kz_grid": kz_grid, "k2_grid": k2_grid,
        "nabla": nabla, "collision_matrix": collision_table(Nn, Nm, Np),
        "sqrt_n_plus": np.sqrt(nn + 1.0), "sqrt_n_minus": np.sqrt(nn * 1.0),
        "sqrt_m_plus": np.sqrt(mm + 1.0), "sqrt_m_minus": np.sqrt(mm * 1.0),
        "sqrt_p_plus": np.sqrt(pp + 1.0), "sqrt_p_minus": np.sqrt(pp * 1.0),
    })
    return p


def make_args(p):
    """The 28-tuple passed to the vector field; spectrax/_simulation.py:154-161."""
    return (p["Nx"], p["Ny"], p["Nz"], p["Nn"], p["Nm"], p["Np"], p["Ns"], p["qs"], p["nu"], p["D"],
            p["Omega_cs"], p["alpha_s"], p["u_s"], p["Lx"], p["Ly"], p["Lz"],
            p["kx_grid"], p["ky_grid"], p["kz_grid"], p["k2_grid"], p["nabla"],
            p["collision_matrix"], p["sqrt_n_plus"], p["sqrt_n_minus"],
            p["sqrt_m_plus"], p["sqrt_m_minus"], p["sqrt_p_plus"], p["sqrt_p_minus"])


def initial_state(p):
    """concat(Ck_0.ravel(), Fk_0.ravel()); spectrax/_simulation.py:148."""
    return np.concatenate([np.asarray(p["Ck_0"], np.complex128).ravel(),
                           np.asarray(p["Fk_0"], np.complex128).ravel()])
