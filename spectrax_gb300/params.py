"""Host-side parameter set-up, mirroring SPECTRAX's configuration layer.

* ``initialize_simulation_parameters`` follows spectrax/_initialization.py:14-156
  (defaults with derived lambdas, the default two-stream state, the user merge,
  k-grids, collision and ladder tables) and returns the same dictionary keys.
* ``load_parameters`` follows spectrax/_initialization.py:158-190 (TOML ->
  ``(input_parameters, solver_parameters)``); the solver entry becomes one of the
  descriptors ``Dopri8()`` / ``ImplicitMidpoint(rtol, atol)`` of this package.
* ``make_problem`` packs a parameter dict into the C ABI's ``spx_problem``.
"""
from __future__ import annotations

import numpy as np

from ._lib import MAX_AXIS, MAX_SPECIES, spx_problem

try:
    import tomllib
except ModuleNotFoundError:  # pragma: no cover
    tomllib = None

MASK_MODES = ("divide", "multiply")
_mask_mode = "divide"


def set_mask_mode(mode: str) -> None:
    """Choose how the 2/3-rule edge bin is rounded (see ``mask_cutoff``)."""
    global _mask_mode
    if mode not in MASK_MODES:
        raise ValueError(f"mask mode must be one of {MASK_MODES}")
    _mask_mode = mode


def get_mask_mode() -> str:
    return _mask_mode


def mask_cutoff(n: int, mode: str | None = None) -> int:
    """Largest |k| the 2/3 mask keeps along an axis of length n (-1: none).

    spectrax/_simulation.py:15-32 keeps |fftshift(fftfreq(n)) * n| <= n // 3.
    fftfreq divides the integer bins by n ("divide", JAX's definition); an XLA
    build that folds the division into a multiply by 1/n ("multiply") drops the
    edge bin for some n (10, 20, 33, ...).  Both are supported.
    """
    mode = mode or _mask_mode
    if mode not in MASK_MODES:
        raise ValueError(f"mask mode must be one of {MASK_MODES}")
    c = n // 3
    best = -1
    # bins k and -k round symmetrically; only k = n//3 can fall either way
    for k in range(0, n // 2 + 1):
        v = (k / float(n)) * n if mode == "divide" else (k * (1.0 / float(n))) * n
        if v <= c:
            best = k
    return best


def _defaults():
    return {
        "Lx": 4 * np.pi, "Ly": 1.0, "Lz": 1.0, "mi_me": 1.0, "Ti_Te": 1.0,
        "qs": np.array([-1, -1]),
        "alpha_e": np.array([0.707107, 0.707107, 0.707107]),
        "alpha_s": lambda d: np.concatenate([d["alpha_e"], d["alpha_e"] * np.sqrt(d["Ti_Te"] / d["mi_me"])]),
        "u_s": np.array([1.0, 0.0, 0.0, -1.0, 0.0, 0.0]),
        "Omega_cs": lambda d: np.array([1.0, 1.0 / d["mi_me"]]),
        "nu": 3.0, "D": 0.0, "t_max": 50.0,
        "nx": 1, "ny": 0, "nz": 0, "dn1": 0.001, "dn2": 0.001,
        "ode_tolerance": 1e-12,
        "vte": lambda d: d["alpha_s"][0] / np.sqrt(2),
        "vti": lambda d: d["vte"] * np.sqrt(1 / d["mi_me"]),
    }


def initialize_simulation_parameters(user_parameters=None, Nx=33, Ny=1, Nz=1, Nn=50, Nm=1, Np=1,
                                     Ns=2, timesteps=500, dt=0.01):
    """Merged parameter dictionary (same keys and values as the reference)."""
    d = _defaults()
    nx = d["nx"]
    mid = int((Nx - 1) / 2)
    O0 = d["Omega_cs"](d)[0]
    def put(arr, row, x, v):
        # JAX .at[].set rules: negative indices wrap once, out-of-range ones are dropped
        x = x + Nx if x < 0 else x
        if 0 <= x < Nx:
            arr[row, 0, x, 0] = v

    Fk_0 = np.zeros((6, 1, Nx, 1), dtype=np.complex128)
    amp = (d["dn1"] + d["dn2"]) * d["Lx"] / (4 * np.pi * nx * O0)
    put(Fk_0, 0, mid - nx, amp)
    put(Fk_0, 0, mid + nx, amp)
    a3 = d["alpha_e"][0] ** 3
    Ck_0 = np.zeros((2 * Nn, 1, Nx, 1), dtype=np.complex128)
    for row, dn in ((0, d["dn1"]), (Nn, d["dn2"])):
        put(Ck_0, row, mid - nx, 1j * (1 / (2 * a3)) * dn)
        put(Ck_0, row, mid, 1 / a3 + 0j)
        put(Ck_0, row, mid + nx, -1j * (1 / (2 * a3)) * dn)
    d.update(Ck_0=Ck_0, Fk_0=Fk_0, Ns=Ns, timesteps=timesteps, dt=dt,
             Nx=Nx, Ny=Ny, Nz=Nz, Nn=Nn, Nm=Nm, Np=Np)
    p = {**d, **(user_parameters or {})}
    for k in list(p):
        v = p[k]
        if callable(v):
            p[k] = v(p)
        if isinstance(v, list):
            p[k] = np.array(v)

    def kaxis(N):
        return (np.arange(-N // 2, N // 2) + 1) * 2 * np.pi

    kxg, kyg, kzg = np.meshgrid(kaxis(Nx), kaxis(Ny), kaxis(Nz), indexing="xy")
    p["kx_grid"], p["ky_grid"], p["kz_grid"] = kxg, kyg, kzg
    p["k2_grid"] = kxg ** 2 + kyg ** 2 + kzg ** 2
    p["nabla"] = np.array([kxg / p["Lx"], kyg / p["Ly"], kzg / p["Lz"]])

    def cc(N, i):
        i = np.asarray(i, np.float64)
        return i * (i - 1) * (i - 2) / ((N - 1) * (N - 2) * (N - 3)) if N > 3 else 0.0 * i

    p["collision_matrix"] = (cc(Nn, np.arange(Nn))[None, None, :] + cc(Nm, np.arange(Nm))[None, :, None]
                             + cc(Np, np.arange(Np))[:, None, None])
    n = np.arange(Nn, dtype=np.float64).reshape(1, 1, 1, Nn, 1, 1, 1)
    m = np.arange(Nm, dtype=np.float64).reshape(1, 1, Nm, 1, 1, 1, 1)
    q = np.arange(Np, dtype=np.float64).reshape(1, Np, 1, 1, 1, 1, 1)
    p.update(sqrt_n_plus=np.sqrt(n + 1), sqrt_n_minus=np.sqrt(n), sqrt_m_plus=np.sqrt(m + 1),
             sqrt_m_minus=np.sqrt(m), sqrt_p_plus=np.sqrt(q + 1), sqrt_p_minus=np.sqrt(q))
    return p


def make_args(p):
    """The 28-tuple ``args`` of spectrax/_simulation.py:154-161."""
    return (p["Nx"], p["Ny"], p["Nz"], p["Nn"], p["Nm"], p["Np"], p["Ns"], p["qs"], p["nu"], p["D"],
            p["Omega_cs"], p["alpha_s"], p["u_s"], p["Lx"], p["Ly"], p["Lz"], p["kx_grid"],
            p["ky_grid"], p["kz_grid"], p["k2_grid"], p["nabla"], p["collision_matrix"],
            p["sqrt_n_plus"], p["sqrt_n_minus"], p["sqrt_m_plus"], p["sqrt_m_minus"],
            p["sqrt_p_plus"], p["sqrt_p_minus"])


def initial_state(p):
    """concat(Ck_0.ravel(), Fk_0.ravel()) as in spectrax/_simulation.py:148."""
    return np.concatenate([np.asarray(p["Ck_0"], np.complex128).ravel(),
                           np.asarray(p["Fk_0"], np.complex128).ravel()])


def landau_initial_state(p, dn=0.01, n=1):
    """Perturbed-Maxwellian 1D1V initial state of the Landau examples
    (Examples/1D_Landau_damping.py:41-54): C_{s,0}(k=0) = 1/alpha_s^3, the
    electrons (species 0) get C_0(-k_n) = +i dn/(2 a^3), C_0(+k_n) = -i dn/(2 a^3)
    at the centred indices (Nx-1)/2 -/+ n, and E_x(+-k_n) = dn Lx / (4 pi n Omega_0)."""
    Nx, Nn, Ns = int(p["Nx"]), int(p["Nn"]), int(p["Ns"])
    if int(p["Ny"]) != 1 or int(p["Nz"]) != 1 or int(p["Nm"]) != 1 or int(p["Np"]) != 1:
        raise ValueError("landau_initial_state builds 1D1V states")
    a = np.asarray(p["alpha_s"], np.float64).reshape(Ns, 3)[:, 0]
    c0 = (Nx - 1) // 2
    Ck = np.zeros((Ns, Nn, Nx), np.complex128)
    for s in range(Ns):
        Ck[s, 0, c0] = 1.0 / a[s] ** 3
    Ck[0, 0, c0 - n] = 1j * dn / (2 * a[0] ** 3)
    Ck[0, 0, c0 + n] = -1j * dn / (2 * a[0] ** 3)
    Fk = np.zeros((6, Nx), np.complex128)
    Om0 = float(np.asarray(p["Omega_cs"], np.float64).ravel()[0])
    Fk[0, c0 - n] = Fk[0, c0 + n] = dn * float(p["Lx"]) / (4 * np.pi * n * Om0)
    return np.concatenate([Ck.ravel(), Fk.ravel()])


def make_problem(Nx, Ny, Nz, Nn, Nm, Np, Ns, qs, nu, D, Omega_cs, alpha_s, u_s, Lx, Ly, Lz,
                 mask_mode: str | None = None) -> spx_problem:
    """Pack shapes and physical scalars into ``spx_problem``."""
    if Ns > MAX_SPECIES:
        raise ValueError(f"at most {MAX_SPECIES} species")
    if max(Nx, Ny, Nz) > MAX_AXIS:
        raise ValueError(f"Fourier axes are limited to {MAX_AXIS} modes")
    pb = spx_problem()
    pb.Nx, pb.Ny, pb.Nz, pb.Nn, pb.Nm, pb.Np, pb.Ns = (int(v) for v in (Nx, Ny, Nz, Nn, Nm, Np, Ns))
    pb.cut_x, pb.cut_y, pb.cut_z = (mask_cutoff(int(v), mask_mode) for v in (Nx, Ny, Nz))
    pb.Lx, pb.Ly, pb.Lz, pb.nu, pb.D = (float(v) for v in (Lx, Ly, Lz, nu, D))
    qs = np.asarray(qs, np.float64).ravel()
    Om = np.asarray(Omega_cs, np.float64).ravel()
    al = np.asarray(alpha_s, np.float64).ravel()
    us = np.asarray(u_s, np.float64).ravel()
    if len(qs) < Ns or len(Om) < Ns or len(al) < 3 * Ns or len(us) < 3 * Ns:
        raise ValueError("species arrays are shorter than Ns")
    for i in range(Ns):
        pb.qs[i] = qs[i]
        pb.Omega_cs[i] = Om[i]
    for i in range(3 * Ns):
        pb.alpha_s[i] = al[i]
        pb.u_s[i] = us[i]
    return pb


def problem_from_params(p, mask_mode: str | None = None) -> spx_problem:
    return make_problem(p["Nx"], p["Ny"], p["Nz"], p["Nn"], p["Nm"], p["Np"], p["Ns"], p["qs"], p["nu"],
                        p["D"], p["Omega_cs"], p["alpha_s"], p["u_s"], p["Lx"], p["Ly"], p["Lz"],
                        mask_mode)


def problem_from_args(Nx, Ny, Nz, Nn, Nm, Np, Ns, args, mask_mode: str | None = None) -> spx_problem:
    """From the reference's ``args`` tuple (entries [7:] per spectrax/_simulation.py:83-86)."""
    qs, nu, D, Omega_cs, alpha_s, u_s, Lx, Ly, Lz = args[7:16]
    return make_problem(Nx, Ny, Nz, Nn, Nm, Np, Ns, qs, nu, D, Omega_cs, alpha_s, u_s, Lx, Ly, Lz,
                        mask_mode)


# ----------------------------------------------------------------- solvers / TOML
class Dopri8:
    """Descriptor for the device Prince-Dormand 8(7) stepper."""
    name = "Dopri8"

    def __repr__(self):
        return "Dopri8()"


class ImplicitMidpoint:
    """Descriptor for the device implicit-midpoint Newton-GMRES stepper
    (spectrax/midpoint_solver.py:10-53)."""
    name = "ImplicitMidpoint"

    def __init__(self, rtol=1e-6, atol=1e-8, max_iters=300, restart=30, gmres_tol=1e-10):
        self.rtol, self.atol, self.max_iters = rtol, atol, max_iters
        self.restart, self.gmres_tol = restart, gmres_tol

    def __repr__(self):
        return f"ImplicitMidpoint(rtol={self.rtol}, atol={self.atol})"


def load_parameters(input_file):
    """TOML -> (input_parameters, solver_parameters); spectrax/_initialization.py:158-190."""
    if tomllib is None:  # pragma: no cover
        raise RuntimeError("tomllib is unavailable")
    with open(input_file, "rb") as fh:
        data = tomllib.load(fh)
    inp = data["input_parameters"]
    sol = data["solver_parameters"]
    sol["adaptive_time_step"] = sol.get("adaptive_time_step", True)
    name = sol.get("solver", "Dopri8")
    if name == "Dopri8":
        sol["solver"] = Dopri8()
    elif name == "ImplicitMidpoint":
        sol["solver"] = ImplicitMidpoint(rtol=inp["ode_tolerance"], atol=inp["ode_tolerance"])
    else:
        raise ValueError(f"Solver '{name}' is not supported. Choose Dopri8 or ImplicitMidpoint.")
    return inp, sol

