"""Hermite-Fourier coefficients of drifting Maxwellians (spectrax/_initialize_maxwellian.py:14-66)
and the 2D3V Orszag-Tang-like initial state (Examples/2D_Orszag_Tang.py:40-77).

C_nmp(x) = sqrt(2^(n+m+p) / (n! m! p!)) / (a_x^(n+1) a_y^(m+1) a_z^(p+1))
           * (U_x - u_x)^n (U_y - u_y)^m (U_z - u_z)^p
sampled on the real-space grid, then fftn(norm="forward") and fftshift over
(y, x, z).  `compute_C_nmp` is the host (NumPy) version; `compute_C_nmp_device`
runs the same on the GPU (`spx_maxwellian`: one CTA per mode plane, samples
formed in shared memory and transformed in place) for large initial states.
"""
from __future__ import annotations

import numpy as np
from scipy.special import factorial


def compute_C_nmp(Us_grid, alpha_s, u_s, Nn, Nm, Np, Ns):
    """Us_grid: (Ns, 3, Ny, Nx, Nz) real velocities -> Ck (Ns, Np, Nm, Nn, Ny, Nx, Nz)."""
    Us = np.asarray(Us_grid, np.float64)
    a = np.asarray(alpha_s, np.float64).reshape(Ns, 3)
    u = np.asarray(u_s, np.float64).reshape(Ns, 3)
    sh = (Ns, 1, 1, 1, 1, 1, 1)
    ax, ay, az = (a[:, i].reshape(sh) for i in range(3))
    ux, uy, uz = (u[:, i].reshape(sh) for i in range(3))
    Ux = Us[:, 0][:, None, None, None]
    Uy = Us[:, 1][:, None, None, None]
    Uz = Us[:, 2][:, None, None, None]
    p = np.arange(Np).reshape(1, Np, 1, 1, 1, 1, 1)
    m = np.arange(Nm).reshape(1, 1, Nm, 1, 1, 1, 1)
    n = np.arange(Nn).reshape(1, 1, 1, Nn, 1, 1, 1)
    C = (np.sqrt(2.0 ** (n + m + p) / (factorial(n) * factorial(m) * factorial(p)))
         * (1.0 / (ax ** (n + 1) * ay ** (m + 1) * az ** (p + 1)))
         * (Ux - ux) ** n * (Uy - uy) ** m * (Uz - uz) ** p)
    ax3 = (-3, -2, -1)
    return np.fft.fftshift(np.fft.fftn(C, axes=ax3, norm="forward"), axes=ax3)


def compute_C_nmp_device(Us_grid, alpha_s, u_s, Nn, Nm, Np, Ns, extra_real=None, device=None):
    """The GPU version of compute_C_nmp: Us_grid (Ns, 3, Ny, Nx, Nz) -> Ck (Ns, Np, Nm,
    Nn, Ny, Nx, Nz) complex128 on the device; `extra_real` (k, Ny, Nx, Nz) real planes
    are transformed the same way and returned second (else None)."""
    import ctypes as C

    import torch

    from . import _lib
    from .params import make_problem
    from .vector_field import _stream_ptr, get_plan
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    Us = torch.as_tensor(np.asarray(Us_grid, np.float64)).to(dev).contiguous()
    _, _, Ny, Nx, Nz = Us.shape
    pb = make_problem(Nx, Ny, Nz, Nn, Nm, Np, Ns, [-1.0] * Ns, 0.0, 0.0, [1.0] * Ns, alpha_s, u_s,
                      1.0, 1.0, 1.0)
    pb.cut_x, pb.cut_y, pb.cut_z = Nx, Ny, Nz           # keep every mode: no 2/3 mask here
    plan = get_plan(pb, dev.index)
    X = None
    nreal = 0
    if extra_real is not None:
        X = torch.as_tensor(np.asarray(extra_real, np.float64)).to(dev).contiguous()
        nreal = X.shape[0]
    plane = Nx * Ny * Nz
    out = torch.empty((Ns * Nn * Nm * Np + nreal) * plane, dtype=torch.complex128, device=dev)
    _lib.check(_lib.lib().spx_maxwellian(plan.handle, C.c_void_p(Us.data_ptr()),
                                         C.c_void_p(X.data_ptr()) if X is not None else None, nreal,
                                         C.c_void_p(out.data_ptr()), _stream_ptr()), "spx_maxwellian")
    nc = Ns * Nn * Nm * Np * plane
    Ck = out[:nc].reshape(Ns, Np, Nm, Nn, Ny, Nx, Nz)
    return Ck, (out[nc:].reshape(nreal, Ny, Nx, Nz) if X is not None else None)


def orszag_tang_state(Nx=64, Ny=64, Nz=1, Nn=8, Nm=8, Np=8, L=50.0, alpha_e=0.25, mi_me=25.0,
                      du=0.2, dB=0.2, Omega_ce=0.5, noise=1e-6, seed=0):
    """Parameters and flat initial state of the 2D3V Orszag-Tang-like workload."""
    from .params import initialize_simulation_parameters
    Ns = 2
    ai = alpha_e / 5.0
    user = dict(Lx=L, Ly=L, Lz=1.0, mi_me=mi_me, qs=[-1.0, 1.0], alpha_s=[alpha_e] * 3 + [ai] * 3,
                u_s=[0.0] * 6, Omega_cs=[Omega_ce, Omega_ce / mi_me], nu=0.5, D=0.0)
    p = initialize_simulation_parameters(user, Nx, Ny, Nz, Nn, Nm, Np, Ns, 2, 0.1)
    kx, ky = 2 * np.pi / L, 2 * np.pi / L
    # the reference samples the fields on linspace(0, L, N) (endpoint included)
    x = np.linspace(0, L, Nx)
    y = np.linspace(0, L, Ny)
    z = np.linspace(0, 1.0, Nz)
    X, Y, Z = np.meshgrid(x, y, z, indexing="xy")
    Ue = np.array([-du * np.sin(ky * Y), du * np.sin(kx * X),
                   -dB * Omega_ce * (2 * kx * np.cos(2 * kx * X) + ky * np.cos(ky * Y))])
    Ui = np.array([-du * np.sin(ky * Y), du * np.sin(kx * X), np.zeros_like(X)])
    Ck = compute_C_nmp(np.stack([Ue, Ui]), p["alpha_s"], p["u_s"], Nn, Nm, Np, Ns)
    B = np.array([-dB * np.sin(ky * Y), dB * np.sin(2 * kx * X), np.ones_like(X)])
    E = np.zeros_like(B)
    ax3 = (-3, -2, -1)
    Fk = np.fft.fftshift(np.fft.fftn(np.concatenate([E, B]), axes=ax3, norm="forward"), axes=ax3)
    y0 = np.concatenate([Ck.ravel(), Fk.ravel()]).astype(np.complex128)
    rng = np.random.default_rng(seed)
    y0 += noise * (rng.standard_normal(y0.shape) + 1j * rng.standard_normal(y0.shape))
    p["Ck_0"] = y0[: Ck.size].reshape(Ns * Np * Nm * Nn, Ny, Nx, Nz)
    p["Fk_0"] = y0[Ck.size:].reshape(6, Ny, Nx, Nz)
    return p, y0
