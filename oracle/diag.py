"""FP64 restatement of SPECTRAX's energy diagnostics (test infrastructure only).

Follows spectrax/_diagnostics.py:71-233: low-order Hermite moments at the k=0
bin (index N//2 per axis, :126-131, :169-198), kinetic energy per species
(:200-215), EM_energy = 0.5 * Omega_c0**2 * sum |Fk|**2 (:217) and total (:219).
"""
from __future__ import annotations

import numpy as np


def _masses(Ns, mi_me=None, ms=None):
    """spectrax/_diagnostics.py:44-68."""
    if ms is not None:
        return np.asarray(ms, dtype=np.float64)
    if Ns == 2 and mi_me is not None:
        return np.array([1.0, float(mi_me)])
    return np.ones(Ns)


def energies(ys, Nx, Ny, Nz, Nn, Nm, Np, Ns, alpha_s, u_s, Omega_cs, mi_me=None, ms=None):
    """Energies of flat states ys (Nt, N).  Returns dict of (Nt,) / (Nt, Ns) arrays."""
    ys = np.atleast_2d(np.asarray(ys, dtype=np.complex128))
    Nt = ys.shape[0]
    NC = Ns * Nn * Nm * Np * Ny * Nx * Nz
    Ck = ys[:, :NC].reshape(Nt, Ns, Nn * Nm * Np, Ny, Nx, Nz)
    Fk = ys[:, NC:].reshape(Nt, 6, Ny, Nx, Nz)
    Hs = Nn * Nm * Np
    cy, cx, cz = Ny // 2, Nx // 2, Nz // 2

    def mode(off):
        if 0 <= off < Hs:
            return Ck[:, :, off, cy, cx, cz]
        return np.zeros((Nt, Ns), dtype=np.complex128)

    C000, C100, C010, C001 = mode(0), mode(1), mode(Nn), mode(Nn * Nm)
    C200, C020, C002 = mode(2), mode(2 * Nn), mode(2 * Nn * Nm)
    a = np.asarray(alpha_s, np.float64).reshape(Ns, 3)
    u = np.asarray(u_s, np.float64).reshape(Ns, 3)
    m = _masses(Ns, mi_me, ms)
    a0, a1, a2 = a[:, 0], a[:, 1], a[:, 2]
    u0, u1, u2 = u[:, 0], u[:, 1], u[:, 2]
    pref = 0.5 * m * a0 * a1 * a2
    term0 = 0.5 * (a0 ** 2 + a1 ** 2 + a2 ** 2) + (u0 ** 2 + u1 ** 2 + u2 ** 2)
    term1 = np.sqrt(2.0) * (a0 * u0 * C100 + a1 * u1 * C010 + a2 * u2 * C001)
    term2 = (1.0 / np.sqrt(2.0)) * (a0 ** 2 * C200 + a1 ** 2 * C020 + a2 ** 2 * C002)
    kes = pref[None, :] * (term0[None, :] * C000 + term1 + term2)
    ke = kes.sum(axis=1)
    em = 0.5 * np.sum(np.abs(Fk) ** 2, axis=(-4, -3, -2, -1)) * float(np.asarray(Omega_cs)[0]) ** 2
    return dict(kinetic_energy_species=kes, kinetic_energy=ke, EM_energy=em, total_energy=ke + em)


def lambda_D_and_k_norm(alpha_s, Lx, Ns, mi_me=None):
    """spectrax/_diagnostics.py:152-163."""
    alpha_s = np.asarray(alpha_s, np.float64)
    if Ns == 2 and mi_me is not None:
        lam = np.sqrt(1.0 / (2.0 * (1.0 / alpha_s[0] ** 2 + 1.0 / (mi_me * alpha_s[3] ** 2))))
    else:
        ax = alpha_s.reshape(Ns, 3)[:, 0]
        lam = np.sqrt(1.0 / (2.0 * np.sum(1.0 / ax ** 2)))
    return lam, np.sqrt(2.0) * np.pi * alpha_s[0] / Lx
