"""FP64 NumPy restatement of the SPECTRAX Hermite-Fourier right-hand side.

TEST INFRASTRUCTURE ONLY (the checker; never imported by the product path).

Follows, operator by operator:
  spectrax/_simulation.py:15-32   ``_twothirds_mask``
  spectrax/_simulation.py:34-53   ``cross_product``
  spectrax/_simulation.py:55-111  ``ode_system`` (the Diffrax vector field)
  spectrax/_model.py:15-72        ``plasma_current``
  spectrax/_model.py:74-97        ``shift_multi`` / ``_pad_hermite_axes``
  spectrax/_model.py:99-212       ``Hermite_Fourier_system``

Layout (identical to the reference): the flat state is
``concat(Ck.ravel(), Fk.ravel())`` with Ck shaped (Ns, Np, Nm, Nn, Ny, Nx, Nz)
and Fk shaped (6, Ny, Nx, Nz) = (Ex, Ey, Ez, Bx, By, Bz); Fourier axes are in
fftshift order (index c <-> wavenumber c - N//2) and the axis order is (y, x, z).
"""
from __future__ import annotations

import numpy as np

_AX = (-3, -2, -1)
SQRT2 = np.sqrt(2.0)

# FFT backend: NumPy (default) or scipy.fft with a worker count, so the CPU
# baseline can use every host core the way XLA's CPU FFT would.
_FFT_WORKERS = None


def set_fft_workers(n):
    """Use scipy.fft with `n` threads (None: NumPy's single-threaded FFT)."""
    global _FFT_WORKERS
    _FFT_WORKERS = n


def _ifftn(x):
    if _FFT_WORKERS:
        import scipy.fft as sf
        return sf.ifftn(x, axes=_AX, norm="forward", workers=_FFT_WORKERS)
    return np.fft.ifftn(x, axes=_AX, norm="forward")


def _fftn(x):
    if _FFT_WORKERS:
        import scipy.fft as sf
        return sf.fftn(x, axes=_AX, norm="forward", workers=_FFT_WORKERS)
    return np.fft.fftn(x, axes=_AX, norm="forward")


# --------------------------------------------------------------------------- mask
def _fftfreq_times_n(n: int, mode: str) -> np.ndarray:
    """``fftshift(fftfreq(n)) * n`` evaluated the way the reference's JAX does it.

    JAX builds the integer bins and then DIVIDES by ``n`` (mode "divide").  When the
    whole mask is traced under ``jit``, XLA's simplifier may instead multiply by the
    constant ``1/n`` (mode "multiply").  The two differ only at the edge bin
    |k| = n//3 for some n (n = 10, 20, 33, 45, ...; at n = 33 "divide" keeps 23
    modes and "multiply" 21).  Which one the live reference takes cannot be run
    here, so the cutoff is an explicit input of the GPU path.
    """
    k = np.empty(n)
    half = (n - 1) // 2 + 1 if n % 2 else n // 2
    k[:half] = np.arange(0, half)
    k[half:] = np.arange(-(n - half), 0)
    if mode == "divide":
        f = k / float(n)
    elif mode == "multiply":
        f = k * (1.0 / float(n))
    else:
        raise ValueError(f"unknown mask mode {mode!r}")
    return np.fft.fftshift(f) * n


def centered_cutoff(n: int, mode: str = "divide") -> int:
    """Largest |k| kept by the 2/3 rule along an axis of length n (-1 keeps nothing).

    The kept set is symmetric and contiguous, so one integer describes it.
    spectrax/_simulation.py:27-32 keeps |k| <= n//3 after the float rounding above.
    """
    kc = np.abs(_fftfreq_times_n(n, mode))
    keep = kc <= (n // 3)
    ints = np.abs(np.arange(n) - n // 2)
    return int(ints[keep].max()) if keep.any() else -1


def twothirds_mask(Ny: int, Nx: int, Nz: int, mode: str = "divide") -> np.ndarray:
    """Boolean (Ny, Nx, Nz) mask; spectrax/_simulation.py:15-32."""
    def axis_keep(n):
        return np.abs(_fftfreq_times_n(n, mode)) <= (n // 3)
    return (axis_keep(Ny)[:, None, None] & axis_keep(Nx)[None, :, None]
            & axis_keep(Nz)[None, None, :])


# --------------------------------------------------------------------------- helpers
def cross_product(k, F):
    """k x F over the leading axis of length 3; spectrax/_simulation.py:34-53."""
    return np.array([k[1] * F[2] - k[2] * F[1],
                     k[2] * F[0] - k[0] * F[2],
                     k[0] * F[1] - k[1] * F[0]])


def hermite_neighbor(C7: np.ndarray, dn: int = 0, dm: int = 0, dp: int = 0) -> np.ndarray:
    """Return D with D[s,p,m,n] = C[s,p+dp,m+dm,n+dn], zero outside the Hermite box.

    This is what spectrax/_model.py:79-97 ``shift_multi(C, dn, dm, dp)`` returns
    (dn=+1 gives C_{n+1}; the docstring there states the opposite).
    """
    Ns, Np, Nm, Nn = C7.shape[:4]
    out = np.zeros_like(C7)
    def rng(N, d):
        dst = slice(max(0, -d), N - max(0, d))
        src = slice(max(0, d), N - max(0, -d))
        return dst, src
    (pd, ps), (md, ms), (nd, ns) = rng(Np, dp), rng(Nm, dm), rng(Nn, dn)
    out[:, pd, md, nd] = C7[:, ps, ms, ns]
    return out


def plasma_current(qs, alpha_s, u_s, Ck, Nn, Nm, Np, Ns):
    """J = sum_s q_s a0 a1 a2 [ (a0 C100, a1 C010, a2 C001)/sqrt2 + u_s C000 ].

    spectrax/_model.py:15-72; uses UNMASKED Fourier Ck; a mode absent because
    its Hermite axis has length 1 reads as zero.
    """
    C7 = Ck.reshape(Ns, Np, Nm, Nn, *Ck.shape[-3:])
    a = np.asarray(alpha_s, dtype=np.float64).reshape(Ns, 3)
    u = np.asarray(u_s, dtype=np.float64).reshape(Ns, 3)
    q = np.asarray(qs, dtype=np.float64)
    C000 = C7[:, 0, 0, 0]
    zero = np.zeros_like(C000)
    C100 = C7[:, 0, 0, 1] if Nn > 1 else zero
    C010 = C7[:, 0, 1, 0] if Nm > 1 else zero
    C001 = C7[:, 1, 0, 0] if Np > 1 else zero
    pre = q * a[:, 0] * a[:, 1] * a[:, 2]
    b = (slice(None), None, None, None)
    Jx = (a[:, 0][b] * C100 / SQRT2 + u[:, 0][b] * C000) * pre[b]
    Jy = (a[:, 1][b] * C010 / SQRT2 + u[:, 1][b] * C000) * pre[b]
    Jz = (a[:, 2][b] * C001 / SQRT2 + u[:, 2][b] * C000) * pre[b]
    return np.stack([Jx.sum(0), Jy.sum(0), Jz.sum(0)])


# --------------------------------------------------------------------------- RHS
def unpack_args(args):
    """Entries [7:] of the 28-tuple built at spectrax/_simulation.py:154-161."""
    (qs, nu, D, Omega_cs, alpha_s, u_s, Lx, Ly, Lz, kx_grid, ky_grid, kz_grid,
     k2_grid, nabla, col, snp, snm, smp, smm, spp, spm) = args[7:]
    return dict(qs=np.asarray(qs, np.float64), nu=float(nu), D=float(D),
                Omega_cs=np.asarray(Omega_cs, np.float64),
                alpha_s=np.asarray(alpha_s, np.float64), u_s=np.asarray(u_s, np.float64),
                Lx=float(Lx), Ly=float(Ly), Lz=float(Lz),
                kx_grid=np.asarray(kx_grid, np.float64), ky_grid=np.asarray(ky_grid, np.float64),
                kz_grid=np.asarray(kz_grid, np.float64), k2_grid=np.asarray(k2_grid, np.float64),
                nabla=np.asarray(nabla, np.float64), col=np.asarray(col, np.float64),
                sqrt_n_plus=np.asarray(snp, np.float64), sqrt_n_minus=np.asarray(snm, np.float64),
                sqrt_m_plus=np.asarray(smp, np.float64), sqrt_m_minus=np.asarray(smm, np.float64),
                sqrt_p_plus=np.asarray(spp, np.float64), sqrt_p_minus=np.asarray(spm, np.float64))


def hermite_fourier_system(Ck, C, F, P, Nn, Nm, Np, Ns, mask):
    """dCk/dt; spectrax/_model.py:99-212.  P is ``unpack_args`` output."""
    Ny, Nx, Nz = Ck.shape[-3:]
    Ck = Ck.reshape(Ns, Np, Nm, Nn, Ny, Nx, Nz)
    C = C.reshape(Ns, Np, Nm, Nn, Ny, Nx, Nz)
    Ex, Ey, Ez, Bx, By, Bz = (F[i][None, None, None, None] for i in range(6))
    sp = (slice(None),) + (None,) * 6
    a = P["alpha_s"].reshape(Ns, 3)
    u = P["u_s"].reshape(Ns, 3)
    a0, a1, a2 = a[:, 0][sp], a[:, 1][sp], a[:, 2][sp]
    u0, u1, u2 = u[:, 0][sp], u[:, 1][sp], u[:, 2][sp]
    q = P["qs"][sp]
    Oc = P["Omega_cs"][sp]
    snp, snm = P["sqrt_n_plus"], P["sqrt_n_minus"]
    smp, smm = P["sqrt_m_plus"], P["sqrt_m_minus"]
    spp, spm = P["sqrt_p_plus"], P["sqrt_p_minus"]
    nb = hermite_neighbor

    # real-space auxiliary combinations (spectrax/_model.py:168-184)
    aux_x = (smm * spm * (a2 / a1 - a1 / a2) * nb(C, 0, -1, -1)
             + smm * spp * (a2 / a1) * nb(C, 0, -1, 1)
             - smp * spm * (a1 / a2) * nb(C, 0, 1, -1)
             + SQRT2 * smm * (u2 / a1) * nb(C, 0, -1, 0)
             - SQRT2 * spm * (u1 / a2) * nb(C, 0, 0, -1))
    aux_y = (snm * spm * (a0 / a2 - a2 / a0) * nb(C, -1, 0, -1)
             + snp * spm * (a0 / a2) * nb(C, 1, 0, -1)
             - snm * spp * (a2 / a0) * nb(C, -1, 0, 1)
             + SQRT2 * spm * (u0 / a2) * nb(C, 0, 0, -1)
             - SQRT2 * snm * (u2 / a0) * nb(C, -1, 0, 0))
    aux_z = (snm * smm * (a1 / a0 - a0 / a1) * nb(C, -1, -1, 0)
             + snm * smp * (a1 / a0) * nb(C, -1, 1, 0)
             - snp * smm * (a0 / a1) * nb(C, 1, -1, 0)
             + SQRT2 * snm * (u1 / a0) * nb(C, -1, 0, 0)
             - SQRT2 * smm * (u0 / a1) * nb(C, 0, -1, 0))

    bracket = ((snm * SQRT2 / a0) * Ex * nb(C, -1, 0, 0)
               + (smm * SQRT2 / a1) * Ey * nb(C, 0, -1, 0)
               + (spm * SQRT2 / a2) * Ez * nb(C, 0, 0, -1)
               + Bx * aux_x + By * aux_y + Bz * aux_z)
    nonlinear = np.fft.fftshift(_fftn(bracket), axes=_AX) * mask

    kx, ky, kz, k2 = P["kx_grid"], P["ky_grid"], P["kz_grid"], P["k2_grid"]
    col = P["col"][None, :, :, :, None, None, None]
    stream = (-(kx * (1j / P["Lx"])) * a0 * (snp / SQRT2 * nb(Ck, 1, 0, 0)
                                            + snm / SQRT2 * nb(Ck, -1, 0, 0) + (u0 / a0) * Ck)
              - (ky * (1j / P["Ly"])) * a1 * (smp / SQRT2 * nb(Ck, 0, 1, 0)
                                             + smm / SQRT2 * nb(Ck, 0, -1, 0) + (u1 / a1) * Ck)
              - (kz * (1j / P["Lz"])) * a2 * (spp / SQRT2 * nb(Ck, 0, 0, 1)
                                             + spm / SQRT2 * nb(Ck, 0, 0, -1) + (u2 / a2) * Ck))
    return stream + q * Oc * nonlinear - P["nu"] * col * Ck - P["D"] * k2 * Ck


def ode_system(Nx, Ny, Nz, Nn, Nm, Np, Ns, t, Ck_Fk, args, mask_mode: str = "divide"):
    """Flat complex128 state -> flat derivative; spectrax/_simulation.py:55-111."""
    del t
    P = unpack_args(args)
    y = np.asarray(Ck_Fk, dtype=np.complex128)
    NC = Nn * Nm * Np * Ns * Nx * Ny * Nz
    Ck = y[:NC].reshape(Nn * Nm * Np * Ns, Ny, Nx, Nz)
    Fk = y[NC:].reshape(6, Ny, Nx, Nz)
    mask = twothirds_mask(Ny, Nx, Nz, mask_mode)
    F = _ifftn(np.fft.ifftshift(Fk * mask, axes=_AX))
    C = _ifftn(np.fft.ifftshift(Ck * mask, axes=_AX))
    dCk = hermite_fourier_system(Ck, C, F, P, Nn, Nm, Np, Ns, mask)
    dBk = -1j * cross_product(P["nabla"], Fk[:3])
    J = plasma_current(P["qs"], P["alpha_s"], P["u_s"], Ck, Nn, Nm, Np, Ns)
    dEk = 1j * cross_product(P["nabla"], Fk[3:]) - J / P["Omega_cs"][0]
    return np.concatenate([dCk.reshape(-1), dEk.reshape(-1), dBk.reshape(-1)])


def rhs(params: dict, y: np.ndarray, mask_mode: str = "divide") -> np.ndarray:
    """Convenience wrapper taking a parameter dict from ``oracle.tables``."""
    from .tables import make_args
    d = params
    return ode_system(d["Nx"], d["Ny"], d["Nz"], d["Nn"], d["Nm"], d["Np"], d["Ns"], 0.0,
                      y, make_args(d), mask_mode)
