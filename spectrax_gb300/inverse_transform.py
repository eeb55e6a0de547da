"""f(x, v) from Hermite-Fourier coefficients on the GPU (spectrax/_inverse_transform.py).

``inverse_HF_transform(Ck, Nn, Nm, Np, xi_x, xi_y, xi_z)`` keeps the reference's
signature and output layout (spectrax/_inverse_transform.py:97-125):

* C = Re ifftn(ifftshift(Ck)) over the last three (y, x, z) axes (1/N
  normalisation, no 2/3 mask), on the device;
* the per-axis basis b_n(xi) = H_n(xi) / (sqrt(pi) 2^(n/2) sqrt(n!)) from the
  ``spx_hermite_basis`` kernel (normalised-function recurrence: finite for every
  n where the reference's H_n overflows), combined into the (n, m, p) product
  basis with the reference's mode order index = (p Nm + m) Nn + n (:61-64);
* the contraction over the modes as one GEMM, times exp(-(xi_x^2 + xi_y^2 +
  xi_z^2)) (:72, :92).

Ck: (..., Nn*Nm*Np, Ny, Nx, Nz) complex; xi_*: arrays of one common shape V.
Returns a real tensor (..., Ny, Nx, Nz, *V) on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .vector_field import _stream_ptr


def hermite_basis(N: int, xi, device=None) -> torch.Tensor:
    """(N, len(xi)) float64: b_n(xi_j) = H_n(xi_j) / (sqrt(pi) 2^(n/2) sqrt(n!))."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    x = torch.as_tensor(xi, dtype=torch.float64).reshape(-1).to(dev).contiguous()
    out = torch.empty((int(N), x.numel()), dtype=torch.float64, device=dev)
    _lib.check(_lib.lib().spx_hermite_basis(int(N), C.c_void_p(x.data_ptr()), x.numel(),
                                            C.c_void_p(out.data_ptr()), _stream_ptr()), "spx_hermite_basis")
    return out


def inverse_HF_transform(Ck, Nn, Nm, Np, xi_x, xi_y, xi_z, device=None):
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    Ck = torch.as_tensor(Ck).to(dev, torch.complex128)
    nmodes = Nn * Nm * Np
    if Ck.dim() < 4 or Ck.shape[-4] != nmodes:
        raise ValueError(f"Ck must end in (Nn*Nm*Np={nmodes}, Ny, Nx, Nz), got {tuple(Ck.shape)}")
    xs = [torch.as_tensor(np.asarray(a, np.float64)) for a in (xi_x, xi_y, xi_z)]
    vshape = tuple(xs[0].shape)
    if any(tuple(a.shape) != vshape for a in xs):
        raise ValueError("xi_x, xi_y, xi_z must have one common shape")
    C_real = torch.fft.ifftn(torch.fft.ifftshift(Ck, dim=(-3, -2, -1)), dim=(-3, -2, -1)).real
    bx, by, bz = (hermite_basis(N, a, dev) for N, a in zip((Nn, Nm, Np), xs))
    nv = bx.shape[1]
    basis = (bz[:, None, None, :] * by[None, :, None, :] * bx[None, None, :, :]).reshape(nmodes, nv)
    xd = [a.reshape(-1).to(dev) for a in xs]
    gauss = torch.exp(-(xd[0] ** 2 + xd[1] ** 2 + xd[2] ** 2))
    lead = C_real.shape[:-4]
    space = C_real.shape[-3:]
    # (..., modes, Ny, Nx, Nz) -> (rows, modes) x (modes, nv)
    Cm = torch.movedim(C_real, -4, -1).reshape(-1, nmodes)
    f = (Cm @ basis) * gauss
    return f.reshape(*lead, *space, *vshape)
