"""f(x, v) from Hermite-Fourier coefficients on the GPU (spectrax/_inverse_transform.py).

``inverse_HF_transform(Ck, Nn, Nm, Np, xi_x, xi_y, xi_z)`` keeps the reference's
signature and output layout (spectrax/_inverse_transform.py:97-125):

* C = Re ifftn(ifftshift(Ck)) over the last three (y, x, z) axes (1/N
  normalisation, no 2/3 mask), by the library's own FFT engine (``spx_fxv``);
* the per-axis basis b_n(xi) = H_n(xi) / (sqrt(pi) 2^(n/2) sqrt(n!)) from the
  ``spx_hermite_basis`` kernel (normalised-function recurrence: finite for every
  n where the reference's H_n overflows), combined into the (n, m, p) product
  basis with the reference's mode order index = (p Nm + m) Nn + n (:61-64);
* the contraction over the modes as an FP64 GEMM kernel of the library, times
  exp(-(xi_x^2 + xi_y^2 + xi_z^2)) (:72, :92).

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
    from .params import make_problem
    from .vector_field import get_plan
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    Ck = torch.as_tensor(Ck).to(dev, torch.complex128).contiguous()
    nmodes = Nn * Nm * Np
    if Ck.dim() < 4 or Ck.shape[-4] != nmodes:
        raise ValueError(f"Ck must end in (Nn*Nm*Np={nmodes}, Ny, Nx, Nz), got {tuple(Ck.shape)}")
    xs = [np.asarray(a, np.float64) for a in (xi_x, xi_y, xi_z)]
    vshape = xs[0].shape
    if any(a.shape != vshape for a in xs):
        raise ValueError("xi_x, xi_y, xi_z must have one common shape")
    Ny, Nx, Nz = (int(v) for v in Ck.shape[-3:])
    lead = tuple(Ck.shape[:-4])
    nlead = int(np.prod(lead)) if lead else 1
    # a one-species plan that keeps every Fourier mode (no 2/3 mask in this transform)
    pb = make_problem(Nx, Ny, Nz, Nn, Nm, Np, 1, [-1.0], 0.0, 0.0, [1.0], [1.0] * 3, [0.0] * 3, 1.0, 1.0, 1.0)
    pb.cut_x, pb.cut_y, pb.cut_z = Nx, Ny, Nz
    plan = get_plan(pb, dev.index)
    xi = torch.from_numpy(np.stack([a.reshape(-1) for a in xs])).to(dev).contiguous()
    nv = xi.shape[1]
    bx, by, bz = (hermite_basis(N, xi[i], dev) for i, N in enumerate((Nn, Nm, Np)))
    L = _lib.lib()
    ws = torch.empty(int(L.spx_fxv_workspace_bytes(plan.handle, nlead)), dtype=torch.uint8, device=dev)
    f = torch.empty((nlead * Nx * Ny * Nz, nv), dtype=torch.float64, device=dev)
    with torch.cuda.device(dev):
        _lib.check(L.spx_fxv(plan.handle, C.c_void_p(Ck.data_ptr()), nlead, C.c_void_p(bx.data_ptr()),
                             C.c_void_p(by.data_ptr()), C.c_void_p(bz.data_ptr()), C.c_void_p(xi.data_ptr()), nv,
                             C.c_void_p(f.data_ptr()), C.c_void_p(ws.data_ptr()), C.c_size_t(ws.numel()),
                             _stream_ptr()), "spx_fxv")
    return f.reshape(*lead, Ny, Nx, Nz, *vshape)
