"""FP64 NumPy restatement of spectrax/_inverse_transform.py (test infrastructure only).

Follows spectrax/_inverse_transform.py:20-38 (Hermite polynomials by a Clenshaw
sum, numpy.polynomial.hermite.hermval in place of orthax's), :41-94 (normalised
product basis, contraction over the modes, Gaussian weight) and :97-125 (Re of
ifftn(ifftshift(Ck)) over the last three axes).  Parity unpinned: JAX and
orthax are not installed here; the formulas are restated from the source.
"""
from __future__ import annotations

import math

import numpy as np
from numpy.polynomial.hermite import hermval


def hermite_basis(N, x):
    """spectrax/_inverse_transform.py:20-38: (N, *x.shape) array of H_n(x)."""
    out = []
    for n in range(N):
        c = np.zeros(N)
        c[n] = 1.0
        out.append(hermval(x, c))
    return np.stack(out)


def inverse_HF_transform(Ck, Nn, Nm, Np, xi_x, xi_y, xi_z):
    """spectrax/_inverse_transform.py:97-125 with generate_Hermite_term (:41-94)."""
    C = np.fft.ifftn(np.fft.ifftshift(Ck, axes=(-3, -2, -1)), axes=(-3, -2, -1)).real
    Hx, Hy, Hz = hermite_basis(Nn, xi_x), hermite_basis(Nm, xi_y), hermite_basis(Np, xi_z)
    idx = np.arange(Nn * Nm * Np)
    p = idx // (Nn * Nm)
    m = (idx % (Nn * Nm)) // Nn
    n = idx % Nn
    gauss = np.exp(-(xi_x ** 2 + xi_y ** 2 + xi_z ** 2))
    fact = np.array([float(math.factorial(k)) for k in range(max(Nn, Nm, Np))])
    norm = np.sqrt(np.pi ** 3) * 2.0 ** ((n + m + p) / 2.0) * np.sqrt(fact[n] * fact[m] * fact[p])
    basis = Hx[n] * Hy[m] * Hz[p] / norm.reshape((-1,) + (1,) * np.ndim(xi_x))
    f = np.tensordot(C, basis, axes=([C.ndim - 4], [0]))
    return f * gauss
