"""Golden vectors of the reference's initial-state builder and f(x, v) reconstruction.

Run once where the SPECTRAX source tree is available:

    python tests/golden/make_builder_golden.py <path to the SPECTRAX source tree>

With the NumPy stand-in of ``make_golden.py`` (``jit`` is the identity, ``jnp``
is NumPy, ``jax.scipy.special.factorial`` is SciPy's) this imports, unmodified,
``spectrax/_initialize_maxwellian.py`` (``compute_C_nmp``) and
``spectrax/_inverse_transform.py`` (``inverse_HF_transform``).  The latter also
needs ``jax.vmap``, stood in by mapping over the first axis and stacking, and
``orthax.hermite.hermval``, stood in by ``numpy.polynomial.hermite.hermval``
(the NumPy function orthax ports to JAX; physicists' Hermite polynomials by the
same Clenshaw recurrence).  Writes builders.npz with the inputs and outputs of
a few seeded cases.
"""
from __future__ import annotations

import importlib
import os
import sys
import types
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import make_golden  # noqa: E402

MAXWELLIAN_CASES = [(2, 8, 1, 1, 1, 33, 1), (2, 3, 3, 3, 6, 5, 1), (1, 2, 2, 3, 4, 5, 3)]
INVERSE_CASES = [(16, 1, 1, 1, 9, 1, (1, 20, 1)), (3, 3, 3, 4, 5, 1, (3, 4, 2)), (2, 3, 2, 1, 6, 3, (2, 2, 3))]


def install_extra_standins():
    jax = sys.modules["jax"]

    def vmap(f):
        return lambda xs: np.stack([np.asarray(f(x)) for x in xs])

    jax.vmap = vmap
    orthax = types.ModuleType("orthax")
    herm = types.ModuleType("orthax.hermite")
    herm.hermval = np.polynomial.hermite.hermval
    orthax.hermite = herm
    sys.modules.update({"orthax": orthax, "orthax.hermite": herm})


def main(ref_root):
    warnings.simplefilter("ignore")
    make_golden.install_standin()
    install_extra_standins()
    pkg = types.ModuleType("spectrax")
    pkg.__path__ = [os.path.join(ref_root, "spectrax")]
    sys.modules["spectrax"] = pkg
    mx = importlib.import_module("spectrax._initialize_maxwellian")
    it = importlib.import_module("spectrax._inverse_transform")
    out = {}
    rng = np.random.default_rng(20261204)
    for i, (Ns, Nn, Nm, Np, Ny, Nx, Nz) in enumerate(MAXWELLIAN_CASES):
        Us = 0.3 * rng.standard_normal((Ns, 3, Ny, Nx, Nz))
        alpha = rng.uniform(0.3, 1.5, 3 * Ns)
        u = rng.uniform(-0.2, 0.2, 3 * Ns)
        Ck = np.asarray(mx.compute_C_nmp(Us, alpha, u, Nn, Nm, Np, Ns))
        out[f"mx{i}/shape"] = np.array([Ns, Nn, Nm, Np, Ny, Nx, Nz])
        out[f"mx{i}/Us"], out[f"mx{i}/alpha"], out[f"mx{i}/u"], out[f"mx{i}/Ck"] = Us, alpha, u, Ck
    for i, (Nn, Nm, Np, Ny, Nx, Nz, V) in enumerate(INVERSE_CASES):
        Ck = (rng.standard_normal((2, Nn * Nm * Np, Ny, Nx, Nz))
              + 1j * rng.standard_normal((2, Nn * Nm * Np, Ny, Nx, Nz)))
        vy, vx, vz = np.linspace(-2.0, 2.0, V[0]), np.linspace(-3.0, 3.0, V[1]), np.linspace(-1.5, 1.5, V[2])
        xi_y, xi_x, xi_z = np.meshgrid(vy, vx, vz, indexing="ij")
        f = np.asarray(it.inverse_HF_transform(Ck, Nn, Nm, Np, xi_x, xi_y, xi_z))
        out[f"inv{i}/shape"] = np.array([Nn, Nm, Np, Ny, Nx, Nz])
        out[f"inv{i}/Ck"], out[f"inv{i}/f"] = Ck, f
        out[f"inv{i}/xi_x"], out[f"inv{i}/xi_y"], out[f"inv{i}/xi_z"] = xi_x, xi_y, xi_z
    np.savez_compressed(os.path.join(HERE, "builders.npz"), **out)
    print("wrote builders.npz:", len(MAXWELLIAN_CASES), "Maxwellian and", len(INVERSE_CASES), "f(x, v) cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_builder_golden.py <path to the SPECTRAX source tree>")
    main(sys.argv[1])
