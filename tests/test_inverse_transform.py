"""f(x, v) reconstruction (spectrax/_inverse_transform.py) against the oracle restatement."""
import math

import numpy as np
import pytest

from conftest import rel_err
from oracle import inverse_transform as oinv


def _normalised(N, x):
    H = oinv.hermite_basis(N, x)
    norm = np.array([math.sqrt(math.pi) * 2.0 ** (n / 2.0) * math.sqrt(math.factorial(n)) for n in range(N)])
    return H / norm.reshape((-1,) + (1,) * np.ndim(x))


def test_oracle_basis_is_orthonormal_under_the_gaussian():
    # Gauss-Hermite quadrature: int e^{-x^2} b_n b_m dx = delta_nm / sqrt(pi)
    x, w = np.polynomial.hermite.hermgauss(40)
    b = _normalised(16, x)
    G = (b * w) @ b.T
    np.testing.assert_allclose(G, np.eye(16) / math.sqrt(math.pi), atol=1e-13)


@pytest.mark.gpu
def test_basis_kernel_matches_oracle():
    from spectrax_gb300.inverse_transform import hermite_basis
    x = np.linspace(-5.0, 5.0, 301)
    ref = _normalised(48, x)
    got = hermite_basis(48, x).cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_basis_kernel_is_finite_where_the_polynomials_overflow():
    from spectrax_gb300.inverse_transform import hermite_basis
    x = np.linspace(-30.0, 30.0, 61)
    got = hermite_basis(400, x).cpu().numpy()
    assert np.all(np.isfinite(got))


@pytest.mark.gpu
@pytest.mark.parametrize("Nn,Nm,Np,Ny,Nx,Nz,V", [
    (16, 1, 1, 1, 9, 1, (1, 20, 1)),
    (3, 3, 3, 4, 5, 1, (3, 4, 2)),
    (2, 3, 2, 1, 6, 3, (2, 2, 3)),
])
def test_inverse_transform_matches_oracle(Nn, Nm, Np, Ny, Nx, Nz, V):
    from spectrax_gb300.inverse_transform import inverse_HF_transform
    rng = np.random.default_rng(Nn * 100 + Nx)
    Ck = rng.standard_normal((2, Nn * Nm * Np, Ny, Nx, Nz)) + 1j * rng.standard_normal((2, Nn * Nm * Np, Ny, Nx, Nz))
    vy = np.linspace(-2.0, 2.0, V[0])
    vx = np.linspace(-3.0, 3.0, V[1])
    vz = np.linspace(-1.5, 1.5, V[2])
    xi_y, xi_x, xi_z = np.meshgrid(vy, vx, vz, indexing="ij")
    ref = oinv.inverse_HF_transform(Ck, Nn, Nm, Np, xi_x, xi_y, xi_z)
    got = inverse_HF_transform(Ck, Nn, Nm, Np, xi_x, xi_y, xi_z).cpu().numpy()
    assert got.shape == ref.shape == (2, Ny, Nx, Nz) + V
    assert rel_err(got, ref) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("Ns,Nn,Nm,Np,Ny,Nx,Nz", [(2, 8, 1, 1, 1, 33, 1), (2, 3, 3, 3, 8, 8, 1), (1, 2, 2, 3, 4, 5, 3)])
def test_device_maxwellian_matches_host(Ns, Nn, Nm, Np, Ny, Nx, Nz):
    # spectrax/_initialize_maxwellian.py on the GPU against the NumPy version,
    # plus the same transform of extra real planes (the fields)
    from spectrax_gb300.maxwellian import compute_C_nmp, compute_C_nmp_device
    rng = np.random.default_rng(Nx * 7 + Nn)
    Us = 0.3 * rng.standard_normal((Ns, 3, Ny, Nx, Nz))
    alpha = rng.uniform(0.3, 1.5, 3 * Ns)
    u = rng.uniform(-0.2, 0.2, 3 * Ns)
    ref = compute_C_nmp(Us, alpha, u, Nn, Nm, Np, Ns)
    F = rng.standard_normal((6, Ny, Nx, Nz))
    got, Fk = compute_C_nmp_device(Us, alpha, u, Nn, Nm, Np, Ns, extra_real=F)
    assert tuple(got.shape) == ref.shape
    assert rel_err(got.cpu().numpy(), ref) < 1e-13
    Fref = np.fft.fftshift(np.fft.fftn(F, axes=(-3, -2, -1), norm="forward"), axes=(-3, -2, -1))
    assert rel_err(Fk.cpu().numpy(), Fref) < 1e-13


def _builders():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "builders.npz"))


def test_restatements_match_reference_builder_vectors():
    # the host Maxwellian builder and the f(x, v) oracle against vectors made by
    # running spectrax/_initialize_maxwellian.py and spectrax/_inverse_transform.py
    from spectrax_gb300.maxwellian import compute_C_nmp
    g = _builders()
    for i in range(3):
        Ns, Nn, Nm, Np, Ny, Nx, Nz = (int(v) for v in g[f"mx{i}/shape"])
        got = compute_C_nmp(g[f"mx{i}/Us"], g[f"mx{i}/alpha"], g[f"mx{i}/u"], Nn, Nm, Np, Ns)
        assert rel_err(got, g[f"mx{i}/Ck"]) < 1e-14
    for i in range(3):
        Nn, Nm, Np = (int(v) for v in g[f"inv{i}/shape"][:3])
        got = oinv.inverse_HF_transform(g[f"inv{i}/Ck"], Nn, Nm, Np, g[f"inv{i}/xi_x"], g[f"inv{i}/xi_y"],
                                        g[f"inv{i}/xi_z"])
        assert rel_err(got, g[f"inv{i}/f"]) < 1e-14


@pytest.mark.gpu
def test_device_builders_match_reference_vectors():
    # spx_maxwellian and the device f(x, v) reconstruction against the reference's own output
    from spectrax_gb300.inverse_transform import inverse_HF_transform
    from spectrax_gb300.maxwellian import compute_C_nmp_device
    g = _builders()
    for i in range(3):
        Ns, Nn, Nm, Np, Ny, Nx, Nz = (int(v) for v in g[f"mx{i}/shape"])
        got, _ = compute_C_nmp_device(g[f"mx{i}/Us"], g[f"mx{i}/alpha"], g[f"mx{i}/u"], Nn, Nm, Np, Ns)
        assert rel_err(got.cpu().numpy(), g[f"mx{i}/Ck"]) < 1e-13
    for i in range(3):
        Nn, Nm, Np = (int(v) for v in g[f"inv{i}/shape"][:3])
        got = inverse_HF_transform(g[f"inv{i}/Ck"], Nn, Nm, Np, g[f"inv{i}/xi_x"], g[f"inv{i}/xi_y"],
                                   g[f"inv{i}/xi_z"]).cpu().numpy()
        assert rel_err(got, g[f"inv{i}/f"]) < 1e-12
