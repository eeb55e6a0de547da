import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: longer GPU integration runs")


def pytest_collection_modifyitems(config, items):
    have_gpu = False
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except Exception:
        pass
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def golden_cases():
    g = np.load(os.path.join(GOLDEN, "rhs_cases.npz"))
    names = sorted({k.split("/")[0] for k in g.files})
    return g, names


def golden_params(g, name):
    """Parameter dict (oracle flavour) for a golden case."""
    from oracle import tables
    Nx, Ny, Nz, Nn, Nm, Np, Ns = (int(v) for v in g[name + "/shape"])
    user = {}
    for k in ("qs", "alpha_s", "u_s", "Omega_cs", "nu", "D", "Lx", "Ly", "Lz"):
        v = g[f"{name}/{k}"]
        user[k] = v.tolist() if v.ndim else float(v)
    return tables.initialize_simulation_parameters(user, Nx, Ny, Nz, Nn, Nm, Np, Ns, 10, 0.01)


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
