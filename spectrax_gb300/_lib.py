"""ctypes binding of ``libspectrax_gb300.so`` (the C ABI in ``include/spectrax_gb300.h``).

The library is built in-tree (``python -m spectrax_gb300.build``).  There is no
fallback: if the shared library is missing or cannot be loaded, every entry
point raises ``SpectraxLibraryError``.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspectrax_gb300.so")

MAX_SPECIES = 8
MAX_AXIS = 256

SPX_OK, SPX_E_ARG, SPX_E_CUDA, SPX_E_WORKSPACE, SPX_E_UNSUPPORTED = 0, -1, -2, -3, -4
KRYLOV_MAX_ROWS = 64   # SPX_KRYLOV_MAX_ROWS

STATUS_NAMES = {0: "RUNNING", 1: "DONE", 2: "MAX_STEPS", 3: "DT_UNDERFLOW", 4: "NONFINITE", 5: "WAIT_TIMEOUT"}
SPX_ST_WAIT_TIMEOUT = 5


class SpectraxLibraryError(RuntimeError):
    pass


class SpectraxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"spectrax_gb300 error {code}: {msg}")
        self.code = code


class spx_problem(C.Structure):
    _fields_ = [
        ("Nx", C.c_int32), ("Ny", C.c_int32), ("Nz", C.c_int32),
        ("Nn", C.c_int32), ("Nm", C.c_int32), ("Np", C.c_int32),
        ("Ns", C.c_int32),
        ("cut_x", C.c_int32), ("cut_y", C.c_int32), ("cut_z", C.c_int32),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("nu", C.c_double), ("D", C.c_double),
        ("qs", C.c_double * MAX_SPECIES),
        ("Omega_cs", C.c_double * MAX_SPECIES),
        ("alpha_s", C.c_double * (3 * MAX_SPECIES)),
        ("u_s", C.c_double * (3 * MAX_SPECIES)),
    ]


class spx_dopri8_opts(C.Structure):
    _fields_ = [
        ("t0", C.c_double), ("t1", C.c_double), ("dt0", C.c_double),
        ("rtol", C.c_double), ("atol", C.c_double),
        ("adaptive", C.c_int32), ("nsave", C.c_int32),
        ("save_ts", C.POINTER(C.c_double)),
        ("max_steps", C.c_int64),
        ("save_states", C.c_int32),
        ("masses", C.POINTER(C.c_double)),
        ("hermitian", C.c_int32),
        ("persistent", C.c_int32),
        ("saveat", C.c_int32),
    ]


class spx_dopri8_stats(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double),
        ("accepted", C.c_int64), ("rejected", C.c_int64), ("rhs_evals", C.c_int64),
        ("status", C.c_int32), ("saved", C.c_int32),
        ("hermitian", C.c_int32), ("persistent", C.c_int32),
    ]


class spx_batch_opts(C.Structure):
    _fields_ = [
        ("t1", C.c_double), ("dt0", C.c_double), ("rtol", C.c_double), ("atol", C.c_double),
        ("max_steps", C.c_int64),
        ("adaptive", C.c_int32), ("nsave", C.c_int32),
        ("save_ts", C.POINTER(C.c_double)),
        ("cluster", C.c_int32), ("tile", C.c_int32),
        ("masses", C.POINTER(C.c_double)),
        ("hermitian", C.c_int32),
        ("saveat", C.c_int32),
        ("costs", C.POINTER(C.c_double)),
    ]


class spx_batch_stats(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double),
        ("accepted", C.c_int64), ("rejected", C.c_int64), ("rhs_evals", C.c_int64),
        ("status", C.c_int32), ("saved", C.c_int32),
        ("hermitian", C.c_int32), ("pad", C.c_int32),
        ("start_s", C.c_double), ("end_s", C.c_double),
    ]


_VP = C.c_void_p
_PROTOS = {
    "spx_last_error": (C.c_char_p, []),
    "spx_version": (C.c_char_p, []),
    "spx_plan_create": (C.c_int, [C.POINTER(spx_problem), C.POINTER(_VP)]),
    "spx_plan_create_ex": (C.c_int, [C.POINTER(spx_problem), C.c_int32, C.c_int32, C.POINTER(_VP)]),
    "spx_plan_destroy": (C.c_int, [_VP]),
    "spx_plan_info": (C.c_int, [_VP, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                C.POINTER(C.c_int32)]),
    "spx_state_len": (C.c_int64, [C.POINTER(spx_problem)]),
    "spx_rhs_workspace_bytes": (C.c_size_t, [_VP]),
    "spx_set_product_grid": (C.c_int, [C.c_int32]),
    "spx_plan_product_grid": (C.c_int, [_VP]),
    "spx_plan_product_radices": (C.c_int, [_VP, C.POINTER(C.c_int32), C.c_int32]),
    "spx_product_grid_for": (C.c_int, [C.c_int32, C.c_int32, C.c_int32]),
    "spx_rhs": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, _VP]),
    "spx_jvp": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_size_t, _VP]),
    "spx_linearize_bytes": (C.c_size_t, [_VP]),
    "spx_linearize": (C.c_int, [_VP, _VP, _VP, C.c_size_t, _VP]),
    "spx_jvp_lin": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_size_t, _VP]),
    "spx_krylov_ws_bytes": (C.c_size_t, [C.c_int64]),
    "spx_hermite_basis": (C.c_int, [C.c_int32, _VP, C.c_int64, _VP, _VP]),
    "spx_fxv_workspace_bytes": (C.c_size_t, [_VP, C.c_int64]),
    "spx_fxv": (C.c_int, [_VP, _VP, C.c_int64, _VP, _VP, _VP, _VP, C.c_int64, _VP, _VP, C.c_size_t, _VP]),
    "spx_maxwellian": (C.c_int, [_VP, _VP, _VP, C.c_int32, _VP, _VP]),
    "spx_krylov_cgs2": (C.c_int, [_VP, C.c_int64, C.c_int32, _VP, _VP, _VP, C.c_size_t, _VP]),
    "spx_krylov_axpy": (C.c_int, [_VP, C.c_int64, C.c_int32, _VP, _VP, _VP]),
    "spx_midpoint_residual": (C.c_int, [C.c_int64, _VP, _VP, _VP, C.c_double, C.c_double, C.c_double, _VP, _VP,
                                        _VP, C.c_size_t, _VP]),
    "spx_midpoint_update": (C.c_int, [C.c_int64, _VP, _VP, _VP, C.c_double, _VP, _VP]),
    "spx_vjp": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_size_t, _VP]),
    "spx_vjp_noalloc": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "spx_dopri8_create": (C.c_int, [_VP, C.POINTER(spx_dopri8_opts), C.POINTER(_VP)]),
    "spx_dopri8_destroy": (C.c_int, [_VP]),
    "spx_dopri8_set_wait_test": (C.c_int, [_VP, C.c_int32, C.c_int32]),
    "spx_dopri8_reset": (C.c_int, [_VP, _VP, _VP]),
    "spx_dopri8_advance": (C.c_int, [_VP, C.c_int64, _VP, C.POINTER(C.c_int32)]),
    "spx_dopri8_run": (C.c_int, [_VP, _VP, C.POINTER(C.c_int32)]),
    "spx_dopri8_enqueue": (C.c_int, [_VP, C.c_int64, _VP]),
    "spx_dopri8_stats_get": (C.c_int, [_VP, C.POINTER(spx_dopri8_stats), _VP]),
    "spx_dopri8_state": (_VP, [_VP]),
    "spx_dopri8_saved_states": (_VP, [_VP]),
    "spx_dopri8_saved_energies": (_VP, [_VP]),
    "spx_dopri8_copy": (C.c_int, [_VP, C.c_int32, _VP, C.c_size_t, _VP]),
    "spx_batch_create": (C.c_int, [C.c_int32, C.POINTER(spx_problem), C.POINTER(spx_batch_opts), C.POINTER(_VP)]),
    "spx_batch_destroy": (C.c_int, [_VP]),
    "spx_batch_offset": (C.c_int64, [_VP, C.c_int32]),
    "spx_batch_energy_offset": (C.c_int32, [_VP, C.c_int32]),
    "spx_batch_grid": (C.c_int32, [_VP]),
    "spx_batch_run": (C.c_int, [_VP, _VP, _VP, _VP]),
    "spx_batch_results": (C.c_int, [_VP, C.POINTER(spx_batch_stats), C.POINTER(C.c_double), _VP]),
    "spx_rk_step_store": (C.c_int, [_VP, _VP, C.c_double, _VP, _VP, _VP, _VP]),
    "spx_rk_step_store_ex": (C.c_int, [_VP, _VP, C.c_double, _VP, _VP, _VP, C.c_int32, _VP]),
    "spx_rk_status": (C.c_int, [C.POINTER(C.c_int32), _VP]),
    "spx_vjp_param": (C.c_int, [_VP, _VP, _VP, _VP, C.POINTER(C.c_double), _VP, C.c_size_t, _VP]),
    "spx_vjp_param_ex": (C.c_int, [_VP, _VP, _VP, _VP, C.POINTER(C.c_double), _VP, C.c_size_t, C.c_int32, _VP]),
    "spx_lincomb": (C.c_int, [C.c_int64, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_double), _VP, _VP]),
    "spx_param_dots": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "spx_probe_fp64": (C.c_int, [_VP, C.c_int, C.c_int, _VP]),
}

_lib = None


def lib():
    """Load the shared library once; raise loudly when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SpectraxLibraryError(
            f"{LIB_PATH} not found: build it with `python -m spectrax_gb300.build` "
            "(this package has no CPU fallback)")
    try:
        L = C.CDLL(LIB_PATH)
    except OSError as e:
        raise SpectraxLibraryError(f"cannot load {LIB_PATH}: {e}") from e
    for name, (res, args) in _PROTOS.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def exported(name: str) -> bool:
    return hasattr(lib(), name)


def check(rc: int, what: str = ""):
    if rc != SPX_OK:
        msg = lib().spx_last_error().decode()
        raise SpectraxError(rc, f"{what}: {msg}" if what else msg)
    return rc
