"""CPU: the C-ABI library loads and exports every function include/*.h declares.

No compute call is made here (no GPU in this environment)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(spx_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_library_exports_header():
    from spectrax_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from spectrax_gb300 import build
        build.build()
    L = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert len(declared_functions()) >= 10


def test_version_and_errors_without_gpu():
    from spectrax_gb300 import _lib
    L = _lib.lib()
    assert b"sm_103a" in L.spx_version()
    # argument validation happens before any CUDA call
    assert L.spx_rhs(None, None, None, None, 0, None) == _lib.SPX_E_ARG
    assert b"null" in L.spx_last_error()


def test_problem_struct_layout():
    from spectrax_gb300 import _lib
    # 10 int32 + 5 doubles + 8 + 8 + 24 + 24 doubles
    assert ctypes.sizeof(_lib.spx_problem) == 40 + 5 * 8 + 64 * 8


def test_no_cpu_fallback_in_product():
    # nothing under the package imports the oracle
    pkg = os.path.join(ROOT, "spectrax_gb300")
    for dp, _, fns in os.walk(pkg):
        for fn in fns:
            if fn.endswith(".py"):
                src = open(os.path.join(dp, fn)).read()
                assert "oracle" not in re.findall(r"^\s*(?:from|import)\s+(\w+)", src, flags=re.M), fn


@pytest.mark.parametrize("nx,cut,mode,expect", [
    (129, 43, 0, 144),   # default: an Nx with a prime factor >= 5 takes a 2^a 3^b grid (4*4*3*3)
    (127, 42, 0, 128),
    (97, 32, 0, 108),
    (251, 83, 0, 256),
    (65, 21, 0, 64),
    (33, 11, 0, 36),
    (17, 5, 0, 16),
    (151, 50, 0, 192),
    (96, 32, 0, 96),     # Nx = 2^a 3^b keeps its own grid
    (129, 43, 2, 136),   # least FP64 count, no extra Stockham stage
    (65, 21, 2, 64),
    (33, 11, 2, 33),
    (129, 43, 1, 129),   # always Nx
    (97, 32, 1, 97),
    (64, 30, 0, 64),     # 3 cut > Nx: the Nx-point product folds more than one term, keep Nx
    (64, 30, 2, 64),
    (127, 43, 0, 127),
])
def test_product_grid_choice_without_gpu(nx, cut, mode, expect):
    # host-side choice of the 1D1V stepper's product grid (no device call)
    from spectrax_gb300 import _lib
    assert _lib.lib().spx_product_grid_for(nx, cut, mode) == expect


def test_product_grid_choice_rejects_bad_arguments():
    from spectrax_gb300 import _lib
    L = _lib.lib()
    assert L.spx_product_grid_for(0, 1, 0) == _lib.SPX_E_ARG
    assert L.spx_product_grid_for(33, 11, 3) == _lib.SPX_E_ARG


def test_product_grid_mode_setter_without_gpu():
    from spectrax_gb300 import vector_field
    with pytest.raises(ValueError):
        vector_field.set_product_grid("bogus")
    try:
        vector_field.set_product_grid("fp64")
        assert vector_field.get_product_grid() == "fp64"
    finally:
        vector_field.set_product_grid("auto")
    assert vector_field.get_product_grid() == "auto"


def test_product_grid_rule_properties_without_gpu():
    # for every Nx up to 300 and the 2/3 cut: the default grid is Nx itself (Nx of
    # the form 2^a 3^b, or a cut whose Nx-point product folds more than one term)
    # or a length M = 2^a 3^b with 3 cut + 1 <= M <= 2 Nx
    from spectrax_gb300 import _lib
    L = _lib.lib()

    def smooth(m):
        for p in (2, 3):
            while m % p == 0:
                m //= p
        return m == 1

    for nx in range(1, 301):
        cut = nx // 3
        m = L.spx_product_grid_for(nx, cut, 0)
        if m == nx:
            assert smooth(nx) or nx < 8 or cut < 1 or 3 * cut > nx or not any(
                smooth(k) for k in range(3 * cut + 1, 2 * nx + 1)), (nx, m)
        else:
            assert not smooth(nx) and smooth(m) and 3 * cut + 1 <= m <= 2 * nx, (nx, cut, m)
