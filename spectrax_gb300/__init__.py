"""spectrax_gb300 — GB300 (sm_103a) Hermite-Fourier Vlasov-Maxwell right-hand side and steppers.

The product path is the in-tree CUDA library ``libspectrax_gb300.so`` (C ABI in
``include/spectrax_gb300.h``), called through ctypes with torch CUDA tensors.
There is no CPU fallback: without the library every compute entry point raises.
"""
from ._lib import SpectraxError, SpectraxLibraryError, spx_problem  # noqa: F401
from .params import (Dopri8, ImplicitMidpoint, get_mask_mode, initial_state,  # noqa: F401
                     initialize_simulation_parameters, load_parameters, make_args, make_problem,
                     mask_cutoff, problem_from_args, problem_from_params, set_mask_mode)

__version__ = "0.1.0"


def __getattr__(name):
    # torch-dependent modules load lazily so that `import spectrax_gb300` stays cheap
    if name in ("ode_system", "rhs", "Plan", "get_plan", "plan_for_params"):
        from . import vector_field as _rhs
        return getattr(_rhs, name)
    raise AttributeError(name)
