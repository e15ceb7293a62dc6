"""nhqg_gb300 -- GB300 (sm_103a) engine for the NHQG ARS(2,2,2) time step.

Drop-in for the time-step path of ksr-ocean/NHQG: ``NHQGConfig``,
``make_grid``, ``Grid``, ``State``, ``imex_step``, ``run`` and the per-operator
functions in ``nhqg_gb300.solver`` / ``nhqg_gb300.spectral`` keep the
reference's names and argument meaning (nhqg/__init__.py:3-5).  The compute
path is the C-ABI library ``libnhqg_gpu.so`` (include/nhqg_gpu.h); building it
needs nvcc, running it needs a CUDA device.
"""

from ._native import build  # noqa: F401
from .config import NHQGConfig  # noqa: F401
from .grid import Grid, make_grid  # noqa: F401
from .initial import theta_perturbation_state  # noqa: F401


def __getattr__(name):
    # torch-backed API loads lazily so that make_grid works without CUDA
    if name in ("State", "imex_step", "run", "step_inplace", "sanitize_state", "to_device", "to_host",
                "make_initial_state"):
        from . import solver
        return getattr(solver, name)
    if name == "compute_diagnostics":
        from . import diagnostics
        return diagnostics.compute_diagnostics
    raise AttributeError(name)
