"""gturbo_gb300: GB300-native (sm_103a, FP64) time-stepping hot path of the Gturbo 2D
alpha-turbulence pseudo-spectral solver, behind the C-ABI of ``include/gturbo.h``."""
from .params import Params, config, famp_for_injection, read_params_dat  # noqa: F401

__all__ = ["Params", "config", "famp_for_injection", "read_params_dat", "Solver", "spec"]


def __getattr__(name):
    # the solver needs torch and the CUDA library; import it lazily
    if name in ("Solver", "spec"):
        from . import solver
        return getattr(solver, name)
    raise AttributeError(name)
