"""GB300-native (sm_103a) hot path of the AMReX/GRTeclyn axion-string code.

The CUDA library ``libaxs_gb300.so`` (C ABI: include/axs.h) implements the
per-level complex-scalar RHS with its classic-RK4 step, the plaquette-winding
string finder and the energy / velocity / xi reductions. This package is the
Python host side: it allocates device memory through torch and calls the
library; it computes nothing itself.
"""
from . import _lib
from ._build import build
from ._lib import AxsError
from .background import (Background, plaquette_count_for_target_xi, xi_from_comoving_length,
                         xi_from_plaquette_count)
from .ensemble import Ensemble
from .level import (AxionStringsLevel, Diagnostics, PeriodicLevel, eval_rhs, fab, fill_periodic_ghosts, lincomb,
                    new_fab, rk4_combine, valid)

__all__ = [
    "AxionStringsLevel", "AxsError", "Background", "Diagnostics", "Ensemble", "PeriodicLevel", "build", "eval_rhs", "fab",
    "fill_periodic_ghosts", "lincomb", "new_fab", "plaquette_count_for_target_xi", "rk4_combine", "valid",
    "xi_from_comoving_length", "xi_from_plaquette_count",
]


def lib():
    """The loaded libaxs_gb300.so (ctypes handle); raises if it cannot be loaded."""
    return _lib.lib()
