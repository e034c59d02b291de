"""`cmtj.utils` names used with the time loop (cmtj/utils/__init__.py):
FieldScan, the resistance helpers, compute_sd and Filters.  The procedures,
FieldScan, the filters and distribute also live in their own submodules
(procedures, linear, filters, parallel), as in the reference."""
from ..procedures import (FieldScan, ResistanceParameters, calculate_resistance_parallel,  # noqa: F401
                          calculate_resistance_series, compute_resistance, compute_sd)
from .filters import Filters  # noqa: F401

__all__ = ["FieldScan", "Filters", "ResistanceParameters", "calculate_resistance_parallel", "calculate_resistance_series",
           "compute_resistance", "compute_sd"]
