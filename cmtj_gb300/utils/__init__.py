"""`cmtj.utils` names used with the time loop (cmtj/utils/__init__.py):
FieldScan, the resistance helpers and compute_sd.  The procedures live in
cmtj_gb300.utils.procedures, as in the reference."""
from ..procedures import (FieldScan, ResistanceParameters, calculate_resistance_parallel,  # noqa: F401
                          calculate_resistance_series, compute_resistance, compute_sd)

__all__ = ["FieldScan", "ResistanceParameters", "calculate_resistance_parallel", "calculate_resistance_series",
           "compute_resistance", "compute_sd"]
