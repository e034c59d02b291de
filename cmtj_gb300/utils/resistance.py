"""`cmtj.utils.resistance` (cmtj/utils/resistance.py): the helpers the
procedures use, implemented in cmtj_gb300.procedures."""
from ..procedures import (calculate_resistance_parallel, calculate_resistance_series,  # noqa: F401
                          compute_resistance, compute_sd)
