"""`cmtj.utils.procedures` (cmtj/utils/procedures.py): PIMM_procedure,
VSD_procedure and their helpers, implemented in cmtj_gb300.procedures."""
from ..procedures import (FieldScan, PIMM_procedure, ResistanceParameters, VSD_procedure,  # noqa: F401
                          calculate_resistance_parallel, calculate_resistance_series, compute_spectrum_strip)
