"""cmtj_gb300 -- GB300-native macrospin solver with the `cmtj` Python API.

`import cmtj_gb300 as cmtj` gives the names the reference's `_cmtj` module
exports (python/cmtj.cpp:35-356): CVector, Layer, Junction, ScalarDriver,
AxialDriver, NullDriver, the driver aliases, the enums (with their values
exported at module level, as pybind11's export_values does), and the
submodules `stack` and `constants`.  Junction.runSimulation runs on the GPU.

Batched and serving entry points beyond the reference API live in
`cmtj_gb300.batch` and `cmtj_gb300.serving`.
"""
from . import constants
from .core import (AdaptiveIntegrationParams, AxialDriver, Axis, CVector, Junction, Layer, NullDriver, Reference,
                   ScalarDriver, SolverMode, UpdateType, c_dot, constantDriver, gaussianImpulseDriver,
                   gaussianStepDriver, posSineDriver, pulseDriver, sineDriver, stepDriver, trapezoidDriver)

__version__ = "0.1.0"

# pybind11 export_values(): enum members are module attributes too.  As in
# the reference, Reference.none is the module-level `none`.
for _enum in (Axis, Reference, SolverMode, UpdateType):
    for _m in _enum:
        globals()[_m.name] = _m
del _enum, _m

__all__ = [
    "AdaptiveIntegrationParams", "AxialDriver", "Axis", "CVector", "Junction", "Layer", "NullDriver", "Reference",
    "ScalarDriver", "SolverMode", "UpdateType", "c_dot", "constantDriver", "gaussianImpulseDriver",
    "gaussianStepDriver", "posSineDriver", "pulseDriver", "sineDriver", "stepDriver", "trapezoidDriver",
    "constants", "stack", "reservoir", "noise",
    "xaxis", "yaxis", "zaxis", "all", "none", "fixed", "top", "bottom", "RK4", "Heun", "EulerHeun",
    "DormandPrince", "constant", "pulse", "sine", "step", "posine", "halfsine", "trapezoid", "gaussimpulse",
    "gaussstep", "custom",
]


def __getattr__(name):
    # submodules bound as attributes of the reference's module (cmtj.stack,
    # cmtj.reservoir, cmtj.noise), imported on first use
    if name in ("stack", "reservoir", "noise"):
        import importlib
        return importlib.import_module(__name__ + "." + name)
    raise AttributeError(name)
