"""ctypes wrapper of the oracle (oracle/_build/libcmtj_oracle.so) for the
tests, the smoke check and bench.py's CPU baseline.  It runs the same packed
inputs that cmtj_gb300 lowers for the GPU, on the CPU restatement."""
import ctypes
import os
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import cmtj_gb300  # noqa: E402
from cmtj_gb300 import _abi  # noqa: E402
from cmtj_gb300._lower import apply_results, lower, plan_run  # noqa: E402

_lib = None


def oracle_lib():
    global _lib
    if _lib is None:
        from oracle.build import build_oracle
        path = build_oracle()
        lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        lib.oracle_run_simulation.restype = ctypes.c_int
        lib.oracle_run_simulation.argtypes = [P, ctypes.c_int32, P, P, P, P, P, ctypes.c_int32]
        lib.oracle_count_flops.restype = ctypes.c_int
        lib.oracle_count_flops.argtypes = [P, P, P, P, P, P]
        lib.oracle_gaussian3.restype = None
        lib.oracle_gaussian3.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, P]
        lib.oracle_log_width.restype = ctypes.c_int
        lib.oracle_log_width.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.oracle_run_group.restype = ctypes.c_int
        lib.oracle_run_group.argtypes = [P, P, P, P, ctypes.c_int32, P, P, P, P, P]
        lib.oracle_alpha_noise.restype = ctypes.c_int
        lib.oracle_alpha_noise.argtypes = [P, ctypes.c_int32, ctypes.c_uint32, P, P, ctypes.c_int32]
        _lib = lib
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def alpha_buffers(specs, n, white=None, threads=8):
    """The oracle's restatement of BufferedAlphaNoise::fillBuffer for the
    cmtj_alpha_noise_t rows `specs` ([rows, n] float32)."""
    lib = oracle_lib()
    out = np.zeros((len(specs), n), dtype=np.float32)
    if white is not None:
        white = np.ascontiguousarray(white, dtype=np.float32)
    rc = lib.oracle_alpha_noise(_p(specs), len(specs), n, _p(white), _p(out), threads)
    assert rc == 0, rc
    return out


# Buffers that the next oracle run uses instead of its own restatement's
# (a test sets it to run the oracle on the GPU's alpha-noise samples).
ALPHA_OVERRIDE = None


def run_lowered(lowered, threads=1):
    """Run a Lowered batch on the oracle; returns (log, status) and updates
    lowered.layers[...]['mag'] in place.  Layers with buffered alpha noise
    read buffers from the oracle's restatement (or ALPHA_OVERRIDE)."""
    global ALPHA_OVERRIDE
    from cmtj_gb300._lower import with_alpha_buffers
    lib = oracle_lib()
    n = len(lowered.junctions)
    n_log = int(lowered.params["n_log"][0])
    log = np.zeros((n, max(n_log, 1), lowered.log_width), dtype=np.float64)
    status = np.zeros(2 * n, dtype=np.uint32)
    layers, bufs = lowered.layers, None
    if lowered.alpha_specs is not None:
        alen = int(layers[lowered.alpha_layers[0]]["alpha_len"])
        bufs = ALPHA_OVERRIDE if ALPHA_OVERRIDE is not None else alpha_buffers(lowered.alpha_specs, alen)
        ALPHA_OVERRIDE = None
        bufs = np.ascontiguousarray(bufs, dtype=np.float32)
        assert bufs.shape == (len(lowered.alpha_specs), alen), bufs.shape
        layers = with_alpha_buffers(lowered, bufs.ctypes.data)
    rc = lib.oracle_run_simulation(_p(lowered.junctions), n, _p(layers), _p(lowered.tables),
                                   _p(lowered.params), _p(log), _p(status), threads)
    assert rc == 0, rc
    if layers is not lowered.layers:
        lowered.layers["mag"] = layers["mag"]
    return log, status


def run_oracle(junctions, totalTime, timeStep=1e-13, writeFrequency=1e-11, verbose=False,
               calculateEnergies=False, solverMode=cmtj_gb300.SolverMode.RK4, threads=1):
    solver = junctions[0].getSolver(solverMode)
    plan = plan_run(totalTime, timeStep, writeFrequency, solver=solver)
    lowered = lower(junctions, plan, solver, calculateEnergies)
    log, status = run_lowered(lowered, threads)
    apply_results(junctions, lowered, log, status, plan)
    return lowered


class OracleJunction(cmtj_gb300.Junction):
    """A cmtj_gb300.Junction whose runSimulation runs on the oracle."""

    def runSimulation(self, totalTime, timeStep=1e-13, writeFrequency=1e-11, verbose=False,
                      calculateEnergies=False, solverMode=cmtj_gb300.SolverMode.RK4):
        run_oracle([self], totalTime, timeStep, writeFrequency, verbose, calculateEnergies, solverMode)


def oracle_module():
    """A stand-in for the `cmtj` module whose Junction runs on the oracle."""
    m = types.SimpleNamespace(**{k: getattr(cmtj_gb300, k) for k in dir(cmtj_gb300) if not k.startswith("__")})
    m.Junction = OracleJunction
    from cmtj_gb300 import reservoir
    m.reservoir = types.SimpleNamespace(**{k: getattr(reservoir, k) for k in dir(reservoir)
                                           if not k.startswith("__")})
    m.reservoir.GroupInteraction = OracleGroupInteraction
    return m


def count_flops(junction, totalTime, timeStep, writeFrequency, solverMode=cmtj_gb300.SolverMode.RK4):
    """[adds, muls, divs, sqrts, transcendentals] of one run of `junction`
    on the counting scalar type."""
    lib = oracle_lib()
    plan = plan_run(totalTime, timeStep, writeFrequency)
    solver = junction.getSolver(solverMode)
    lowered = lower([junction], plan, solver, False)
    log = np.zeros((max(plan.n_log, 1), lowered.log_width), dtype=np.float64)
    out = np.zeros(5, dtype=np.uint64)
    lib.oracle_count_flops(_p(lowered.junctions), _p(lowered.layers), _p(lowered.tables), _p(lowered.params),
                           _p(log), _p(out))
    return out


def gaussian3(seed_lo, seed_hi, step):
    g = np.zeros(3, dtype=np.float64)
    oracle_lib().oracle_gaussian3(seed_lo, seed_hi, step, _p(g))
    return g


def run_groups_oracle(groups, totalTime, timeStep=1e-13, writeFrequency=1e-11):
    """cmtj_gb300.reservoir.run_groups with the oracle in place of the GPU
    (same host preparation, same records)."""
    from cmtj_gb300 import reservoir
    plan, junctions, low, grec, tops, pairs = reservoir.prepare_groups(groups, totalTime, timeStep, writeFrequency)
    from cmtj_gb300._lower import with_alpha_buffers
    n = len(junctions)
    log = np.zeros((n, max(plan.n_log, 1), low.log_width), dtype=np.float64)
    status = np.zeros(2 * n, dtype=np.uint32)
    layers, bufs = low.layers, None
    if low.alpha_specs is not None:
        bufs = alpha_buffers(low.alpha_specs, int(layers[low.alpha_layers[0]]["alpha_len"]))
        layers = with_alpha_buffers(low, bufs.ctypes.data)
    rc = oracle_lib().oracle_run_group(_p(low.junctions), _p(layers), _p(low.tables), _p(grec), len(groups),
                                       _p(pairs), _p(tops), _p(low.params), _p(log), _p(status))
    assert rc == 0, rc
    if layers is not low.layers:
        low.layers["mag"] = layers["mag"]
        for k in range(3):
            low.layers["drv"][:, _abi.SLOT_HRES + k] = layers["drv"][:, _abi.SLOT_HRES + k]
    apply_results(junctions, low, log, status, plan)
    reservoir.finish_groups(groups, junctions, low, tops)


class OracleGroupInteraction(cmtj_gb300.reservoir.GroupInteraction):
    """A GroupInteraction whose runSimulation runs on the oracle."""

    def runSimulation(self, totalTime, timeStep=1e-13, writeFrequency=1e-11):
        run_groups_oracle([self], totalTime, timeStep, writeFrequency)
