"""numpy mirrors of the POD structs in include/cmtj_gpu.h and the ctypes
prototypes of libcmtj_gpu.so.

Every struct is declared field by field in the header's order with C
alignment (``align=True``); ``check_layout`` compares the numpy item sizes
with the sizes the compiled library reports, so a header change that is not
mirrored here fails at load time instead of corrupting memory.
"""
import ctypes
import os

import numpy as np

ABI_VERSION = 2  # CMTJ_ABI_VERSION
MAX_LAYERS = 8
ALPHA_MAX_LEN = 8388608  # CMTJ_ALPHA_MAX_LEN: samples per alpha-noise buffer
MAX_LAYERS_F32 = 4
NUM_SLOTS = 30
ENERGY_COLS = 29

# enum cmtj_update_type (drivers.hpp:18-29)
DRV_CONSTANT, DRV_PULSE, DRV_SINE, DRV_STEP, DRV_POSINE, DRV_HALFSINE = 0, 1, 2, 3, 4, 5
DRV_TRAPEZOID, DRV_GAUSSIMPULSE, DRV_GAUSSSTEP, DRV_TABLE = 6, 7, 8, 100

# enum cmtj_driver_slot (junction.hpp:147-163)
SLOT_TEMPERATURE = 0
SLOT_IEC_TOP, SLOT_IEC_BOTTOM, SLOT_IECQ_TOP, SLOT_IECQ_BOTTOM = 1, 2, 3, 4
SLOT_CURRENT, SLOT_ANIS, SLOT_ANIS2 = 5, 6, 7
SLOT_FL, SLOT_DL, SLOT_FL2, SLOT_DL2 = 8, 9, 10, 11
SLOT_HEXT, SLOT_HOE, SLOT_HDMI, SLOT_HRES, SLOT_IDMI_TOP, SLOT_IDMI_BOTTOM = 12, 15, 18, 21, 24, 27

REF_NONE, REF_FIXED, REF_TOP, REF_BOTTOM = 0, 1, 2, 3
EULER_HEUN, RK4, DORMAND_PRINCE, HEUN = 0, 1, 2, 3
MR_NONE, MR_CLASSIC, MR_STRIP = 0, 1, 2

CMTJ_OK, CMTJ_ERR_ARG, CMTJ_ERR_CUDA, CMTJ_ERR_RUNTIME, CMTJ_ERR_LIMIT = 0, -1, -2, -3, -4
STATUS_OK, STATUS_NAN, STATUS_NOT_RUN, STATUS_BAD_INPUT, STATUS_DP_STALL, STATUS_LIMIT = 0, 1, 2, 3, 4, 5

DRIVER_DTYPE = np.dtype(
    [("update", "<i4"), ("reserved", "<i4"), ("table_offset", "<i8"),
     ("constantValue", "<f8"), ("amplitude", "<f8"), ("frequency", "<f8"), ("phase", "<f8"),
     ("period", "<f8"), ("cycle", "<f8"), ("timeStart", "<f8"), ("timeStop", "<f8"),
     ("edgeTime", "<f8"), ("steadyTime", "<f8")], align=True)

ADAPTIVE_DTYPE = np.dtype(
    [("abs_tol", "<f8"), ("rel_tol", "<f8"), ("max_factor", "<f8"), ("min_factor", "<f8"),
     ("safety_factor", "<f8"), ("ki", "<f8"), ("kp", "<f8"), ("kd", "<f8"), ("prev_error_ratio", "<f8"),
     ("integral_error", "<f8"), ("use_pid_control", "<i4"), ("reserved", "<i4")], align=True)

LAYER_DTYPE = np.dtype(
    [("mag", "<f8", 3), ("anis", "<f8", 3), ("ref", "<f8", 3), ("ref2", "<f8", 3),
     ("demag", "<f8", 9), ("dipole_top", "<f8", 9), ("dipole_bottom", "<f8", 9),
     ("Ms", "<f8"), ("thickness", "<f8"), ("cellSurface", "<f8"), ("cellVolume", "<f8"),
     ("damping", "<f8"), ("fieldLikeTorque", "<f8"), ("dampingLikeTorque", "<f8"),
     ("slonczewski", "<f8"), ("beta", "<f8"), ("kappa", "<f8"), ("spinPolarisation", "<f8"),
     ("referenceType", "<i4"), ("includeSTT", "<i4"), ("includeSOT", "<i4"), ("dynamicSOT", "<i4"),
     ("alternativeSTT", "<i4"), ("temperatureSet", "<i4"),
     ("seed_lo", "<u4"), ("seed_hi", "<u4"), ("noise_step", "<u8"),
     ("drv", DRIVER_DTYPE, NUM_SLOTS), ("adaptive", ADAPTIVE_DTYPE),
     ("conv_term", "<f8"), ("stoch_conv", "<f8"), ("ms_over_mu0", "<f8"), ("zero_terms", "<u4"),
     ("reserved2", "<u4"), ("alpha_buf", "<u8"), ("alpha_scale", "<f8"), ("alpha_len", "<u4"),
     ("alpha_axis", "<i4")], align=True)

# cmtj_alpha_noise_t: one buffer row of BufferedAlphaNoise::fillBuffer.
ALPHA_NOISE_DTYPE = np.dtype(
    [("alpha", "<f8"), ("std", "<f8"), ("seed_lo", "<u4"), ("seed_hi", "<u4"), ("counter", "<u8"),
     ("component", "<i4"), ("reserved", "<i4")], align=True)

ZERO_DIPOLE, ZERO_IDMI, ZERO_K2, ZERO_J2 = 1, 2, 4, 8

JUNCTION_DTYPE = np.dtype(
    [("n_layers", "<i4"), ("mr_mode", "<i4"), ("layer_offset", "<i4"), ("reserved", "<i4"),
     ("Rp", "<f8"), ("Rap", "<f8"),
     ("Rx0", "<f8", MAX_LAYERS), ("Ry0", "<f8", MAX_LAYERS), ("AMR_X", "<f8", MAX_LAYERS),
     ("AMR_Y", "<f8", MAX_LAYERS), ("SMR_X", "<f8", MAX_LAYERS), ("SMR_Y", "<f8", MAX_LAYERS),
     ("AHE", "<f8", MAX_LAYERS)], align=True)

CONSTANTS_DTYPE = np.dtype(
    [("mu0", "<f8"), ("gyro", "<f8"), ("TtoAm", "<f8"), ("hbar", "<f8"), ("echarge", "<f8"),
     ("kB", "<f8")], align=True)

SIM_PARAMS_DTYPE = np.dtype(
    [("time_step", "<f8"), ("total_iterations", "<u4"), ("write_every", "<u4"), ("n_log", "<u4"),
     ("solver", "<i4"), ("calculate_energies", "<i4"), ("log_width", "<i4"),
     ("c", CONSTANTS_DTYPE), ("total_time", "<f8"), ("write_frequency", "<f8"), ("max_attempts", "<u8"),
     ("max_layers", "<i4"), ("lanes_per_layer", "<i4"), ("arithmetic", "<i4"), ("reserved", "<i4")],
    align=True)

# enum cmtj_arithmetic
ARITH_REFERENCE, ARITH_FUSED = 0, 1
ARITHMETIC = {"reference": ARITH_REFERENCE, "fused": ARITH_FUSED}

# Order of cmtj_struct_sizes() output.
STRUCT_SIZES = {
    "cmtj_driver_t": DRIVER_DTYPE.itemsize,
    "cmtj_layer_t": LAYER_DTYPE.itemsize,
    "cmtj_junction_t": JUNCTION_DTYPE.itemsize,
    "cmtj_constants_t": CONSTANTS_DTYPE.itemsize,
    "cmtj_sim_params_t": SIM_PARAMS_DTYPE.itemsize,
}


def log_width(n_layers, calculate_energies):
    """Doubles per log row (cmtj_log_width in include/cmtj_gpu.h)."""
    return n_layers * (ENERGY_COLS if calculate_energies else 3) + 4


# --------------------------------------------------------------------------
# Shared library loading.
# --------------------------------------------------------------------------
PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libcmtj_gpu.so")

_P = ctypes.c_void_p
_I32 = ctypes.c_int32

# name -> (restype, argtypes); every symbol declared in include/*.h.
PROTOTYPES = {
    "cmtj_abi_version": (ctypes.c_int, []),
    "cmtj_last_error": (ctypes.c_char_p, []),
    "cmtj_device_info": (ctypes.c_int, [ctypes.c_int, _P, _P, _P]),
    "cmtj_log_width": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "cmtj_struct_sizes": (ctypes.c_int, [_P, _I32]),
    "cmtj_run_simulation_f64": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P, _P, _P]),
    "cmtj_batch_run_f32": (ctypes.c_int, [_P, _P, _P, _P, _I32, _I32, _I32, _P, _P, _P, _I32, _P]),
    "cmtj_batch_variant_f32": (ctypes.c_int, [_I32, _I32, _I32]),
    "cmtj_batch_bounds_f32": (ctypes.c_int, [_I32, _I32, _I32, _P, _I32]),
    "cmtj_batch_run_f32_noalloc": (ctypes.c_int, [_P, _P, _P, _P, _I32, _I32, _I32, _P, _P, _I32, _I32, _P]),
    "cmtj_spectrum_f32": (ctypes.c_int, [_P, ctypes.c_int64, _I32, _I32, _I32, _I32, _I32, _P, _P]),
    "cmtj_run_stack_f64": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P, _P, _P, _P, _P, _I32, _I32, _P, _P]),
    "cmtj_run_group_f64": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P, _P, _P, _P, _I32, _P, _P]),
    "cmtj_alpha_noise_scratch_bytes": (ctypes.c_size_t, [ctypes.c_uint32]),
    "cmtj_alpha_noise_f32": (ctypes.c_int, [_P, _I32, ctypes.c_uint32, _P, _P, _P, ctypes.c_size_t, _P]),
}

_lib = None


class LibraryMissing(RuntimeError):
    pass


def load(path=None):
    """Load libcmtj_gpu.so (built by __graft_entry__.build()).  Raises
    LibraryMissing, never falls back to another implementation."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise LibraryMissing(
            "libcmtj_gpu.so is not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"`" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    check_layout(lib)
    if path is None:
        _lib = lib
    return lib


def check_layout(lib):
    from .batch import STRUCT_SIZES_F32
    from .reservoir import GROUP_DTYPE, PAIR_DTYPE
    from .stack import STACK_DTYPE
    sizes = dict(STRUCT_SIZES)
    sizes.update(STRUCT_SIZES_F32)
    sizes["cmtj_stack_t"] = STACK_DTYPE.itemsize
    sizes["cmtj_group_t"] = GROUP_DTYPE.itemsize
    sizes["cmtj_pair_t"] = PAIR_DTYPE.itemsize
    sizes["cmtj_alpha_noise_t"] = ALPHA_NOISE_DTYPE.itemsize
    n = len(sizes)
    buf = (ctypes.c_int32 * n)()
    lib.cmtj_struct_sizes(ctypes.cast(buf, _P), n)
    for (name, size), got in zip(sizes.items(), buf):
        if size != got:
            raise RuntimeError("ABI mismatch for %s: numpy %d bytes, library %d bytes" % (name, size, got))
    if lib.cmtj_abi_version() != ABI_VERSION:
        raise RuntimeError("unexpected libcmtj_gpu ABI version %d" % lib.cmtj_abi_version())


def last_error(lib=None):
    lib = lib or load()
    msg = lib.cmtj_last_error()
    return msg.decode() if msg else ""


def check(rc, lib=None):
    """Map a C-ABI return code to the reference's Python exception types."""
    if rc == CMTJ_OK:
        return
    msg = last_error(lib)
    if rc == CMTJ_ERR_ARG:
        raise ValueError(msg)
    if rc == CMTJ_ERR_LIMIT:
        raise ValueError(msg)
    raise RuntimeError(msg)
