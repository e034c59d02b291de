"""GPU execution of lowered junctions through libcmtj_gpu.so.

Device memory and streams come from PyTorch; the compute is the library's
CUDA kernels.  There is no CPU path: without a CUDA device or without the
built library every entry point raises.
"""
import ctypes

import numpy as np

from . import _abi
from ._lower import RunPlan, apply_results, lower, plan_run  # noqa: F401

_torch = None


def torch():
    global _torch
    if _torch is None:
        import torch as t
        _torch = t
    return _torch


def require_gpu():
    t = torch()
    if not t.cuda.is_available():
        raise RuntimeError("cmtj_gb300 runs on a CUDA GPU (sm_103a); no CUDA device is available")
    return _abi.load()


def to_device(arr):
    """numpy array -> device tensor holding the same bytes."""
    t = torch()
    flat = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
    return t.from_numpy(flat.copy()).to("cuda", non_blocking=False)


def ptr(tensor):
    return ctypes.c_void_p(tensor.data_ptr()) if tensor is not None else None


def stream_ptr(stream=None):
    t = torch()
    s = stream if stream is not None else t.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def device_layers(lowered, stream=None):
    """Upload the layer records of a lowered run.  Layers with buffered
    alpha noise first get this run's buffers, filled on the GPU
    (cmtj_alpha_noise_f32) and referenced from their records.  Returns
    (layers tensor, buffers tensor or None); keep both until the run ends."""
    if lowered.alpha_specs is None:
        return to_device(lowered.layers), None
    from .noise import device_buffers
    n = int(lowered.layers[lowered.alpha_layers[0]]["alpha_len"])
    bufs = device_buffers(lowered.alpha_specs, n, stream=stream)
    from ._lower import with_alpha_buffers
    return to_device(with_alpha_buffers(lowered, bufs.data_ptr())), bufs


# fixed-step batches below this many layer-steps run the library's own
# lane pick: trial launches would cost more than they could save
TUNE_F64_MIN_LAYER_STEPS = 2e7


def tuned_f64_params(lowered, d_j, d_l, d_tab, stream=None):
    """The launch parameters of a lowered FP64 batch, with the lane layout
    (threads per junction) the run-time autotuner chose for this kind of
    batch (cmtj_gb300.autotune; the layout changes no result)."""
    from . import autotune
    p = lowered.params
    solver = int(p["solver"][0])
    n = len(lowered.junctions)
    work = float(n) * float(p["total_iterations"][0]) * float(lowered.junctions["n_layers"].mean() if n else 0)
    if (not autotune.enabled() or solver == _abi.DORMAND_PRINCE or int(p["lanes_per_layer"][0]) != 0
            or work < TUNE_F64_MIN_LAYER_STEPS):
        return p
    key = autotune.f64_key(int(p["max_layers"][0]), solver, n)
    c = autotune.lookup(key)
    if c is None:
        t = torch()
        c = autotune.tune_f64(lowered, d_j, d_l, d_tab, stream if stream is not None else t.cuda.current_stream())
        if c is None:
            return p
        autotune.store(key, c)
    p = p.copy()
    p["lanes_per_layer"] = int(c["lanes"])
    return p


def run_lowered_f64(lowered, stream=None):
    """Run a lowered batch on the FP64 plain form; returns host arrays
    (log [n][n_log][width], status [n*2], updated layers)."""
    lib = require_gpu()
    t = torch()
    n = len(lowered.junctions)
    p = lowered.params
    n_log = int(p["n_log"][0])
    width = lowered.log_width
    d_j = to_device(lowered.junctions)
    d_l, alpha = device_layers(lowered, stream)
    d_tab = to_device(lowered.tables) if lowered.tables is not None else None
    p = tuned_f64_params(lowered, d_j, d_l, d_tab, stream)
    d_log = t.empty((n, max(n_log, 1), width), dtype=t.float64, device="cuda")
    d_status = t.zeros(2 * n, dtype=t.int32, device="cuda")
    rc = lib.cmtj_run_simulation_f64(ptr(d_j), n, ptr(d_l), ptr(d_tab), p.ctypes.data, ptr(d_log), ptr(d_status),
                                     stream_ptr(stream))
    _abi.check(rc, lib)
    log = d_log.cpu().numpy()
    status = d_status.cpu().numpy().view(np.uint32)
    layers = d_l.cpu().numpy().view(_abi.LAYER_DTYPE).copy()
    del alpha
    return log, status, layers


def run_junctions(junctions, plan, solver, calculate_energies=False, arithmetic="reference"):
    """Junction::runSimulation for a list of junctions sharing one plan
    (each junction keeps its own layers, drivers and log).  arithmetic:
    "reference" (the reference's bits) or "fused" (cmtj_arithmetic)."""
    plan = plan.for_solver(solver)
    lowered = lower(junctions, plan, solver, calculate_energies, arithmetic)
    require_gpu()
    log, status, layers = run_lowered_f64(lowered)
    lowered.layers = layers
    apply_results(junctions, lowered, log, status, plan)
    return lowered
