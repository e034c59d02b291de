"""Run-time launch tuning.

The launch choices below change no result (a junction's arithmetic does
not depend on them: the log tile only sets when staged samples are
written, the resident-CTA bound only how many registers a thread may use,
the lane layout is proven bit-identical), only the speed.  Each is chosen
the first time a kind of launch is met, by timing short trial launches of
the real batch on scratch state, and kept in a table:

* FP32 batched form, per partition (layer count, solver, kernel variant,
  log channels, weighted reduction, size class): the log tile (samples
  staged per thread in shared memory before one bulk store) and the
  resident-CTA bound of the variant (two instantiations are compiled:
  cmtj_batch_bounds_f32).
* FP64 plain form, per (layer group, solver, size class): lanes per layer,
  1 (a layer per lane) or 4 (a layer's x, y, z on a quad), i.e. the
  threads per junction.

The size class is floor(log2(junctions)).  The table lives in memory and in
cmtj_gb300/_build/autotune.json, keyed by the GPU's name and the library's
build time.  CMTJ_AUTOTUNE=0 turns tuning off: the fixed defaults
(batch.default_tile, the default bound, the library's own lane pick) run.
"""
import json
import math
import os
import threading

import numpy as np

from . import _abi

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")
_lock = threading.Lock()
_table = None
_prefix = None


def enabled():
    return os.environ.get("CMTJ_AUTOTUNE", "1") != "0"


def _device_prefix():
    global _prefix
    if _prefix is None:
        from . import engine
        t = engine.torch()
        name = t.cuda.get_device_name(t.cuda.current_device())
        try:
            build = int(os.path.getmtime(_abi.LIB_PATH))
        except OSError:
            build = 0
        _prefix = "%s|%d" % (name, build)
    return _prefix


def _load():
    global _table
    if _table is None:
        _table = {}
        try:
            with open(PATH) as f:
                data = json.load(f)
            _table = data.get(_device_prefix(), {})
        except (OSError, ValueError):
            _table = {}
    return _table


def _save():
    try:
        data = {}
        if os.path.exists(PATH):
            with open(PATH) as f:
                data = json.load(f)
        data[_device_prefix()] = _table
        os.makedirs(os.path.dirname(PATH), exist_ok=True)
        tmp = PATH + ".%d.tmp" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, PATH)
    except (OSError, ValueError):
        pass


def lookup(key):
    with _lock:
        return _load().get(key)


def store(key, choice):
    with _lock:
        _load()[key] = choice
        _save()


def size_class(n):
    return int(math.floor(math.log2(max(int(n), 1))))


# ------------------------------------------------------------ FP32 batched
def f32_key(n_layers, solver, code, channels, weighted, n):
    return "f32|L%d|s%d|v%x|c%d|w%d|n%d" % (n_layers, int(solver), code & 0xffffff, channels, int(bool(weighted)),
                                           size_class(n))


def tile_candidates(channels, log_every, chunk_steps):
    """Log tiles to try: multiples of 4 with tile * channels <= 96 floats,
    at most 6 of them spread over the range; under chunked launches only
    those a chunk holds whole."""
    if channels <= 0:
        return [0]
    hi = max(4, (96 // channels) // 4 * 4)
    cands = sorted({t for t in (4, 8, 12, 16, 24, 32, 48, 64, 96) if t <= hi})
    if chunk_steps is not None:
        cands = [t for t in cands if int(chunk_steps) % (log_every * t) == 0]
    return cands


def tune_f32_partition(run, q, stream, chunk_steps=None, trial_steps=2000, reps=2):
    """Times trial launches of partition q of BatchRun `run` over its
    (bound, tile) candidates on a copy of the batch state, restores the
    state, and returns the best choice {"bound", "tile", "ms", "trials"}.
    The trials write log samples of their first steps, which the real run
    writes again with the same values."""
    from . import engine
    from .batch import log_channels
    t = engine.torch()
    nl, d_order, cnt, code = run.parts[q]
    channels = log_channels(run.log_mode, nl)
    base = code & 0xffffff
    import ctypes
    arr = (ctypes.c_int32 * 4)()
    nb = run.lib.cmtj_batch_bounds_f32(nl, int(run.solver), base, ctypes.cast(arr, ctypes.c_void_p), 4)
    bounds = [int(arr[k]) for k in range(nb)] if nb > 0 else [(code >> 24) & 0xf]
    tiles = tile_candidates(channels, run.log_every, chunk_steps)
    if not tiles:
        return None
    steps = run.lowered.n_steps[np.asarray(run.part_rows[q])]
    step = (run.log_every * int(np.lcm.reduce(tiles))) if channels > 0 else 1
    k = min(int(steps.min()), trial_steps)
    if chunk_steps is not None:
        k = min(k, int(chunk_steps))
    k = k // step * step
    if k <= 0:
        return None
    saved = run.d_s.clone()
    trials = []
    try:
        for bound in bounds:
            for tile in tiles:
                best = None
                for _ in range(reps):
                    run.d_s.copy_(saved)
                    a, b = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
                    a.record(stream)
                    run._launch_part(q, k, stream, tile, base | (bound << 24), 0)
                    b.record(stream)
                    b.synchronize()
                    ms = a.elapsed_time(b)
                    best = ms if best is None else min(best, ms)
                trials.append({"bound": bound, "tile": tile, "ms": best})
    finally:
        run.d_s.copy_(saved)
        stream.synchronize()
    win = min(trials, key=lambda r: r["ms"])
    return {"bound": win["bound"], "tile": win["tile"], "ms": win["ms"], "trial_steps": k, "trials": trials}


# ------------------------------------------------------------ FP64 plain
def f64_key(max_layers, solver, n):
    g = 1 if max_layers <= 1 else (2 if max_layers <= 2 else (4 if max_layers <= 4 else 8))
    return "f64|G%d|s%d|n%d" % (g, int(solver), size_class(n))


def tune_f64(lowered, d_j, d_l, d_tab, stream, trial_steps=500, reps=2):
    """Times trial launches of a lowered FP64 fixed-step batch with a layer
    per lane and with a layer per quad, on a copy of its layer records
    and a scratch log; returns {"lanes", "ms", "trials"}."""
    from . import engine
    t = engine.torch()
    lib = engine.require_gpu()
    p = lowered.params.copy()
    k = int(min(int(p["total_iterations"][0]), trial_steps))
    if k <= 0:
        return None
    we = int(p["write_every"][0])
    p["total_iterations"] = k
    p["n_log"] = (k + we - 1) // we
    n = len(lowered.junctions)
    log = t.empty((n, int(p["n_log"][0]), lowered.log_width), dtype=t.float64, device="cuda")
    status = t.zeros(2 * n, dtype=t.int32, device="cuda")
    scratch = d_l.clone()
    trials = []
    for lanes in (1, 4):
        p["lanes_per_layer"] = lanes
        best = None
        for _ in range(reps):
            scratch.copy_(d_l)
            a, b = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
            a.record(stream)
            rc = lib.cmtj_run_simulation_f64(engine.ptr(d_j), n, engine.ptr(scratch), engine.ptr(d_tab),
                                             p.ctypes.data, engine.ptr(log), engine.ptr(status),
                                             engine.stream_ptr(stream))
            _abi.check(rc, lib)
            b.record(stream)
            b.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        trials.append({"lanes": lanes, "ms": best})
    win = min(trials, key=lambda r: r["ms"])
    return {"lanes": win["lanes"], "ms": win["ms"], "trial_steps": k, "trials": trials}
