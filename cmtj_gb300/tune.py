"""Launch-shape tuner of the FP32 batched kernel.

The specialised k_batch variants are compiled with
__launch_bounds__(128, CMTJ_BATCH_MINB): the number of resident 128-thread
CTAs per SM the register allocator must allow.  More CTAs hide more latency
but force fewer registers (and spills).  This tool builds the library once
per candidate bound into cmtj_gb300/_build/tune_mb<k>/ (only the units of
the layer counts named by --layers are recompiled), times the same 2-layer
PIMM batch on each with CUDA events (best of `reps` launches after one
warm-up), and prints one JSON line per candidate plus the best.

    python -m cmtj_gb300.tune [--minb 4 5 6] [--layers 2] [--steps 5000] [--n-h 512 --n-draw 512]

The default build uses the CMTJ_BATCH_MINB and CMTJ_BATCH_MINB_PACKED
defaults in csrc/batch_f32.cuh.
"""
import argparse
import json
import os
import subprocess
import sys

from . import build as B


def build_variant(minb, layers=(2,)):
    """libcmtj_gpu.so whose batch units for the layer counts in `layers` are
    compiled with every specialised variant (packed ones included) bounded
    to `minb` resident CTAs per SM; every other unit is the default build's
    object.  Returns the library path."""
    B.build()
    out = os.path.join(B.BUILD, "tune_mb%d" % minb)
    os.makedirs(out, exist_ok=True)
    flags = ["-DCMTJ_BATCH_MINB=%d" % minb, "-DCMTJ_BATCH_MINB_PACKED=%d" % minb,
             "-DCMTJ_BATCH_MINB_WIDE=%d" % minb]
    tuned = {"batch_f32_l%d.cu" % L for L in layers}
    objs = []
    jobs = []
    for unit, uflags in B.UNITS.items():
        if unit in tuned:
            obj = os.path.join(out, unit.replace(".cu", ".o"))
            jobs.append([B._nvcc(), *B.ARCH, *B.COMMON, *uflags, *flags, "-c", os.path.join(B.CSRC, unit), "-o",
                         obj])
        else:
            obj = os.path.join(B.BUILD, unit.replace(".cu", ".o"))
        objs.append(obj)
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for r in res:
        if r.returncode:
            raise RuntimeError("nvcc failed:\n%s" % r.stderr)
    lib = os.path.join(out, "libcmtj_gpu.so")
    subprocess.check_call([B._nvcc(), *B.ARCH, "-shared", "-o", lib, *objs])
    return lib


def time_library(lib, n_h, n_draw, steps, reps, workload="pimm"):
    """Runs in a fresh process: loads `lib` and times one batch: the 2-layer
    PIMM sweep, or (workload "vsd") the uneven 1-4-layer spin-diode sweep
    at its own durations."""
    import numpy as np
    import torch
    from . import _abi
    _abi.LIB_PATH = lib
    from . import batch, sweeps
    dt = 1e-13
    if workload == "vsd":
        spec, ns = sweeps.vsd_config(dt=dt)
        low = batch.lower(spec, dt, ns)
        run = batch.BatchRun(low, dt, batch.SolverMode.RK4, batch.LOG_NONE, 0, red_every=1)
        layer_steps = float((ns * spec.n_layers).sum())
    else:
        spec, ns = sweeps.pimm_config(n_h=n_h, n_draw=n_draw, dt=dt, total=steps * dt)
        low = batch.lower(spec, dt, ns)
        run = batch.BatchRun(low, dt, batch.SolverMode.RK4, batch.LOG_MIX, 10)
        layer_steps = float(spec.n * ns * 2)
    zero = torch.zeros_like(run.d_s)
    times = []
    for k in range(reps + 1):
        run.d_s.copy_(zero)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        run.launch()
        b.record()
        torch.cuda.synchronize()
        if k:
            times.append(a.elapsed_time(b))
    st = run.state()
    best = min(times)
    return {"lib": lib, "workload": workload, "ms": times, "best_ms": best,
            "layer_steps_per_s": layer_steps / (best / 1e3), "all_ok": bool(np.all(st["status"] == 0))}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--minb", type=int, nargs="+", default=[4, 5, 6])
    ap.add_argument("--layers", type=int, nargs="+", default=[2], help="layer counts whose units are rebuilt")
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--n-h", type=int, default=512)
    ap.add_argument("--n-draw", type=int, default=512)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--workload", default="pimm", choices=["pimm", "vsd"])
    ap.add_argument("--time-lib", help=argparse.SUPPRESS)
    a = ap.parse_args(argv)
    if a.time_lib:
        print(json.dumps(time_library(a.time_lib, a.n_h, a.n_draw, a.steps, a.reps, a.workload)), flush=True)
        return
    results = []
    for mb in a.minb:
        lib = build_variant(mb, a.layers)
        out = subprocess.run([sys.executable, "-m", "cmtj_gb300.tune", "--time-lib", lib, "--steps", str(a.steps),
                              "--n-h", str(a.n_h), "--n-draw", str(a.n_draw), "--reps", str(a.reps),
                              "--workload", a.workload],
                             capture_output=True, text=True, cwd=os.path.dirname(B.PKG))
        if out.returncode:
            raise RuntimeError(out.stderr)
        r = json.loads(out.stdout.strip().splitlines()[-1])
        r["minb"] = mb
        print(json.dumps(r), flush=True)
        results.append(r)
    best = max(results, key=lambda r: r["layer_steps_per_s"])
    print(json.dumps({"best_minb": best["minb"], "layer_steps_per_s": best["layer_steps_per_s"]}), flush=True)


if __name__ == "__main__":
    main()
