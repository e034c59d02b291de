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

With --fp64 it times the FP64 plain form's fixed-step kernel instead, on
the R(H) sweep of the 2-layer MTJ (Hx over +-800 kA/m, RK4, R logged every
step), for each batch size in --n and each lane layout in --lanes (1: a
layer per lane, 4: a layer's x, y, z on a quad of lanes, 0: the library's
own pick), one JSON line each:

    python -m cmtj_gb300.tune --fp64 [--n 1 64 1024 16384] [--lanes 0 1 4] [--steps 2000]
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
             "-DCMTJ_BATCH_MINB_WIDE=%d" % minb, "-DCMTJ_BATCH_MINB_STOCH=%d" % minb]
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


def time_library(lib, n_h, n_draw, steps, reps, workload="pimm", vsd_shape=(128, 1024, 5.0, 50.0)):
    """Runs in a fresh process: loads `lib` and times one batch: the 2-layer
    PIMM sweep, (workload "vsd") the uneven 1-4-layer spin-diode sweep at
    its own durations, or (workload "pbit") the thermal single-layer p-bit
    sweep, n_h currents x n_draw junctions, Euler-Heun at 300 K."""
    import numpy as np
    import torch
    from . import _abi
    _abi.LIB_PATH = lib
    from . import batch, sweeps
    dt = 1e-13
    if workload == "vsd":
        n_f, n_hv, t_lo, t_hi = vsd_shape
        spec, ns = sweeps.vsd_config(n_f=int(n_f), n_h=int(n_hv), dt=dt, t_min=t_lo * 1e-9, t_max=t_hi * 1e-9)
        low = batch.lower(spec, dt, ns)
        run = batch.BatchRun(low, dt, batch.SolverMode.RK4, batch.LOG_NONE, 0, red_every=1)
        layer_steps = float((ns * spec.n_layers).sum())
    elif workload == "pbit":
        # n_h currents x n_draw junctions, `steps` Euler-Heun steps each at 300 K
        spec, _, _ = sweeps.pbit_config(n_j=n_h, n_per=n_draw, dt=dt, t_min=steps * dt, t_max=steps * dt)
        ns = np.full(spec.n, steps, dtype=np.int64)
        low = batch.lower(spec, dt, ns)
        run = batch.BatchRun(low, dt, batch.SolverMode.EulerHeun, batch.LOG_NONE, 0)
        layer_steps = float(spec.n * steps)
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


def rh_junctions(n, total):
    """n 2-layer MTJs of the R(H) sweep: free Ms 1.2 T, Ku 3e5 J/m^3,
    t 1.5 nm; reference Ms 1.5 T, Ku 1e6 J/m^3, t 2 nm; both along z,
    alpha 0.01, demag diag(0.0024, 0.0024, 0.9952), surface 1e-16 m^2,
    IEC J = -5e-5 J/m^2, Rp 100, Rap 200, m along +z; Hx evenly over
    +-800 kA/m."""
    import numpy as np
    from . import core
    V = core.CVector
    demag = [V(0.0024, 0, 0), V(0, 0.0024, 0), V(0, 0, 0.9952)]
    js = []
    for h in np.linspace(-800e3, 800e3, n):
        free = core.Layer("free", mag=V(0, 0, 1), anis=V(0, 0, 1), Ms=1.2, thickness=1.5e-9, cellSurface=1e-16,
                          demagTensor=demag, damping=0.01)
        ref = core.Layer("ref", mag=V(0, 0, 1), anis=V(0, 0, 1), Ms=1.5, thickness=2e-9, cellSurface=1e-16,
                         demagTensor=demag, damping=0.01)
        j = core.Junction([free, ref], 100, 200)
        j.setLayerAnisotropyDriver("free", core.constantDriver(3e5))
        j.setLayerAnisotropyDriver("ref", core.constantDriver(1e6))
        j.setIECDriver("free", "ref", core.constantDriver(-5e-5))
        j.setLayerExternalFieldDriver("all", core.AxialDriver(float(h), 0, 0))
        js.append(j)
    return js


def time_fp64(n, steps, reps, lanes, dt=1e-13, arithmetic="reference"):
    """Best-of-`reps` CUDA-event time of one cmtj_run_simulation_f64 launch
    (after one warm-up launch) on the R(H) batch of n junctions."""
    import numpy as np
    import torch
    from . import _abi, engine
    from ._lower import lower, plan_run
    from .core import SolverMode
    plan = plan_run(steps * dt, dt, dt).for_solver(SolverMode.RK4)
    low = lower(rh_junctions(n, steps * dt), plan, SolverMode.RK4, False, arithmetic)
    low.params["lanes_per_layer"] = lanes
    lib = engine.require_gpu()
    d_j, d_l0 = engine.to_device(low.junctions), engine.to_device(low.layers)
    d_log = torch.empty((n, int(low.params["n_log"][0]), low.log_width), dtype=torch.float64, device="cuda")
    d_st = torch.zeros(2 * n, dtype=torch.int32, device="cuda")
    times = []
    for k in range(reps + 1):
        d_l = d_l0.clone()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        rc = lib.cmtj_run_simulation_f64(engine.ptr(d_j), n, engine.ptr(d_l), None, low.params.ctypes.data,
                                         engine.ptr(d_log), engine.ptr(d_st), engine.stream_ptr())
        b.record()
        _abi.check(rc, lib)
        torch.cuda.synchronize()
        if k:
            times.append(a.elapsed_time(b))
    st = d_st.cpu().numpy().view(np.uint32)
    best = min(times)
    return {"workload": "fp64_rh", "n": n, "lanes_per_layer": lanes, "arithmetic": arithmetic, "steps": steps,
            "ms": times, "best_ms": best,
            "us_per_step": best * 1e3 / steps, "layer_steps_per_s": n * steps * 2 / (best / 1e3),
            "all_ok": bool(np.all(st[0::2] == 0) and np.all(st[1::2] == steps))}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--minb", type=int, nargs="+", default=[4, 5, 6])
    ap.add_argument("--layers", type=int, nargs="+", default=[2], help="layer counts whose units are rebuilt")
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--n-h", type=int, default=512)
    ap.add_argument("--n-draw", type=int, default=512)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--workload", default="pimm", choices=["pimm", "vsd", "pbit"])
    ap.add_argument("--fp64", action="store_true", help="time the FP64 fixed-step lane layouts instead")
    ap.add_argument("--n", type=int, nargs="+", default=[1, 64, 1024, 16384], help="--fp64 batch sizes")
    ap.add_argument("--lanes", type=int, nargs="+", default=[0, 1, 4], help="--fp64 lanes per layer")
    ap.add_argument("--arithmetic", nargs="+", default=["reference"], choices=["reference", "fused"],
                    help="--fp64 arithmetic (cmtj_arithmetic)")
    ap.add_argument("--vsd-shape", type=float, nargs=4, default=[128, 1024, 5.0, 50.0],
                    metavar=("FREQS", "FIELDS", "T_MIN_NS", "T_MAX_NS"),
                    help="spin-diode sweep: frequencies x fields, durations uniform in [T_MIN, T_MAX] ns")
    ap.add_argument("--time-lib", help=argparse.SUPPRESS)
    a = ap.parse_args(argv)
    if a.fp64:
        B.build()
        for n in a.n:
            for lanes in a.lanes:
                for arith in a.arithmetic:
                    print(json.dumps(time_fp64(n, a.steps, a.reps, lanes, arithmetic=arith)), flush=True)
        return
    if a.time_lib:
        print(json.dumps(time_library(a.time_lib, a.n_h, a.n_draw, a.steps, a.reps, a.workload,
                                      tuple(a.vsd_shape))), flush=True)
        return
    results = []
    for mb in a.minb:
        lib = build_variant(mb, a.layers)
        out = subprocess.run([sys.executable, "-m", "cmtj_gb300.tune", "--time-lib", lib, "--steps", str(a.steps),
                              "--n-h", str(a.n_h), "--n-draw", str(a.n_draw), "--reps", str(a.reps),
                              "--workload", a.workload, "--vsd-shape", *[str(x) for x in a.vsd_shape]],
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
