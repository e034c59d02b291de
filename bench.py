"""Benchmark of the macrospin hot path on one GB300.

Workload (value, e2e): batched FP32 PIMM -- 262,144 independent 2-layer
junctions (512 fields over +-600 kA/m along x x 512 seeded draws of
Ku(free) ~ U[1e5, 6e5] J/m^3 and J ~ U[-1e-4, 1e-4] J/m^2), a 1 ps
1 kA/m Oersted step along x, 5 ns at dt = 1e-13 s (50,000 RK4 steps), the
Ms*t-weighted m_x logged every 1 ps, and a 4096-point device FFT of each
junction's last 4096 samples.  One step = one pass of that whole batch.

Metric: layer-steps/s of the FP32 batched form (one layer-step = one
integration step of one layer), beside the FP64 plain form (the reference's
arithmetic on the GPU, one launch per solve and one launch per batch), the
FP32-vs-FP64 max|dm| on a sample of the same junctions, and the reference's
CPU path (the oracle restatement, bit-identical to the reference) on the
host cores.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

N_H, N_DRAW = 512, 512
DT = 1e-13
TOTAL = 5e-9
LOG_EVERY = 10       # 1 ps
N_FFT = 4096
MAX_FREQ = 80e9      # PIMM_procedure default max_frequency (procedures.py:52)

METRIC = "layer-steps/s FP32-batched vs FP64-plain @max|Δm|≤1e-4; p50/p99 request latency"
UNIT = "layer-steps/s"
RELAX_STEPS = 50000  # 5 ns at alpha = 1: static equilibrium before the ringing run (untimed setup)
WORKLOAD = ("batched FP32 PIMM: 262144 2-layer MTJs (512 H x 512 seeded Ku/J draws) from their relaxed "
            "equilibrium, 1 ps 1 kA/m Oersted step, 5 ns @ dt=1e-13 (RK4), m_x mix logged every 1 ps, "
            "4096-pt device FFT")


def fp32_flops_per_layer_step(n_layers=2, waves_per_junction=1, quiet_fraction=0.0):
    """FP32 operations per layer-step of the batched RK4 integrator for the
    PIMM junction (FMA = 2, rsqrt = 1), counted from its formulation.  The
    field terms are stored pre-multiplied by gamma dt/6, and the anisotropy
    (axis along z) and the diagonal demag fold into one diagonal tensor M.
    Per RHS (4 per step) and layer: M m 6, m x H 9, m x (m x H) 9, alpha
    FMA 6.  Per layer-step: stage states 18, RK4 accumulation 15,
    m + increment 3, renormalisation 9.  Field base per layer: while a
    step driver is on, h0 + wave 6 per wave and IEC neighbour 6 per
    neighbour at 3 stage times; in quiet bursts (driver off for the whole
    burst) only the IEC term, once per step.  `quiet_fraction` is the share
    of steps run in quiet bursts."""
    nb = 2.0 * (n_layers - 1) / n_layers
    rk4 = 4 * (6 + 9 + 9 + 6) + 18 + 15 + 3 + 9
    loud = rk4 + 3 * (6 * float(waves_per_junction) + 6 * nb)
    quiet = rk4 + 6 * nb
    return quiet_fraction * quiet + (1.0 - quiet_fraction) * loud


def pimm_quiet_fraction(n_steps):
    """Share of the PIMM run's steps in quiet bursts: bursts end at every
    log step (LOG_EVERY), and the bursts that overlap the pulse's stage
    windows ([0, pulse_len] inclusive) evaluate the waves."""
    from cmtj_gb300.sweeps import step_window
    on, off = step_window(0.0, 1e-12, DT, None)
    last = int(np.max(off))
    loud = (last // LOG_EVERY + 1) * LOG_EVERY
    return max(0.0, 1.0 - loud / float(n_steps))


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed
    region (every 100 ms).  Entering waits (at most 5 s) for the first
    sample, so nvidia-smi's start-up (its first device query held up a
    device-to-host copy by ~20 ms) falls before the timed region; the
    summary covers the samples taken after that."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.mark = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()
            while not self.rows and self.proc.poll() is None and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
            self.mark = len(self.rows)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        if len(self.rows) > self.mark:
            self.rows = self.rows[self.mark:]
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower() == "active"})
        pw = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_min_mhz": min(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "power_w_max": max(pw) if pw else None,
                "reasons": reasons, "samples": len(self.rows)}


def flops_per_layer_step():
    """FLOPs of one layer-step of the 2-layer PIMM junction, counted by running
    the oracle (the reference's arithmetic) on a counting scalar type."""
    import cases  # noqa: F401
    import oracle_harness
    import cmtj_gb300 as cm
    j, _ = __import__("cases").mtj_rh_point(cm, hx=-3e5, total=1e-11)
    j.setLayerOerstedFieldDriver("all", cm.AxialDriver(cm.stepDriver(0, 1e3, 0, 1e-12), cm.NullDriver(),
                                                        cm.NullDriver()))
    steps = 200
    c = oracle_harness.count_flops(j, steps * DT, DT, DT * LOG_EVERY)
    return float(c.sum()) / (steps * 2), [int(x) for x in c]


def build_workload(n_h=N_H, n_draw=N_DRAW, total=TOTAL, relax=True, seed=1):
    """The PIMM batch of one rank.  Under N ranks the job is N x 262,144
    junctions: rank r draws its Ku/J with seed 1 + r, so ranks hold disjoint
    shards and never exchange data."""
    from cmtj_gb300 import batch, sweeps
    spec, n_steps = sweeps.pimm_config(n_h=n_h, n_draw=n_draw, seed=seed, dt=DT, total=total)
    if relax:
        batch.relax(spec, DT, RELAX_STEPS, alpha=1.0)
    low = batch.lower(spec, DT, n_steps)
    return spec, low, n_steps


def fft_bins():
    freqs = np.fft.fftfreq(N_FFT, DT * LOG_EVERY)[: N_FFT // 2]
    hi = int(np.searchsorted(freqs, MAX_FREQ, side="right"))
    return 1, hi


def run_reference_arm(args):
    """The reference's CPU path (oracle restatement, bit-identical to the
    reference build; the reference itself does not build on the GPU machine)
    on all host cores, on bounded samples of the same workload."""
    import oracle_harness
    from cmtj_gb300 import _lower, sweeps
    rank, world, _ = dist_info()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n = cores * 8
    spec, steps = sweeps.pimm_config(n_h=n, n_draw=1, dt=DT, total=TOTAL)
    js = spec_to_junctions(spec)
    vals = []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for j in js:
            j.clearLog()
        oracle_harness.run_oracle(js, steps * DT, DT, DT * LOG_EVERY, threads=cores)
        el = time.perf_counter() - t0
        if it >= args.warmup:
            vals.append(n * steps * 2 / el)
    v = float(np.median(vals))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * n * steps * 2 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": "%d junctions x %d steps per step" % (n, steps)},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d PIMM junctions x %d RK4 steps (whole 5 ns solves), one oracle pass per step"
                                       % (n, steps)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def spec_to_junctions(spec):
    """Junction objects equal to the first rows of a pimm_config spec."""
    import cmtj_gb300 as cm
    import cases
    out = []
    for k in range(spec.n):
        j, _ = cases.mtj_rh_point(cm, hx=float(spec.Hc[k, 0, 0]), total=1e-9)
        j.setLayerAnisotropyDriver("free", cm.constantDriver(float(spec.K[k, 0])))
        j.setIECDriver("free", "ref", cm.constantDriver(float(spec.Jt[k, 0])))
        j.setLayerOerstedFieldDriver("all", cm.AxialDriver(cm.stepDriver(0, 1e3, 0, 1e-12), cm.NullDriver(),
                                                            cm.NullDriver()))
        out.append(j)
    return out


def dp_junctions(cm, n=4096):
    """n single free layers (Ms 1.2 T, Ku 3e5 J/m^3 along z, t 1.5 nm,
    alpha 0.01, demag diag(0.0024, 0.0024, 0.9952), m tilted 0.1 from z)
    driven by a 5 kA/m Oersted sine along x at 2-12 GHz."""
    V = cm.CVector
    demag = [V(0.0024, 0, 0), V(0, 0.0024, 0), V(0, 0, 0.9952)]
    js = []
    for k in range(n):
        f = 2e9 + 10e9 * k / max(n - 1, 1)
        layer = cm.Layer("free", mag=V(0.1, 0, 0.995), anis=V(0, 0, 1), Ms=1.2, thickness=1.5e-9,
                         cellSurface=1e-16, demagTensor=demag, damping=0.01)
        j = cm.Junction([layer])
        j.setLayerAnisotropyDriver("free", cm.constantDriver(3e5))
        j.setLayerOerstedFieldDriver("free", cm.AxialDriver(cm.sineDriver(0, 5e3, f, 0), cm.NullDriver(),
                                                            cm.NullDriver()))
        js.append(j)
    return js


def groups_16(cm, n_groups=64):
    """n_groups GroupInteractions of 16 single-layer junctions each on a
    4 x 4 grid at 60 nm pitch, Kanao et al. dipole coupling (the module's
    default), initial m varied over junctions and groups."""
    import group_cases
    out = []
    for q in range(n_groups):
        js = [group_cases._single(cm, (0.1 + 0.01 * k, 0.2 - 0.002 * q, 0.97)) for k in range(16)]
        pos = [cm.CVector(60e-9 * (k % 4), 60e-9 * (k // 4), 0) for k in range(16)]
        out.append(cm.reservoir.GroupInteraction(pos, js))
    return out


def pimm_procedure_case(cm):
    """PIMM_procedure over a list of 64 two-layer MTJs (the R(H) sweep's
    junction with Ku(free) over 1e5..6e5 J/m^3) swept from saturation
    downwards along +x (800 to 350 kA/m, 10 fields, no switching on the way:
    a well-conditioned chain), 0.5 ns per point, a 20 kA/m Oersted step."""
    import cases
    from cmtj_gb300 import procedures
    js = []
    for k in range(64):
        j, _ = cases.mtj_rh_point(cm, hx=0.0)
        j.setLayerAnisotropyDriver("free", cm.constantDriver(1e5 + 5e5 * k / 63))
        j.setLayerMagnetisation("free", cm.CVector(1, 0, 0.1))
        j.setLayerMagnetisation("ref", cm.CVector(1, 0, 0.2))
        js.append(j)
    H = np.linspace(800e3, 350e3, 10)
    RP = procedures.ResistanceParameters
    kw = dict(Hvecs=np.stack([H, 0 * H, 0 * H], 1), int_step=DT,
              resistance_params=[RP(Rxx0=100, Rxy0=5, Ramr=-0.24, Rahe=-0.3, Rsmr=-0.46, w=3e-5, l=2e-5)] * 2,
              Hoe_excitation=2e4, simulation_duration=5e-10, disturbance=0.0, take_last_n=50, max_frequency=80e9,
              disable_tqdm=True)
    return js, kw


def rh_logs(junctions):
    """m of both layers [n, rows, 6] and R [n, rows] from the R(H) logs."""
    lg = [j.getLogArrays() for j in junctions]
    m = np.stack([np.stack([g[k] for k in ("free_mx", "free_my", "free_mz", "ref_mx", "ref_my", "ref_mz")], 1)
                  for g in lg])
    return m, np.stack([g["R_free_ref"] for g in lg])


def final_m(junctions):
    return np.array([[(l.mag.x, l.mag.y, l.mag.z) for l in j.layers] for j in junctions])


def cpu_baseline(budget_s=15.0):
    """The oracle (the reference's arithmetic, bit-identical on the pinned
    cases) on all host cores: a pilot of whole 5 ns PIMM solves on 2
    junctions per core, then as many junctions as fill about budget_s."""
    import oracle_harness
    from cmtj_gb300 import sweeps
    cores = os.cpu_count() or 1
    n = cores * 2
    spec, n_steps = sweeps.pimm_config(n_h=n, n_draw=1, dt=DT, total=TOTAL)
    js = spec_to_junctions(spec)
    t0 = time.perf_counter()
    oracle_harness.run_oracle(js, n_steps * DT, DT, DT * LOG_EVERY, threads=cores)
    el = time.perf_counter() - t0
    per_junction_s = el / n
    n2 = max(cores, int(budget_s / per_junction_s) // cores * cores)
    spec, _ = sweeps.pimm_config(n_h=n2, n_draw=1, dt=DT, total=TOTAL)
    js = spec_to_junctions(spec)
    t0 = time.perf_counter()
    oracle_harness.run_oracle(js, n_steps * DT, DT, DT * LOG_EVERY, threads=cores)
    el = time.perf_counter() - t0
    rate = n2 * n_steps * 2 / el
    ref_fpls, fcount = flops_per_layer_step()
    # the R(H) sweep in full (64 fields x 10 ns, 100,000 RK4 steps, m and R
    # logged every step), one solve per task on all host cores
    from cmtj_gb300 import tune
    js = tune.rh_junctions(64, 1e-8)
    t0 = time.perf_counter()
    oracle_harness.run_oracle(js, 1e-8, DT, DT, threads=cores)
    rh_el = time.perf_counter() - t0
    rh = {"seconds": rh_el, "cores": cores, "layer_steps_per_s": 64 * 100_000 * 2 / rh_el,
          "mean_R_last_2ns": [float(np.mean(j.getLogArrays()["R_free_ref"][-20_000:])) for j in js],
          "logs": rh_logs(js)}
    # Dormand-Prince and a dipole-coupled group, the same runs as the GPU legs
    ocm = oracle_harness.oracle_module()
    js = dp_junctions(ocm)
    t0 = time.perf_counter()
    oracle_harness.run_oracle(js, 5e-9, DT, 1e-11, solverMode=ocm.SolverMode.DormandPrince, threads=cores)
    dp = {"seconds": time.perf_counter() - t0, "cores": cores, "final_m": final_m(js)}
    gs = groups_16(ocm)
    t0 = time.perf_counter()
    oracle_harness.run_groups_oracle(gs, 2e-10, DT, 1e-12)
    grp = {"seconds": time.perf_counter() - t0, "cores": 1,
           "final_m": np.concatenate([final_m(g.junctionList) for g in gs])}
    # PIMM_procedure with the oracle as its FP64 runner
    from cmtj_gb300 import procedures
    js, kw = pimm_procedure_case(ocm)
    run_f64 = procedures._run_f64
    procedures._run_f64 = lambda junctions, duration, int_step: oracle_harness.run_oracle(
        junctions, duration, int_step, int_step, threads=cores)
    try:
        t0 = time.perf_counter()
        res = procedures.PIMM_procedure(js, precision="f64", **kw)
        proc = {"seconds": time.perf_counter() - t0, "cores": cores,
                "spectra": np.stack([r[0] for r in res])}
    finally:
        procedures._run_f64 = run_f64
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "rh_config0": rh, "dp": dp, "group": grp,
            "procedure": proc,
            "reference_flop_per_layer_step": ref_fpls, "reference_flop_breakdown": fcount,
            "sample": "%d PIMM junctions x %d RK4 steps (full 5 ns solves) on %d threads (%.1f s)"
                      % (n2, n_steps, cores, el)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--profile", action="store_true",
                    help="262144 junctions x 2000 steps, no extra measurements (for ncu captures)")
    ap.add_argument("--main-only", action="store_true",
                    help="the full-size timed leg and the end-to-end leg only, no extra measurements (for the "
                         "ncu launch list of the benchmark's own kernels)")
    ap.add_argument("--profile-alpha", action="store_true",
                    help="the alpha-noise generator alone: 192 buffers of 100,000 samples, a warm-up call and one "
                         "timed call (for ncu captures)")
    ap.add_argument("--profile-fft", type=int, metavar="ROWS", default=0,
                    help="the spectrum kernel alone on ROWS log rows of the benchmark's shape (5000 samples, "
                         "4096-point FFT, the benchmark's bins): a warm-up call and three timed calls")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.profile_alpha:
        profile_alpha()
        return
    if args.profile_fft:
        profile_fft(args.profile_fft)
        return

    import torch
    from cmtj_gb300 import _abi, batch, engine
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = engine.require_gpu()
    stream = torch.cuda.current_stream()

    if args.profile:
        spec, low, n_steps = build_workload(N_H, N_DRAW, total=2000 * DT, relax=False, seed=1 + rank)
    else:
        spec, low, n_steps = build_workload(N_H, N_DRAW, seed=1 + rank)
    n = spec.n
    layer_steps = float(n) * n_steps * 2
    run = batch.BatchRun(low, DT, batch.SolverMode.RK4, batch.LOG_MIX, LOG_EVERY, log_axis=0)
    samples = int(run.samples[0])
    n_fft = min(N_FFT, 1 << int(np.log2(samples)))
    row_stride = int(run.log_pad[0])
    b_lo, b_hi = fft_bins()
    b_hi = min(b_hi, n_fft // 2)
    d_spec = torch.empty((n, b_hi - b_lo), dtype=torch.float32, device="cuda")
    state0 = torch.zeros_like(run.d_s)

    def spectrum():
        rc = lib.cmtj_spectrum_f32(engine.ptr(run.d_log), row_stride, n, samples, n_fft, b_lo, b_hi,
                                   engine.ptr(d_spec), engine.stream_ptr())
        _abi.check(rc, lib)

    def one_step():
        run.d_s.copy_(state0)
        run.launch()
        spectrum()

    # --- device-resident timing (value): each step replays two CUDA
    # graphs, the state reset + batched launch and the FFT, with CUDA
    # events between them on the replay stream
    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    g_run, g_fft = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
    run.tune()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        with torch.cuda.graph(g_run, stream=side):
            run.d_s.copy_(state0)
            run.launch(stream=side)
        with torch.cuda.graph(g_fft, stream=side):
            spectrum()
    stream.wait_stream(side)
    g_run.replay()
    g_fft.replay()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps + 2)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    kern_ms = []
    fft_ms = []
    with ClockSampler(local) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for k in range(args.steps):
            ev[2 * k].record(stream)
            g_run.replay()
            ev[2 * k + 1].record(stream)
            g_fft.replay()
            e = torch.cuda.Event(enable_timing=True)
            e.record(stream)
            fft_ms.append(e)
        t_end.record(stream)
        torch.cuda.synchronize()
    elapsed = t_start.elapsed_time(t_end) / 1e3
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    kern_ms = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(args.steps)]
    fft_only = [ev[2 * k + 1].elapsed_time(fft_ms[k]) for k in range(args.steps)]
    value = world * layer_steps * args.steps / elapsed
    clocks = clk.summary()

    st = run.state()
    ok = bool(np.all(st["status"] == 0) and np.all(st["step"] == n_steps))

    # --- end to end through the C ABI with host buffers (pinned): H2D of
    # the junction/layer records, the batched run, the device FFT, D2H of
    # the spectra and final states, every step.  Two device buffer sets
    # alternate, so step k's upload and step k-1's download overlap the
    # neighbouring compute; every copy stays inside the timed region.
    h_j = torch.from_numpy(low.junctions.view(np.uint8).copy()).pin_memory()
    h_l = torch.from_numpy(low.layers.view(np.uint8).copy()).pin_memory()
    runs = [run, batch.BatchRun(low, DT, batch.SolverMode.RK4, batch.LOG_MIX, LOG_EVERY, log_axis=0)]
    specs = [d_spec, torch.empty_like(d_spec)]
    h_specs = [torch.empty(d_spec.shape, dtype=torch.float32).pin_memory() for _ in range(2)]
    h_states = [torch.empty(run.d_s.shape, dtype=run.d_s.dtype).pin_memory() for _ in range(2)]
    # uploads and downloads on their own streams (one copy engine each way),
    # so step k+1's upload never queues behind step k's download
    up_stream, down_stream = torch.cuda.Stream(), torch.cuda.Stream()
    out_done = [None, None]  # per buffer set: its last outputs are on the host

    def spectrum_of(r, out):
        rc = lib.cmtj_spectrum_f32(engine.ptr(r.d_log), row_stride, n, samples, n_fft, b_lo, b_hi,
                                   engine.ptr(out), engine.stream_ptr())
        _abi.check(rc, lib)

    marks = []  # per timed step: (upload start, upload end, compute start, compute end, download start, end)

    def e2e_step(k, timed=False):
        q = k % 2
        r = runs[q]
        ev = [torch.cuda.Event(enable_timing=timed) for _ in range(6)]
        with torch.cuda.stream(up_stream):
            if out_done[q] is not None:
                up_stream.wait_event(out_done[q])
            ev[0].record(up_stream)
            r.d_j.copy_(h_j, non_blocking=True)
            r.d_l.copy_(h_l, non_blocking=True)
            ev[1].record(up_stream)
        stream.wait_event(ev[1])
        with torch.cuda.stream(stream):
            ev[2].record(stream)
            r.d_s.copy_(state0)
            r.launch(stream=stream)
            # the FFT writes the step's spectra straight into pinned host
            # memory (device-addressable under unified addressing, over
            # NVLink-C2C on GB300): no copy-engine transfer for the result
            spectrum_of(r, h_specs[q])
            ev[3].record(stream)
        with torch.cuda.stream(down_stream):
            down_stream.wait_event(ev[3])
            ev[4].record(down_stream)
            h_states[q].copy_(r.d_s, non_blocking=True)
            ev[5].record(down_stream)
            out_done[q] = ev[5]
        if timed:
            marks.append(ev)

    for k in range(max(2, args.warmup // 2)):
        e2e_step(k)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as e2e_clk:
        a.record(stream)
        for k in range(args.steps):
            e2e_step(k, timed=True)
        for e in out_done:
            stream.wait_event(e)
        b.record(stream)
        torch.cuda.synchronize()
    e2e_s = a.elapsed_time(b) / 1e3
    up_ms = [m[0].elapsed_time(m[1]) for m in marks]
    comp_ms = [m[2].elapsed_time(m[3]) for m in marks]
    down_ms = [m[4].elapsed_time(m[5]) for m in marks]
    # how long the compute stream sat idle between steps, and the fill and
    # drain of the pipeline (first upload, last download)
    gaps_ms = [marks[k][3].elapsed_time(marks[k + 1][2]) for k in range(len(marks) - 1)]
    fill_ms = a.elapsed_time(marks[0][2]) if marks else 0.0
    drain_ms = marks[-1][3].elapsed_time(b) if marks else 0.0
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    h_spec, h_state = h_specs[0], h_states[0]
    # the spectra the FFT wrote into host memory equal the resident leg's
    # (same inputs, same kernels)
    spectra_equal = bool(torch.equal(h_specs[(args.steps - 1) % 2], d_spec.cpu()))
    e2e = {"value": world * layer_steps * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(h_j.numel() + h_l.numel()),
           "d2h_bytes_per_step": int(h_spec.numel() * 4 + h_state.numel()),
           "pipelining": "two device buffer sets; copies of one step overlap the neighbouring step's compute; "
                         "the FFT writes the spectra into pinned host memory, the states are copied",
           "spectra_equal_resident_leg": spectra_equal,
           "timeline_ms": {"upload": up_ms, "compute": comp_ms, "download_states": down_ms,
                           "compute_idle_between_steps": gaps_ms, "fill": fill_ms, "drain": drain_ms,
                           "h2d_gbs": [(h_j.numel() + h_l.numel()) / (u / 1e3) / 1e9 for u in up_ms],
                           "d2h_states_gbs": [h_state.numel() / (d / 1e3) / 1e9 for d in down_ms]},
           "clocks": e2e_clk.summary()}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "junctions_per_gpu": n, "layers": 2, "steps_per_junction": n_steps,
                       "parallelism": ("%d disjoint shards (rank r: draws seeded 1 + r), no data-path collective"
                                       % world) if world > 1 else "single",
                       "l2": "inputs and logs (5.2 GB) larger than L2", "all_ok": ok,
                       "replay": "each timed step replays two CUDA graphs: state reset + batched launch, FFT"},
            "e2e": e2e, "clocks": clocks,
            "gpu_launches": args.steps * 2,
            "autotune": {"enabled": os.environ.get("CMTJ_AUTOTUNE", "1") != "0",
                         "partitions": [None if tu is None else {"key": tu[0], **tu[1]} for tu in run.tuning],
                         "defaults": {"log_tile": 32, "bound": 5}}}

    if rank == 0 and not (args.profile or args.main_only):
        extra = measure_rest(run, low, spec, n_steps, kern_ms, fft_only, lib)
        line.update(extra)
        f64 = line["fp64_plain"]
        f64["fp32_over_fp64_per_solve"] = value / f64["per_solve_launch_layer_steps_per_s"]
        f64["fp32_over_fp64_batched"] = value / f64["batched_launch_layer_steps_per_s"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def profile_alpha(rows=192, n=100_000):
    """The buffered alpha-noise generator (cmtj_alpha_noise_f32) on `rows`
    buffers of n samples (three axes of rows / 3 layers; FFT size 262,144
    for n = 100,000): one warm-up call, one call timed with CUDA events."""
    import torch
    from cmtj_gb300 import noise
    specs = noise.specs_array([(1.0, 1.0, 77 + r // 3, 0, r % 3) for r in range(rows)])
    noise.device_buffers(specs, n)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    noise.device_buffers(specs, n)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    print(json.dumps({"alpha_noise_generator": {"rows": rows, "samples": n, "ms": ms,
                                                "samples_per_s": rows * n / (ms / 1e3)}}))


def profile_fft(rows, samples=5000):
    """cmtj_spectrum_f32 alone on `rows` seeded Gaussian rows of `samples`
    floats (the benchmark's log rows: 5000 samples, the last 4096
    transformed, the benchmark's bins): one warm-up call, three calls timed
    with CUDA events, each after writing a buffer larger than L2."""
    import torch
    from cmtj_gb300 import _abi, engine
    lib = engine.require_gpu()
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    series = torch.randn((rows, samples), generator=g, device="cuda", dtype=torch.float32)
    b_lo, b_hi = fft_bins()
    out = torch.empty((rows, b_hi - b_lo), device="cuda", dtype=torch.float32)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def call():
        rc = lib.cmtj_spectrum_f32(engine.ptr(series), samples, rows, samples, N_FFT, b_lo, b_hi, engine.ptr(out),
                                   engine.stream_ptr())
        _abi.check(rc, lib)

    call()
    ms = []
    for _ in range(3):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        call()
        b.record()
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    nbytes = 4.0 * rows * (N_FFT + (b_hi - b_lo))
    print(json.dumps({"spectrum": {"rows": rows, "n_fft": N_FFT, "bins": b_hi - b_lo, "ms": ms,
                                   "algorithmic_bytes": nbytes, "gbs": nbytes / (min(ms) / 1e3) / 1e9,
                                   "checksum": float(out.double().sum())}}))


def build_peak_probe():
    """Compile bench_peak.cu (the FP32 FMA throughput probe that gives the
    roofline its denominator) into _build/libbench_peak.so."""
    from cmtj_gb300 import build as cbuild
    src = os.path.join(ROOT, "bench_peak.cu")
    out_dir = os.path.join(ROOT, "_build")
    lib = os.path.join(out_dir, "libbench_peak.so")
    os.makedirs(out_dir, exist_ok=True)
    if not os.path.exists(lib) or os.path.getmtime(src) > os.path.getmtime(lib):
        subprocess.check_call([cbuild._nvcc(), *cbuild.ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                               src, "-o", lib + ".tmp"])
        os.replace(lib + ".tmp", lib)
    return lib


def measure_rest(run, low, spec, n_steps, kern_ms, fft_ms, lib):
    """Roofline, FP64 plain comparisons, FP32-vs-FP64 accuracy, CPU baseline."""
    import torch
    from cmtj_gb300 import batch, engine
    out = {}
    # roofline of the dominant kernel (the FP32 batch integrator)
    quiet = pimm_quiet_fraction(n_steps)
    fpls = fp32_flops_per_layer_step(2, 1, quiet)
    n = spec.n
    kavg = float(np.mean(kern_ms)) / 1e3
    achieved = fpls * n * n_steps * 2 / kavg / 1e12
    import ctypes
    probe = ctypes.CDLL(build_peak_probe())
    peaks = {}
    for name in ("cmtj_probe_fp32_peak", "cmtj_probe_fp32x2_peak"):
        fn = getattr(probe, name)
        fn.restype = ctypes.c_double
        fn.argtypes = [ctypes.c_int]
        peaks[name] = fn(5) / 1e12
    # the FP32 ceiling is the larger of scalar FFMA and packed FFMA2 issue
    peak = max(peaks.values())
    # SM cycles a warp spends per FP64 FMA (one chain: latency; four
    # independent chains: whether a warp's FP64 instructions overlap)
    fn = probe.cmtj_probe_fp64_cycles
    fn.restype = ctypes.c_double
    fn.argtypes = [ctypes.c_int]
    fp64_cycles = {"one_chain": fn(1), "four_chains": fn(4)}
    # DRAM traffic of k_batch per launch: the reads measured by ncu on the
    # 2000-step case of the same batch (profiles/k_batch_pimm_262k_2000steps.md:
    # 313.5 MB, the records read once, the same at any length), plus the
    # writes at their algorithmic count (every decimated log sample and the
    # final states).  The capture's own 176 MB of writes understate a launch:
    # the last tiles were still in L2 when that kernel ended.
    log_write = 4.0 * float(np.sum(run.samples)) + n * batch.F32_STATE_DTYPE.itemsize
    traffic = 313.5e6 + log_write
    out["roofline"] = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                       "frac": achieved / peak, "traffic": traffic,
                       "traffic_source": "ncu dram__bytes_read of the 2000-step capture (records, read once) + "
                                         "algorithmic log and state writes",
                       "flop_per_layer_step": fpls,
                       "flop_model": "171 per layer-step in quiet bursts, 201 while the pulse is on; "
                                     "quiet share %.5f" % quiet,
                       "peak_source": "measured FP32 FMA probe on this GPU, best of scalar FFMA and packed FFMA2 "
                                      "(MEASURED_PEAKS.json has no FP32 figure)",
                       "peak_scalar_ffma": peaks["cmtj_probe_fp32_peak"],
                       "peak_packed_ffma2": peaks["cmtj_probe_fp32x2_peak"],
                       "kernel_ms_avg": kavg * 1e3, "fft_ms_avg": float(np.mean(fft_ms))}
    # HBM view of both kernels against MEASURED_PEAKS.json's copy bandwidth:
    # k_batch moves its records once plus the decimated log; the FFT reads
    # each row's last n_fft samples and writes the kept bins
    hbm_peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak = float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        pass
    rec_bytes = low.junctions.nbytes + low.layers.nbytes + n * batch.F32_STATE_DTYPE.itemsize
    log_bytes = 4.0 * float(np.sum(run.samples))
    b_lo, b_hi = fft_bins()
    fft_bytes = 4.0 * n * (N_FFT + (b_hi - b_lo))
    k_gbs = (rec_bytes + log_bytes) / kavg / 1e9
    f_gbs = fft_bytes / (float(np.mean(fft_ms)) / 1e3) / 1e9
    out["roofline"]["hbm_secondary"] = {
        "peak_gbs": hbm_peak, "peak_source": "MEASURED_PEAKS.json hbm_gbs" if hbm_peak else None,
        "k_batch": {"algorithmic_bytes": rec_bytes + log_bytes, "achieved_gbs": k_gbs,
                    "frac": k_gbs / hbm_peak if hbm_peak else None},
        "k_spectrum": {"algorithmic_bytes": fft_bytes, "achieved_gbs": f_gbs,
                       "frac": f_gbs / hbm_peak if hbm_peak else None}}

    # FP64 plain form and accuracy on a sample of the same junctions
    rows = np.arange(0, n, max(1, n // 256))[:256]
    plan = engine.plan_run(n_steps * DT, DT, DT * LOG_EVERY)
    from cmtj_gb300.core import SolverMode
    # one launch per solve (2 solves of 2000 steps, 1 thread each)
    solo = spec_to_junctions_rows(spec, rows[:2])
    plan_s = engine.plan_run(2000 * DT, DT, DT * LOG_EVERY)
    engine.run_junctions([spec_to_junctions_rows(spec, rows[:1])[0]], engine.plan_run(10 * DT, DT, DT),
                         SolverMode.RK4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for j in solo:
        engine.run_junctions([j], plan_s, SolverMode.RK4)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    fp64_solo = len(solo) * 2000 * 2 / el
    # one launch for the 256 sampled solves over the full duration, timed
    # after an untimed run of the same batch (which makes the run-time
    # autotuner's lane-layout trials for this batch shape, once)
    engine.run_junctions(spec_to_junctions_rows(spec, rows), plan, SolverMode.RK4)
    js = spec_to_junctions_rows(spec, rows)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.run_junctions(js, plan, SolverMode.RK4)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    fp64_batch = len(rows) * n_steps * 2 / el
    # FP32 vs FP64 on those junctions: final m and the logged m_x mix
    st = run.state()
    m32 = st["m"][rows, :2, :].astype(np.float64)
    m64 = np.stack([[[l.mag.x, l.mag.y, l.mag.z] for l in j.layers] for j in js])
    dm_final = float(np.max(np.abs(m32 - m64)))
    log32 = run.d_log.cpu().numpy()
    dmix = 0.0
    for q, k in enumerate(rows):
        lg = js[q].getLogArrays()
        w = spec.mix_w[k, :2]
        mix64 = w[0] * lg["free_mx"] + w[1] * lg["ref_mx"]
        mix32 = run.log_of(int(k), log32)[:, 0]
        dmix = max(dmix, float(np.max(np.abs(mix32 - mix64))))
    out["fp64_plain"] = {"per_solve_launch_layer_steps_per_s": fp64_solo,
                         "batched_launch_layer_steps_per_s": fp64_batch,
                         "sample": "2 solo launches x 2000 steps; one launch of %d junctions x %d steps"
                                   % (len(rows), n_steps)}
    out["accuracy"] = {"max_abs_dm_final_vs_fp64": dm_final, "max_abs_dmix_logged_vs_fp64": dmix,
                       "tolerance": 1e-4, "sample_junctions": 256, "pass": max(dm_final, dmix) <= 1e-4,
                       "start": "relaxed equilibrium (the timed workload)",
                       "literal_start": literal_start_accuracy(rows, n_steps)}
    out["serving"] = serving_leg()
    out["other_workloads"] = other_workloads()
    out["cpu_baseline"] = cpu_baseline()
    rh_cpu = out["cpu_baseline"].pop("rh_config0")
    rh_gpu = out["other_workloads"]["rh_config0_fp64"]
    rh_gpu["max_abs_dR_mean_vs_cpu_ohm"] = float(np.max(np.abs(np.array(rh_gpu.pop("mean_R_last_2ns")) -
                                                               np.array(rh_cpu["mean_R_last_2ns"]))))
    (m64, r64), (mo, ro) = rh_gpu.pop("logs"), rh_cpu.pop("logs")
    rh_gpu["vs_oracle_full_logs"] = {
        "max_abs_dm": float(np.max(np.abs(m64 - mo))), "max_rel_dR": float(np.max(np.abs(r64 - ro) / np.abs(ro))),
        "rows": int(m64.shape[0] * m64.shape[1]), "tolerance": "max|dm| <= 1e-9, R relative <= 1e-9",
        "pass": bool(np.max(np.abs(m64 - mo)) <= 1e-9 and np.max(np.abs(r64 - ro) / np.abs(ro)) <= 1e-9)}
    rh_gpu["cpu_oracle"] = {k: v for k, v in rh_cpu.items() if k != "mean_R_last_2ns"}
    rh_gpu["fp64_pipe_probe"] = {
        "cycles_per_dfma": fp64_cycles,
        "note": "one warp, clock64 around dependent DFMA chains (bench_peak.cu); a step of the FP64 plain "
                "form costs about this per FP64 instruction on its warp"}
    fz = rh_gpu["fused"]
    mf, rf = fz.pop("logs")
    dmf = np.max(np.abs(mf - mo), axis=(1, 2))
    rel = np.max(np.abs(rf - ro) / np.abs(ro), axis=1)
    ok = (dmf <= 1e-9) & (rel <= 1e-9)
    spread = np.load(os.path.join(ROOT, "tests", "golden", "rh_fma_spread.npz"))
    fz["vs_oracle_full_logs"] = {
        "max_abs_dm": float(dmf.max()), "max_rel_dR": float(rel.max()),
        "fields_within_1e-9": int(ok.sum()), "fields": int(len(ok)),
        "other_fields": [{"field_index": int(i), "max_abs_dm": float(dmf[i]), "max_rel_dR": float(rel[i]),
                          "fma_built_reference_max_abs_dm": float(spread["max_abs_dm"][i])}
                         for i in np.flatnonzero(~ok)],
        "fma_built_reference_fields_within_1e-9": int(np.sum(spread["max_abs_dm"] <= 1e-9)),
        "note": "fma_built_reference: the reference compiled with FMA contraction (GCC's default on aarch64) "
                "against its x86-64 build, per field, from tests/golden/rh_fma_spread.npz"}
    fz["vs_cpu_oracle"] = rh_cpu["seconds"] / fz["kernel_s"]
    del mf, rf
    for key, leg in (("dp", "dormand_prince_fmr_4096"), ("group", "groups_dipole_64x16")):
        cpu = out["cpu_baseline"].pop(key)
        gpu = out["other_workloads"][leg]
        gpu["max_abs_dm_vs_oracle"] = float(np.max(np.abs(gpu.pop("final_m") - cpu.pop("final_m"))))
        gpu["cpu_oracle"] = cpu
    cpu = out["cpu_baseline"].pop("procedure")
    gpu = out["other_workloads"]["pimm_procedure_64x10"]
    ref = cpu.pop("spectra")
    gpu["max_rel_spectrum_diff_fp64_vs_oracle"] = float(np.max(np.abs(gpu.pop("spectra_f64") - ref)) / np.max(ref))
    gpu["max_rel_spectrum_diff_fp32_vs_oracle"] = float(np.max(np.abs(gpu.pop("spectra_f32") - ref)) / np.max(ref))
    gpu["cpu_oracle"] = cpu
    # the reference's own arithmetic per layer-step, counted in the CPU leg
    out["roofline"]["reference_flop_per_layer_step"] = out["cpu_baseline"].pop("reference_flop_per_layer_step")
    out["roofline"]["reference_flop_breakdown_add_mul_div_sqrt_trans"] = out["cpu_baseline"].pop(
        "reference_flop_breakdown")
    return out


def literal_start_accuracy(rows, n_steps):
    """The PIMM workload's sample rows from the literal start of the R(H)
    MTJ (m along +z, no relaxation) instead of the relaxed equilibrium:
    the FP32 batched form against the FP64 plain form, and the FP64 plain
    form against itself with m0 nudged by 1e-7 along x (its conditioning:
    how far a 1e-7 change of the start moves FP64 itself)."""
    import cmtj_gb300 as cm
    from cmtj_gb300 import batch, engine, sweeps
    spec, _ = sweeps.pimm_config(n_h=N_H, n_draw=N_DRAW, seed=1, dt=DT, total=TOTAL)
    sub = spec.take(rows)
    run = batch.BatchRun(batch.lower(sub, DT, n_steps), DT, batch.SolverMode.RK4, batch.LOG_MIX, LOG_EVERY,
                         log_axis=0)
    run.launch()
    m32 = run.state()["m"][:, :2, :].astype(np.float64)
    plan = engine.plan_run(n_steps * DT, DT, DT * LOG_EVERY)
    js = spec_to_junctions_rows(spec, rows)
    engine.run_junctions(js, plan, cm.SolverMode.RK4)
    m64 = final_m(js)
    nudged = spec_to_junctions_rows(spec, rows)
    for j in nudged:
        for layer in j.layers:
            layer.mag = cm.CVector(layer.mag.x + 1e-7, layer.mag.y, layer.mag.z)
    engine.run_junctions(nudged, plan, cm.SolverMode.RK4)
    d32 = np.max(np.abs(m32 - m64), axis=(1, 2))
    cond = np.max(np.abs(final_m(nudged) - m64), axis=(1, 2))
    well = cond <= 3e-5
    return {"sample_junctions": len(rows), "max_abs_dm_final_fp32_vs_fp64": float(np.max(d32)),
            "median_abs_dm_final_fp32_vs_fp64": float(np.median(d32)),
            "fp64_nudge_1e-7_max_abs_dm": float(np.max(cond)),
            "fp64_nudge_1e-7_median_abs_dm": float(np.median(cond)),
            "well_conditioned_junctions": int(np.sum(well)),
            "max_abs_dm_fp32_vs_fp64_well_conditioned": float(np.max(d32[well])) if np.any(well) else None,
            "junctions_within_1e-4": int(np.sum(d32 <= 1e-4)),
            "note": "well conditioned: FP64 moves <= 3e-5 under the 1e-7 nudge"}


def fp64_rows_at(js, ends, every, solver):
    """The FP64 plain form on `js` for the longest of `ends` iterations,
    logged every `every` steps; for each junction the log row of the state
    after every * floor((end - 1) / every) + 1 steps (gathered on the
    device).  Returns (rows [n, width], status)."""
    import torch
    from cmtj_gb300 import _abi, engine
    lib = engine.require_gpu()
    plan = engine.plan_run(int(max(ends)) * DT, DT, every * DT)
    low = engine.lower(js, plan, solver, False)
    n, p = len(js), low.params
    d_j = engine.to_device(low.junctions)
    d_l, alpha = engine.device_layers(low)
    d_tab = engine.to_device(low.tables) if low.tables is not None else None
    d_log = torch.empty((n, int(p["n_log"][0]), low.log_width), dtype=torch.float64, device="cuda")
    d_status = torch.zeros(2 * n, dtype=torch.int32, device="cuda")
    _abi.check(lib.cmtj_run_simulation_f64(engine.ptr(d_j), n, engine.ptr(d_l), engine.ptr(d_tab), p.ctypes.data,
                                           engine.ptr(d_log), engine.ptr(d_status), engine.stream_ptr()), lib)
    idx = torch.from_numpy((np.asarray(ends, dtype=np.int64) - 1) // every).cuda()
    out = d_log[torch.arange(n, device="cuda"), idx].cpu().numpy()
    del alpha
    return out, d_status.cpu().numpy().view(np.uint32)


def pbit_accuracy(spec, n_steps, jd, mz32):
    """The p-bit sweep's P(switch) against the reference's counts
    (tests/golden/pbit_sweep.npz: 17 of the 64 currents, 2048 runs each,
    3-sigma binomial bound), and 4 seeded junctions per current (256) on the
    FP64 plain form under the same Philox noise words: how often the two
    forms end on the same side."""
    import cmtj_gb300 as cm
    import thermal_cases
    g = np.load(os.path.join(ROOT, "tests", "golden", "pbit_sweep.npz"))
    cur, sw, runs = g["currents"], g["switched"], g["runs"]
    rows = []
    for q, c in enumerate(cur):
        sel = jd == c
        n = int(sel.sum())
        k = int(np.sum(mz32[sel] < 0))
        p1, p2 = k / n, sw[q] / runs[q]
        p = (k + sw[q]) / (n + runs[q])
        bound = 3 * np.sqrt(max(p * (1 - p), 1.0 / (n + runs[q])) * (1.0 / n + 1.0 / runs[q]))
        rows.append((float(c), p1, float(p2), abs(p1 - p2), float(bound)))
    within = sum(1 for r in rows if r[3] <= r[4])
    # FP64 sample under the same noise
    pick = np.concatenate([np.nonzero(jd == c)[0][:4] for c in np.unique(jd)])
    js = []
    for k in pick:
        j, _ = thermal_cases.pbit_sweep_junction(cm, float(jd[k]), n_steps[k] * DT)
        j.layers[0].noise_seed = int(spec.seed[k, 0])
        js.append(j)
    r64, st64 = fp64_rows_at(js, n_steps[pick], 100, cm.SolverMode.EulerHeun)
    same = np.mean((r64[:, 2] < 0) == (mz32[pick] < 0))
    return {"vs_reference": {"currents": len(rows), "within_3sigma": within,
                             "max_abs_dP": float(max(r[3] for r in rows)),
                             "per_current": [[round(r[0], 1), round(r[1], 4), round(r[2], 4), round(r[4], 4)]
                                             for r in rows],
                             "columns": "current A/m^2, P fp32 (16,384 runs), P reference (2048 runs), 3-sigma"},
            "vs_fp64_same_noise": {"sample_junctions": int(len(pick)), "same_final_side": float(same),
                                   "fp64_ok": bool(np.all(st64[0::2] == 0)),
                                   "note": "FP64 read at the last 10 ps log row at or before each run's end"}}


def vsd_accuracy(spec, n_steps, st, n_sample=64, seed=5):
    """A seeded sample of the spin-diode sweep on the oracle (FP64, every
    step logged, each row its own duration, all host cores): the on-device
    <I R>, time-averaged R, mixing covariance <I R> - <I><R> and the
    Butterworth-filtered voltage (compute_sd) against the same quantities of
    the FP64 trajectory."""
    from concurrent.futures import ThreadPoolExecutor
    import cmtj_gb300 as cm
    import oracle_harness
    from cases import junctions_from_spec
    from scipy.signal import butter, lfilter
    rows = np.sort(np.random.default_rng(seed).choice(spec.n, n_sample, replace=False))
    sub = spec.take(rows)
    oracle_harness.oracle_lib()
    b, a = butter(3, 10e6 / (0.5 / DT), btype="low", analog=False)

    def one(q):
        j = junctions_from_spec(sub, [q], lambda k: cm.AxialDriver(
            cm.NullDriver(), cm.sineDriver(0, 500.0, float(sub.vsd_freq[k]), 0), cm.NullDriver()))[0]
        ns = int(n_steps[rows[q]])
        oracle_harness.run_oracle([j], ns * DT, DT, DT)
        lg = j.getLogArrays()
        L = int(sub.n_layers[q])
        if sub.mr_mode[q] == 1:
            R = lg["R"] if L == 1 else lg["R_L0_L1"]
            scale = sub.Rap[q] - sub.Rp[q]
        else:
            R = sum(sub.strip[q, 0, l] + sub.strip[q, 2, l] * lg["L%d_mx" % l] ** 2 +
                    sub.strip[q, 4, l] * lg["L%d_my" % l] ** 2 for l in range(L))
            scale = sum(abs(sub.strip[q, 2, l]) + abs(sub.strip[q, 4, l]) for l in range(L))
        I = np.sin(2 * np.pi * sub.vsd_freq[q] * lg["time"])
        return (float(np.mean(I * R)), float(np.mean(R)), float(np.mean(I)),
                float(np.mean(lfilter(b, a, -I * R))), float(scale))

    t0 = time.perf_counter()
    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        ref = list(ex.map(one, range(len(rows))))
    el = time.perf_counter() - t0
    ns = n_steps[rows].astype(np.float64)
    v32 = (st["v_sum"][rows].astype(np.float64) + st["v_c"][rows]) / ns
    r32 = (st["r_sum"][rows].astype(np.float64) + st["r_c"][rows]) / ns
    sd32 = -(st["vw_sum"][rows].astype(np.float64) + st["vw_c"][rows]) / ns
    v64, r64, i64, sd64, scale = (np.array(x) for x in zip(*ref))
    cov64, cov32 = v64 - i64 * r64, v32 - i64 * r32
    return {"sample_junctions": len(rows), "oracle_seconds": el,
            "max_abs_dV_over_mr_scale": float(np.max(np.abs(v32 - v64) / scale)),
            "max_abs_dR_mean_over_mr_scale": float(np.max(np.abs(r32 - r64) / scale)),
            "max_abs_dcov_over_mr_scale": float(np.max(np.abs(cov32 - cov64) / scale)),
            "median_rel_dcov": float(np.median(np.abs(cov32 - cov64) / np.maximum(np.abs(cov64), 1e-30))),
            "max_abs_dV_filtered_over_mr_scale": float(np.max(np.abs(sd32 - sd64) / scale)),
            "max_abs_dV_ohm": float(np.max(np.abs(v32 - v64))),
            "median_abs_cov64_ohm": float(np.median(np.abs(cov64))),
            "note": "V = <I R> per unit drive current; MR scale = Rap - Rp (classic) or sum |AMR_X| + |SMR_X| "
                    "(series Rx)"}


def _timed_run(run, warm_steps=2000):
    """One full launch of a BatchRun timed with CUDA events on its stream.
    Outside the timed region: its launch choices are resolved, and a chunk
    of warm_steps steps runs once and is undone (the state is put back),
    so that the timed launch does not pay for the GPU's first work after the
    host-side setup.  Without it, the first launch after a setup whose
    choices were already tuned took 3.8-4.9 s instead of 1.3 s."""
    import math
    import torch
    from cmtj_gb300 import batch
    state0 = run.d_s.clone()
    choices = run.tune()
    if run.log_mode != batch.LOG_NONE:
        # a chunk must hold whole log tiles of every partition
        unit = run.log_every * math.lcm(*[int(tile) for tile, _ in choices])
        warm_steps = unit * max(1, -(-warm_steps // unit))
    run.launch(chunk_steps=warm_steps)
    torch.cuda.synchronize()
    run.d_s.copy_(state0)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    run.launch()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3


def other_workloads():
    """The remaining sweep families at full size, each one timed launch:
    the stochastic p-bit sweep (64 currents x 16,384 single-layer STT
    junctions, Euler-Heun at 300 K, 5-20 ns each), the uneven spin-diode
    sweep (128 frequencies x 1024 fields, 1-4 layers, 5-50 ns, plain and
    Butterworth-filtered <I R> on the device), and a 16-junction series
    stack in the FP64 form (2000 steps)."""
    import torch
    import cmtj_gb300 as cm
    import cases
    from cmtj_gb300 import batch, stack, sweeps
    out = {}
    # p-bit
    spec, n_steps, jd = sweeps.pbit_config(dt=DT)
    low = batch.lower(spec, DT, n_steps)
    run = batch.BatchRun(low, DT, batch.SolverMode.EulerHeun, batch.LOG_NONE, 0)
    el = _timed_run(run)
    st = run.state()
    mz = st["m"][:, 0, 2]
    cur = np.unique(jd)
    p_sw = [float(np.mean(mz[jd == c] < 0)) for c in cur]
    norm = np.linalg.norm(st["m"][:, 0, :].astype(np.float64), axis=1)
    out["pbit_1M"] = {"layer_steps_per_s": float(n_steps.sum()) / el, "seconds": el, "junctions": spec.n,
                      "layer_steps": float(n_steps.sum()), "all_ok": bool(np.all(st["status"] == 0)),
                      "p_switch_first_last": [p_sw[0], p_sw[-1]], "max_norm_drift": float(np.max(np.abs(norm - 1))),
                      "accuracy": pbit_accuracy(spec, n_steps, jd, mz)}
    del run, low, spec
    torch.cuda.empty_cache()
    # uneven spin-diode sweep with both voltage forms
    spec, n_steps = sweeps.vsd_config(dt=DT)
    low = batch.lower(spec, DT, n_steps)
    w = batch.lowpass_step_response(int(n_steps.max()), 1.0 / DT)
    run = batch.BatchRun(low, DT, batch.SolverMode.RK4, batch.LOG_NONE, 0, red_every=1, red_weights=w)
    el = _timed_run(run)
    st = run.state()
    ls = float((n_steps * spec.n_layers).sum())
    out["vsd_uneven_131k"] = {"layer_steps_per_s": ls / el, "seconds": el, "junctions": spec.n, "layer_steps": ls,
                              "all_ok": bool(np.all(st["status"] == 0)),
                              "variants": [[int(a), int(b), int(c)] for a, b, c in run.variants()],
                              "reductions": "plain and Butterworth-weighted <I R>, every step",
                              "accuracy": vsd_accuracy(spec, n_steps, st)}
    del run, low, spec
    torch.cuda.empty_cache()
    # R(H) sweep of the 2-layer MTJ: 64 fields over +-800 kA/m along x, 1 ns
    # at dt = 1e-13 with R logged every step; one FP64 plain launch and one
    # FP32 batched launch, and the mean R over the last 20 % of each
    from cmtj_gb300 import engine
    js = [cases.mtj_rh_point(cm, hx=float(h), total=1e-9)[0] for h in np.linspace(-800e3, 800e3, 64)]
    js32 = [cases.mtj_rh_point(cm, hx=float(h), total=1e-9)[0] for h in np.linspace(-800e3, 800e3, 64)]
    plan = engine.plan_run(1e-9, DT, DT)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.run_junctions(js, plan, batch.SolverMode.RK4)
    torch.cuda.synchronize()
    el64 = time.perf_counter() - t0
    spec = batch.BatchSpec.from_junctions(js32)
    run = batch.BatchRun(batch.lower(spec, DT, plan.total_iterations), DT, batch.SolverMode.RK4, batch.LOG_R, 1)
    el32 = _timed_run(run)
    log32 = run.d_log.cpu().numpy()
    tail = plan.total_iterations // 5
    r64 = np.array([np.mean(j.getLogArrays()["R_free_ref"][-tail:]) for j in js])
    r32 = np.array([np.mean(run.log_of(k, log32)[-tail:, 0].astype(np.float64)) for k in range(len(js))])
    ls = 64.0 * plan.total_iterations * 2
    out["rh_sweep_64"] = {"fp64_plain_layer_steps_per_s": ls / el64, "fp32_batched_layer_steps_per_s": ls / el32,
                          "max_abs_dR_mean_ohm": float(np.max(np.abs(r32 - r64))),
                          "sample": "64 fields x 10,000 steps, R logged every step, mean over the last 2,000"}
    del run
    # The R(H) sweep in full on the FP64 plain form: 64 fields x 10 ns
    # (100,000 RK4 steps), m and R logged every step.  Kernel time alone
    # (CUDA events, best of one after a warm-up launch), and end to end
    # through the public API (lowering, copies, the 512 MB log back, log
    # columns per junction)
    from cmtj_gb300 import tune
    k = tune.time_fp64(64, 100_000, 1, 0)
    js = tune.rh_junctions(64, 1e-8)
    plan = engine.plan_run(1e-8, DT, DT)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.run_junctions(js, plan, batch.SolverMode.RK4)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    out["rh_config0_fp64"] = {"kernel_s": k["best_ms"] / 1e3, "e2e_s": el, "us_per_step": k["us_per_step"],
                              "layer_steps_per_s_kernel": k["layer_steps_per_s"], "all_ok": k["all_ok"],
                              "mean_R_last_2ns": [float(np.mean(j.getLogArrays()["R_free_ref"][-20_000:]))
                                                  for j in js],
                              "logs": rh_logs(js),
                              "sample": "64 fields x 100,000 RK4 steps, log every step"}
    del js
    # The same sweep in the fused FP64 arithmetic (cmtj_arithmetic
    # CMTJ_ARITH_FUSED); its error is set beside how far the reference itself
    # moves when compiled with FMA contraction (tests/golden/rh_fma_spread.npz,
    # made by tests/golden/make_rh_fma.py from both builds of the reference)
    kf = tune.time_fp64(64, 100_000, 1, 0, arithmetic="fused")
    js = tune.rh_junctions(64, 1e-8)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.run_junctions(js, plan, batch.SolverMode.RK4, arithmetic="fused")
    torch.cuda.synchronize()
    elf = time.perf_counter() - t0
    out["rh_config0_fp64"]["fused"] = {
        "kernel_s": kf["best_ms"] / 1e3, "e2e_s": elf, "us_per_step": kf["us_per_step"],
        "layer_steps_per_s_kernel": kf["layer_steps_per_s"], "all_ok": kf["all_ok"], "logs": rh_logs(js),
        "arithmetic": "CMTJ_ARITH_FUSED: H = Hconst + A m, FMA contraction, series normalisation"}
    del js
    # Dormand-Prince: 4096 sine-driven free layers, 5 ns, adaptive steps
    js = dp_junctions(cm)
    plan = engine.plan_run(5e-9, DT, 1e-11)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.run_junctions(js, plan, cm.SolverMode.DormandPrince)
    torch.cuda.synchronize()
    out["dormand_prince_fmr_4096"] = {"seconds": time.perf_counter() - t0, "final_m": final_m(js),
                                      "rows_logged": int(js[0].logLength),
                                      "sample": "4096 free layers under a 2-12 GHz Oersted sine, 5 ns, FP64 "
                                                "plain form, one launch"}
    # dipole-coupled groups (cmtj.reservoir.GroupInteraction): 64 groups of
    # 16 junctions, 2000 steps, one launch
    from cmtj_gb300 import reservoir
    gs = groups_16(cm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reservoir.run_groups(gs, 2e-10, DT, 1e-12)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    out["groups_dipole_64x16"] = {"seconds": el, "layer_steps_per_s": 64 * 16 * 2000 / el,
                                  "final_m": np.concatenate([final_m(g.junctionList) for g in gs]),
                                  "sample": "64 groups of 16 junctions on a 4x4 grid, Kanao dipole coupling, "
                                            "2000 RK4 steps, FP64 plain form, one CTA per group"}
    # PIMM_procedure (the procedure front-end) over 64 junctions x 10 fields,
    # each point one launch for all 64 chains, FP64 plain and FP32 batched
    from cmtj_gb300 import procedures
    leg = {"sample": "PIMM_procedure on a list of 64 two-layer MTJs, 10 fields, 0.5 ns per point"}
    for prec in ("f64", "f32"):
        js, kw = pimm_procedure_case(cm)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = procedures.PIMM_procedure(js, precision=prec, **kw)
        torch.cuda.synchronize()
        leg["seconds_" + prec] = time.perf_counter() - t0
        leg["spectra_" + prec] = np.stack([r[0] for r in res])
    out["pimm_procedure_64x10"] = leg
    # buffered 1/f^alpha noise: the generator alone (3072 buffers of
    # 100,000 samples: one 10 ns run of 1024 noisy layers), and 1024 p-bit
    # layers with thermal noise and alpha noise, 10 ns Euler-Heun on the
    # FP64 plain form through Junction.runSimulation's path
    from cmtj_gb300 import noise
    import thermal_cases
    specs = noise.specs_array([(1.0, 1.0, 77 + r // 3, 0, r % 3) for r in range(3072)])
    noise.device_buffers(specs[:3], 100_000)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    bufs = noise.device_buffers(specs, 100_000)
    b.record()
    torch.cuda.synchronize()
    gen_s = a.elapsed_time(b) / 1e3
    del bufs
    def alpha_junctions():
        js = []
        for k in range(1024):
            j, _ = thermal_cases.pbit_sweep_junction(cm, 1e11, 1e-8)
            j.layers[0].setAlphaNoise(1.0, 1.0, 0.05, cm.Axis.all)
            j.layers[0].noise_seed = 5000 + k
            js.append(j)
        return js

    plan = engine.plan_run(1e-8, DT, 1e-9)
    # an untimed run of the same batch first: it makes the run-time
    # autotuner's lane-layout trials for this batch shape, once
    engine.run_junctions(alpha_junctions(), plan, cm.SolverMode.EulerHeun)
    js = alpha_junctions()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    engine.run_junctions(js, plan, cm.SolverMode.EulerHeun)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    out["alpha_noise_fp64_1024"] = {
        "generator_s_3072x100k": gen_s, "generator_samples_per_s": 3072 * 100_000 / gen_s,
        "run_seconds": el, "layer_steps_per_s": 1024 * plan.total_iterations / el,
        "sample": "1024 p-bit layers (alpha 1, scale 0.05, axis all, plus 300 K), 10 ns Euler-Heun, FP64 plain "
                  "form, buffers generated on the device per run"}
    del js
    # 16-junction series stack, FP64 plain form
    js = [cases._stt_junction(cm, 1.0 + 0.02 * k, 1e3 + 50 * k, (0.1, 0.2, 1), (1, 0, 0)) for k in range(16)]
    s = cm.stack.SeriesStack(js)
    s.setCouplingStrength(0.3)
    s.setCoupledCurrentDriver(cm.constantDriver(5e10))
    steps = 2000
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.runSimulation(steps * DT, DT, DT * 10)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    out["series_stack_16_fp64"] = {"layer_steps_per_s": 16 * steps / el, "seconds": el,
                                   "sample": "16 STT junctions x %d steps, KCL, one CTA" % steps}
    return out


def serving_leg(n_sat=200, sat_rate_hz=200.0, n_requests=1000, loads=(0.5, 0.8, 1.2)):
    """Serving trace (cmtj_gb300.serving, continuous batching): Poisson
    arrivals of requests holding 64-16,384 solves (log-uniform) of three
    kinds -- PIMM-style 2-layer RK4, thermal 1-layer p-bit Euler-Heun at
    300 K, uneven 1-4-layer spin-diode RK4 with on-device <I R> -- each
    solve 2-40 ns at dt = 1e-13, 5 % of requests FP64 plain.

    1. Capacity: 200 requests at 200 req/s (about 3x overload), shortest
       job first and FIFO; the delivered layer-steps/s is the capacity.
    2. Latency against load: 1000 requests at 0.5, 0.8 and 1.2 x that
       capacity (arrival rate = load x capacity / mean request size).
    3. FP64 plain alone, measured: 8 sampled FP32 requests of the 0.8 x run,
       each run alone on the FP64 plain form (all its solves, one launch,
       for 2000 steps, scaled to its longest solve), beside the same request
       run alone on the FP32 form and its latency in the mix.
    Latency = completion minus arrival, wall clock."""
    from cmtj_gb300 import serving
    f64_fraction = 0.05
    out = {}
    fifo = serving.ServingEngine(hbm_budget_bytes=8 << 30, chunk_steps=4000, policy="fifo")
    t0 = time.perf_counter()
    done_fifo = fifo.run(serving.make_trace(n_sat, rate_hz=sat_rate_hz, seed=3, f64_fraction=f64_fraction))
    fifo_summary = serving.summary(done_fifo, time.perf_counter() - t0)
    eng = serving.ServingEngine(hbm_budget_bytes=8 << 30, chunk_steps=4000, policy="sjf")
    t0 = time.perf_counter()
    done = eng.run(serving.make_trace(n_sat, rate_hz=sat_rate_hz, seed=3, f64_fraction=f64_fraction))
    sat = serving.summary(done, time.perf_counter() - t0)
    offered = sum(r.layer_steps for r in done)
    capacity = sat["layer_steps_per_s"]
    out["saturated"] = dict(sat, policy="sjf: smallest layer-steps first among arrived requests",
                            fifo={k: fifo_summary[k] for k in ("p50_ms", "p99_ms", "layer_steps_per_s", "wall_s")},
                            offered_over_span=offered / max(done[-1].arrival, 1e-9),
                            trace="%d requests, Poisson %.0f req/s" % (n_sat, sat_rate_hz),
                            ticks=eng.stats["ticks"], host_s=eng.stats["host_s"])
    probe = serving.make_trace(400, rate_hz=1.0, seed=11, f64_fraction=f64_fraction)
    mean_ls = float(np.mean([serving._work_estimate(r) for r in probe]))
    curve, mid = [], None
    for q, load in enumerate(loads):
        rate = load * capacity / mean_ls
        reqs = serving.make_trace(n_requests, rate_hz=rate, seed=20 + q, f64_fraction=f64_fraction)
        e = serving.ServingEngine(hbm_budget_bytes=8 << 30, chunk_steps=4000, policy="sjf")
        t0 = time.perf_counter()
        d = e.run(reqs)
        wall = time.perf_counter() - t0
        lat = np.array([r.latency for r in d]) * 1e3
        ls = sum(r.layer_steps for r in d)
        curve.append({"load": load, "rate_hz": rate, "requests": len(d),
                      "offered_layer_steps_per_s": ls / max(d[-1].arrival, 1e-9),
                      "delivered_layer_steps_per_s": ls / wall, "p50_ms": float(np.percentile(lat, 50)),
                      "p90_ms": float(np.percentile(lat, 90)), "p99_ms": float(np.percentile(lat, 99)),
                      "max_ms": float(np.max(lat)), "wall_s": wall})
        if abs(load - 0.8) < 1e-9:
            mid = d
    out["latency_vs_load"] = {"capacity_layer_steps_per_s": capacity, "mean_request_layer_steps": mean_ls,
                              "points": curve, "policy": "sjf"}
    out["fp64_alone"] = fp64_alone_sample(mid if mid is not None else done)
    return out


def request_junctions(req):
    """Junction objects equal to the solves of an FP32 serving request."""
    import cmtj_gb300 as cm
    import thermal_cases
    from cases import junctions_from_spec
    sp = req.spec
    if req.tag == "pimm":
        return spec_to_junctions(sp)
    if req.tag == "pbit":
        out = []
        for k in range(sp.n):
            j, _ = thermal_cases.pbit_sweep_junction(cm, float(sp.wave_table["amp"][k, 0]), 1e-9)
            j.layers[0].noise_seed = int(sp.seed[k, 0])
            out.append(j)
        return out
    return junctions_from_spec(sp, range(sp.n), lambda k: cm.AxialDriver(
        cm.NullDriver(), cm.sineDriver(0, float(sp.wave_table["amp"][k, 0]), float(sp.vsd_freq[k]), 0),
        cm.NullDriver()))


def fp64_alone_sample(done, n_sample=8, probe_steps=2000, seed=4):
    """Eight FP32 requests of a served trace, each run alone: on the FP64
    plain form (all its solves in one launch, logging what its result
    needs -- R every step for the spin-diode kind, the final state
    otherwise), timed over probe_steps and scaled to its longest solve; and
    on the FP32 batched form through a fresh serving engine.  The smallest
    sampled request also runs in full on the FP64 form, to check the
    scaling."""
    import torch
    import cmtj_gb300 as cm
    from cmtj_gb300 import engine, serving
    rng = np.random.default_rng(seed)
    f32 = [r for r in done if r.precision == "f32"]
    pick = sorted(rng.choice(len(f32), min(n_sample, len(f32)), replace=False).tolist(),
                  key=lambda i: f32[i].layer_steps)
    rows = []
    for q, i in enumerate(pick):
        req = f32[i]
        steps = np.broadcast_to(np.asarray(req.n_steps), (req.spec.n,))
        mode = cm.SolverMode.EulerHeun if req.tag == "pbit" else cm.SolverMode.RK4
        every = 1 if req.tag == "vsd" else probe_steps
        js = request_junctions(req)
        plan = engine.plan_run(probe_steps * DT, DT, every * DT)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        engine.run_junctions(js, plan, mode)
        torch.cuda.synchronize()
        t64 = (time.perf_counter() - t0) * float(steps.max()) / probe_steps
        full = None
        if q == 0 and req.tag != "vsd" and req.layer_steps <= 2e9:
            js = request_junctions(req)
            plan = engine.plan_run(float(steps.max()) * DT, DT, float(steps.max()) * DT)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            engine.run_junctions(js, plan, mode)
            torch.cuda.synchronize()
            full = time.perf_counter() - t0
        alone = serving.Request(spec=req.spec, n_steps=req.n_steps, solver=req.solver, tag=req.tag,
                                red_every=req.red_every, arrival=0.0)
        e = serving.ServingEngine(hbm_budget_bytes=8 << 30, chunk_steps=4000, policy="sjf")
        t0 = time.perf_counter()
        e.run([alone])
        t32 = time.perf_counter() - t0
        rows.append({"kind": req.tag, "solves": int(req.spec.n), "layer_steps": float(req.layer_steps),
                     "fp64_alone_s": t64, "fp64_alone_full_run_s": full, "fp32_alone_s": t32,
                     "latency_in_mix_s": float(req.latency),
                     "fp64_alone_over_latency_in_mix": t64 / float(req.latency)})
    ratios = [r["fp64_alone_over_latency_in_mix"] for r in rows]
    return {"requests": rows, "median_fp64_alone_over_latency_in_mix": float(np.median(ratios)),
            "median_fp64_alone_over_fp32_alone": float(np.median([r["fp64_alone_s"] / r["fp32_alone_s"]
                                                                  for r in rows])),
            "method": "FP64 plain form, all solves of the request in one launch, %d steps timed and scaled to "
                      "the longest solve (fp64_alone_full_run_s: the smallest request run in full)" % probe_steps}


def spec_to_junctions_rows(spec, rows):
    """Junction objects for the given rows of the PIMM spec, starting from
    the spec's m0 exactly (no renormalisation)."""
    import cmtj_gb300 as cm
    import cases
    out = []
    for k in rows:
        j, _ = cases.mtj_rh_point(cm, hx=float(spec.Hc[k, 0, 0]), total=1e-9)
        for l in range(2):
            j.layers[l].mag = cm.CVector(*spec.m0[k, l])
        j.setLayerAnisotropyDriver("free", cm.constantDriver(float(spec.K[k, 0])))
        j.setIECDriver("free", "ref", cm.constantDriver(float(spec.Jt[k, 0])))
        j.setLayerOerstedFieldDriver("all", cm.AxialDriver(cm.stepDriver(0, 1e3, 0, 1e-12), cm.NullDriver(),
                                                            cm.NullDriver()))
        out.append(j)
    return out


if __name__ == "__main__":
    main()
