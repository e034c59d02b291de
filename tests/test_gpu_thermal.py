"""Stochastic parity on the GPU: switching statistics of the FP32 batched
and FP64 plain forms against the reference (3-sigma binomial bound), the
FP64 GPU path against the oracle under identical Philox noise (pathwise),
and the Boltzmann m_z density from the FP32 form."""
import numpy as np
import pytest

import cmtj_gb300
import oracle_harness
import thermal_cases
from cmtj_gb300 import batch, engine
from test_thermal import binomial_ok, check_density, load_ref, seeded_pbits


@pytest.mark.gpu
def test_fp32_batch_switching_matches_reference(gpu_lib):
    cur, sw, runs = load_ref()
    n = 8192
    js, counts = [], []
    for q, jd in enumerate(cur):
        part, run = seeded_pbits(cmtj_gb300, float(jd), n, 10_000_000 + 100_000 * q)
        js += part
    spec = batch.BatchSpec.from_junctions(js)
    plan = engine.plan_run(run["totalTime"], run["timeStep"], run["writeFrequency"])
    low = batch.lower(spec, plan.time_step, plan.total_iterations)
    r = batch.BatchRun(low, plan.time_step, cmtj_gb300.SolverMode.EulerHeun)
    r.launch()
    st = r.state()
    assert np.all(st["status"] == 0)
    mz = st["m"][:, 0, 2]
    for q, jd in enumerate(cur):
        k = int(np.sum(mz[q * n:(q + 1) * n] < 0))
        ok, d, b = binomial_ok(k, n, int(sw[q]), int(runs[q]))
        assert ok, (jd, k / n, sw[q] / runs[q], d, b)


@pytest.mark.gpu
def test_fp64_plain_switching_matches_reference(gpu_lib):
    cur, sw, runs = load_ref()
    n = 1024
    js = []
    for q, jd in enumerate(cur):
        part, run = seeded_pbits(cmtj_gb300, float(jd), n, 20_000_000 + 100_000 * q)
        js += part
    plan = engine.plan_run(run["totalTime"], run["timeStep"], run["writeFrequency"])
    engine.run_junctions(js, plan, cmtj_gb300.SolverMode.EulerHeun)
    for q, jd in enumerate(cur):
        k = sum(1 for j in js[q * n:(q + 1) * n] if j.getLayerMagnetisation("free").z < 0)
        ok, d, b = binomial_ok(k, n, int(sw[q]), int(runs[q]))
        assert ok, (jd, k / n, sw[q] / runs[q], d, b)


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["EulerHeun", "Heun"])
def test_fp64_gpu_equals_oracle_under_same_noise(gpu_lib, solver):
    """Same Philox stream on both sides: trajectories agree to 1e-9 over
    2000 steps (differences come only from CUDA vs glibc log/sin/cos)."""
    mode = getattr(cmtj_gb300.SolverMode, solver)
    a, _ = seeded_pbits(cmtj_gb300, 8e10, 4, 4242)
    b, _ = seeded_pbits(oracle_harness.oracle_module(), 8e10, 4, 4242)
    for j in a:
        j.runSimulation(2e-10, 1e-13, 1e-12, solverMode=mode)
    for j in b:
        j.runSimulation(2e-10, 1e-13, 1e-12, solverMode=mode)
    for x, y in zip(a, b):
        la, lb = x.getLogArrays(), y.getLogArrays()
        for k in ("free_mx", "free_my", "free_mz"):
            assert np.max(np.abs(la[k] - lb[k])) <= 1e-9, (k, np.max(np.abs(la[k] - lb[k])))


@pytest.mark.gpu
def test_fp32_batch_boltzmann_equilibrium(gpu_lib):
    V = 7e-17 * 1.2e-9
    Ku = 1.5 * 1.380649e-23 * 300 / V
    js = []
    for k in range(4096):
        j, _ = thermal_cases.pbit_junction(cmtj_gb300, 0.0, Ku=Ku)
        j.layers[0].noise_seed = 555 + k
        if k % 2:
            j.setLayerMagnetisation("free", cmtj_gb300.CVector(0, 0, -1))  # both wells start populated
        js.append(j)
    spec = batch.BatchSpec.from_junctions(js)
    # intra-well relaxation takes 1/(alpha gamma Hk) ~ 1.5 ns: 2 ns burn-in, 10 ns sampled
    low = batch.lower(spec, 1e-13, 120000)
    r = batch.BatchRun(low, 1e-13, cmtj_gb300.SolverMode.EulerHeun, batch.LOG_M, 200)
    r.launch()
    log = r.d_log.cpu().numpy()
    mz = np.concatenate([r.log_of(k, log)[100:, 2] for k in range(len(js))])
    check_density(mz, Ku, V)


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["EulerHeun", "Heun"])
def test_fp32_and_fp64_forms_share_the_noise_stream(gpu_lib, solver):
    """The same seeded p-bit junctions, 300 Euler-Heun (or Heun) steps at
    300 K, in the FP32 batched form and the FP64 plain form: the same Philox
    words drive both, so the trajectories agree to the FP32 bound.
    Independent (or sign-flipped) noise would leave them about 1e-2 apart."""
    mode = getattr(cmtj_gb300.SolverMode, solver)
    a, run = seeded_pbits(cmtj_gb300, 8e10, 32, 31337)
    b, _ = seeded_pbits(cmtj_gb300, 8e10, 32, 31337)
    steps, dt = 300, run["timeStep"]
    spec = batch.BatchSpec.from_junctions(a)
    r = batch.BatchRun(batch.lower(spec, dt, steps), dt, mode)
    r.launch()
    st = r.state()
    assert np.all(st["status"] == 0)
    engine.run_junctions(b, engine.plan_run(steps * dt, dt, 10 * dt), mode)
    m32 = st["m"][:, 0, :].astype(np.float64)
    m64 = np.array([[j.layers[0].mag.x, j.layers[0].mag.y, j.layers[0].mag.z] for j in b])
    m0 = np.array([[j.layers[0].mag.x, j.layers[0].mag.y, j.layers[0].mag.z] for j in seeded_pbits(
        cmtj_gb300, 8e10, 32, 31337)[0]])
    assert np.max(np.abs(m64 - m0)) > 1e-2  # the noise moved m
    assert np.max(np.abs(m32 - m64)) <= 1e-4, np.max(np.abs(m32 - m64))


@pytest.mark.gpu
def test_fp32_batch_full_pbit_sweep_matches_reference(gpu_lib):
    """The whole stochastic p-bit sweep in the FP32 batched form: 64 current
    densities over [0, 5e11] A/m^2 x 16,384 single-layer STT junctions
    (1,048,576), Ku 2.5e5 J/m^3, Euler-Heun at 300 K, each junction's
    duration drawn from U[5, 20] ns.  At the 17 currents the reference ran
    (2048 runs each, tests/golden/pbit_sweep.npz), P(m_z < 0 at the end) is
    within the 3-sigma binomial bound; |m| stays 1 to FP32 rounding."""
    from cmtj_gb300 import sweeps
    from test_thermal import load_sweep_ref
    dt = 1e-13
    spec, n_steps, jd = sweeps.pbit_config(dt=dt)
    run = batch.BatchRun(batch.lower(spec, dt, n_steps), dt, cmtj_gb300.SolverMode.EulerHeun)
    run.launch()
    st = run.state()
    assert np.all(st["status"] == 0) and np.all(st["step"] == n_steps)
    m = st["m"][:, 0, :].astype(np.float64)
    assert np.max(np.abs(np.linalg.norm(m, axis=1) - 1)) <= 1e-6
    cur, sw, runs = load_sweep_ref()
    for q, c in enumerate(cur):
        sel = jd == c
        n = int(sel.sum())
        assert n == 16384, c
        k = int(np.sum(m[sel, 2] < 0))
        ok, d, b = binomial_ok(k, n, int(sw[q]), int(runs[q]))
        assert ok, (c, k / n, sw[q] / runs[q], d, b)


def _run_f64_rows(js, plan, solver, every_rows):
    """The FP64 plain form on `js`, returning only log rows every_rows[k] of
    junction k (gathered on the device)."""
    from cmtj_gb300 import _abi
    t = engine.torch()
    lib = engine.require_gpu()
    low = engine.lower(js, plan, solver, False)
    n, p = len(js), low.params
    n_log, width = int(p["n_log"][0]), low.log_width
    d_j, d_l = engine.to_device(low.junctions), engine.to_device(low.layers)
    d_tab = engine.to_device(low.tables) if low.tables is not None else None
    d_log = t.empty((n, n_log, width), dtype=t.float64, device="cuda")
    d_status = t.zeros(2 * n, dtype=t.int32, device="cuda")
    _abi.check(lib.cmtj_run_simulation_f64(engine.ptr(d_j), n, engine.ptr(d_l), engine.ptr(d_tab), p.ctypes.data,
                                           engine.ptr(d_log), engine.ptr(d_status), engine.stream_ptr()), lib)
    idx = t.from_numpy(np.asarray(every_rows, dtype=np.int64)).cuda()
    rows = d_log[t.arange(n, device="cuda"), idx].cpu().numpy()
    return rows, d_status.cpu().numpy().view(np.uint32)


@pytest.mark.gpu
def test_fp64_plain_full_pbit_sweep_matches_reference(gpu_lib):
    """The FP64 plain form on the same 17 currents of the full p-bit sweep,
    512 runs each with their own U[5, 20] ns durations, in one launch of
    the longest duration logged every 100 steps: a run of n steps is read
    from the last log row at or before its end (the state after
    100 * floor((n - 1) / 100) + 1 steps, at most 10 ps early).  P(m_z < 0)
    is within the 3-sigma binomial bound of the reference's counts."""
    from test_thermal import load_sweep_ref
    cur, sw, runs = load_sweep_ref()
    dt, every, n = 1e-13, 100, 512
    js, last = [], []
    for q, c in enumerate(cur):
        for k, d in enumerate(thermal_cases.sweep_durations(n, 900 + q)):
            j, _ = thermal_cases.pbit_sweep_junction(cmtj_gb300, float(c), d)
            j.layers[0].noise_seed = 40_000_000 + 100_000 * q + k
            js.append(j)
            last.append((int(d / dt) - 1) // every)
    plan = engine.plan_run(thermal_cases.SWEEP_T_MAX, dt, every * dt)
    rows, status = _run_f64_rows(js, plan, cmtj_gb300.SolverMode.EulerHeun, last)
    assert np.all(status[0::2] == 0)
    mz = rows[:, 2]
    for q, c in enumerate(cur):
        k = int(np.sum(mz[q * n:(q + 1) * n] < 0))
        ok, d, b = binomial_ok(k, n, int(sw[q]), int(runs[q]))
        assert ok, (c, k / n, sw[q] / runs[q], d, b)
