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
def test_fp32_and_fp64_forms_share_the_noise_stream(gpu_lib):
    """The same seeded p-bit junctions, 300 Euler-Heun steps at 300 K, in the
    FP32 batched form and the FP64 plain form: the same Philox words drive
    both, so the trajectories agree to the FP32 bound.  Independent (or
    sign-flipped) noise would leave them about 1e-2 apart."""
    a, run = seeded_pbits(cmtj_gb300, 8e10, 32, 31337)
    b, _ = seeded_pbits(cmtj_gb300, 8e10, 32, 31337)
    steps, dt = 300, run["timeStep"]
    spec = batch.BatchSpec.from_junctions(a)
    r = batch.BatchRun(batch.lower(spec, dt, steps), dt, cmtj_gb300.SolverMode.EulerHeun)
    r.launch()
    st = r.state()
    assert np.all(st["status"] == 0)
    engine.run_junctions(b, engine.plan_run(steps * dt, dt, 10 * dt), cmtj_gb300.SolverMode.EulerHeun)
    m32 = st["m"][:, 0, :].astype(np.float64)
    m64 = np.array([[j.layers[0].mag.x, j.layers[0].mag.y, j.layers[0].mag.z] for j in b])
    m0 = np.array([[j.layers[0].mag.x, j.layers[0].mag.y, j.layers[0].mag.z] for j in seeded_pbits(
        cmtj_gb300, 8e10, 32, 31337)[0]])
    assert np.max(np.abs(m64 - m0)) > 1e-2  # the noise moved m
    assert np.max(np.abs(m32 - m64)) <= 1e-4, np.max(np.abs(m32 - m64))
