"""Buffered 1/f^alpha noise on the GPU: cmtj_alpha_noise_f32 against the
reference's own buffers (same white draws) and against the oracle's
restatement (same Philox draws), its statistics, and the FP64 plain form's
Euler-Heun and Heun runs with alpha noise against the oracle fed the same
buffers (pathwise, 1e-9)."""
import numpy as np
import pytest

import cmtj_gb300 as cm
import oracle_harness
from cmtj_gb300 import _abi, engine, noise
from cmtj_gb300.noise import specs_array
from test_alpha_noise import GOLDEN, _weights


def _buffers(specs, n, white=None, scratch_rows=None):
    """cmtj_alpha_noise_f32 through the C ABI, with scratch for
    `scratch_rows` rows at a time (all rows when None)."""
    t = engine.torch()
    lib = engine.require_gpu()
    rows = len(specs)
    per_row = int(lib.cmtj_alpha_noise_scratch_bytes(n))
    k = rows if scratch_rows is None else scratch_rows
    scratch = t.empty(k * per_row, dtype=t.uint8, device="cuda")
    out = t.full((rows, n), float("nan"), dtype=t.float32, device="cuda")
    d_specs = engine.to_device(specs)
    d_white = None if white is None else t.from_numpy(np.ascontiguousarray(white, dtype=np.float32)).cuda()
    rc = lib.cmtj_alpha_noise_f32(engine.ptr(d_specs), rows, n, engine.ptr(d_white), engine.ptr(out),
                                  engine.ptr(scratch), k * per_row, engine.stream_ptr())
    _abi.check(rc, lib)
    return out.cpu().numpy()


@pytest.mark.gpu
def test_device_fill_matches_reference_buffers(gpu_lib):
    """The reference's white draws in, the reference's buffers out, within
    the float rounding of the FFT convolution (n = 1 to 1537, alpha 0-2)."""
    g = np.load(GOLDEN)
    for k, (n, alpha, std) in enumerate(g["cases"]):
        n = int(n)
        ref = g["out_%d" % k]
        got = _buffers(specs_array([(alpha, std, 0, 0, 0)]), n, white=g["white_%d" % k][None, :])[0]
        tol = 2e-6 * max(float(np.max(np.abs(ref))), 1e-30)
        assert np.max(np.abs(got - ref)) <= tol, (n, alpha, float(np.max(np.abs(got - ref))), tol)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [3, 1000, 100_000])
def test_device_fill_matches_oracle_on_philox_draws(gpu_lib, n):
    """Philox white draws on both sides (several seeds, counters and
    components; scratch for two rows at a time, so rows go in batches):
    the device buffers equal the oracle's FP64 restatement to float
    rounding."""
    specs = specs_array([(a, s, 1000 + r, 77 * r, r % 3) for r, (a, s) in
                         enumerate([(0.0, 1.0), (0.5, 0.3), (1.0, 1.0), (1.5, 2.0), (2.0, 1.0)])])
    got = _buffers(specs, n, scratch_rows=2)
    want = oracle_harness.alpha_buffers(specs, n)
    for r in range(len(specs)):
        scale = max(float(np.max(np.abs(want[r]))), 1e-30)
        tol = (2e-6 if n <= 1000 else 1e-5) * scale
        assert np.max(np.abs(got[r] - want[r])) <= tol, (n, r, float(np.max(np.abs(got[r] - want[r]))), tol)


@pytest.mark.gpu
def test_device_fill_statistics(gpu_lib):
    """Variance along the buffer follows std^2 sum_{j<=m} h_j^2 and the
    periodogram falls as 1/f^alpha, on 1536 device buffers."""
    n, rows, std = 4096, 512, 0.5
    for alpha in (0.5, 1.0, 1.5):
        specs = specs_array([(alpha, std, 31337, 10_000 * r, r % 3) for r in range(rows)])
        buf = _buffers(specs, n).astype(np.float64)
        h = _weights(n, alpha)
        theory = std ** 2 * np.cumsum(h * h)
        for lo, hi in ((64, 512), (512, 4096)):
            v, t = float(np.mean(buf[:, lo:hi] ** 2)), float(np.mean(theory[lo:hi]))
            assert abs(v / t - 1) < 0.12, (alpha, lo, hi, v, t)
        p = np.mean(np.abs(np.fft.rfft(buf - buf.mean(axis=1, keepdims=True), axis=1)) ** 2, axis=0)
        f = np.arange(p.size)
        sel = (f >= 32) & (f <= n // 16)
        slope = np.polyfit(np.log(f[sel]), np.log(p[sel]), 1)[0]
        assert abs(slope + alpha) < 0.1, (alpha, slope)


@pytest.mark.gpu
def test_device_fill_rejects_bad_sizes(gpu_lib):
    lib = engine.require_gpu()
    assert lib.cmtj_alpha_noise_scratch_bytes(0) == 0
    assert lib.cmtj_alpha_noise_scratch_bytes(_abi.ALPHA_MAX_LEN + 1) == 0
    t = engine.torch()
    scratch = t.empty(1024, dtype=t.uint8, device="cuda")
    d_specs = engine.to_device(specs_array([(1.0, 1.0, 0, 0, 0)]))
    out = t.empty(4096, dtype=t.float32, device="cuda")
    rc = lib.cmtj_alpha_noise_f32(engine.ptr(d_specs), 1, 4096, None, engine.ptr(out), engine.ptr(scratch), 1024,
                                  engine.stream_ptr())
    assert rc == _abi.CMTJ_ERR_LIMIT and "holds no buffer row" in _abi.last_error(lib)


def _mtj(alpha_axis, T, seed):
    """A 2-layer MTJ (free layer with alpha noise, optionally both layers at
    temperature T) under a small in-plane field."""
    demag = [cm.CVector(0.0024, 0, 0), cm.CVector(0, 0.0024, 0), cm.CVector(0, 0, 0.9952)]
    free = cm.Layer("free", cm.CVector(0, 0.1, 0.99), cm.CVector(0, 0, 1), 1.2, 1.5e-9, 1e-16, demag, 0.01)
    ref = cm.Layer("ref", cm.CVector(0, 0, 1), cm.CVector(0, 0, 1), 1.5, 2e-9, 1e-16, demag, 0.01)
    free.setAlphaNoise(1.0, 1.0, 0.05, alpha_axis)
    free.noise_seed, ref.noise_seed = seed, seed + 1
    j = cm.Junction([free, ref], 100, 200)
    j.setLayerAnisotropyDriver("free", cm.constantDriver(3e5))
    j.setLayerAnisotropyDriver("ref", cm.constantDriver(1e6))
    j.setIECDriver("free", "ref", cm.constantDriver(-5e-5))
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(2e4, 0, 0))
    if T:
        j.setLayerTemperatureDriver("all", cm.constantDriver(T))
    return j


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["EulerHeun", "Heun"])
@pytest.mark.parametrize("axis,T", [(cm.Axis.all, 0.0), (cm.Axis.all, 300.0), (cm.Axis.xaxis, 300.0)])
def test_fp64_runs_with_alpha_noise_match_oracle(gpu_lib, solver, axis, T):
    """Runs of 3000 steps through Junction.runSimulation on the GPU against
    the oracle given the same buffers (the generator is deterministic, so
    the same records give the same bits): trajectories agree to 1e-9."""
    mode = getattr(cm.SolverMode, solver)
    steps, dt = 3000, 1e-13
    gpu = [_mtj(axis, T, 900 + k) for k in range(3)]
    cpu = [_mtj(axis, T, 900 + k) for k in range(3)]
    plan = engine.plan_run(steps * dt, dt, 10 * dt)
    low = engine.lower(cpu, plan, mode, False)
    n = int(low.layers[low.alpha_layers[0]]["alpha_len"])
    bufs = noise.fill_buffers(low.alpha_specs, n)
    engine.run_junctions(gpu, plan, mode)
    oracle_harness.ALPHA_OVERRIDE = bufs
    oracle_harness.run_oracle(cpu, steps * dt, dt, 10 * dt, solverMode=mode)
    moved = 0.0
    for a, b in zip(gpu, cpu):
        la, lb = a.getLogArrays(), b.getLogArrays()
        for k in ("free_mx", "free_my", "free_mz", "ref_mx", "ref_my", "ref_mz"):
            assert np.max(np.abs(la[k] - lb[k])) <= 1e-9, (k, float(np.max(np.abs(la[k] - lb[k]))))
        moved = max(moved, float(np.max(np.abs(la["free_my"] - la["free_my"][0]))))
    assert moved > 1e-3  # the noise moved m


@pytest.mark.gpu
def test_fp64_alpha_noise_switching_matches_reference(gpu_lib):
    """The FP64 plain form on every alpha-noise p-bit case (alpha 0.5-1.5,
    scale 0.01-0.03, axis all or x, with and without 300 K), 1024 runs
    each in one launch: P(m_z < 0) within the 3-sigma binomial bound of the
    reference's counts (its BufferedAlphaNoise on mt19937)."""
    import thermal_cases
    from test_thermal import binomial_ok, load_alpha_ref
    cases, sw, runs = load_alpha_ref()
    n = 1024
    js = []
    for q, case in enumerate(thermal_cases.ALPHA_CASES):
        for k in range(n):
            j, run = thermal_cases.alpha_pbit_junction(cm, *case)
            j.layers[0].noise_seed = 7_000_000 + 100_000 * q + k
            js.append(j)
    plan = engine.plan_run(run["totalTime"], run["timeStep"], run["writeFrequency"])
    engine.run_junctions(js, plan, cm.SolverMode.EulerHeun)
    for q, case in enumerate(thermal_cases.ALPHA_CASES):
        k = sum(1 for j in js[q * n:(q + 1) * n] if j.getLayerMagnetisation("free").z < 0)
        ok, d, b = binomial_ok(k, n, int(sw[q]), int(runs[q]))
        assert ok, (case, k / n, sw[q] / runs[q], d, b)


@pytest.mark.gpu
def test_noise_module_classes(gpu_lib):
    """cmtj.noise (python/cmtj.cpp:448-462): BufferedAlphaNoise.tick walks
    the device buffer times its scale and draws a new buffer when it wraps;
    VectorAlphaNoise.tickVector is the normalised sample vector times the
    scale for Axis.all (one axis otherwise) and keeps the previous sample;
    Layer.getOneFVector ticks the layer's buffered noise."""
    import cmtj
    b = cmtj.noise.BufferedAlphaNoise(64, 1.0, 2.0, 3.0)
    first = [b.tick() for _ in range(64)]
    buf = b.getFullBuffer()
    assert np.allclose(first, 3.0 * buf.astype(np.float64))
    second = [b.tick() for _ in range(64)]
    assert not np.allclose(first, second)  # a fresh buffer after the wrap
    v = cmtj.noise.VectorAlphaNoise(32, 1.0, 1.0, 0.5, cm.Axis.all)
    prev = None
    for _ in range(40):
        s = v.tickVector()
        assert abs(s.length() - 0.5) < 1e-12
        if prev is not None:
            assert v.getPrevSample().tolist() == [x / 0.5 for x in prev.tolist()]
        prev = s
    z = cmtj.noise.VectorAlphaNoise(32, 1.0, 1.0, 2.0, cm.Axis.zaxis)
    s = z.tickVector()
    assert s.x == 0.0 and s.y == 0.0 and s.z != 0.0
    demag = [cm.CVector(0, 0, 0)] * 3
    layer = cm.Layer("free", cm.CVector(0, 0, 1), cm.CVector(0, 0, 1), 1.0, 1e-9, 1e-16, demag, 0.01)
    layer.setAlphaNoise(1.0, 1.0, 0.25)
    layer.createBufferedAlphaNoise(16)
    assert abs(layer.getOneFVector().length() - 0.25) < 1e-12
