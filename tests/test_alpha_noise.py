"""Buffered 1/f^alpha noise (core/noise.hpp:138-308, junction.hpp:406-424,
1130-1136, 1891-1931) on the CPU: the oracle's restatement of
BufferedAlphaNoise::fillBuffer against the reference's own buffers
(tests/golden/alpha_noise.npz, recorded with their white draws), the
buffers' statistics, and how the Euler-Heun and Heun runners consume them
(getOneFVector: the normalised sample vector times the scale, added to the
thermal dW)."""
import numpy as np
import pytest

import cmtj_gb300 as cm
import oracle_harness
from cmtj_gb300 import _abi
from cmtj_gb300.noise import specs_array

GOLDEN = "%s/golden/alpha_noise.npz" % oracle_harness.__file__.rsplit("/", 1)[0]


def _spec(alpha, std, seed=0, counter=0, component=0):
    return specs_array([(alpha, std, seed, counter, component)])


def test_oracle_fill_matches_reference_buffers():
    """Given the reference's white draws, the restatement reproduces the
    reference's buffers to float rounding, from n = 1 (its one bin halved
    twice) to n = 1537 (odd, not a power of two), alpha 0 to 2."""
    g = np.load(GOLDEN)
    for k, (n, alpha, std) in enumerate(g["cases"]):
        n = int(n)
        ref = g["out_%d" % k]
        got = oracle_harness.alpha_buffers(_spec(alpha, std), n, white=g["white_%d" % k][None, :])[0]
        tol = 4e-7 * max(float(np.max(np.abs(ref))), 1e-30)
        assert np.max(np.abs(got - ref)) <= tol, (n, alpha, np.max(np.abs(got - ref)), tol)


def _weights(n, alpha):
    h = np.zeros(n, np.float64)
    h[0] = 1.0
    for i in range(1, n):
        h[i] = h[i - 1] * np.float32(np.float32(0.5 * alpha + np.float32(i - 1)) / np.float32(i))
    return h


def test_oracle_fill_variance_follows_the_filter():
    """Philox white draws: the variance of sample m over many buffers is
    std^2 sum_{j<=m} h_j^2 (the causal filter; the top-bin term is of
    order std / sqrt(n)), within sampling error, for alpha 0.5, 1, 1.5."""
    n, rows, std = 512, 768, 0.7
    for alpha in (0.5, 1.0, 1.5):
        specs = specs_array([(alpha, std, 99, 1000 * r, r % 3) for r in range(rows)])
        buf = oracle_harness.alpha_buffers(specs, n).astype(np.float64)
        h = _weights(n, alpha)
        theory = std ** 2 * np.cumsum(h * h)
        for lo, hi in ((16, 64), (64, 256), (256, 512)):
            v = float(np.mean(buf[:, lo:hi] ** 2))
            t = float(np.mean(theory[lo:hi]))
            # chi-square of `rows` draws per sample, correlated along m
            assert abs(v / t - 1) < 0.15, (alpha, lo, hi, v, t)


def test_oracle_fill_spectrum_slope_is_minus_alpha():
    """The averaged periodogram of the buffers falls as 1/f^alpha over the
    middle of the band (the Kasdin filter's design)."""
    n, rows = 2048, 96
    for alpha in (0.5, 1.0, 1.5):
        specs = specs_array([(alpha, 1.0, 7, 5000 * r, 0) for r in range(rows)])
        buf = oracle_harness.alpha_buffers(specs, n).astype(np.float64)
        p = np.mean(np.abs(np.fft.rfft(buf - buf.mean(axis=1, keepdims=True), axis=1)) ** 2, axis=0)
        f = np.arange(p.size)
        sel = (f >= 16) & (f <= n // 16)
        slope = np.polyfit(np.log(f[sel]), np.log(p[sel]), 1)[0]
        assert abs(slope + alpha) < 0.15, (alpha, slope)


def test_set_alpha_noise_checks_range_and_forces_euler_heun(capsys):
    z = cm.CVector(0, 0, 0)
    l = cm.Layer("free", cm.CVector(0, 0, 1), cm.CVector(0, 0, 1), 1.0, 1e-9, 1e-16, [z, z, z], 0.02)
    with pytest.raises(RuntimeError, match="alpha must be between 0 and 2"):
        l.setAlphaNoise(2.5, 1.0, 1.0)
    l.setAlphaNoise(1.0, 1.0, 0.5)
    j = cm.Junction([l])
    assert j.getSolver(cm.SolverMode.RK4) == cm.SolverMode.EulerHeun
    assert j.getSolver(cm.SolverMode.Heun) == cm.SolverMode.Heun
    assert "Solver automatically changed to Euler Heun" in capsys.readouterr().out
    with pytest.raises(RuntimeError, match="createBufferedAlphaNoise"):
        l.getOneFVector()
    l2 = cm.Layer("x", cm.CVector(0, 0, 1), cm.CVector(0, 0, 1), 1.0, 1e-9, 1e-16, [z, z, z], 0.02)
    assert l2.getOneFVector().tolist() == [0.0, 0.0, 0.0]  # scale 0: no noise


def _free_layer(alpha_axis=cm.Axis.all, scale=0.05, T=None, seed=4321):
    """A layer with no field at all (no anisotropy, demag or drivers), so the
    Euler-Heun step is the stochastic torque alone."""
    z = cm.CVector(0, 0, 0)
    l = cm.Layer("free", cm.CVector(0.6, 0, 0.8), cm.CVector(0, 0, 1), 1.0, 1.2e-9, 7e-17, [z, z, z], 0.02)
    l.setAlphaNoise(1.0, 1.0, scale, alpha_axis)
    if T is not None:
        l.setTemperatureDriver(cm.constantDriver(T))
    l.noise_seed = seed
    return l


def _euler_heun_by_hand(m, samples, scale, axis, damping, gyro, dt):
    """eulerHeunSolverStep (junction.hpp:1709-1754) for a layer with no
    field: dW = getOneFVector (the normalised sample times the scale, or the
    one axis), m' = normalise(m + (g(m) + g(m + g(m) sqrt dt)) sqrt dt / 2)."""
    conv = -gyro / (1 + damping ** 2)

    def g(m, dW):
        th = np.cross(m, dW)
        return (th + np.cross(m, th) * damping) * conv
    out = []
    for s in samples:
        v = np.zeros(3)
        if axis == 3:
            v = s.astype(np.float64)
            v = v / np.sqrt(v @ v)
        else:
            v[axis] = float(s[axis])
        dW = v * scale
        g1 = g(m, dW)
        g2 = g(m + g1 * np.sqrt(dt), dW)
        m = m + 0.5 * (g1 + g2) * np.sqrt(dt)
        m = m / np.sqrt(m @ m)
        out.append(m)
    return np.array(out)


@pytest.mark.parametrize("axis", [cm.Axis.all, cm.Axis.zaxis])
def test_oracle_runner_consumes_the_buffer_as_get_one_f_vector(axis):
    """The oracle's Euler-Heun run of a field-free layer against the step
    written out by hand from the same buffers: the noise enters only
    through getOneFVector."""
    dt, steps = 1e-13, 40
    j = cm.Junction([_free_layer(axis)])
    l = j.layers[0]
    specs = specs_array([(1.0, 1.0, l.noise_seed, 0, c) for c in range(3)])
    bufs = oracle_harness.alpha_buffers(specs, steps)
    oracle_harness.ALPHA_OVERRIDE = bufs
    oracle_harness.run_oracle([j], steps * dt, dt, dt, solverMode=cm.SolverMode.EulerHeun)
    lg = j.getLogArrays()
    got = np.stack([lg["free_mx"], lg["free_my"], lg["free_mz"]], 1)
    gyro = cm.constants.PhysicalConstants.gyromagnetic_ratio()
    want = _euler_heun_by_hand(np.array([0.6, 0, 0.8]), bufs.T, 0.05, int(axis), 0.02, gyro, dt)
    assert np.max(np.abs(got - want)) <= 1e-12, np.max(np.abs(got - want))


def test_oracle_alpha_noise_draws_new_buffers_each_run():
    """Each runSimulation creates new buffers (junction.hpp:1912-1916): a
    second run of a layer sees new noise, while a layer with the same seed
    replays the first run exactly."""
    dt = 1e-13
    a = cm.Junction([_free_layer()])
    b = cm.Junction([_free_layer()])
    for j in (a, b):
        oracle_harness.run_oracle([j], 50 * dt, dt, dt, solverMode=cm.SolverMode.EulerHeun)
    assert np.array_equal(a.getLogArrays()["free_mx"], b.getLogArrays()["free_mx"])
    a.clearLog()
    oracle_harness.run_oracle([a], 50 * dt, dt, dt, solverMode=cm.SolverMode.EulerHeun)
    second = a.getLogArrays()["free_mx"]
    first = b.getLogArrays()["free_mx"]
    assert not np.allclose(np.diff(second), np.diff(first))


def test_vector_alpha_noise_api_shapes():
    """cmtj.noise's classes without a GPU: the axis check of
    VectorAlphaNoise (noise.hpp:297-299)."""
    from cmtj_gb300.noise import VectorAlphaNoise
    with pytest.raises(RuntimeError, match="Invalid axis specified"):
        VectorAlphaNoise(16, 1.0, 1.0, 1.0, cm.Axis.none)
    v = VectorAlphaNoise(16, 1.0, 1.0, 2.0, cm.Axis.yaxis)
    assert v.getScale() == 2.0 and not v.normalized
    assert _abi.ALPHA_NOISE_DTYPE.itemsize == 40
