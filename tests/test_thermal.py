"""Stochastic (sLLGS) parity on the CPU: the oracle's Philox thermal field
against the reference's own switching statistics (tests/golden/
pbit_switching.npz, from the reference extension with its mt19937) within a
3-sigma binomial bound, and the stationary m_z density against the
Boltzmann distribution of the uniaxial macrospin."""
import numpy as np

import cmtj_gb300
import oracle_harness
import thermal_cases


def load_ref():
    g = np.load("%s/golden/pbit_switching.npz" % thermal_cases.__file__.rsplit("/", 1)[0])
    return g["currents"], g["switched"], g["runs"]


def load_sweep_ref():
    """Reference switching counts of the full p-bit sweep (Ku 2.5e5, 17 of
    its 64 currents, durations U[5, 20] ns): tests/golden/pbit_sweep.npz."""
    g = np.load("%s/golden/pbit_sweep.npz" % thermal_cases.__file__.rsplit("/", 1)[0])
    return g["currents"], g["switched"], g["runs"]


def binomial_ok(k1, n1, k2, n2):
    p1, p2 = k1 / n1, k2 / n2
    p = (k1 + k2) / (n1 + n2)
    bound = 3 * np.sqrt(max(p * (1 - p), 1.0 / (n1 + n2)) * (1.0 / n1 + 1.0 / n2))
    return abs(p1 - p2) <= bound, abs(p1 - p2), bound


def seeded_pbits(cm, j_density, n, seed0):
    out = []
    for k in range(n):
        j, run = thermal_cases.pbit_junction(cm, j_density)
        j.layers[0].noise_seed = seed0 + k
        out.append(j)
    return out, run


def test_oracle_switching_matches_reference_statistics():
    cur, sw, runs = load_ref()
    n = 1024
    for q, jd in enumerate(cur):
        js, run = seeded_pbits(cmtj_gb300, float(jd), n, 1000 * q + 17)
        r = dict(run)
        oracle_harness.run_oracle(js, r.pop("totalTime"), threads=8, **r)
        k = sum(1 for j in js if j.getLayerMagnetisation("free").z < 0)
        ok, d, b = binomial_ok(k, n, int(sw[q]), int(runs[q]))
        assert ok, (jd, k / n, sw[q] / runs[q], d, b)


def test_oracle_boltzmann_equilibrium():
    """j = 0, barrier 1.5 kT: pooled m_z samples after 1 ns of burn-in
    follow p(m_z) ~ exp(Ku V m_z^2 / kT) (histogram within 4 sigma)."""
    V = 7e-17 * 1.2e-9
    Ku = 1.5 * 1.380649e-23 * 300 / V
    js = []
    for k in range(128):
        j, run = thermal_cases.pbit_junction(cmtj_gb300, 0.0, Ku=Ku)
        j.layers[0].noise_seed = 77 + k
        if k % 2:
            j.setLayerMagnetisation("free", cmtj_gb300.CVector(0, 0, -1))  # both wells start populated
        js.append(j)
    oracle_harness.run_oracle(js, 1.2e-8, 1e-13, 2e-11, solverMode=cmtj_gb300.SolverMode.EulerHeun, threads=8)
    mz = np.concatenate([np.asarray(j.getLogArrays()["free_mz"])[100:] for j in js])
    check_density(mz, Ku, V)


def check_density(mz, Ku, V, bins=10, sigmas=4.0):
    """Histogram of |m_z| against the folded Boltzmann density.  The density
    is even in m_z; folding removes the slow population exchange between the
    two wells, whose few independent samples say nothing about the shape."""
    a = np.abs(np.asarray(mz))
    edges = np.linspace(0, 1, bins + 1)
    h, _ = np.histogram(a, bins=edges)
    x = np.linspace(0, 1, 20001)
    p = 2 * thermal_cases.boltzmann_mz_density(x, Ku, V, 300.0)
    expect = np.array([np.trapezoid(p[(x >= lo) & (x <= hi)], x[(x >= lo) & (x <= hi)])
                       for lo, hi in zip(edges[:-1], edges[1:])]) * a.size
    # samples are correlated in time: inflate the Poisson variance
    corr = 8.0
    z = (h - expect) / np.sqrt(corr * np.maximum(expect, 1.0))
    assert np.max(np.abs(z)) < sigmas, (np.round(z, 2), h, np.round(expect))


def test_sweep_fixture_matches_its_generator():
    """The full-sweep fixture holds the 17 currents of thermal_cases (every
    4th of the sweep's 64 plus the last), 2048 runs each, and its switching
    probability rises with the current from the thermal floor."""
    cur, sw, runs = load_sweep_ref()
    assert np.array_equal(cur, np.asarray(thermal_cases.SWEEP_CURRENTS))
    assert np.all(runs == 2048)
    p = sw / runs
    assert 0.1 < p[0] < 0.3 and p[-1] > 0.7 and p[5] > p[1]


def test_oracle_full_sweep_statistics_match_reference():
    """The oracle (Philox noise) on three currents of the full p-bit sweep,
    512 runs each with their own U[5, 20] ns durations, within the 3-sigma
    binomial bound of the reference's counts."""
    from concurrent.futures import ThreadPoolExecutor
    cur, sw, runs = load_sweep_ref()
    oracle_harness.oracle_lib()
    n = 512
    for q in (0, 2, 16):
        jd = float(cur[q])
        durs = thermal_cases.sweep_durations(n, 500 + q)

        def one(k):
            j, run = thermal_cases.pbit_sweep_junction(cmtj_gb300, jd, durs[k])
            j.layers[0].noise_seed = 3_000_000 + 10_000 * q + k
            r = dict(run)
            oracle_harness.run_oracle([j], r.pop("totalTime"), **r)
            return j.getLayerMagnetisation("free").z < 0

        with ThreadPoolExecutor(8) as ex:
            k = sum(ex.map(one, range(n)))
        ok, d, b = binomial_ok(k, n, int(sw[q]), int(runs[q]))
        assert ok, (jd, k / n, sw[q] / runs[q], d, b)


def load_alpha_ref():
    """The reference's switching counts of the p-bit layer with buffered
    alpha noise (tests/golden/alpha_switching.npz: thermal_cases.ALPHA_CASES,
    1024 runs each, the reference's BufferedAlphaNoise on mt19937)."""
    g = np.load("%s/golden/alpha_switching.npz" % thermal_cases.__file__.rsplit("/", 1)[0])
    return g["cases"], g["switched"], g["runs"]


def test_oracle_alpha_noise_switching_matches_reference():
    """The oracle (Philox white draws, its own restatement of fillBuffer) on
    the first alpha-noise case, 384 runs: P(m_z < 0) within the 3-sigma
    binomial bound of the reference's count."""
    from concurrent.futures import ThreadPoolExecutor
    cases, sw, runs = load_alpha_ref()
    assert [tuple(c) for c in cases] == [tuple(map(float, c)) for c in thermal_cases.ALPHA_CASES]
    oracle_harness.oracle_lib()
    n, q = 384, 0

    def one(k):
        j, run = thermal_cases.alpha_pbit_junction(cmtj_gb300, *thermal_cases.ALPHA_CASES[q])
        j.layers[0].noise_seed = 6_000_000 + k
        r = dict(run)
        oracle_harness.run_oracle([j], r.pop("totalTime"), **r)
        return j.getLayerMagnetisation("free").z < 0

    with ThreadPoolExecutor(8) as ex:
        k = sum(ex.map(one, range(n)))
    ok, d, b = binomial_ok(k, n, int(sw[q]), int(runs[q]))
    assert ok, (k / n, sw[q] / runs[q], d, b)


def test_rh_fma_spread_fixture():
    """The committed spread of the FMA-built reference on the R(H) sweep
    (tests/golden/make_rh_fma.py): 64 fields over +-800 kA/m; the builds
    agree to 1e-10 except near the switching fields of the free layer, and
    the sweep is symmetric in H, so mirrored fields move alike."""
    import os
    import numpy as np
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "rh_fma_spread.npz"))
    assert np.array_equal(d["fields"], np.linspace(-800e3, 800e3, 64))
    dm = d["max_abs_dm"]
    assert np.all(np.isfinite(dm)) and np.all(dm >= 0)
    rough = set(np.flatnonzero(dm > 1e-10).tolist())
    assert rough == {27, 28, 35, 36}, rough
    assert np.allclose(dm, dm[::-1], rtol=0.5, atol=1e-10)
