"""On-device reductions against FP64:

* spin-diode mixing <I(t) R(t)> (compute.hpp:75-76 form; resistance.py:12-22
  without the low-pass) accumulated in the FP32 batch kernel with
  compensated sums, on uneven 1-4 layer junctions of the spin-diode sweep,
  against the mean over the oracle's FP64 trajectory;
* the low-passed form of resistance.py:12-22 (compute_sd) as a weighted
  on-device sum, against compute_sd on the oracle's FP64 trajectory;
* the PIMM spectrum (procedures.py:28-39): cmtj_spectrum_f32 on the FP32 log
  against numpy's FFT of the same log (the FFT itself) and of the FP64
  trajectory (end to end)."""
import numpy as np
import pytest

import cmtj_gb300 as cm
import oracle_harness
from cases import junctions_from_spec
from cmtj_gb300 import _abi, batch, engine, sweeps

DT = 1e-13


# Rows of the uneven spin-diode sweep itself (sweeps.vsd_config defaults:
# 131,072 junctions, seed 3, 500 A/m sine Oersted field, durations U[5, 50]
# ns, from their literal start).  Four per layer count, the strip (series
# Rx) junctions at 3 and 4 layers, picked among rows of at most 15 ns whose
# FP64 trajectory moves by at most 3e-5 under a 1e-7 nudge of m0 (the
# trajectories the FP32 bound applies to) and whose mixing covariance
# <I R> - <I><R> is well above the tolerance (checked below).
VSD_ROWS = [82121, 119468, 1678, 95069,        # 1 layer, classic R
            109839, 124315, 91883, 105362,     # 2 layers, classic R
            40864, 92767, 19241, 10835,        # 3 layers, series Rx
            100206, 100563, 81789, 121478]     # 4 layers, series Rx


def _vsd_rows(rows):
    spec, n_steps = sweeps.vsd_config(dt=DT)
    return spec.take(rows), n_steps[rows]


def _vsd_fp64(spec, n_steps):
    """Each row on the oracle for its own duration, logged every step:
    (R(t), I(t) = sin(2 pi f t), MR scale) per row."""
    from concurrent.futures import ThreadPoolExecutor
    oracle_harness.oracle_lib()

    def one(k):
        j = junctions_from_spec(spec, [k], lambda q: cm.AxialDriver(
            cm.NullDriver(), cm.sineDriver(0, 500.0, float(spec.vsd_freq[q]), 0), cm.NullDriver()))[0]
        oracle_harness.run_oracle([j], int(n_steps[k]) * DT, DT, DT)
        lg = j.getLogArrays()
        L = int(spec.n_layers[k])
        if spec.mr_mode[k] == 1:
            R = lg["R"] if L == 1 else lg["R_L0_L1"]
            scale = spec.Rap[k] - spec.Rp[k]
        else:
            R = sum(spec.strip[k, 0, l] + spec.strip[k, 2, l] * lg["L%d_mx" % l] ** 2 +
                    spec.strip[k, 4, l] * lg["L%d_my" % l] ** 2 for l in range(L))
            scale = sum(abs(spec.strip[k, 2, l]) + abs(spec.strip[k, 4, l]) for l in range(L))
        m = np.array([[lg["L%d_m%s" % (l, c)][-1] for c in "xyz"] for l in range(L)])
        return R, np.sin(2 * np.pi * spec.vsd_freq[k] * lg["time"]), scale, m

    with ThreadPoolExecutor(8) as ex:
        return list(ex.map(one, range(spec.n)))


def _vsd_tolerance(scale, r_mean, r_coef=1e-8):
    """Tolerance of an FP32 <I(t) R(t)> against FP64: 2e-6 of the MR scale
    (the trajectory's error, averaged against the oscillating drive) plus
    r_coef of the mean R (the FP32 sine of the drive phase and the FP32
    filter weights multiply the whole of R).  Measured on these rows: at
    most 2.3e-8 of the scale and 4e-9 of R for the plain mean, 7e-8 of R
    for the filtered one."""
    return 2e-6 * scale + r_coef * r_mean


def _mean_r_tolerance(scale, r_mean):
    """Error bound of the FP32 time-averaged R: the FP32 trajectory bound
    max|dm| <= 1e-4 (reached in the transient from the literal start) moves
    R by at most 2e-4 per unit of MR scale, plus FP32 rounding of R."""
    return 2e-4 * scale + 2e-7 * r_mean


@pytest.mark.gpu
def test_vsd_mixing_voltage_matches_fp64(gpu_lib):
    """Config-3 rows at their own 500 A/m drive and 5-15 ns durations: the
    on-device compensated <I R> (compute.hpp:75-76 form), the on-device
    time-averaged R (procedures.py:292-296) and their mixing covariance
    <I R> - <I><R> against the same means over the oracle's FP64
    trajectory.  Every row's covariance is at least 10x the tolerance, so a
    zero or unrelated answer fails."""
    spec, n_steps = _vsd_rows(VSD_ROWS)
    run = batch.BatchRun(batch.lower(spec, DT, n_steps), DT, cm.SolverMode.RK4, batch.LOG_NONE, 0, red_every=1)
    run.launch()
    st = run.state()
    assert np.all(st["status"] == 0) and np.all(st["n_red"] == n_steps)
    v32 = (st["v_sum"].astype(np.float64) + st["v_c"]) / n_steps
    r32 = (st["r_sum"].astype(np.float64) + st["r_c"]) / n_steps
    ref = _vsd_fp64(spec, n_steps)
    report = []
    for k, (R, I, scale, m64) in enumerate(ref):
        L = int(spec.n_layers[k])
        v64, r64, i64 = float(np.mean(I * R)), float(np.mean(R)), float(np.mean(I))
        cov64, cov32 = v64 - i64 * r64, v32[k] - i64 * r32[k]
        dm = float(np.max(np.abs(st["m"][k, :L].astype(np.float64) - m64)))
        tol = _vsd_tolerance(scale, abs(r64))
        tol_r = _mean_r_tolerance(scale, abs(r64))
        report.append((VSD_ROWS[k], L, dm, v64, v32[k] - v64, r32[k] - r64, tol_r, cov64, cov32 - cov64, tol))
    print("\nrow L max|dm| v64 dv dR tolR cov64 dcov tol")
    for r in report:
        print("%d %d %.2e %.5g %.2e %.2e %.2e %.4e %.2e %.2e" % r)
    for row, L, dm, v64, dv, dr, tol_r, cov64, dcov, tol in report:
        assert dm <= 1e-4, (row, dm)
        assert abs(cov64) > 10 * tol, (row, cov64, tol)
        assert abs(dv) <= tol, (row, L, dv, tol)
        assert abs(dr) <= tol_r, (row, L, dr, tol_r)
        assert abs(dcov) <= tol, (row, L, dcov, tol)
        assert abs(dcov) <= 0.01 * abs(cov64), (row, L, dcov, cov64)


def compute_sd_f64(R, I, dt):
    """The reference's filtered spin-diode voltage on an FP64 trajectory
    (cmtj/utils/resistance.py:12-22 with filters.py:33-43): mean of the
    3rd-order 10 MHz Butterworth low-pass of -I R."""
    from scipy.signal import butter, lfilter
    b, a = butter(3, 10e6 / (0.5 / dt), btype="low", analog=False)
    return float(np.mean(lfilter(b, a, -I * R)))


@pytest.mark.gpu
def test_vsd_filtered_voltage_matches_compute_sd(gpu_lib):
    """The weighted on-device sum (weights = the filter's step response)
    against compute_sd run on the oracle's FP64 trajectory, on the same
    config-3 rows (500 A/m, 5-15 ns, 1-4 layers)."""
    spec, n_steps = _vsd_rows(VSD_ROWS)
    w = batch.lowpass_step_response(int(n_steps.max()), 1.0 / DT)
    run = batch.BatchRun(batch.lower(spec, DT, n_steps), DT, cm.SolverMode.RK4, batch.LOG_NONE, 0, red_every=1,
                         red_weights=w)
    run.launch()
    st = run.state()
    assert np.all(st["status"] == 0) and np.all(st["n_red"] == n_steps)
    v32 = -(st["vw_sum"].astype(np.float64) + st["vw_c"]) / n_steps
    ref = _vsd_fp64(spec, n_steps)
    print("\nrow L sd64 dsd tol")
    worst = []
    for k, (R, I, scale, _) in enumerate(ref):
        v64 = compute_sd_f64(R, I, DT)
        tol = _vsd_tolerance(scale, float(np.mean(np.abs(R))), r_coef=1e-7)
        print("%d %d %.5g %.2e %.2e" % (VSD_ROWS[k], int(spec.n_layers[k]), v64, v32[k] - v64, tol))
        worst.append((abs(v32[k] - v64) / tol, VSD_ROWS[k], v64, v32[k]))
    assert max(worst)[0] <= 1.0, max(worst)


@pytest.mark.gpu
def test_pimm_spectrum_matches_numpy_and_fp64(gpu_lib):
    spec, _ = sweeps.pimm_config(n_h=16, n_draw=1, dt=DT)
    batch.relax(spec, DT, 30000, alpha=1.0)
    n_steps, every, nfft = 10240, 10, 1024
    low = batch.lower(spec, DT, n_steps)
    run = batch.BatchRun(low, DT, cm.SolverMode.RK4, batch.LOG_MIX, every, log_axis=0)
    run.launch()
    lib = _abi.load()
    t = engine.torch()
    samples = int(run.samples[0])
    out = t.empty((spec.n, nfft // 2 - 1), dtype=t.float32, device="cuda")
    rc = lib.cmtj_spectrum_f32(engine.ptr(run.d_log), int(run.log_pad[0]), spec.n, samples, nfft, 1, nfft // 2,
                               engine.ptr(out), engine.stream_ptr())
    _abi.check(rc, lib)
    gpu = out.cpu().numpy()
    log = run.d_log.cpu().numpy()
    js = junctions_from_spec(spec, range(spec.n), lambda k: cm.AxialDriver(cm.stepDriver(0, 1e3, 0, 1e-12),
                                                                            cm.NullDriver(), cm.NullDriver()))
    for j in js:
        j.setLayerAnisotropyDriver("L1", cm.constantDriver(1e6))
    oracle_harness.run_oracle(js, n_steps * DT, DT, DT * every, threads=8)
    eps32 = np.finfo(np.float32).eps
    errs = []
    for k in range(spec.n):
        x32 = run.log_of(k, log)[:, 0].astype(np.float64)
        ref_fft = np.abs(np.fft.fft(x32[-nfft:]))[1:nfft // 2]
        # FP32 FFT rounding: per bin about eps * log2(N) * ||x||_2 (the DC
        # part of x dominates ||x||, not the ringing)
        fft_tol = 4 * eps32 * np.log2(nfft) * np.linalg.norm(x32[-nfft:])
        assert np.max(np.abs(gpu[k] - ref_fft)) <= fft_tol, (k, np.max(np.abs(gpu[k] - ref_fft)), fft_tol)
        lg = js[k].getLogArrays()
        w = spec.mix_w[k, :2]
        x64 = w[0] * lg["L0_mx"] + w[1] * lg["L1_mx"]
        fft64 = np.abs(np.fft.fft(x64[-nfft:]))[1:nfft // 2]
        # end to end (FP32 trajectory, log and FFT against the FP64
        # trajectory's spectrum), relative to the ringing's spectral peak.
        # The 1 ps, 1 kA/m pulse rings at about 1e-4 of |m|, so the FP32
        # trajectory's ~1e-6 errors are percent-level of the peak; at the
        # field grid's ends m is saturated along the pulse and does not ring
        # (peak 0): there only the FFT rounding remains
        peak = float(np.max(fft64))
        err = float(np.max(np.abs(gpu[k] - fft64)))
        print("row %d: peak %.3e  max|d spectrum| %.2e  fft_tol %.2e" % (k, peak, err, fft_tol))
        errs.append((err, peak, fft_tol))
    for k, (err, peak, fft_tol) in enumerate(errs):
        assert err <= 5e-2 * peak + fft_tol, (k, err, peak, fft_tol)


@pytest.mark.gpu
@pytest.mark.parametrize("nfft", [64, 128, 256, 512, 4096, 8192])
def test_spectrum_kernel_matches_numpy(gpu_lib, nfft):
    """Radix-8 Stockham stages with a radix-4 or radix-2 tail: |FFT| of
    random rows (taken from the end of longer rows) against numpy."""
    t = engine.torch()
    lib = _abi.load()
    rng = np.random.default_rng(nfft)
    rows, length, stride = 37, nfft + 13, nfft + 20
    x = rng.standard_normal((rows, stride)).astype(np.float32) + 0.5
    d_x = t.from_numpy(x.ravel().copy()).cuda()
    full = np.abs(np.fft.fft(x[:, length - nfft:length].astype(np.float64), axis=1))
    tol = 4 * np.finfo(np.float32).eps * np.log2(nfft) * np.linalg.norm(x[:, length - nfft:length], axis=1)
    # the lower half with bin n/2, and a window across n/2 to the last bin
    # (|X[k]| = |X[n-k]| above n/2)
    for lo, hi in ((0, nfft // 2 + 1), (nfft // 2 - 5, nfft)):
        out = t.empty((rows, hi - lo), dtype=t.float32, device="cuda")
        rc = lib.cmtj_spectrum_f32(engine.ptr(d_x), stride, rows, length, nfft, lo, hi, engine.ptr(out),
                                   engine.stream_ptr())
        _abi.check(rc, lib)
        got = out.cpu().numpy()
        assert np.all(np.max(np.abs(got - full[:, lo:hi]), axis=1) <= tol), (lo, hi)


@pytest.mark.gpu
def test_windowed_mean_r_matches_fp64(gpu_lib):
    """The on-device time-averaged R over a window (the R(H) sweep's mean over
    its last fifth; procedures.py:292-296, compute.hpp:75-76): the 2-layer
    MTJ of the R(H) sweep from +z under fields of 400-800 kA/m along +-x
    (FP64 moves <= 5e-6 under a 1e-7 nudge of m0 here), 20,000 RK4 steps,
    R summed on the device over the last 4,000, against the mean of the
    oracle's FP64 R log over the same steps.  The window matters: the mean
    over the whole run differs by 10-15 ohm."""
    import cases
    n, w0 = 20000, 16000
    fields = [-8e5, -7e5, -6e5, -5e5, -4e5, 4e5, 5e5, 6e5, 7e5, 8e5]
    js32 = [cases.mtj_rh_point(cm, hx=h, total=n * DT)[0] for h in fields]
    js64 = [cases.mtj_rh_point(cm, hx=h, total=n * DT)[0] for h in fields]
    spec = batch.BatchSpec.from_junctions(js32)
    run = batch.BatchRun(batch.lower(spec, DT, n, win_start=w0), DT, cm.SolverMode.RK4, batch.LOG_NONE, 0,
                         red_every=1)
    run.launch()
    st = run.state()
    assert np.all(st["status"] == 0) and np.all(st["n_red"] == n - w0)
    r32 = (st["r_sum"].astype(np.float64) + st["r_c"]) / (n - w0)
    oracle_harness.run_oracle(js64, n * DT, DT, DT, threads=8)
    for k, j in enumerate(js64):
        R = j.getLogArrays()["R_free_ref"]
        r64, r_all = float(np.mean(R[w0:])), float(np.mean(R))
        assert abs(r_all - r64) > 5.0, (fields[k], r_all, r64)
        tol = _mean_r_tolerance(100.0, r64)
        assert abs(r32[k] - r64) <= tol, (fields[k], r32[k], r64, tol)


@pytest.mark.gpu
def test_largest_shared_memory_layout_keeps_logs_and_reductions(gpu_lib):
    """4-layer spin-diode junctions with every layer's m logged every step
    in 8-sample tiles (96 floats per thread), the Butterworth-weighted sum
    and the cached reduction constants: 59 KB of shared memory per CTA,
    above the 48 KB a launch gets without opting in.  Logging leaves the
    reductions bit for bit as a run without a log gives them, and reducing
    leaves the log bit for bit as a run without reductions gives it."""
    spec, ns = sweeps.vsd_config(n_f=4, n_h=64, dt=DT, t_min=1e-10, t_max=2e-10)
    keep = np.nonzero(spec.n_layers == 4)[0]
    spec, ns = spec.take(keep), ns[keep]
    rows = batch.BatchRun(batch.lower(spec, DT, ns), DT, cm.SolverMode.RK4).part_rows[0]  # one kernel variant
    spec, ns = spec.take(rows), ns[rows]
    low = batch.lower(spec, DT, ns)
    w = batch.lowpass_step_response(int(ns.max()), 1 / DT)
    tile = 8
    assert 128 * (tile * 12 + 2 + 18) * 4 > 48 * 1024

    def run(logged, reduced):
        mode = batch.LOG_M if logged else batch.LOG_NONE
        kw = dict(red_every=1, red_weights=w) if reduced else {}
        r = batch.BatchRun(low, DT, cm.SolverMode.RK4, mode, 1 if logged else 0, **kw)
        assert len(r.parts) == 1
        code = r.parts[0][3]
        r._launch_part(0, None, engine.torch().cuda.current_stream(), tile if logged else 0, code)
        st = r.state()
        assert np.all(st["status"] == 0) and np.all(st["step"] == ns)
        log = r.d_log.cpu().numpy()
        samples = [r.log_of(k, log).copy() for k in range(r.n)] if logged else None
        return st, samples

    both, log_both = run(True, True)
    red_only, _ = run(False, True)
    log_only, log_alone = run(True, False)
    for f in ("m", "n_red", "r_sum", "r_c", "v_sum", "v_c", "vw_sum", "vw_c"):
        assert both[f].tobytes() == red_only[f].tobytes(), f
    assert np.all(both["n_red"] == ns) and np.all(np.abs(both["v_sum"]) > 0)
    assert both["m"].tobytes() == log_only["m"].tobytes()
    assert np.array_equal(both["n_logged"], log_only["n_logged"]) and np.all(both["n_logged"] == ns)
    for a, b in zip(log_both, log_alone):
        assert a.shape == (a.shape[0], 12) and a.tobytes() == b.tobytes()
