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


@pytest.mark.gpu
def test_vsd_mixing_voltage_matches_fp64(gpu_lib):
    spec, _ = sweeps.vsd_config(n_f=4, n_h=8, seed=9, dt=DT, amp=5e3)
    batch.relax(spec, DT, 20000, alpha=1.0)
    n_steps = 20000
    low = batch.lower(spec, DT, n_steps)
    run = batch.BatchRun(low, DT, cm.SolverMode.RK4, batch.LOG_NONE, 0, red_every=1)
    run.launch()
    st = run.state()
    assert np.all(st["status"] == 0) and np.all(st["n_red"] == n_steps)
    v32 = (st["v_sum"].astype(np.float64) + st["v_c"]) / n_steps
    rows = list(range(spec.n))
    js = junctions_from_spec(spec, rows, lambda k: cm.AxialDriver(cm.NullDriver(),
                                                                     cm.sineDriver(0, 5e3, float(spec.vsd_freq[k]), 0),
                                                                     cm.NullDriver()))
    oracle_harness.run_oracle(js, n_steps * DT, DT, DT, threads=8)
    for q, k in enumerate(rows):
        lg = js[q].getLogArrays()
        L = int(spec.n_layers[k])
        t = lg["time"]
        if spec.mr_mode[k] == 1:
            R = lg["R"] if L == 1 else lg["R_L0_L1"]
            scale = spec.Rap[k] - spec.Rp[k]
        else:
            R = sum(spec.strip[k, 0, l] + spec.strip[k, 2, l] * lg["L%d_mx" % l] ** 2 +
                    spec.strip[k, 4, l] * lg["L%d_my" % l] ** 2 for l in range(L))
            scale = sum(abs(spec.strip[k, 2, l]) + abs(spec.strip[k, 4, l]) for l in range(L))
        I = np.sin(2 * np.pi * spec.vsd_freq[k] * t)
        v64 = float(np.mean(I * R))
        assert abs(v32[k] - v64) <= 1e-4 * scale, (k, L, v32[k], v64)


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
    against compute_sd run on the oracle's FP64 trajectory."""
    spec, _ = sweeps.vsd_config(n_f=4, n_h=6, seed=13, dt=DT, amp=5e3)
    batch.relax(spec, DT, 20000, alpha=1.0)
    n_steps = 30000
    low = batch.lower(spec, DT, n_steps)
    w = batch.lowpass_step_response(n_steps, 1.0 / DT)
    run = batch.BatchRun(low, DT, cm.SolverMode.RK4, batch.LOG_NONE, 0, red_every=1, red_weights=w)
    run.launch()
    st = run.state()
    assert np.all(st["status"] == 0) and np.all(st["n_red"] == n_steps)
    v32 = -(st["vw_sum"].astype(np.float64) + st["vw_c"]) / n_steps
    plain32 = (st["v_sum"].astype(np.float64) + st["v_c"]) / n_steps
    rows = list(range(spec.n))
    js = junctions_from_spec(spec, rows, lambda k: cm.AxialDriver(cm.NullDriver(),
                                                                     cm.sineDriver(0, 5e3, float(spec.vsd_freq[k]), 0),
                                                                     cm.NullDriver()))
    oracle_harness.run_oracle(js, n_steps * DT, DT, DT, threads=8)
    for q, k in enumerate(rows):
        lg = js[q].getLogArrays()
        L = int(spec.n_layers[k])
        if spec.mr_mode[k] == 1:
            R = lg["R"] if L == 1 else lg["R_L0_L1"]
            scale = spec.Rap[k] - spec.Rp[k]
        else:
            R = sum(spec.strip[k, 0, l] + spec.strip[k, 2, l] * lg["L%d_mx" % l] ** 2 +
                    spec.strip[k, 4, l] * lg["L%d_my" % l] ** 2 for l in range(L))
            scale = sum(abs(spec.strip[k, 2, l]) + abs(spec.strip[k, 4, l]) for l in range(L))
        I = np.sin(2 * np.pi * spec.vsd_freq[k] * lg["time"])
        v64 = compute_sd_f64(R, I, DT)
        assert abs(v32[k] - v64) <= 1e-4 * scale, (k, L, v32[k], v64)
        # the filter removes part of the plain mean: the two differ
        assert np.isfinite(plain32[k])


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
        # trajectory error (max|dm| <= 1e-4 per sample) plus FFT rounding
        traj_tol = 1e-4 * nfft
        assert np.max(np.abs(gpu[k] - fft64)) <= traj_tol + fft_tol, k


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
    lo, hi = 0, nfft // 2 + 1
    out = t.empty((rows, hi - lo), dtype=t.float32, device="cuda")
    rc = lib.cmtj_spectrum_f32(engine.ptr(d_x), stride, rows, length, nfft, lo, hi, engine.ptr(out),
                               engine.stream_ptr())
    _abi.check(rc, lib)
    got = out.cpu().numpy()
    ref = np.abs(np.fft.fft(x[:, length - nfft:length].astype(np.float64), axis=1))[:, lo:hi]
    tol = 4 * np.finfo(np.float32).eps * np.log2(nfft) * np.linalg.norm(x[:, length - nfft:length], axis=1)
    assert np.all(np.max(np.abs(got - ref), axis=1) <= tol)
