"""PIMM and spin-diode (VSD) procedures on the GPU solver.

The reference's procedures (cmtj/utils/procedures.py:42-331) sweep one
junction through field points (and frequencies) in a Python loop.  Each
point is a warm start from the previous point's final state, plus an
optional random disturbance, followed by one `runSimulation` and numpy/scipy
post-processing of the log.  That chain is sequential by construction.

Here the same functions take either one Junction (the reference's call,
same results) or a list of Junctions.  With a list, every junction runs its
own chain, and all chains advance together: one device launch per field
point for the whole list.  `precision="f64"` runs the FP64 plain form (the
reference's arithmetic); `precision="f32"` runs the FP32 batched form, with
the logs taken on the device at every step.

The helpers the procedures use are restated from cmtj/utils: resistance
(resistance.py:30-150), the Butterworth low-pass mean (resistance.py:12-22
with filters.py:33-43), the spectrum strip (procedures.py:28-39) and
FieldScan.amplitude_scan (linear.py:57-84).
"""
from collections import defaultdict
from dataclasses import dataclass

import numpy as np

from .core import AxialDriver, Axis, CVector, NullDriver, ScalarDriver, SolverMode


@dataclass
class ResistanceParameters:
    """procedures.py:14-25."""
    Rxx0: float = 0
    Rxy0: float = 0
    Rahe: float = 0
    Rsmr: float = 0
    Ramr: float = 0
    w: float = 0
    l: float = 0


# ---------------------------------------------------------------- helpers
def compute_resistance(Rx0, Ry0, AMR, AHE, SMR, m, l, w):
    """Per-layer Sx, Sy (resistance.py:30-66); m is [layers, 3] or
    [layers, 3, T]."""
    n = len(Rx0)
    m = np.asarray(m)
    shape = (n,) if m.ndim == 2 else (n, m.shape[2])
    Sx = np.zeros(shape)
    Sy = np.zeros(shape)
    for i in range(n):
        wl = w[i] / l[i]
        Sx[i] = Rx0[i] + (AMR[i] * m[i, 0] ** 2 + SMR[i] * m[i, 1] ** 2)
        Sy[i] = Ry0[i] + 0.5 * AHE[i] * m[i, 2] + (wl) * (SMR[i] + AMR[i]) * m[i, 0] * m[i, 1]
    return Sx, Sy


def calculate_resistance_series(Rx0, Ry0, AMR, AHE, SMR, m, l, w):
    """Series Rx, Ry (resistance.py:121-150)."""
    Sx, Sy = compute_resistance(Rx0, Ry0, AMR, AHE, SMR, m, l, w)
    return np.sum(Sx, axis=0), np.sum(Sy, axis=0)


def calculate_resistance_parallel(Rx0, Ry0, AMR, AHE, SMR, m, l, w):
    """Parallel Rx, Ry (resistance.py:91-118)."""
    Sx, Sy = compute_resistance(Rx0, Ry0, AMR, AHE, SMR, m, l, w)
    return 1.0 / np.sum(1.0 / Sx, axis=0), 1.0 / np.sum(1.0 / Sy, axis=0)


def compute_sd(dynamic_r, dynamic_i, integration_step):
    """Mean of the 3rd-order 10 MHz Butterworth low-pass of -I R
    (resistance.py:12-22, filters.py:33-43)."""
    from scipy.signal import butter, lfilter
    sd = -np.asarray(dynamic_i) * np.asarray(dynamic_r)
    fs = 1.0 / integration_step
    b, a = butter(3, 10e6 / (0.5 * fs), btype="low", analog=False)
    return np.mean(lfilter(b, a, sd, zi=None))


def compute_spectrum_strip(input_m, int_step, max_frequency):
    """|FFT| and frequencies up to max_frequency (procedures.py:28-39)."""
    from scipy.fft import fft, fftfreq
    yf = np.abs(fft(input_m))
    freqs = fftfreq(len(yf), int_step)
    freqs = freqs[: len(freqs) // 2]
    yf = yf[: len(yf) // 2]
    findx = np.argwhere(freqs <= max_frequency)
    return yf[findx], freqs[findx]


class FieldScan:
    """cmtj/utils/linear.py:6-124: field-vector constructors for sweeps.
    The arithmetic (sin/cos of the degree angles, then the products in the
    reference's order) is the reference's, so sweeps built here equal its
    own to the bit."""

    @staticmethod
    def _trig_compute(theta, phi):
        """(sin theta, cos theta, sin phi, cos phi), angles in degrees."""
        return (np.sin(np.deg2rad(theta)), np.cos(np.deg2rad(theta)), np.sin(np.deg2rad(phi)),
                np.cos(np.deg2rad(phi)))

    @staticmethod
    def angle2vector(theta, phi, amplitude=1):
        sin_t, cos_t, sin_p, cos_p = FieldScan._trig_compute(theta, phi)
        return CVector(sin_t * cos_p * amplitude, sin_t * sin_p * amplitude, cos_t * amplitude)

    @staticmethod
    def vector2angle(x, y, z):
        """(theta, phi, r) in degrees of a cartesian vector."""
        norm = np.sqrt(x ** 2 + y ** 2 + z ** 2)
        return np.rad2deg(np.arctan2(np.sqrt(x ** 2 + y ** 2), z)), np.rad2deg(np.arctan2(y, x)), norm

    @staticmethod
    def cvector2angle(vector):
        return FieldScan.vector2angle(vector.x, vector.y, vector.z)

    @staticmethod
    def theta_scan(start, stop, steps, amplitude, phi):
        """Polar-angle sweep at fixed amplitude and azimuth (degrees)."""
        angles = np.linspace(start, stop, endpoint=True, num=steps)
        sin_t, cos_t, sin_p, cos_p = FieldScan._trig_compute(angles, phi)
        return angles, np.vstack((sin_t * cos_p * amplitude, sin_t * sin_p * amplitude, cos_t * amplitude)).T

    @staticmethod
    def phi_scan(start, stop, steps, amplitude, theta):
        """Azimuth sweep at fixed amplitude and polar angle (degrees)."""
        angles = np.linspace(start, stop, endpoint=True, num=steps)
        sin_t, cos_t, sin_p, cos_p = FieldScan._trig_compute(theta, angles)
        y_part = sin_t * sin_p * amplitude
        return angles, np.vstack((sin_t * cos_p * amplitude, y_part, cos_t * amplitude * np.ones_like(y_part))).T

    @staticmethod
    def amplitude_scan(start, stop, steps, theta, phi, back=False):
        """Field-magnitude sweep along a fixed direction; with `back` the
        sweep returns to its start (the turning point once)."""
        magnitudes = np.linspace(start, stop, endpoint=True, num=steps)
        sin_t, cos_t, sin_p, cos_p = FieldScan._trig_compute(theta, phi)
        vectors = np.vstack((sin_t * cos_p * magnitudes, sin_t * sin_p * magnitudes, cos_t * magnitudes)).T
        if back:
            return (np.concatenate((magnitudes[:-1], magnitudes[::-1]), axis=0),
                    np.concatenate((vectors[:-1], vectors[::-1]), axis=0))
        return magnitudes, vectors


# ---------------------------------------------------------------- engine
def _oersted(direction, driver):
    if direction == Axis.zaxis:
        return AxialDriver(NullDriver(), NullDriver(), driver), "z"
    if direction == Axis.yaxis:
        return AxialDriver(NullDriver(), driver, NullDriver()), "y"
    return AxialDriver(driver, NullDriver(), NullDriver()), "x"


def _prepare(junctions, H, oedriver, disturbance):
    """The per-point set-up of both procedures, in the reference's order:
    constant Hext, the Oersted driver, then the disturbance (three normal
    draws per layer from numpy's global generator, then normalise)."""
    for j in junctions:
        j.clearLog()
        j.setLayerExternalFieldDriver("all", AxialDriver(ScalarDriver.getConstantDriver(H[0]),
                                                         ScalarDriver.getConstantDriver(H[1]),
                                                         ScalarDriver.getConstantDriver(H[2])))
        j.setLayerOerstedFieldDriver("all", oedriver)
        if disturbance:
            for lid in j.getLayerIds():
                old = j.getLayerMagnetisation(lid)
                new = CVector(old.x + np.random.normal(0, disturbance), old.y + np.random.normal(0, disturbance),
                              old.z + np.random.normal(0, disturbance))
                new.normalize()
                j.setLayerMagnetisation(lid, new)


def _run_f64(junctions, duration, int_step):
    """runSimulation(duration, int_step, int_step) of every junction in one
    FP64 plain-form launch; each junction gets its own log."""
    from . import engine
    plan = engine.plan_run(duration, int_step, int_step)
    solver = junctions[0].getSolver(SolverMode.RK4)
    engine.run_junctions(junctions, plan, solver)


def _run_point(junctions, duration, int_step, precision):
    """Run every junction for `duration` at writeFrequency = int_step and
    return, per junction, its log dict (numpy arrays) with the reference's
    keys for m, R and time."""
    if precision == "f64":
        _run_f64(junctions, duration, int_step)
        return [j.getLogArrays() for j in junctions]
    if precision != "f32":
        raise ValueError("precision must be 'f64' or 'f32'")
    from . import batch
    from ._lower import plan_run
    plan = plan_run(duration, int_step, int_step)
    solver = junctions[0].getSolver(SolverMode.RK4)
    spec = batch.BatchSpec.from_junctions(junctions)
    low = batch.lower(spec, plan.time_step, plan.total_iterations)
    run = batch.BatchRun(low, plan.time_step, solver, batch.LOG_M, 1)
    run.launch()
    st = run.state()
    log = run.d_log.cpu().numpy()
    out = []
    t = np.arange(plan.total_iterations, dtype=np.float64) * plan.time_step
    for k, j in enumerate(junctions):
        a = run.log_of(k, log).astype(np.float64)
        cols = {}
        for l, lid in enumerate(j.getLayerIds()):
            for c, ax in enumerate("xyz"):
                cols["%s_m%s" % (lid, ax)] = a[:, 3 * l + c]
            m = st["m"][k, l].astype(np.float64)
            j.setLayerMagnetisation(lid, CVector(*m))
        ids = j.getLayerIds()
        if j.MR_mode == 1 and len(ids) == 2:  # classic R of the two layers, from the logged m
            cosT = sum(cols["%s_m%s" % (ids[0], ax)] * cols["%s_m%s" % (ids[1], ax)] for ax in "xyz")
            cols["R_%s_%s" % (ids[0], ids[1])] = j.Rp + ((j.Rap - j.Rp) / 2.0) * (1.0 - cosT)
        cols["time"] = t
        out.append(cols)
    if np.any(st["status"] != 0):
        raise RuntimeError("NAN magnetisation")
    return out


def _as_list(junction):
    return (list(junction), False) if isinstance(junction, (list, tuple)) else ([junction], True)


# ---------------------------------------------------------------- procedures
def PIMM_procedure(junction, Hvecs, int_step, resistance_params, Hoe_direction=Axis.zaxis, Hoe_excitation=50,
                   Hoe_duration=3, simulation_duration=5e-9, wait_time=0e-9, max_frequency=80e9,
                   resistance_fn=calculate_resistance_series, disturbance=1e-3, take_last_n=100,
                   full_output=False, disable_tqdm=False, static_only=False, precision="f64"):
    """Pulse-induced microwave magnetometry (procedures.py:42-199).  Returns
    (spectrum, frequencies, output) like the reference for one junction; for
    a list of junctions, a list of such triples in the same order (all
    chains run together, one launch per field point)."""
    if wait_time > simulation_duration:
        raise ValueError("wait_time must be smaller than simulation_duration!")
    js, single = _as_list(junction)
    oedriver, comp = _oersted(Hoe_direction, ScalarDriver.getStepDriver(0, Hoe_excitation, 0,
                                                                        int_step * Hoe_duration))
    for j in js:
        if len(j.getLayerIds()) != len(resistance_params):
            raise ValueError("The number of layers in the junction must match the number of resistance "
                             "parameters!")
    spectra = [[] for _ in js]
    outputs = [defaultdict(list) for _ in js]
    freqs = None
    for H in Hvecs:
        _prepare(js, H, oedriver, disturbance)
        logs = _run_point(js, simulation_duration, int_step, precision)
        for q, (j, log) in enumerate(zip(js, logs)):
            norm = np.sum([layer.thickness * layer.Ms for layer in j.layers])
            indx = np.argwhere(np.asarray(log["time"]) >= wait_time).ravel()
            m_traj = np.asarray([np.asarray([log[f"{layer.id}_mx"], log[f"{layer.id}_my"], log[f"{layer.id}_mz"]]) *
                                 layer.thickness * layer.Ms / norm for layer in j.layers])
            m = m_traj[:, :, -take_last_n:]
            Rx, Ry = resistance_fn([r.Rxx0 for r in resistance_params], [r.Rxy0 for r in resistance_params],
                                   [r.Ramr for r in resistance_params], [r.Rahe for r in resistance_params],
                                   [r.Rsmr for r in resistance_params], m, l=[r.l for r in resistance_params],
                                   w=[r.w for r in resistance_params])
            out = outputs[q]
            if not static_only:
                mixed = np.asarray([np.asarray(log[f"{layer.id}_m{comp}"])[indx] * layer.thickness * layer.Ms / norm
                                    for layer in j.layers])
                yf, freqs = compute_spectrum_strip(mixed.sum(axis=0), int_step, max_frequency)
                spectra[q].append(yf)
            out["H"].append(H)
            out["Rx"].append(Rx)
            out["Ry"].append(Ry)
            out["m_avg"].append(m_traj[:, :, -1].sum(0))
            if full_output and not static_only:
                out["m_traj"].append(m_traj)
                for li, lid in enumerate(j.getLayerIds()):
                    y, _ = compute_spectrum_strip(mixed[li], int_step, max_frequency)
                    out[lid].append(y)
    results = []
    for q, j in enumerate(js):
        out = outputs[q]
        if full_output:
            for lid in j.getLayerIds():
                out[lid] = np.asarray(out[lid]).squeeze()
        results.append((np.squeeze(np.asarray(spectra[q])), freqs, out))
    return results[0] if single else results


def VSD_procedure(junction, Hvecs, frequencies, int_step, resistance_params=None, Hoe_direction=Axis.yaxis,
                  Hoe_excitation=50, simulation_duration=30e-9, disturbance=1e-3, Rtype="Rz",
                  resistance_fn=calculate_resistance_series, disable_tqdm=False, precision="f64"):
    """Spin-diode voltage over fields x frequencies (procedures.py:200-331):
    [len(Hvecs), len(frequencies)] per junction (a list of them for a list
    of junctions, all chains run together)."""
    if resistance_params is None:
        resistance_params = []
    js, single = _as_list(junction)
    for j in js:
        ids = j.getLayerIds()
        if Rtype == "Rz" and len(ids) > 2:
            raise ValueError("Rz can only be used for 2 layer junctions. Use Rx or Ry instead.")
        elif len(resistance_params) != len(ids):
            raise ValueError("The number of layers in the junction must match the number of resistance "
                             "parameters!")
    spectra = [np.zeros((len(Hvecs), len(frequencies))) for _ in js]
    for h, H in enumerate(Hvecs):
        for fi, f in enumerate(frequencies):
            oedriver, _ = _oersted(Hoe_direction, ScalarDriver.getSineDriver(0, Hoe_excitation, f, 0))
            _prepare(js, H, oedriver, disturbance)
            logs = _run_point(js, simulation_duration, int_step, precision)
            for q, (j, log) in enumerate(zip(js, logs)):
                ids = j.getLayerIds()
                m_traj = np.asarray([[log[f"{ids[i]}_mx"], log[f"{ids[i]}_my"], log[f"{ids[i]}_mz"]]
                                     for i in range(len(ids))])
                if Rtype == "Rz":
                    if len(ids) == 2:
                        R = log[f"R_{ids[0]}_{ids[1]}"]
                    elif len(ids) == 1:
                        R = log["Resistance"]  # the reference's key (procedures.py:297)
                    else:
                        raise ValueError("Resistance definition ambiguous!")
                else:
                    Rx, Ry = resistance_fn([r.Rxx0 for r in resistance_params], [r.Rxy0 for r in resistance_params],
                                           [r.Ramr for r in resistance_params], [r.Rahe for r in resistance_params],
                                           [r.Rsmr for r in resistance_params], m_traj,
                                           l=[r.l for r in resistance_params], w=[r.w for r in resistance_params])
                    if Rtype == "Rx":
                        R = Rx
                    elif Rtype == "Ry":
                        R = Ry
                    else:
                        raise ValueError("Rtype must be either Rx or Ry or Rz")
                dynamicI = np.sin(2 * np.pi * f * np.asarray(log["time"]))
                spectra[q][h, fi] = compute_sd(R, dynamicI, int_step)
    return spectra[0] if single else spectra
