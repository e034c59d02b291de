"""FP32 batched form: many independent junctions in one persistent launch.

Two ways in:
  * `BatchSpec.from_junctions(junctions)` takes ordinary Junction objects
    (any mix of 1-4 layers, drivers, STT/SOT, temperature);
  * `BatchSpec` fields can also be filled directly with numpy arrays for
    sweeps of 10^5-10^6 junctions (see cmtj_gb300.sweeps).
`lower(spec, time_step, n_steps)` folds constant drivers into the per-layer
coefficients of cmtj_f32_layer_t, turns each time-dependent driver into a
cmtj_wave_t and groups junctions by layer count; `run(...)` launches
cmtj_batch_run_f32 once per layer count (or resumes in chunks).

Driver time is never an FP32 variable: sine phases are Q0.64 fixed point
(cycles), step drivers become per-stage integer step windows found by
evaluating the reference's own FP64 comparisons (t = i*dt, t + 0.5*dt,
t + dt; junction.hpp:1974, 1020-1033), and the remaining waveforms use
t - t0 formed from integer step differences.
"""
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from . import constants as _constants
from .core import MR_CLASSIC, MR_NONE, MR_STRIP, Reference, SolverMode, UpdateType

MR_SERIES = 3

# cmtj_wave_target
TGT_HX, TGT_HY, TGT_HZ, TGT_K, TGT_K2, TGT_JB, TGT_JT, TGT_J2B, TGT_J2T = range(9)
TGT_I, TGT_FL, TGT_DL, TGT_FL2, TGT_DL2, TGT_T = 9, 10, 11, 12, 13, 14

FEAT_FULL_DEMAG, FEAT_DIPOLE, FEAT_IDMI, FEAT_K2 = 1, 2, 4, 8
FEAT_STT, FEAT_SOT, FEAT_WAVES, FEAT_SCALAR_WAVES, FEAT_IEC2 = 16, 32, 64, 128, 256
FEAT_OFFAXIS, FEAT_ALL = 512, 1023

F32_STT, F32_SOT, F32_SOT_STATIC, F32_ALT_STT = 1, 2, 4, 8
LOG_NONE, LOG_M, LOG_MIX, LOG_R = 0, 1, 2, 3
MAX_WAVES = 4

WAVE_DTYPE = np.dtype(
    [("target", "<i4"), ("kind", "<i4"), ("amp", "<f4"), ("p0", "<f4"), ("p1", "<f4"), ("p2", "<f4"),
     ("thr32", "<u4"), ("i0", "<i4"), ("ph0", "<u8"), ("dph", "<u8"), ("dph_half", "<u8"),
     ("on", "<u4", 3), ("off", "<u4", 3), ("layer_mask", "<i4"), ("reserved", "<i4")], align=True)

F32_LAYER_DTYPE = np.dtype(
    [("m", "<f4", 3), ("anis", "<f4", 3), ("kc", "<f4"), ("k2c", "<f4"), ("demag", "<f4", 9),
     ("dip_b", "<f4", 9), ("dip_t", "<f4", 9), ("h0", "<f4", 3), ("jb", "<f4"), ("jt", "<f4"), ("j2b", "<f4"),
     ("j2t", "<f4"), ("dmi_b", "<f4", 3), ("dmi_t", "<f4", 3), ("gam", "<f4"), ("alpha", "<f4"),
     ("ref", "<f4", 3), ("ref2", "<f4", 3), ("ref_type", "<i4"), ("flags", "<i4"), ("stt_c", "<f4"),
     ("stt_p", "<f4"), ("stt_l", "<f4"), ("stt_beta", "<f4"), ("stt_kappa", "<f4"), ("i0", "<f4"),
     ("fl0", "<f4"), ("dl0", "<f4"), ("fl20", "<f4"), ("dl20", "<f4"), ("sig_c", "<f4"), ("t0", "<f4"),
     ("seed_lo", "<u4"), ("seed_hi", "<u4"), ("noise_step_lo", "<u4"), ("noise_step_hi", "<u4"),
     ("gdt", "<f4"), ("gdt6", "<f4"), ("stt_cdt", "<f4"), ("stt_cdt6", "<f4")], align=True)

F32_JUNCTION_DTYPE = np.dtype(
    [("n_layers", "<i4"), ("mr_mode", "<i4"), ("layer_offset", "<i4"), ("n_steps", "<u4"),
     ("win_start", "<u4"), ("log_offset", "<u4"), ("Rp", "<f4"), ("Rap", "<f4"),
     ("Rx0", "<f4", 4), ("Ry0", "<f4", 4), ("AMR_X", "<f4", 4), ("AMR_Y", "<f4", 4), ("SMR_X", "<f4", 4),
     ("SMR_Y", "<f4", 4), ("AHE", "<f4", 4), ("mix_w", "<f4", 4), ("vsd_ph0", "<u8"), ("vsd_dph", "<u8"),
     ("n_waves", "<i4"), ("red_total", "<u4"), ("waves", WAVE_DTYPE, MAX_WAVES)], align=True)

F32_STATE_DTYPE = np.dtype(
    [("m", "<f4", (4, 3)), ("step", "<u4"), ("status", "<u4"), ("n_logged", "<u4"), ("n_red", "<u4"),
     ("r_sum", "<f4"), ("r_c", "<f4"), ("v_sum", "<f4"), ("v_c", "<f4"), ("vw_sum", "<f4"), ("vw_c", "<f4")],
    align=True)

F32_PARAMS_DTYPE = np.dtype(
    [("dt", "<f8"), ("chunk_steps", "<u4"), ("solver", "<i4"), ("log_mode", "<i4"), ("log_axis", "<i4"),
     ("log_every", "<u4"), ("log_tile", "<u4"), ("red_every", "<u4"), ("reserved", "<i4"),
     ("red_weights", "<u8")], align=True)

STRUCT_SIZES_F32 = {
    "cmtj_wave_t": WAVE_DTYPE.itemsize, "cmtj_f32_layer_t": F32_LAYER_DTYPE.itemsize,
    "cmtj_f32_junction_t": F32_JUNCTION_DTYPE.itemsize, "cmtj_f32_state_t": F32_STATE_DTYPE.itemsize,
    "cmtj_f32_params_t": F32_PARAMS_DTYPE.itemsize,
}


# --------------------------------------------------------------------------
# Fixed point and exact step windows
# --------------------------------------------------------------------------
_Q64 = float(2 ** 64)


def q64_frac(x):
    """Fractional part of x (cycles) as Q0.64, elementwise, x float64."""
    x = np.asarray(x, dtype=np.float64)
    f = x - np.floor(x)
    hi = np.floor(f * 2.0 ** 32)
    lo = np.floor((f * 2.0 ** 32 - hi) * 2.0 ** 32)
    return (hi.astype(np.uint64) << np.uint64(32)) | np.clip(lo, 0, 2 ** 32 - 1).astype(np.uint64)


def stage_time(i, dt, s):
    """Stage time exactly as the reference forms it: t = i*dt, then
    t + 0.5*dt or t + dt (double precision)."""
    t = np.asarray(i, dtype=np.float64) * dt
    if s == 1:
        return t + 0.5 * dt
    if s == 2:
        return t + dt
    return t


def step_window(t_start, t_stop, dt, n_steps):
    """Per stage s: inclusive [on_s, off_s] of steps i with
    t_start <= t_s(i) <= t_stop (drivers.hpp:73-78), found with the same
    FP64 arithmetic the reference uses; empty windows are on > off."""
    on = np.zeros(3, dtype=np.uint32)
    off = np.zeros(3, dtype=np.uint32)
    big = 2 ** 32 + 16

    def guess_of(x):
        q = x / dt
        if not np.isfinite(q):
            return big if q > 0 else 0
        return int(min(max(np.floor(q), 0), big))

    for s in range(3):
        lo = max(guess_of(t_start) - 4, 0)
        cand = np.arange(lo, lo + 10, dtype=np.int64)
        ok = stage_time(cand, dt, s) >= t_start
        first = int(cand[np.argmax(ok)]) if ok.any() else lo + 10
        lo2 = max(guess_of(t_stop) - 4, 0)
        cand = np.arange(lo2, lo2 + 10, dtype=np.int64)
        ok = stage_time(cand, dt, s) <= t_stop
        last = int(cand[ok][-1]) if ok.any() else -1
        if last < first:
            on[s], off[s] = 1, 0
        else:
            on[s] = min(first, 2 ** 32 - 1)
            off[s] = min(last, 2 ** 32 - 1)
    return on, off


def wave_from_driver(d, target, amp_scale, layer_mask, dt):
    """cmtj_wave_t for the time-dependent part of ScalarDriver d (its
    constantValue is folded by the caller), or None if d is constant."""
    u = d.update
    if u == UpdateType.constant:
        return None
    if u == UpdateType.custom:
        raise ValueError("custom (Python callback) drivers are supported by the FP64 plain form only")
    w = np.zeros((), dtype=WAVE_DTYPE)
    w["target"] = target
    w["layer_mask"] = layer_mask
    w["amp"] = d.amplitude * amp_scale
    if u in (UpdateType.sine, UpdateType.posine, UpdateType.halfsine):
        w["kind"] = int(u)
        w["ph0"] = q64_frac(d.phase / (2 * np.pi))
        w["dph"] = q64_frac(d.frequency * dt)
        w["dph_half"] = q64_frac(d.frequency * dt * 0.5)
        if u == UpdateType.posine:
            w["amp"] = abs(d.amplitude * amp_scale)
        if u == UpdateType.halfsine:
            w["p0"] = 1.0 if d.amplitude >= 0 else -1.0
    elif u == UpdateType.pulse:
        w["kind"] = int(u)
        w["dph"] = q64_frac(dt / d.period)
        w["dph_half"] = q64_frac(0.5 * dt / d.period)
        w["thr32"] = np.uint32(min(max(d.cycle, 0.0), 1.0 - 2 ** -33) * 2 ** 32)
    elif u == UpdateType.step:
        w["kind"] = int(u)
        on, off = step_window(d.timeStart, d.timeStop, dt, None)
        w["on"] = on
        w["off"] = off
    elif u in (UpdateType.trapezoid, UpdateType.gaussimpulse, UpdateType.gaussstep):
        w["kind"] = int(u)
        i0 = int(round(d.timeStart / dt))
        w["i0"] = i0
        w["p2"] = i0 * dt - d.timeStart
        if u == UpdateType.trapezoid:
            w["p0"] = d.edgeTime
            w["p1"] = d.steadyTime
        elif u == UpdateType.gaussimpulse:
            w["p0"] = 1.0 / d.edgeTime
        else:
            w["p0"] = 1.0 / (np.sqrt(2.0) * d.edgeTime)
    else:
        raise ValueError("unsupported driver type %r" % (u,))
    return w


# --------------------------------------------------------------------------
# Batch specification (structure of arrays, float64 on the host)
# --------------------------------------------------------------------------
@dataclass
class BatchSpec:
    """Structure-of-arrays description of n junctions with up to 4 layers.
    Per-layer arrays are [n, 4, ...]; unused layers are ignored."""
    n: int
    n_layers: np.ndarray                  # [n] int
    m0: np.ndarray                        # [n,4,3]
    anis: np.ndarray                      # [n,4,3]
    Ms: np.ndarray                        # [n,4]
    thickness: np.ndarray                 # [n,4]
    surface: np.ndarray                   # [n,4]
    alpha: np.ndarray                     # [n,4]
    demag: np.ndarray                     # [n,4,9]
    dip_b: np.ndarray                     # [n,4,9]
    dip_t: np.ndarray                     # [n,4,9]
    K: np.ndarray                         # [n,4] constant parts
    K2: np.ndarray
    Jb: np.ndarray
    Jt: np.ndarray
    J2b: np.ndarray
    J2t: np.ndarray
    Hc: np.ndarray                        # [n,4,3] constant Hext+Hoe+Hdmi+Hres
    Db: np.ndarray                        # [n,4,3] IDMI vectors
    Dt: np.ndarray
    I: np.ndarray                         # [n,4] constant current
    FL: np.ndarray
    DL: np.ndarray
    FL2: np.ndarray
    DL2: np.ndarray
    T: np.ndarray                         # [n,4] constant temperature
    temperature: np.ndarray               # [n,4] bool: thermal field on
    ref: np.ndarray                       # [n,4,3]
    ref2: np.ndarray
    ref_type: np.ndarray                  # [n,4] int
    flags: np.ndarray                     # [n,4] int (F32_*)
    stt_p: np.ndarray
    stt_l: np.ndarray
    stt_beta: np.ndarray
    stt_kappa: np.ndarray
    sot_fl: np.ndarray                    # static SOT coefficients
    sot_dl: np.ndarray
    seed: np.ndarray                      # [n,4] uint64
    noise_step: np.ndarray                # [n,4] uint64
    mr_mode: np.ndarray                   # [n] int
    Rp: np.ndarray
    Rap: np.ndarray
    strip: np.ndarray                     # [n,7,4]: Rx0, Ry0, AMR_X, AMR_Y, SMR_X, SMR_Y, AHE
    mix_w: np.ndarray                     # [n,4]
    vsd_freq: np.ndarray                  # [n] Hz (0: no I*R reduction)
    waves: list = field(default_factory=list)   # per junction: list of cmtj_wave_t drafts (scalar)
    wave_drivers: list = field(default_factory=list)  # per junction: list of (driver, target, layer_mask, layer)
    wave_table: np.ndarray = None         # [n, MAX_WAVES] WAVE_DTYPE, vectorised sweeps
    wave_count: np.ndarray = None         # [n] waves used in wave_table

    @staticmethod
    def empty(n):
        z = lambda *s: np.zeros((n,) + s, dtype=np.float64)
        sp = BatchSpec(
            n=n, n_layers=np.ones(n, dtype=np.int32), m0=z(4, 3), anis=z(4, 3), Ms=np.ones((n, 4)),
            thickness=np.ones((n, 4)), surface=z(4), alpha=z(4), demag=z(4, 9), dip_b=z(4, 9), dip_t=z(4, 9),
            K=z(4), K2=z(4), Jb=z(4), Jt=z(4), J2b=z(4), J2t=z(4), Hc=z(4, 3), Db=z(4, 3), Dt=z(4, 3), I=z(4),
            FL=z(4), DL=z(4), FL2=z(4), DL2=z(4), T=z(4), temperature=np.zeros((n, 4), dtype=bool), ref=z(4, 3),
            ref2=z(4, 3), ref_type=np.zeros((n, 4), dtype=np.int32), flags=np.zeros((n, 4), dtype=np.int32),
            stt_p=z(4), stt_l=z(4), stt_beta=z(4), stt_kappa=np.ones((n, 4)), sot_fl=z(4), sot_dl=z(4),
            seed=np.zeros((n, 4), dtype=np.uint64), noise_step=np.zeros((n, 4), dtype=np.uint64),
            mr_mode=np.zeros(n, dtype=np.int32), Rp=z(), Rap=z(), strip=z(7, 4), mix_w=z(4), vsd_freq=z())
        sp.wave_drivers = [[] for _ in range(n)]
        sp.m0[:, :, 2] = 1.0
        sp.anis[:, :, 2] = 1.0
        return sp

    def take(self, rows):
        """A new BatchSpec holding rows `rows` (in that order) of this one."""
        import dataclasses
        rows = np.asarray(rows, dtype=np.int64)
        out = {}
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if f.name == "n":
                out["n"] = len(rows)
            elif isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == self.n:
                out[f.name] = v[rows].copy()
            elif isinstance(v, list) and len(v) == self.n:
                out[f.name] = [v[k] for k in rows]
            else:
                out[f.name] = v
        return BatchSpec(**out)

    @staticmethod
    def from_junctions(junctions):
        sp = BatchSpec.empty(len(junctions))
        for k, j in enumerate(junctions):
            sp.set_junction(k, j)
        return sp

    def set_junction(self, k, j):
        """Fill row k from a Junction object (junction.hpp semantics)."""
        from .core import _AXIAL_SLOTS
        if j.layerNo > 4:
            raise ValueError("the FP32 batched form supports 1-4 layers, got %d" % j.layerNo)
        L = j.layerNo
        self.n_layers[k] = L
        self.mr_mode[k] = j.MR_mode
        self.Rp[k], self.Rap[k] = j.Rp, j.Rap
        if j.MR_mode == MR_STRIP:
            for q, key in enumerate(("Rx0", "Ry0", "AMR_X", "AMR_Y", "SMR_X", "SMR_Y", "AHE")):
                self.strip[k, q, :L] = j.strip[key]
        self.wave_drivers[k] = []
        for l, ly in enumerate(j.layers):
            if ly.alphaNoiseScale != 0:
                raise RuntimeError("the FP32 batched form has no buffered alpha noise; the FP64 plain form "
                                   "(Junction.runSimulation) runs it")
            self.m0[k, l] = ly.mag.tolist()
            self.anis[k, l] = ly.anis.tolist()
            self.Ms[k, l], self.thickness[k, l] = ly.Ms, ly.thickness
            self.surface[k, l], self.alpha[k, l] = ly.cellSurface, ly.damping
            self.demag[k, l] = [c for r in ly.demagTensor for c in (r.x, r.y, r.z)]
            self.dip_b[k, l] = [c for r in ly.dipoleBottom for c in (r.x, r.y, r.z)]
            self.dip_t[k, l] = [c for r in ly.dipoleTop for c in (r.x, r.y, r.z)]
            sc = ly.scalar
            self.K[k, l] = sc["anis"].constantValue
            self.K2[k, l] = sc["anis2"].constantValue
            self.Jb[k, l], self.Jt[k, l] = sc["iec_bottom"].constantValue, sc["iec_top"].constantValue
            self.J2b[k, l], self.J2t[k, l] = sc["iecq_bottom"].constantValue, sc["iecq_top"].constantValue
            self.I[k, l] = sc["current"].constantValue
            self.FL[k, l], self.DL[k, l] = sc["fl"].constantValue, sc["dl"].constantValue
            self.FL2[k, l], self.DL2[k, l] = sc["fl2"].constantValue, sc["dl2"].constantValue
            self.T[k, l] = sc["temperature"].constantValue
            self.temperature[k, l] = ly.temperatureSet
            hc = np.zeros(3)
            for name in ("hext", "hoe", "hdmi", "hres"):
                hc += [d.constantValue for d in ly.axial[name].drivers]
            self.Hc[k, l] = hc
            self.Db[k, l] = [d.constantValue for d in ly.axial["idmi_bottom"].drivers]
            self.Dt[k, l] = [d.constantValue for d in ly.axial["idmi_top"].drivers]
            self.ref[k, l] = ly.referenceLayer.tolist()
            self.ref2[k, l] = ly.secondaryReferenceLayer.tolist()
            self.ref_type[k, l] = int(ly.referenceType)
            fl = 0
            if ly.includeSTT:
                fl |= F32_STT
            elif ly.includeSOT:
                fl |= F32_SOT | (0 if ly.dynamicSOT else F32_SOT_STATIC)
            if ly.alternativeSTT:
                fl |= F32_ALT_STT
            self.flags[k, l] = fl
            self.stt_p[k, l], self.stt_l[k, l] = ly.spinPolarisation, ly.SlonczewskiSpacerLayerParameter
            self.stt_beta[k, l], self.stt_kappa[k, l] = ly.beta, ly.kappa
            self.sot_fl[k, l], self.sot_dl[k, l] = ly.fieldLikeTorque, ly.dampingLikeTorque
            self.seed[k, l] = ly.noise_seed
            self.noise_step[k, l] = ly.noise_step
            # time-dependent drivers
            for name, tgt in (("anis", TGT_K), ("anis2", TGT_K2), ("iec_bottom", TGT_JB), ("iec_top", TGT_JT),
                              ("iecq_bottom", TGT_J2B), ("iecq_top", TGT_J2T), ("current", TGT_I),
                              ("fl", TGT_FL), ("dl", TGT_DL), ("fl2", TGT_FL2), ("dl2", TGT_DL2),
                              ("temperature", TGT_T)):
                d = sc[name]
                if d.update != UpdateType.constant:
                    self.wave_drivers[k].append((d, tgt, 1 << l, l))
            for name in ("hext", "hoe", "hdmi", "hres"):
                for ax, d in enumerate(ly.axial[name].drivers):
                    if d.update != UpdateType.constant:
                        self.wave_drivers[k].append((d, TGT_HX + ax, 1 << l, l))
            for name in ("idmi_bottom", "idmi_top"):
                if any(d.update != UpdateType.constant for d in ly.axial[name].drivers):
                    raise ValueError("time-dependent IDMI drivers are supported by the FP64 plain form only")
        self.mix_w[k, :L] = 1.0 / L


def _merge_waves(drivers, spec, k, dt):
    """Scale each time-dependent driver to its target term and merge copies
    of one driver on several layers into one wave with a layer mask."""
    out = []
    keyed = {}
    for d, tgt, mask, l in drivers:
        Ms, t = spec.Ms[k, l], spec.thickness[k, l]
        if tgt == TGT_K:
            scale = 2.0 / Ms
        elif tgt == TGT_K2:
            scale = 4.0 / Ms
        elif tgt in (TGT_JB, TGT_JT):
            scale = 1.0 / (Ms * t)
        elif tgt in (TGT_J2B, TGT_J2T):
            scale = 2.0 / (Ms * t)
        else:
            scale = 1.0
        key = (tgt, int(d.update), d.amplitude * scale, d.frequency, d.phase, d.period, d.cycle, d.timeStart,
               d.timeStop, d.edgeTime, d.steadyTime)
        if key in keyed:
            out[keyed[key]]["layer_mask"] |= mask
            continue
        w = wave_from_driver(d, tgt, scale, mask, dt)
        keyed[key] = len(out)
        out.append(w)
    return out


@dataclass
class LoweredF32:
    junctions: np.ndarray    # [n] F32_JUNCTION_DTYPE
    layers: np.ndarray       # [sum L] F32_LAYER_DTYPE
    features: np.ndarray     # [n] int feature bits needed
    n_waves: np.ndarray      # [n]
    n_steps: np.ndarray      # [n]


def lower(spec, time_step, n_steps, win_start=None):
    """BatchSpec -> packed FP32 records.  n_steps: scalar or [n]."""
    n = spec.n
    c = _constants.snapshot()
    dt = float(time_step)
    n_steps = np.broadcast_to(np.asarray(n_steps, dtype=np.int64), (n,))
    if np.any(n_steps < 0) or np.any(n_steps >= 2 ** 32):
        raise ValueError("step counts must fit an unsigned 32-bit integer")
    L = spec.n_layers.astype(np.int64)
    if np.any(L < 1) or np.any(L > 4):
        raise ValueError("the FP32 batched form supports 1-4 layers per junction")
    offsets = np.zeros(n, dtype=np.int64)
    offsets[1:] = np.cumsum(L)[:-1]
    total = int(L.sum())
    # flat (junction, layer) index of every real layer
    jj = np.repeat(np.arange(n), L)
    ll = np.arange(total) - np.repeat(offsets, L)
    g = lambda a: a[jj, ll]
    Ms, t, alpha = g(spec.Ms), g(spec.thickness), g(spec.alpha)
    if np.any(Ms * t == 0):
        raise RuntimeError("Failed to divide vector by zero!")
    mst = Ms * t
    lay = np.zeros(total, dtype=F32_LAYER_DTYPE)
    lay["m"] = g(spec.m0)
    lay["anis"] = g(spec.anis)
    lay["kc"] = 2.0 * g(spec.K) / Ms
    lay["k2c"] = 4.0 * g(spec.K2) / Ms
    scale_mu = (Ms / c["mu0"])[:, None]
    lay["demag"] = g(spec.demag) * scale_mu
    lay["dip_b"] = g(spec.dip_b) * scale_mu
    lay["dip_t"] = g(spec.dip_t) * scale_mu
    lay["h0"] = g(spec.Hc)
    lay["jb"] = g(spec.Jb) / mst
    lay["jt"] = g(spec.Jt) / mst
    lay["j2b"] = 2.0 * g(spec.J2b) / mst
    lay["j2t"] = 2.0 * g(spec.J2t) / mst
    lay["dmi_b"] = g(spec.Db) / mst[:, None]
    lay["dmi_t"] = g(spec.Dt) / mst[:, None]
    conv = 1.0 / (1.0 + alpha * alpha)
    lay["gam"] = -c["gyro"] * conv
    lay["gdt"] = -c["gyro"] * conv * dt
    lay["gdt6"] = -c["gyro"] * conv * dt / 6.0
    lay["alpha"] = alpha
    lay["ref"] = g(spec.ref)
    lay["ref2"] = g(spec.ref2)
    lay["ref_type"] = g(spec.ref_type)
    flags = g(spec.flags)
    lay["flags"] = flags
    lay["stt_c"] = c["gyro"] * c["hbar"] / (c["echarge"] * mst) * conv
    lay["stt_cdt"] = c["gyro"] * c["hbar"] / (c["echarge"] * mst) * conv * dt
    lay["stt_cdt6"] = c["gyro"] * c["hbar"] / (c["echarge"] * mst) * conv * dt / 6.0
    lay["stt_p"] = g(spec.stt_p)
    lay["stt_l"] = g(spec.stt_l)
    lay["stt_beta"] = g(spec.stt_beta)
    lay["stt_kappa"] = g(spec.stt_kappa)
    lay["i0"] = g(spec.I)
    static = (flags & F32_SOT_STATIC) != 0
    lay["fl0"] = np.where(static, g(spec.sot_fl), g(spec.FL))
    lay["dl0"] = np.where(static, g(spec.sot_dl), g(spec.DL))
    lay["fl20"] = g(spec.FL2)
    lay["dl20"] = g(spec.DL2)
    vol = g(spec.surface) * t
    temp_on = g(spec.temperature)
    if np.any(temp_on & (vol == 0)):
        raise RuntimeError("Cell surface cannot be 0 during temp. calculations!")
    with np.errstate(divide="ignore", invalid="ignore"):
        sig_c = np.where(temp_on, 2.0 * alpha * c["kB"] / (Ms * vol * c["gyro"]), 0.0)
    lay["sig_c"] = sig_c
    lay["t0"] = np.where(temp_on, g(spec.T), 0.0)
    seed = g(spec.seed).astype(np.uint64)
    lay["seed_lo"] = (seed & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    lay["seed_hi"] = (seed >> np.uint64(32)).astype(np.uint32)
    ns = g(spec.noise_step).astype(np.uint64)
    lay["noise_step_lo"] = (ns & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    lay["noise_step_hi"] = (ns >> np.uint64(32)).astype(np.uint32)

    jun = np.zeros(n, dtype=F32_JUNCTION_DTYPE)
    jun["n_layers"] = L
    jun["mr_mode"] = spec.mr_mode
    jun["layer_offset"] = offsets
    jun["n_steps"] = n_steps
    jun["win_start"] = 0 if win_start is None else np.broadcast_to(np.asarray(win_start), (n,))
    jun["Rp"] = spec.Rp
    jun["Rap"] = spec.Rap
    for q, key in enumerate(("Rx0", "Ry0", "AMR_X", "AMR_Y", "SMR_X", "SMR_Y", "AHE")):
        jun[key] = spec.strip[:, q, :]
    jun["mix_w"] = spec.mix_w
    jun["vsd_dph"] = np.where(spec.vsd_freq != 0, q64_frac(spec.vsd_freq * dt), np.uint64(0))

    # feature bits per junction
    feat = np.zeros(n, dtype=np.int64)
    offdiag = np.abs(spec.demag[:, :, [1, 2, 3, 5, 6, 7]]).sum(axis=2)
    lmask = np.arange(4)[None, :] < L[:, None]
    feat |= np.where(((offdiag > 0) & lmask).any(axis=1), FEAT_FULL_DEMAG, 0)
    feat |= np.where((((np.abs(spec.dip_b).sum(2) + np.abs(spec.dip_t).sum(2)) > 0) & lmask).any(axis=1),
                     FEAT_DIPOLE, 0)
    feat |= np.where((((np.abs(spec.Db).sum(2) + np.abs(spec.Dt).sum(2)) > 0) & lmask).any(axis=1), FEAT_IDMI, 0)
    feat |= np.where(((spec.K2 != 0) & lmask).any(axis=1), FEAT_K2, 0)
    feat |= np.where((((spec.anis != 0).sum(axis=2) > 1) & lmask).any(axis=1), FEAT_OFFAXIS, 0)
    feat |= np.where((((spec.J2b != 0) | (spec.J2t != 0)) & lmask).any(axis=1), FEAT_IEC2, 0)
    feat |= np.where((((spec.flags & F32_STT) != 0) & lmask).any(axis=1), FEAT_STT, 0)
    feat |= np.where((((spec.flags & F32_SOT) != 0) & lmask).any(axis=1), FEAT_SOT, 0)
    n_waves = np.zeros(n, dtype=np.int64)
    if spec.wave_table is not None:
        jun["waves"] = spec.wave_table
        n_waves[:] = spec.wave_count
        jun["n_waves"] = n_waves
        used = np.arange(MAX_WAVES)[None, :] < n_waves[:, None]
        tg = spec.wave_table["target"]
        scal = np.isin(tg, [TGT_K, TGT_K2, TGT_JB, TGT_JT, TGT_J2B, TGT_J2T, TGT_T]) & used
        feat |= np.where((np.isin(tg, [TGT_J2B, TGT_J2T]) & used).any(axis=1), FEAT_IEC2, 0)
        feat |= np.where(scal.any(axis=1), FEAT_SCALAR_WAVES, 0)
        feat |= np.where(((tg == TGT_K2) & used).any(axis=1), FEAT_K2, 0)
        feat |= np.where(n_waves > 0, FEAT_WAVES, 0)
    for k in range(n if spec.wave_table is None else 0):
        ws = list(spec.waves[k]) if spec.waves else []
        if spec.wave_drivers and spec.wave_drivers[k]:
            ws += _merge_waves(spec.wave_drivers[k], spec, k, dt)
        if not ws:
            continue
        if len(ws) > MAX_WAVES:
            raise ValueError("junction %d has %d time-dependent drivers; the FP32 form takes at most %d"
                             % (k, len(ws), MAX_WAVES))
        for q, w in enumerate(ws):
            jun["waves"][k, q] = w
            tg = int(w["target"])
            if tg in (TGT_K, TGT_JB, TGT_JT, TGT_J2B, TGT_J2T, TGT_T):
                feat[k] |= FEAT_SCALAR_WAVES
            if tg in (TGT_J2B, TGT_J2T):
                feat[k] |= FEAT_IEC2
            if tg == TGT_K2:
                feat[k] |= FEAT_SCALAR_WAVES | FEAT_K2
        n_waves[k] = len(ws)
        jun["n_waves"][k] = len(ws)
        feat[k] |= FEAT_WAVES
    return LoweredF32(jun, lay, feat, n_waves, n_steps.astype(np.int64))


# --------------------------------------------------------------------------
# Launch
# --------------------------------------------------------------------------
def log_channels(log_mode, n_layers):
    return 3 * n_layers if log_mode == LOG_M else (0 if log_mode == LOG_NONE else 1)


def default_tile(channels):
    if channels <= 0:
        return 0
    t = max(4, (32 // channels) // 4 * 4)
    while t * channels > 96:
        t -= 4
    return t


class BatchRun:
    """Device-resident batch: records, state, log and per-partition order
    lists.  Call `launch()` (once, or repeatedly with chunk_steps) and
    `fetch()` to read results back."""

    def __init__(self, lowered, time_step, solver=SolverMode.RK4, log_mode=LOG_NONE, log_every=0, log_axis=0,
                 red_every=0, red_weights=None, device="cuda"):
        from . import engine
        t = engine.torch()
        engine.require_gpu()
        self.lib = _abi.load()
        self.lowered = lowered
        self.n = len(lowered.junctions)
        self.dt = float(time_step)
        self.solver = SolverMode(int(solver))
        self.log_mode, self.log_every, self.log_axis, self.red_every = log_mode, int(log_every), log_axis, red_every
        L = lowered.junctions["n_layers"].astype(np.int64)
        # log layout: per junction ceil4(samples) * channels floats
        self.samples = np.zeros(self.n, dtype=np.int64)
        if log_mode != LOG_NONE:
            if self.log_every < 1:
                raise ValueError("log_every must be >= 1 when logging")
            self.samples = (lowered.n_steps + self.log_every - 1) // self.log_every
        pad = (self.samples + 3) // 4 * 4
        chans = np.array([log_channels(log_mode, int(x)) for x in range(5)])[L]
        # each junction owns ceil4(samples) * channels floats; rows start on
        # 16-byte boundaries (log_offset counts units of 4 floats)
        floats = pad * chans
        starts = np.zeros(self.n, dtype=np.int64)
        starts[1:] = np.cumsum(floats)[:-1]
        if np.any(starts // 4 >= 2 ** 32):
            raise ValueError("log buffer beyond 2^34 floats")
        lowered.junctions["log_offset"] = (starts // 4).astype(np.uint32)
        self.log_starts, self.log_pad, self.log_chans = starts, pad, chans
        total_floats = int(floats.sum())
        if total_floats >= 2 ** 32 * 4:
            raise ValueError("log too large")
        self.d_j = engine.to_device(lowered.junctions)
        self.d_l = engine.to_device(lowered.layers)
        st = np.zeros(self.n, dtype=F32_STATE_DTYPE)
        self.d_s = engine.to_device(st)
        self.d_log = t.zeros(max(total_floats, 4), dtype=t.float32, device=device)
        # one work ticket per partition, 64 B apart: partitions run concurrently
        self.d_ticket = t.zeros(16 * 5 * 16, dtype=t.int32, device=device)
        self._streams = None
        # Partitions: one per (layer count, kernel variant).  The variant is
        # chosen from each junction's own features, never from its batch
        # partners, so a junction runs the same code (and gives the same
        # bits) alone or inside any mix.  Longest junctions first.
        own = lowered.features | (np.where(lowered.n_waves > 1, 4, np.where(lowered.n_waves > 0, 1, 0)) << 16)
        variant = np.zeros(self.n, dtype=np.int64)
        keys = L * (1 << 24) + own
        for key in np.unique(keys):
            nl, code = int(key >> 24), int(key & ((1 << 24) - 1))
            v = self.lib.cmtj_batch_variant_f32(nl, int(self.solver), code)
            if v < 0:
                raise ValueError("no FP32 kernel variant for layers=%d features=0x%x" % (nl, code))
            variant[keys == key] = v
        self.parts = []
        self.part_rows = []
        for nl in range(1, 5):
            for v in sorted(set(variant[L == nl].tolist())):
                idx = np.nonzero((L == nl) & (variant == v))[0]
                idx = idx[np.argsort(-lowered.n_steps[idx], kind="stable")]
                self.parts.append((nl, engine.to_device(idx.astype(np.int32)), int(idx.size), int(v)))
                self.part_rows.append(idx)
        self.launch_order = submission_order(
            [(nl, int(lowered.n_steps[rows[0]])) for (nl, _, _, _), rows in zip(self.parts, self.part_rows)])
        # run-time launch choices per partition (cmtj_gb300.autotune):
        # (key, {"bound", "tile", ...}); None: the fixed defaults
        self.tuning = [None] * len(self.parts)
        self.params = np.zeros(1, dtype=F32_PARAMS_DTYPE)
        self.params["dt"] = self.dt
        self.params["solver"] = int(self.solver)
        self.params["log_mode"] = log_mode
        self.params["log_axis"] = log_axis
        self.params["log_every"] = self.log_every
        self.params["red_every"] = red_every
        self.d_w = None
        if red_weights is not None:
            # weighted I*R sum: sample k of N gets red_weights[N-1-k]
            if not red_every:
                raise ValueError("red_weights need red_every >= 1")
            total = reduction_samples(lowered.n_steps, lowered.junctions["win_start"].astype(np.int64),
                                      int(red_every))
            w = np.ascontiguousarray(red_weights, dtype=np.float32).ravel()
            if total.max(initial=0) > w.size:
                raise ValueError("red_weights holds %d values; a junction takes %d samples" % (w.size, total.max()))
            lowered.junctions["red_total"] = total.astype(np.uint32)
            self.d_j = engine.to_device(lowered.junctions)
            self.d_w = t.from_numpy(w.copy()).to(device)
            self.params["red_weights"] = self.d_w.data_ptr()

    def variants(self):
        """[(n_layers, variant code, junction count)] of the partitions."""
        return [(nl, code, cnt) for nl, _, cnt, code in self.parts]

    def launch(self, chunk_steps=None, stream=None, grid_blocks=0):
        """Advance every junction by up to chunk_steps iterations (all of
        them when None).  A chunk must hold whole log tiles so that resumed
        logs stay 16-byte aligned.  Partitions (layer count x kernel
        variant) run concurrently, each on its own stream with its own work
        ticket, so a small partition's long junctions overlap the others
        instead of adding their tail; `stream` waits for all of them.  They
        are submitted in submission_order (longest critical path first), so
        that the CTAs of the partition holding the longest junction reach
        the SMs before the others fill them.  Each
        partition's log tile and resident-CTA bound come from the run-time
        autotuner (cmtj_gb300.autotune), which times them once per kind of
        partition; the choices change no result."""
        from . import engine
        t = engine.torch()
        if len(self.parts) > 80:
            raise ValueError("more than 80 partitions in one batch")
        main = stream if stream is not None else t.cuda.current_stream()
        choices = [self._choice(q, chunk_steps, main) for q in range(len(self.parts))]
        if chunk_steps is not None and self.log_mode != LOG_NONE:
            for (nl, _, _, _), (tile, _) in zip(self.parts, choices):
                if int(chunk_steps) % (self.log_every * tile):
                    raise ValueError("chunk_steps must be a multiple of log_every * %d" % tile)
        multi = len(self.parts) > 1
        if multi and self._streams is None:
            self._streams = [t.cuda.Stream() for _ in range(min(len(self.parts), 8))]
        start = t.cuda.Event()
        if multi:
            start.record(main)
        ends = []
        for i, q in enumerate(self.launch_order):
            s = self._streams[i % len(self._streams)] if multi else main
            if multi:
                s.wait_event(start)
            tile, code = choices[q]
            self._launch_part(q, chunk_steps, s, tile, code, grid_blocks)
            if multi:
                e = t.cuda.Event()
                e.record(s)
                ends.append(e)
        for e in ends:
            main.wait_event(e)

    def graph(self, chunk_steps=None):
        """A CUDA graph of one launch() -- every partition on its stream,
        forked from and joined to the capture stream -- for replay with
        graph.replay(): each replay advances every junction by up to
        chunk_steps iterations from the state it finds, with no host work.
        Launch choices are resolved before the capture."""
        from . import engine
        t = engine.torch()
        self.tune(chunk_steps)
        if len(self.parts) > 1 and self._streams is None:
            self._streams = [t.cuda.Stream() for _ in range(min(len(self.parts), 8))]
        g = t.cuda.CUDAGraph()
        side = t.cuda.Stream()
        side.wait_stream(t.cuda.current_stream())
        with t.cuda.stream(side):
            with t.cuda.graph(g, stream=side):
                self.launch(chunk_steps, stream=side)
        t.cuda.current_stream().wait_stream(side)
        return g

    def tune(self, chunk_steps=None, stream=None):
        """Resolve every partition's launch choices now (trial launches for
        kinds of partition the autotuner has not met), so that a later
        launch() runs no trials."""
        from . import engine
        main = stream if stream is not None else engine.torch().cuda.current_stream()
        return [self._choice(q, chunk_steps, main) for q in range(len(self.parts))]

    def _choice(self, q, chunk_steps, stream):
        """(log tile, variant code) of partition q: the autotuner's choice
        (tuned now if this kind of partition is new), else the defaults."""
        from . import autotune
        nl, _, cnt, code = self.parts[q]
        channels = log_channels(self.log_mode, nl)
        tile, chosen = default_tile(channels), code
        if not autotune.enabled() or cnt == 0:
            return tile, chosen
        key = autotune.f32_key(nl, self.solver, code, channels, self.d_w is not None, cnt)
        c = autotune.lookup(key)
        if c is None:
            c = autotune.tune_f32_partition(self, q, stream, chunk_steps)
            if c is None:
                return tile, chosen
            autotune.store(key, c)
        if channels > 0 and (chunk_steps is None or int(chunk_steps) % (self.log_every * int(c["tile"])) == 0):
            tile = int(c["tile"])
        chosen = (code & 0xffffff) | (int(c["bound"]) << 24)
        self.tuning[q] = (key, {"tile": tile, "bound": int(c["bound"])})
        return tile, chosen

    def _launch_part(self, q, chunk_steps, stream, tile, code, grid_blocks=0):
        """One cmtj_batch_run_f32 launch of partition q on `stream`."""
        from . import engine
        nl, d_order, cnt, _ = self.parts[q]
        pq = self.params.copy()  # the library copies params at launch; one record per partition
        pq["chunk_steps"] = 2 ** 32 - 1 if chunk_steps is None else int(chunk_steps)
        pq["log_tile"] = tile
        ticket = self.d_ticket[16 * q:]
        rc = self.lib.cmtj_batch_run_f32(engine.ptr(self.d_j), engine.ptr(self.d_l), engine.ptr(self.d_s),
                                         engine.ptr(d_order), cnt, nl, code, pq.ctypes.data, engine.ptr(self.d_log),
                                         engine.ptr(ticket), grid_blocks, engine.stream_ptr(stream))
        _abi.check(rc, self.lib)

    def state(self):
        return self.d_s.cpu().numpy().view(F32_STATE_DTYPE)

    def log_of(self, k, log=None):
        """Junction k's log as [samples, channels]."""
        log = self.d_log.cpu().numpy() if log is None else log
        s, c = int(self.samples[k]), int(self.log_chans[k])
        a = log[self.log_starts[k]: self.log_starts[k] + self.log_pad[k] * c].reshape(-1, c)
        return a[:s]


def submission_order(parts):
    """Order in which launch() submits partitions, given (layer count,
    longest junction's steps) per partition: longest critical path first.

    One thread runs a junction from start to end, so a sweep can end no
    sooner than its longest junction takes, at the speed one thread reaches
    among the warps it shares an SM with.  The block scheduler places the
    CTAs of concurrent launches roughly in submission order, and a mixed
    sweep holds more CTAs than fit on the GPU at once (the 3- and 4-layer
    kernels use up to 255 registers a thread), so a partition submitted
    last waits for SM room that the others free only as their queues run
    dry.  A thread's step costs about one unit per layer pair (the 1-layer
    kernel: one unit), so the key is steps x ceil(layers / 2), ties going to
    more layers, then to the earlier partition."""
    def cost(q):
        nl, steps = parts[q]
        return (-int(steps) * ((int(nl) + 1) // 2), -int(nl), q)
    return sorted(range(len(parts)), key=cost)


def reduction_samples(n_steps, win_start, red_every):
    """Samples each junction's on-device reductions take: steps s in
    [win_start, n_steps) with (s - win_start) % red_every == 0."""
    n_steps = np.asarray(n_steps, dtype=np.int64)
    win = np.broadcast_to(np.asarray(win_start, dtype=np.int64), n_steps.shape)
    return np.where(n_steps > win, (n_steps - 1 - win) // red_every + 1, 0)


def lowpass_step_response(n, fs, cutoff=10e6, order=3):
    """Step response s[0..n-1] of the digital Butterworth low-pass that
    cmtj/utils/filters.py:33-43 applies (scipy.signal.butter(order,
    cutoff / (fs/2)) run through lfilter from rest).  For x_0..x_{N-1},
    mean(lfilter(b, a, x)) = sum_k s[N-1-k] x_k / N, so these are the
    red_weights of the filtered spin-diode mean."""
    from scipy.signal import butter, lfilter
    b, a = butter(order, cutoff / (0.5 * fs), btype="low", analog=False)
    return lfilter(b, a, np.ones(int(n)))


def simulate_junctions_f32(junctions, totalTime, timeStep=1e-13, writeFrequency=1e-11,
                           solverMode=SolverMode.RK4):
    """Run Junction objects on the FP32 batched form, logging every layer's
    m at the reference's write cadence.  Returns (BatchRun, [m logs]) where
    each m log is [samples, n_layers, 3]; it does not touch the junctions'
    own logs or state."""
    from ._lower import plan_run
    plan = plan_run(totalTime, timeStep, writeFrequency)
    solver = junctions[0].getSolver(solverMode)
    spec = BatchSpec.from_junctions(junctions)
    low = lower(spec, plan.time_step, plan.total_iterations)
    run = BatchRun(low, plan.time_step, solver, LOG_M, plan.write_every)
    run.launch()
    log = run.d_log.cpu().numpy()
    out = [run.log_of(k, log).reshape(-1, junctions[k].layerNo, 3) for k in range(len(junctions))]
    return run, out


def relax(spec, time_step, n_steps, alpha=1.0):
    """Bring every junction of `spec` close to its static equilibrium: run
    the FP32 form for n_steps with damping `alpha`, no time-dependent
    drivers and no thermal field, then store the final m as spec.m0 (the
    warm start PIMM_procedure gets by sweeping H, procedures.py:114-141).
    Returns the relaxed m [n, 4, 3]."""
    import copy as _copy
    sp = _copy.copy(spec)
    sp.alpha = np.where(spec.alpha > 0, alpha, alpha)
    sp.temperature = np.zeros_like(spec.temperature)
    sp.wave_table = None
    sp.wave_count = None
    sp.waves = []
    sp.wave_drivers = [[] for _ in range(spec.n)]
    low = lower(sp, time_step, n_steps)
    run = BatchRun(low, time_step, SolverMode.RK4, LOG_NONE, 0)
    run.launch()
    m = run.state()["m"].astype(np.float64)
    L = spec.n_layers
    mask = np.arange(4)[None, :] < L[:, None]
    spec.m0 = np.where(mask[..., None], m, spec.m0)
    return spec.m0
