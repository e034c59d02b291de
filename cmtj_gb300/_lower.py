"""Lowering of host-side Junction descriptions into the packed structs of
include/cmtj_gpu.h, and decoding of the solver's log rows back into the
reference's log dictionary (junction.hpp:1580-1636)."""
import operator
from dataclasses import dataclass

import numpy as np

from . import _abi
from . import constants as _constants
from .core import (MR_CLASSIC, MR_NONE, MR_STRIP, SolverMode, UpdateType, _AXIAL_SLOTS, _SCALAR_SLOTS,
                   _UNSET_DRIVER)

# driver slot order of cmtj_layer_t.drv: the scalar slots in _SCALAR_SLOTS
# order, then three per axial slot in _AXIAL_SLOTS order
if [i for i, _ in enumerate(_SCALAR_SLOTS)] + [b + k for b in _AXIAL_SLOTS.values() for k in range(3)] != \
        list(range(_abi.NUM_SLOTS)):
    raise ImportError("driver slot tables do not match cmtj_layer_t.drv")

# stages each solver evaluates drivers at: 0 -> t, 1 -> t + dt/2, 2 -> t + dt
_SOLVER_STAGES = {
    SolverMode.RK4: (0, 1, 2),
    SolverMode.EulerHeun: (0,),
    SolverMode.Heun: (0, 2),
}


@dataclass
class RunPlan:
    """Junction::runSimulation arguments resolved as the reference does
    (junction.hpp:1952-1959): truncating casts of totalTime/timeStep and
    writeFrequency/timeStep.  `adaptive` marks a Dormand-Prince run
    (junction.hpp:1982-2045), whose log length depends on the step sizes
    it picks: at most floor(totalTime / writeFrequency) + 2 rows."""
    time_step: float
    total_iterations: int
    write_every: int
    total_time: float = 0.0
    write_frequency: float = 0.0
    adaptive: bool = False

    @property
    def n_log(self):
        if self.adaptive:
            return int(self.total_time / self.write_frequency) + 2
        if self.total_iterations == 0:
            return 0
        return (self.total_iterations + self.write_every - 1) // self.write_every

    def for_solver(self, solver):
        """This plan for `solver` (Dormand-Prince plans are adaptive)."""
        import dataclasses
        return dataclasses.replace(self, adaptive=SolverMode(int(solver)) == SolverMode.DormandPrince)

    @property
    def max_attempts(self):
        """Dormand-Prince step attempts before the run stops with an error:
        100 attempts per initial step of the horizon, at least 10^6."""
        return int(max(1e6, 100.0 * self.total_time / self.time_step))


def plan_run(totalTime, timeStep=1e-13, writeFrequency=1e-11, solver=None):
    totalTime, timeStep, writeFrequency = float(totalTime), float(timeStep), float(writeFrequency)
    if timeStep > writeFrequency:
        raise RuntimeError("The time step cannot be larger than write frequency!")
    total = totalTime / timeStep
    we = writeFrequency / timeStep
    if not (0 <= total < 2 ** 32) or not (1 <= we < 2 ** 32):
        raise ValueError("totalTime/timeStep and writeFrequency/timeStep must fit an unsigned 32-bit count")
    plan = RunPlan(timeStep, int(total), int(we), totalTime, writeFrequency)
    return plan.for_solver(solver) if solver is not None else plan


class TableBuilder:
    """Samples custom (Python callback) drivers at every time the solver
    asks for: t = i*dt, i*dt + 0.5*dt and i*dt + dt (junction.hpp:1974,
    1024-1031), each formed in double precision like the reference."""

    def __init__(self, plan, solver):
        self.plan = plan
        self.stages = _SOLVER_STAGES.get(SolverMode(int(solver)))
        self.chunks = []
        self.size = 0
        self._cache = {}

    def add(self, driver):
        if self.stages is None:
            raise RuntimeError("custom (Python) drivers cannot be sampled ahead of time at the adaptive times "
                               "of SolverMode.DormandPrince")
        key = id(driver.callback)
        if key in self._cache:
            return self._cache[key]
        n = self.plan.total_iterations
        dt = self.plan.time_step
        tab = np.zeros((n, 3), dtype=np.float64)
        from .core import _call_custom
        for i in range(n):
            t = float(i) * dt
            for s in self.stages:
                ts = t if s == 0 else (t + 0.5 * dt if s == 1 else t + dt)
                tab[i, s] = _call_custom(driver.callback, ts)
        off = self.size
        self.chunks.append(tab.ravel())
        self.size += tab.size
        self._cache[key] = off
        return off

    def array(self):
        if not self.chunks:
            return None
        return np.concatenate(self.chunks)


def _driver_record(d, tables):
    """One cmtj_driver_t as a tuple in DRIVER_DTYPE field order."""
    u = d.update
    if u is _CUSTOM:
        if tables is None:
            raise RuntimeError("custom drivers need a run plan")
        return (_abi.DRV_TABLE, 0, tables.add(d), 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    return (int(u), 0, 0, d.constantValue, d.amplitude, d.frequency, d.phase, d.period, d.cycle,
            d.timeStart, d.timeStop, d.edgeTime, d.steadyTime)


_CUSTOM = UpdateType.custom
_UNSET_RECORD = np.array(_driver_record(_UNSET_DRIVER, None), dtype=_abi.DRIVER_DTYPE)


def _tensor9(rows):
    return [v for r in rows for v in (r.x, r.y, r.z)]


_LAYER_SCALARS = (("Ms", "Ms"), ("thickness", "thickness"), ("cellSurface", "cellSurface"),
                  ("cellVolume", "cellVolume"), ("damping", "damping"), ("fieldLikeTorque", "fieldLikeTorque"),
                  ("dampingLikeTorque", "dampingLikeTorque"), ("slonczewski", "SlonczewskiSpacerLayerParameter"),
                  ("beta", "beta"), ("kappa", "kappa"), ("spinPolarisation", "spinPolarisation"),
                  ("noise_step", "noise_step"))
_LAYER_FLOATS = tuple(fa for fa in _LAYER_SCALARS if fa[0] != "noise_step")
_LAYER_FLOAT_VALUES = operator.attrgetter(*(attr for _, attr in _LAYER_FLOATS))
_LAYER_FLAGS = ("includeSTT", "includeSOT", "dynamicSOT", "alternativeSTT", "temperatureSet")
_ADAPTIVE_FIELDS = ("abs_tol", "rel_tol", "max_factor", "min_factor", "safety_factor", "ki", "kp", "kd",
                    "prev_error_ratio", "integral_error")
_ADAPTIVE_VALUES = operator.attrgetter(*_ADAPTIVE_FIELDS)


def lower_layers(layers, larr, tables=None):
    """cmtj_layer_t records of `layers` into larr (same length), column by
    column; custom drivers are tabulated in layer order, scalar slots before
    axial ones."""
    larr["mag"] = [(l.mag.x, l.mag.y, l.mag.z) for l in layers]
    larr["anis"] = [(l.anis.x, l.anis.y, l.anis.z) for l in layers]
    larr["ref"] = [tuple(l.referenceLayer) for l in layers]
    larr["ref2"] = [tuple(l.secondaryReferenceLayer) for l in layers]
    larr["demag"] = [_tensor9(l.demagTensor) for l in layers]
    larr["dipole_top"] = [_tensor9(l.dipoleTop) for l in layers]
    larr["dipole_bottom"] = [_tensor9(l.dipoleBottom) for l in layers]
    n = len(layers)
    # the FP64 scalars of all layers as one [n][k] array, then column by column
    vals = np.array([_LAYER_FLOAT_VALUES(l) for l in layers], dtype=np.float64).reshape(n, len(_LAYER_FLOATS))
    for c, (field, _) in enumerate(_LAYER_FLOATS):
        larr[field] = vals[:, c]
    larr["noise_step"] = [l.noise_step for l in layers]
    larr["referenceType"] = [int(l.referenceType) for l in layers]
    for field in _LAYER_FLAGS:
        larr[field] = [int(getattr(l, field)) for l in layers]
    larr["seed_lo"] = [l.noise_seed & 0xFFFFFFFF for l in layers]
    larr["seed_hi"] = [(l.noise_seed >> 32) & 0xFFFFFFFF for l in layers]
    ap = larr["adaptive"]
    aps = [l.adaptiveParams for l in layers]
    vals = np.array([_ADAPTIVE_VALUES(a) for a in aps], dtype=np.float64).reshape(n, len(_ADAPTIVE_FIELDS))
    for c, field in enumerate(_ADAPTIVE_FIELDS):
        ap[field] = vals[:, c]
    ap["use_pid_control"] = [int(bool(a.use_pid_control)) for a in aps]
    if layers:
        larr["drv"] = _driver_slots(layers, tables)
    derive_layers(larr)


def _driver_slots(layers, tables):
    """The [layer][slot] cmtj_driver_t records.  Slot order: the scalar
    slots in _SCALAR_SLOTS order, then three per axial slot in _AXIAL_SLOTS
    order (checked at import).  Slots a layer was never given a driver for
    hold the shared unset driver and start as its record; only the others
    are converted, in layer and slot order (the order custom drivers are
    tabulated in)."""
    drv = np.empty(len(layers) * _abi.NUM_SLOTS, dtype=_abi.DRIVER_DTYPE)
    drv[:] = _UNSET_RECORD
    idx, recs = [], []
    unset, rec = _UNSET_DRIVER, _driver_record
    axial_names = tuple(_AXIAL_SLOTS)
    s = 0
    for l in layers:
        sc, ax = l.scalar, l.axial
        for name in _SCALAR_SLOTS:
            d = sc[name]
            if d is not unset:
                idx.append(s)
                recs.append(rec(d, tables))
            s += 1
        for name in axial_names:
            for d in ax[name].drivers:
                if d is not unset:
                    idx.append(s)
                    recs.append(rec(d, tables))
                s += 1
    if idx:
        drv[idx] = np.array(recs, dtype=_abi.DRIVER_DTYPE)
    return drv.reshape(len(layers), _abi.NUM_SLOTS)


def _const_zero(drv, slot):
    return (drv["update"][:, slot] == _abi.DRV_CONSTANT) & (drv["constantValue"][:, slot] == 0.0)


def derive_layers(larr):
    """The derived fields of cmtj_layer_t records: the reference's constant
    sub-expressions, evaluated once in FP64 exactly as it writes them
    (element-wise numpy arithmetic rounds each operation like the scalar
    form), and the CMTJ_ZERO_* mask of field terms that are identically
    zero."""
    c = _constants.snapshot()
    d = larr["damping"]
    larr["conv_term"] = 1 / (1 + d * d)
    larr["stoch_conv"] = -c["gyro"] / (1. + d * d)
    larr["ms_over_mu0"] = larr["Ms"] / c["mu0"]
    drv = larr["drv"]
    z = np.zeros(len(larr), dtype=np.uint32)
    z[~np.any(larr["dipole_top"] != 0, axis=1) & ~np.any(larr["dipole_bottom"] != 0, axis=1)] |= _abi.ZERO_DIPOLE
    idmi = np.ones(len(larr), dtype=bool)
    for k in range(3):
        idmi &= _const_zero(drv, _abi.SLOT_IDMI_TOP + k) & _const_zero(drv, _abi.SLOT_IDMI_BOTTOM + k)
    z[idmi] |= _abi.ZERO_IDMI
    z[_const_zero(drv, _abi.SLOT_ANIS2)] |= _abi.ZERO_K2
    z[_const_zero(drv, _abi.SLOT_IECQ_TOP) & _const_zero(drv, _abi.SLOT_IECQ_BOTTOM)] |= _abi.ZERO_J2
    larr["zero_terms"] = z


def lower_junction(junction, rec, layer_offset):
    rec["n_layers"] = junction.layerNo
    rec["mr_mode"] = junction.MR_mode
    rec["layer_offset"] = layer_offset
    rec["Rp"] = junction.Rp
    rec["Rap"] = junction.Rap
    if junction.MR_mode == MR_STRIP:
        for k, v in junction.strip.items():
            arr = np.zeros(_abi.MAX_LAYERS)
            arr[:len(v)] = v
            rec[k] = arr


def validate(junctions, solver, max_layers=_abi.MAX_LAYERS):
    """Reference exceptions that depend only on the inputs, raised before
    any work is launched (the reference raises them at the first step)."""
    for j in junctions:
        if j.layerNo > max_layers:
            raise ValueError("the GPU solver supports at most %d layers per junction, got %d" %
                             (max_layers, j.layerNo))
        for l in j.layers:
            if l.alphaNoiseScale != 0 and solver not in (SolverMode.EulerHeun, SolverMode.Heun):
                raise RuntimeError("buffered alpha noise runs under Euler-Heun or Heun (getSolver forces them)")
            if l.Ms * l.thickness == 0:
                raise RuntimeError("Failed to divide vector by zero!")
            if l.temperatureSet and solver in (SolverMode.EulerHeun, SolverMode.Heun) and l.cellVolume == 0.0:
                raise RuntimeError("Cell surface cannot be 0 during temp. calculations!")


@dataclass
class Lowered:
    junctions: np.ndarray
    layers: np.ndarray
    tables: np.ndarray
    params: np.ndarray
    log_width: int
    # buffered alpha noise of this run: cmtj_alpha_noise_t rows (x, y, z of
    # each noisy layer in turn) and the layer index each triple belongs to;
    # the runner fills the buffers and sets layers[q]["alpha_buf"]
    alpha_specs: np.ndarray = None
    alpha_layers: np.ndarray = None


def alpha_noise_rows(layers, larr, plan):
    """cmtj_alpha_noise_t rows of the layers with a non-zero alpha-noise
    scale (createBufferedAlphaNoise(totalIterations) per layer and run,
    junction.hpp:1912-1916): three rows (normals 0, 1, 2 of the layer's
    alpha-noise stream at counter noise_step + m) per noisy layer; fills
    the layers' alpha_scale, alpha_axis and alpha_len."""
    from .noise import specs_array
    rows, which = [], []
    for q, l in enumerate(layers):
        if l.alphaNoiseScale == 0:
            continue
        which.append(q)
        rows += [(l.alphaNoise, l.alphaNoiseStd, l.noise_seed, l.noise_step, c) for c in range(3)]
        larr[q]["alpha_scale"] = l.alphaNoiseScale
        larr[q]["alpha_axis"] = int(l.alphaNoiseAxis)
        larr[q]["alpha_len"] = plan.total_iterations
    if not which:
        return None, None
    if plan.total_iterations > _abi.ALPHA_MAX_LEN:
        raise ValueError("alpha noise: %d iterations exceed the %d samples of a buffer" %
                         (plan.total_iterations, _abi.ALPHA_MAX_LEN))
    return specs_array(rows), np.asarray(which, dtype=np.int64)


def lower(junctions, plan, solver, calculate_energies, arithmetic="reference"):
    solver = SolverMode(int(solver))
    plan = plan.for_solver(solver)
    validate(junctions, solver)
    n_layers = sum(j.layerNo for j in junctions)
    jarr = np.zeros(len(junctions), dtype=_abi.JUNCTION_DTYPE)
    larr = np.zeros(n_layers, dtype=_abi.LAYER_DTYPE)
    tables = TableBuilder(plan, solver)
    off = 0
    for k, j in enumerate(junctions):
        lower_junction(j, jarr[k], off)
        off += j.layerNo
    all_layers = [l for j in junctions for l in j.layers]
    lower_layers(all_layers, larr, tables)
    alpha_specs, alpha_layers = (alpha_noise_rows(all_layers, larr, plan) if plan.total_iterations
                                 else (None, None))
    max_layers = max(j.layerNo for j in junctions)
    width = _abi.log_width(max_layers, calculate_energies)
    params = make_params(plan, solver, calculate_energies, width, max_layers, arithmetic)
    return Lowered(jarr, larr, tables.array(), params, width, alpha_specs, alpha_layers)


def with_alpha_buffers(lowered, base_address):
    """The layer records with alpha_buf pointing into a buffer array at
    base_address ([rows][alpha_len] float32, rows in alpha_specs order)."""
    larr = lowered.layers
    if lowered.alpha_specs is None:
        return larr
    larr = larr.copy()
    n = int(larr[lowered.alpha_layers[0]]["alpha_len"])
    for a, q in enumerate(lowered.alpha_layers.tolist()):
        larr[q]["alpha_buf"] = base_address + 4 * 3 * a * n
    return larr


def make_params(plan, solver, calculate_energies, width, max_layers=0, arithmetic="reference"):
    """cmtj_sim_params_t of a run.  arithmetic: "reference" (the reference's
    operations in its order: its bits) or "fused" (CMTJ_ARITH_FUSED: field-only
    RK4 layers with constant anisotropy and IEC in fused FP64 arithmetic, not
    bit-identical)."""
    if arithmetic not in _abi.ARITHMETIC:
        raise ValueError("arithmetic must be one of %s, not %r" % (sorted(_abi.ARITHMETIC), arithmetic))
    p = np.zeros(1, dtype=_abi.SIM_PARAMS_DTYPE)
    p["arithmetic"] = _abi.ARITHMETIC[arithmetic]
    p["max_layers"] = max_layers
    p["time_step"] = plan.time_step
    p["total_iterations"] = plan.total_iterations
    p["write_every"] = plan.write_every
    p["n_log"] = plan.n_log
    p["solver"] = int(solver)
    p["calculate_energies"] = int(bool(calculate_energies))
    p["log_width"] = width
    p["total_time"] = plan.total_time
    p["write_frequency"] = plan.write_frequency
    p["max_attempts"] = plan.max_attempts
    c = _constants.snapshot()
    for k in ("mu0", "gyro", "TtoAm", "hbar", "echarge", "kB"):
        p["c"][k] = c[k]
    return p


_ENERGY_VEC = ("Hext", "Hiec", "Hanis", "Hdemag", "Hth", "Hfl", "Hdl")


def decode_log(junction, rows, calculate_energies):
    """One junction's [n_rows][width] log rows -> ordered column dict with
    the reference's keys."""
    cols = {}
    c = 0
    for l in junction.layers:
        lid = l.id
        if calculate_energies:
            I = rows[:, c + 4]
            cols[lid + "_K"] = rows[:, c]
            cols[lid + "_K2"] = rows[:, c + 1]
            cols[lid + "_Jbottom"] = rows[:, c + 2]
            cols[lid + "_Jtop"] = rows[:, c + 3]
            # junction.hpp:1593 and 1611-1612: "_I" gets a second entry per
            # row when the layer has STT or SOT.
            cols[lid + "_I"] = np.repeat(I, 2) if (l.includeSTT or l.includeSOT) else I
            for q, name in enumerate(_ENERGY_VEC):
                if name in ("Hfl", "Hdl") and not l.includeSOT:
                    continue
                for a, ax in enumerate("xyz"):
                    cols[lid + "_" + name + ax] = rows[:, c + 5 + 3 * q + a]
            c += _abi.ENERGY_COLS - 3
        cols[lid + "_mx"] = rows[:, c]
        cols[lid + "_my"] = rows[:, c + 1]
        cols[lid + "_mz"] = rows[:, c + 2]
        c += 3
    if junction.MR_mode == MR_CLASSIC and junction.layerNo == 1:
        cols["R"] = rows[:, c]
    elif junction.MR_mode == MR_CLASSIC and junction.layerNo > 1:
        cols[junction.Rtag] = rows[:, c]
    elif junction.MR_mode == MR_STRIP:
        cols["Rx"] = rows[:, c]
        cols["Ry"] = rows[:, c + 1]
        cols["Rz"] = rows[:, c + 2]
    cols["time"] = rows[:, c + 3]
    return cols


def apply_results(junctions, lowered, log, status, plan):
    """Write final magnetisations back, append logs, raise on NaN."""
    nan = False
    # whole columns as Python lists: one conversion instead of a record
    # lookup per layer (the values are the same doubles)
    offsets = lowered.junctions["layer_offset"].tolist()
    codes = np.asarray(status).tolist()
    mags = lowered.layers["mag"].tolist()
    if plan.adaptive:
        prev_ratio = lowered.layers["adaptive"]["prev_error_ratio"].tolist()
        integral = lowered.layers["adaptive"]["integral_error"].tolist()
    energies = bool(lowered.params["calculate_energies"][0])
    for k, j in enumerate(junctions):
        off = offsets[k]
        code, rows = codes[2 * k], codes[2 * k + 1]
        for i, l in enumerate(j.layers):
            l.mag.x, l.mag.y, l.mag.z = mags[off + i]
            l.noise_step += plan.total_iterations
            if plan.adaptive:
                l.adaptiveParams.prev_error_ratio = prev_ratio[off + i]
                l.adaptiveParams.integral_error = integral[off + i]
        if rows:
            j._append_log(decode_log(j, log[k, :rows], energies), rows)
        if code == _abi.STATUS_NAN:
            nan = True
        elif code == _abi.STATUS_DP_STALL:
            raise RuntimeError(
                "Dormand-Prince: a layer of a multi-layer junction rejected a step; the reference then uses the "
                "unassigned Layer::hopt (-1) as the step and does not terminate (junction.hpp:1700-1705)")
        elif code == _abi.STATUS_LIMIT:
            raise RuntimeError("Dormand-Prince: no end after %d step attempts" % plan.max_attempts)
        elif code != _abi.STATUS_OK:
            raise RuntimeError("solver status %d for junction %d" % (code, k))
    if nan:
        raise RuntimeError("NAN magnetisation")
