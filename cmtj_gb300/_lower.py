"""Lowering of host-side Junction descriptions into the packed structs of
include/cmtj_gpu.h, and decoding of the solver's log rows back into the
reference's log dictionary (junction.hpp:1580-1636)."""
from dataclasses import dataclass

import numpy as np

from . import _abi
from . import constants as _constants
from .core import MR_CLASSIC, MR_NONE, MR_STRIP, SolverMode, UpdateType, _AXIAL_SLOTS, _SCALAR_SLOTS

_SCALAR_INDEX = {name: i for i, name in enumerate(_SCALAR_SLOTS)}

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
    writeFrequency/timeStep."""
    time_step: float
    total_iterations: int
    write_every: int

    @property
    def n_log(self):
        if self.total_iterations == 0:
            return 0
        return (self.total_iterations + self.write_every - 1) // self.write_every


def plan_run(totalTime, timeStep=1e-13, writeFrequency=1e-11):
    totalTime, timeStep, writeFrequency = float(totalTime), float(timeStep), float(writeFrequency)
    if timeStep > writeFrequency:
        raise RuntimeError("The time step cannot be larger than write frequency!")
    total = totalTime / timeStep
    we = writeFrequency / timeStep
    if not (0 <= total < 2 ** 32) or not (1 <= we < 2 ** 32):
        raise ValueError("totalTime/timeStep and writeFrequency/timeStep must fit an unsigned 32-bit count")
    return RunPlan(timeStep, int(total), int(we))


class TableBuilder:
    """Samples custom (Python callback) drivers at every time the solver
    asks for: t = i*dt, i*dt + 0.5*dt and i*dt + dt (junction.hpp:1974,
    1024-1031), each formed in double precision like the reference."""

    def __init__(self, plan, solver):
        self.plan = plan
        self.stages = _SOLVER_STAGES[SolverMode(int(solver))]
        self.chunks = []
        self.size = 0
        self._cache = {}

    def add(self, driver):
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


def _fill_driver(rec, d, tables):
    if d.update == UpdateType.custom:
        if tables is None:
            raise RuntimeError("custom drivers need a run plan")
        rec["update"] = _abi.DRV_TABLE
        rec["table_offset"] = tables.add(d)
        return
    rec["update"] = int(d.update)
    rec["table_offset"] = 0
    for f in ("constantValue", "amplitude", "frequency", "phase", "period", "cycle", "timeStart", "timeStop",
              "edgeTime", "steadyTime"):
        rec[f] = getattr(d, f)


def _tensor9(rows):
    return np.array([[r.x, r.y, r.z] for r in rows], dtype=np.float64).ravel()


def lower_layer(layer, rec, tables=None):
    rec["mag"] = (layer.mag.x, layer.mag.y, layer.mag.z)
    rec["anis"] = (layer.anis.x, layer.anis.y, layer.anis.z)
    rec["ref"] = tuple(layer.referenceLayer)
    rec["ref2"] = tuple(layer.secondaryReferenceLayer)
    rec["demag"] = _tensor9(layer.demagTensor)
    rec["dipole_top"] = _tensor9(layer.dipoleTop)
    rec["dipole_bottom"] = _tensor9(layer.dipoleBottom)
    rec["Ms"] = layer.Ms
    rec["thickness"] = layer.thickness
    rec["cellSurface"] = layer.cellSurface
    rec["cellVolume"] = layer.cellVolume
    rec["damping"] = layer.damping
    rec["fieldLikeTorque"] = layer.fieldLikeTorque
    rec["dampingLikeTorque"] = layer.dampingLikeTorque
    rec["slonczewski"] = layer.SlonczewskiSpacerLayerParameter
    rec["beta"] = layer.beta
    rec["kappa"] = layer.kappa
    rec["spinPolarisation"] = layer.spinPolarisation
    rec["referenceType"] = int(layer.referenceType)
    rec["includeSTT"] = int(layer.includeSTT)
    rec["includeSOT"] = int(layer.includeSOT)
    rec["dynamicSOT"] = int(layer.dynamicSOT)
    rec["alternativeSTT"] = int(layer.alternativeSTT)
    rec["temperatureSet"] = int(layer.temperatureSet)
    rec["seed_lo"] = layer.noise_seed & 0xFFFFFFFF
    rec["seed_hi"] = (layer.noise_seed >> 32) & 0xFFFFFFFF
    rec["noise_step"] = layer.noise_step
    drv = rec["drv"]
    for name, idx in _SCALAR_INDEX.items():
        _fill_driver(drv[idx], layer.scalar[name], tables)
    for name, base in _AXIAL_SLOTS.items():
        for k in range(3):
            _fill_driver(drv[base + k], layer.axial[name].drivers[k], tables)


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
            if l.alphaNoiseScale != 0:
                raise RuntimeError("buffered 1/f alpha noise (core/noise.hpp) is not supported by the GPU solver")
            if l.Ms * l.thickness == 0:
                raise RuntimeError("Failed to divide vector by zero!")
            if l.temperatureSet and solver in (SolverMode.EulerHeun, SolverMode.Heun) and l.cellVolume == 0.0:
                raise RuntimeError("Cell surface cannot be 0 during temp. calculations!")
    if solver == SolverMode.DormandPrince:
        raise RuntimeError("SolverMode.DormandPrince is not implemented by the GPU solver")


@dataclass
class Lowered:
    junctions: np.ndarray
    layers: np.ndarray
    tables: np.ndarray
    params: np.ndarray
    log_width: int


def lower(junctions, plan, solver, calculate_energies):
    solver = SolverMode(int(solver))
    validate(junctions, solver)
    n_layers = sum(j.layerNo for j in junctions)
    jarr = np.zeros(len(junctions), dtype=_abi.JUNCTION_DTYPE)
    larr = np.zeros(n_layers, dtype=_abi.LAYER_DTYPE)
    tables = TableBuilder(plan, solver)
    off = 0
    for k, j in enumerate(junctions):
        lower_junction(j, jarr[k], off)
        for l in j.layers:
            lower_layer(l, larr[off], tables)
            off += 1
    width = _abi.log_width(max(j.layerNo for j in junctions), calculate_energies)
    params = make_params(plan, solver, calculate_energies, width)
    return Lowered(jarr, larr, tables.array(), params, width)


def make_params(plan, solver, calculate_energies, width):
    p = np.zeros(1, dtype=_abi.SIM_PARAMS_DTYPE)
    p["time_step"] = plan.time_step
    p["total_iterations"] = plan.total_iterations
    p["write_every"] = plan.write_every
    p["n_log"] = plan.n_log
    p["solver"] = int(solver)
    p["calculate_energies"] = int(bool(calculate_energies))
    p["log_width"] = width
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
    for k, j in enumerate(junctions):
        off = int(lowered.junctions[k]["layer_offset"])
        code, rows = int(status[2 * k]), int(status[2 * k + 1])
        for i, l in enumerate(j.layers):
            m = lowered.layers[off + i]["mag"]
            l.mag.x, l.mag.y, l.mag.z = float(m[0]), float(m[1]), float(m[2])
            l.noise_step += plan.total_iterations
        if rows:
            j._append_log(decode_log(j, log[k, :rows], bool(lowered.params["calculate_energies"][0])), rows)
        if code == _abi.STATUS_NAN:
            nan = True
        elif code != _abi.STATUS_OK:
            raise RuntimeError("solver status %d for junction %d" % (code, k))
    if nan:
        raise RuntimeError("NAN magnetisation")
