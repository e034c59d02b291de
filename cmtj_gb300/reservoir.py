"""`cmtj.reservoir`: dipole-coupled junction groups (core/reservoir.hpp,
bound at python/cmtj.cpp:428-445).

GroupInteraction keeps the reference's constructor checks, interaction
functions, per-step semantics and per-junction logs.  Its run is one device
launch (cmtj_run_group_f64): one CTA per group, each junction's layers on
lanes (one thread per junction for groups too wide for that), the FP64
plain form's device physics.  The pair geometry the interaction uses
(separations and their 3rd and 5th powers, or the dipole tensors) never
changes during a run, so the host forms it once here with the same libm
calls and operand order as the reference, and the device evaluates only the
part that depends on the magnetisations.
"""
import copy
import math

import numpy as np

from . import _abi
from .core import CVector, AxialDriver, SolverMode

GROUP_DTYPE = np.dtype(
    [("first_junction", "<i4"), ("n_junctions", "<i4"), ("interaction", "<i4"), ("single_layer_runner", "<i4"),
     ("pair_offset", "<i8")], align=True)
PAIR_DTYPE = np.dtype([("g", "<f8", 9), ("scale", "<f8")], align=True)

INTERACTION_NULL, INTERACTION_DIPOLE, INTERACTION_NOUMRA = 0, 1, 2
MAX_GROUP_JUNCTIONS = 256


def _mu0():
    from . import constants
    return constants.snapshot()["mu0"]


def _v(a):
    return (float(a.x), float(a.y), float(a.z))


def _length(v):
    # CVector::length: sqrt(pow(x,2) + pow(y,2) + pow(z,2)), pow(.,2) = x*x
    return math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])


def _dipole_geometry(r1, r2):
    """rij = r1 - r2, |rij|^3 and |rij|^5 (reservoir.hpp:82-90)."""
    rij = (r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2])
    n = _length(rij)
    if n < 1e-10:
        raise RuntimeError("Points are too close for stable dipole calculation")
    return rij, math.pow(n, 3), math.pow(n, 5)


def _dipole_tensor(r1, r2):
    """getDipoleTensorFromRelPositions (reservoir.hpp:37-57), row-major."""
    rij = (r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2])
    n = _length(rij)
    if n < 1e-14:
        raise RuntimeError("Points are too close for stable dipole calculation")
    r_mag = n * n
    mult = 3 / (4 * math.pi * math.pow(n, 5))
    x, y, z = rij
    rows = ((x * x - (r_mag / 3), x * y, x * z), (x * y, y * y - (r_mag / 3), y * z),
            (x * z, y * z, z * z - (r_mag / 3)))
    return [c * mult for r in rows for c in r]


def nullDipoleInteraction(r1, r2, layer1, layer2):
    """reservoir.hpp:61-66."""
    return CVector(0, 0, 0)


def computeDipoleInteraction(r1, r2, layer1, layer2):
    """Kanao et al. (2019) form (reservoir.hpp:68-97): the field at r1 from
    layer2's moment at r2."""
    rij, r3, r5 = _dipole_geometry(_v(r1), _v(r2))
    m = _v(layer2.mag)
    V = layer2.thickness * layer2.cellSurface
    pref = (layer2.Ms / _mu0()) * V
    s = 3 * (m[0] * rij[0] + m[1] * rij[1] + m[2] * rij[2])
    out = [pref * ((s * rij[k]) / r5 - m[k] / r3) for k in range(3)]
    return CVector(*out)


def computeDipoleInteractionNoumra(r1, r2, layer1, layer2):
    """Nomura et al. (2019) form (reservoir.hpp:99-122)."""
    t = _dipole_tensor(_v(r1), _v(r2))
    m = _v(layer2.mag)
    V = layer2.thickness * layer2.cellSurface
    scale = (layer2.Ms * V) / _mu0()
    out = [(t[3 * r] * m[0] + t[3 * r + 1] * m[1] + t[3 * r + 2] * m[2]) * scale for r in range(3)]
    return CVector(*out)


_KIND = {nullDipoleInteraction: INTERACTION_NULL, computeDipoleInteraction: INTERACTION_DIPOLE,
         computeDipoleInteractionNoumra: INTERACTION_NOUMRA}


class GroupInteraction:
    """reservoir.hpp:122-245.  The junctions are copied on construction (the
    binding converts the list to std::vector<Junction>), and getLog(id)
    returns the group's copy's log."""

    def __init__(self, coordinateMatrix, junctionList, topId="free"):
        coords = [CVector._coerce(c) for c in coordinateMatrix]
        if len(coords) != len(junctionList):
            raise RuntimeError("Coordinate matrix and junction list must have the same size!")
        if not coords or not junctionList:
            raise RuntimeError("Coordinate matrix and junction list cannot be empty!")
        for i in range(len(coords)):
            for j in range(i + 1, len(coords)):
                if _v(coords[i]) == _v(coords[j]):
                    raise RuntimeError("Coordinate vectors must be unique!")
        self.topId = str(topId)
        self.coordinateMatrix = coords
        self.junctionList = [copy.deepcopy(j) for j in junctionList]
        self.noElements = len(self.junctionList)
        self.interactionFunc = computeDipoleInteraction

    def setInteractionFunction(self, interactionFunc):
        self.interactionFunc = interactionFunc

    def clearLogs(self):
        for j in self.junctionList:
            j.clearLog()

    def getLog(self, id):
        if 0 <= int(id) < len(self.junctionList):
            return self.junctionList[int(id)].getLog()
        raise RuntimeError("Asking for id of a non-existing junction!")

    def _pairs(self, kind):
        n = self.noElements
        pairs = np.zeros(n * n, dtype=PAIR_DTYPE)
        if kind == INTERACTION_NULL:
            return pairs
        mu0 = _mu0()
        tops = [j.getLayer(self.topId) for j in self.junctionList]
        pos = [_v(c) for c in self.coordinateMatrix]
        # the scale depends only on the source junction k
        if kind == INTERACTION_DIPOLE:
            scale = [(L2.Ms / mu0) * (L2.thickness * L2.cellSurface) for L2 in tops]
        else:
            scale = [(L2.Ms * (L2.thickness * L2.cellSurface)) / mu0 for L2 in tops]
        idx, rows = [], []
        for i in range(n):
            for k in range(n):
                if i == k:
                    continue
                idx.append(i * n + k)
                if kind == INTERACTION_DIPOLE:
                    rij, r3, r5 = _dipole_geometry(pos[i], pos[k])
                    rows.append((rij[0], rij[1], rij[2], r3, r5))
                else:
                    rows.append(_dipole_tensor(pos[i], pos[k]))
        if idx:
            width = 5 if kind == INTERACTION_DIPOLE else 9
            pairs["g"][idx, :width] = np.array(rows, dtype=np.float64)
            pairs["scale"][idx] = np.array(scale, dtype=np.float64)[np.array(idx) % n]
        return pairs

    def runSimulation(self, totalTime, timeStep=1e-13, writeFrequency=1e-11):
        """reservoir.hpp:185-230 on the GPU."""
        run_groups([self], totalTime, timeStep, writeFrequency)


def _setup(group):
    kind = _KIND.get(group.interactionFunc)
    if kind is None:
        raise RuntimeError("GroupInteraction on the GPU takes nullDipoleInteraction, computeDipoleInteraction or "
                           "computeDipoleInteractionNoumra as the interaction function")
    if group.noElements > MAX_GROUP_JUNCTIONS:
        raise ValueError("the GPU group solver takes at most %d junctions per group" % MAX_GROUP_JUNCTIONS)
    # getSolver(RK4) per junction; all modes equal (reservoir.hpp:196-212);
    # the runner is the last junction's
    modes = [j.getSolver(SolverMode.RK4) for j in group.junctionList]
    if any(m != modes[0] for m in modes):
        raise RuntimeError("Junctions have different solver modes! Set the same solver mode for all junctions "
                           "explicitly. Do not mix stochastic and deterministic solvers!")
    last = group.junctionList[-1]
    single = modes[0] == SolverMode.RK4 and last.layerNo == 1
    tops = []
    for j in group.junctionList:
        j.getLayer(group.topId)  # raises for a missing topId, like getLayer
        tops.append([l.id for l in j.layers].index(group.topId))
    return kind, modes[0], single, tops, group._pairs(kind)


def prepare_groups(groups, totalTime, timeStep=1e-13, writeFrequency=1e-11):
    """Host side of a group run: the time plan, the lowered junctions and
    the group, top-layer and pair records (checks as the reference)."""
    from ._lower import lower, plan_run
    if timeStep > writeFrequency:
        raise RuntimeError("The time step cannot be larger than write frequency!")
    plan = plan_run(totalTime, timeStep, writeFrequency)
    setups = [_setup(g) for g in groups]
    modes = {s[1] for s in setups}
    if len(modes) != 1:
        raise RuntimeError("groups run together must share the solver mode")
    solver = modes.pop()
    junctions = [j for g in groups for j in g.junctionList]
    low = lower(junctions, plan, solver, False)
    grec = np.zeros(len(groups), dtype=GROUP_DTYPE)
    tops = np.zeros(len(junctions), dtype=np.int32)
    pairs = []
    first, poff = 0, 0
    for k, (g, (kind, _, single, top, pr)) in enumerate(zip(groups, setups)):
        grec[k] = (first, g.noElements, kind, int(single), poff)
        tops[first:first + g.noElements] = top
        pairs.append(pr)
        first += g.noElements
        poff += pr.size
    return plan, junctions, low, grec, tops, np.concatenate(pairs)


def run_groups(groups, totalTime, timeStep=1e-13, writeFrequency=1e-11):
    """Run several groups (same time plan) in one launch, one CTA each."""
    from . import engine
    from ._lower import apply_results
    plan, junctions, low, grec, tops, pairs = prepare_groups(groups, totalTime, timeStep, writeFrequency)
    lib = engine.require_gpu()
    t = engine.torch()
    n = len(junctions)
    d_g, d_p = engine.to_device(grec), engine.to_device(pairs)
    d_j = engine.to_device(low.junctions)
    d_l, alpha = engine.device_layers(low)  # alpha: this run's noise buffers, kept until it ends
    d_tab = engine.to_device(low.tables) if low.tables is not None else None
    d_top = engine.to_device(tops)
    d_log = t.empty((n, max(plan.n_log, 1), low.log_width), dtype=t.float64, device="cuda")
    d_status = t.zeros(2 * n, dtype=t.int32, device="cuda")
    maxn = max(g.noElements for g in groups)
    rc = lib.cmtj_run_group_f64(engine.ptr(d_g), len(groups), engine.ptr(d_p), engine.ptr(d_j), engine.ptr(d_top),
                                engine.ptr(d_l), engine.ptr(d_tab), low.params.ctypes.data, engine.ptr(d_log), maxn,
                                engine.ptr(d_status), engine.stream_ptr())
    _abi.check(rc, lib)
    log = d_log.cpu().numpy()
    status = d_status.cpu().numpy().view(np.uint32)
    low.layers = d_l.cpu().numpy().view(_abi.LAYER_DTYPE).copy()
    apply_results(junctions, low, log, status, plan)
    finish_groups(groups, junctions, low, tops)
    return low


def finish_groups(groups, junctions, low, tops):
    """After a run each top layer keeps its last interaction field as its
    reserved-interaction driver, as setLayerReservedInteractionField left it."""
    for q, j in enumerate(junctions):
        off = int(low.junctions[q]["layer_offset"])
        rec = low.layers[off + int(tops[q])]
        h = [float(rec["drv"][_abi.SLOT_HRES + k]["constantValue"]) for k in range(3)]
        j.layers[int(tops[q])].setReservedInteractionField(AxialDriver(*h))
