"""Electrically coupled junction stacks (core/stack.hpp, bound as
cmtj.stack in python/cmtj.cpp:358-426): SeriesStack and ParallelStack.

runSimulation lowers every junction of the stack into the FP64 structs of
include/cmtj_gpu.h and runs cmtj_run_stack_f64: one CTA per stack, one
thread per junction, the KCL current or the non-KCL coupling chain formed
per step in the reference's order."""
import copy

import numpy as np

from . import _abi
from .core import MR_CLASSIC, CVector, ScalarDriver, SolverMode, constantDriver

STACK_SERIES, STACK_PARALLEL = 0, 1
MAX_STACK_JUNCTIONS = 256

STACK_DTYPE = np.dtype(
    [("first_junction", "<i4"), ("n_junctions", "<i4"), ("kind", "<i4"), ("use_kcl", "<i4"), ("delayed", "<i4"),
     ("single_layer_runner", "<i4"), ("coupling_offset", "<i4"), ("n_coupling", "<i4"),
     ("phase_offset", "<f8"), ("pol", "<f8", 3), ("current", _abi.DRIVER_DTYPE)], align=True)


class _Stack:
    _kind = STACK_SERIES

    def __init__(self, junctionList, topId_a="free", bottomId="bottom", phaseOffset=0.0, useKCL=True):
        self.topId = str(topId_a)
        self.bottomId = str(bottomId)
        self.phaseOffset = float(phaseOffset)
        self.useKCL = bool(useKCL)
        if len(junctionList) < 2:
            raise RuntimeError("Stack must have at least 2 junctions!")
        self.junctionList = [copy.deepcopy(j) for j in junctionList]
        if any(j.MR_mode != MR_CLASSIC for j in self.junctionList):
            raise RuntimeError("Junction has a non-classic magnetoresitance mode! "
                               "Define the junction with Rp and Rap resistance values.")
        self.stackSize = len(self.junctionList)
        self.couplingStrength = [0.0]
        self.delayed = True
        self.currentDriver = ScalarDriver()
        self._log_chunks = {}
        self._log_order = []

    # ------------------------------------------------------------ settings
    def getCoupling(self, order):
        if not self.couplingStrength:
            raise RuntimeError("Coupling strength is not set!")
        if len(self.couplingStrength) == 1:
            return self.couplingStrength[0]
        return self.couplingStrength[order]

    def setCouplingStrength(self, coupling):
        if isinstance(coupling, (list, tuple, np.ndarray)):
            if len(coupling) != self.stackSize - 1:
                raise RuntimeError("Coupling strength vector must have size of stack size - 1!")
            self.couplingStrength = [float(c) for c in coupling]
        else:
            self.couplingStrength = [float(coupling)]

    def isTwoLayerMemberStack(self):
        for j in self.junctionList:
            if j.layerNo >= 3:
                raise RuntimeError("At least one junction has more than 2 layers! It's not supported now.")
            if j.layerNo != 2:
                return False
        return True

    def setDelayed(self, delayed):
        if not delayed and not self.isTwoLayerMemberStack():
            raise RuntimeError("Non delayed coupling is only supported for 2 layer stacks!")
        self.delayed = bool(delayed)

    def setMagnetisation(self, junction, layerId, mag):
        self.junctionList[junction].setLayerMagnetisation(layerId, mag)

    def getMagnetisation(self, junction, layerId):
        return self.junctionList[junction].getLayerMagnetisation(layerId)

    def getJunction(self, junctionId):
        if not isinstance(junctionId, (int, np.integer)) or junctionId < 0:
            raise TypeError("getJunction(): junctionId must be a non-negative integer")
        if junctionId >= len(self.junctionList):
            raise IndexError("junction index out of range")
        return self.junctionList[junctionId]

    def setJunctionAnisotropyDriver(self, junctionId, layerId, k):
        self.junctionList[junctionId].setLayerAnisotropyDriver(layerId, k)

    def setOerstedFieldDriver(self, driver):
        for j in self.junctionList:
            j.setLayerOerstedFieldDriver("all", driver)

    def setExternalFieldDriver(self, driver):
        for j in self.junctionList:
            j.setLayerExternalFieldDriver("all", driver)

    def resetCoupledCurrentDriver(self):
        self.currentDriver = ScalarDriver()
        for j in self.junctionList:
            j.setLayerCurrentDriver("all", self.currentDriver)

    def setCoupledCurrentDriver(self, driver):
        self.currentDriver = driver.copy()
        for j in self.junctionList:
            j.setLayerCurrentDriver("all", self.currentDriver)

    # ------------------------------------------------------------ logs
    def clearLogs(self):
        for j in self.junctionList:
            j.clearLog()
        self._log_chunks = {}
        self._log_order = []

    def getLog(self, id=None):
        if id is None:
            return {k: (np.concatenate(v) if len(v) > 1 else v[0]).tolist()
                    for k, v in ((k, self._log_chunks[k]) for k in self._log_order)}
        if isinstance(id, bool) or not isinstance(id, (int, np.integer)) or id < 0:
            raise TypeError("getLog(): incompatible function arguments (id must be a non-negative integer)")
        if id < len(self.junctionList):
            return self.junctionList[id].getLog()
        raise RuntimeError("Asking for id of a non-existing junction!")

    def _append(self, cols):
        for k, v in cols.items():
            if k not in self._log_chunks:
                self._log_chunks[k] = []
                self._log_order.append(k)
            self._log_chunks[k].append(np.asarray(v, dtype=np.float64))

    # ------------------------------------------------------------ run
    def getPolarisationVector(self):
        probe = self.junctionList[0].getLayer(self.topId).referenceLayer
        for j in self.junctionList[1:]:
            if probe != j.getLayer(self.topId).referenceLayer:
                raise RuntimeError("Polarisation vectors are not equal in stack")
        if not probe.length():
            raise RuntimeError("Polarisation is not set!")
        return probe

    def runSimulation(self, totalTime, timeStep=1e-13, writeFrequency=1e-11):
        run_stacks([self], totalTime, timeStep, writeFrequency)


class SeriesStack(_Stack):
    _kind = STACK_SERIES


class ParallelStack(_Stack):
    _kind = STACK_PARALLEL


def _setup(stack, plan):
    """initializeSimulation (stack.hpp:33-64) and the per-junction layer
    indices storeMagnetisations reads (66-77)."""
    modes = [j.getSolver(SolverMode.RK4) for j in stack.junctionList]
    if any(m != modes[0] for m in modes[1:]):
        raise RuntimeError("Junctions have different solver modes! Set the same solver mode for all junctions "
                           "explicitly. Do not mix stochastic and deterministic solvers!")
    two = stack.isTwoLayerMemberStack()
    tb = []
    for j in stack.junctionList:
        top = j.getLayerIds().index(stack.topId) if stack.topId in j.getLayerIds() else None
        if top is None:
            j.getLayer(stack.topId)  # raises the reference's error
        bot = -1
        if two:
            if stack.bottomId not in j.getLayerIds():
                j.getLayer(stack.bottomId)
            bot = j.getLayerIds().index(stack.bottomId)
        tb.append((top, bot))
    pol = (0.0, 0.0, 0.0) if two else tuple(stack.getPolarisationVector())
    single = modes[-1] == SolverMode.RK4 and stack.junctionList[-1].layerNo == 1
    return modes[0], tb, pol, single


def run_stacks(stacks, totalTime, timeStep=1e-13, writeFrequency=1e-11):
    """Run several stacks (same time plan) in one launch, one CTA each."""
    from . import engine
    from ._lower import apply_results, lower, make_params, plan_run
    from . import _abi as abi
    if timeStep > writeFrequency:
        raise RuntimeError("The time step cannot be larger than write frequency!")
    plan = plan_run(totalTime, timeStep, writeFrequency)
    setups = [_setup(s, plan) for s in stacks]
    solvers = {st[0] for st in setups}
    if len(solvers) != 1:
        raise RuntimeError("stacks run together must share the solver mode")
    solver = solvers.pop()
    maxn = max(s.stackSize for s in stacks)
    if maxn > MAX_STACK_JUNCTIONS:
        raise ValueError("the GPU stack solver takes at most %d junctions per stack" % MAX_STACK_JUNCTIONS)
    junctions = [j for s in stacks for j in s.junctionList]
    low = lower(junctions, plan, solver, False)
    # the stack's current driver goes through the same lowering (tables for callbacks)
    from ._lower import TableBuilder, _driver_record
    tables = TableBuilder(plan, solver)
    base = 0 if low.tables is None else low.tables.size
    srec = np.zeros(len(stacks), dtype=STACK_DTYPE)
    couplings = []
    tbarr = np.zeros((len(junctions), 2), dtype=np.int32)
    first = 0
    for k, (s, (_, tb, pol, single)) in enumerate(zip(stacks, setups)):
        srec[k]["first_junction"] = first
        srec[k]["n_junctions"] = s.stackSize
        srec[k]["kind"] = s._kind
        srec[k]["use_kcl"] = int(s.useKCL)
        srec[k]["delayed"] = int(s.delayed)
        srec[k]["single_layer_runner"] = int(single)
        srec[k]["coupling_offset"] = len(couplings)
        srec[k]["n_coupling"] = len(s.couplingStrength)
        couplings.extend(s.couplingStrength)
        srec[k]["phase_offset"] = s.phaseOffset
        srec[k]["pol"] = pol
        srec[k]["current"] = _driver_record(s.currentDriver, tables)
        if srec[k]["current"]["update"] == abi.DRV_TABLE:
            srec[k]["current"]["table_offset"] += base
        for q, (t, b) in enumerate(tb):
            tbarr[first + q] = (t, b)
        first += s.stackSize
    extra = tables.array()
    if extra is not None:
        low.tables = extra if low.tables is None else np.concatenate([low.tables, extra])
    width = 2 * maxn + 1
    lib = engine.require_gpu()
    t = engine.torch()
    n = len(junctions)
    n_log = plan.n_log
    d_j = engine.to_device(low.junctions)
    d_l, alpha = engine.device_layers(low)  # alpha: this run's noise buffers, kept until it ends
    d_tab = engine.to_device(low.tables) if low.tables is not None else None
    d_s = engine.to_device(srec)
    d_c = engine.to_device(np.asarray(couplings, dtype=np.float64))
    d_tb = engine.to_device(tbarr)
    d_log = t.empty((n, max(n_log, 1), low.log_width), dtype=t.float64, device="cuda")
    d_slog = t.empty((len(stacks), max(n_log, 1), width), dtype=t.float64, device="cuda")
    d_status = t.zeros(2 * n, dtype=t.int32, device="cuda")
    rc = lib.cmtj_run_stack_f64(engine.ptr(d_s), len(stacks), engine.ptr(d_c), engine.ptr(d_j), engine.ptr(d_tb),
                                engine.ptr(d_l), engine.ptr(d_tab), low.params.ctypes.data, engine.ptr(d_log),
                                engine.ptr(d_slog), width, maxn, engine.ptr(d_status), engine.stream_ptr())
    abi.check(rc, lib)
    log = d_log.cpu().numpy()
    slog = d_slog.cpu().numpy()
    status = d_status.cpu().numpy().view(np.uint32)
    low.layers = d_l.cpu().numpy().view(abi.LAYER_DTYPE).copy()
    rows = int(status[1]) if n else 0
    for k, s in enumerate(stacks):
        N = s.stackSize
        if rows:
            sl = slog[k, :rows]
            cols = {"Resistance": sl[:, 0]}
            for q in range(N):
                cols["I_%d" % q] = sl[:, 1 + q]
                if q < N - 1:
                    cols["C_%d_%d" % (q, q + 1)] = sl[:, 1 + N + q]
            cols["time"] = sl[:, 2 * N]
            s._append(cols)
    apply_results(junctions, low, log, status, plan)
