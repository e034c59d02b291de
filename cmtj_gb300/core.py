"""Drop-in host API of the reference's `_cmtj` module.

Class names, constructor and method signatures, defaults, log keys and error
types follow the reference's pybind11 bindings (python/cmtj.cpp:35-356) and
the C++ classes behind them (core/cvector.hpp, core/drivers.hpp,
core/junction.hpp).  Objects here are descriptions: runSimulation lowers a
Junction into the packed structs of include/cmtj_gpu.h and runs it on the
GPU through libcmtj_gpu.so (see cmtj_gb300.engine).  There is no CPU solver
in this package.
"""
import copy
import enum
import math
import os
import sys
import time as _time

import numpy as np

from . import constants as _constants

# --------------------------------------------------------------------------
# Enums (python/cmtj.cpp:129-176).  Values match the C++ enums.
# --------------------------------------------------------------------------


class Axis(enum.IntEnum):
    xaxis = 0
    yaxis = 1
    zaxis = 2
    all = 3
    none = 4


class Reference(enum.IntEnum):
    none = 0
    fixed = 1
    top = 2
    bottom = 3


class SolverMode(enum.IntEnum):
    EulerHeun = 0
    RK4 = 1
    DormandPrince = 2
    Heun = 3


class UpdateType(enum.IntEnum):
    constant = 0
    pulse = 1
    sine = 2
    step = 3
    posine = 4
    halfsine = 5
    trapezoid = 6
    gaussimpulse = 7
    gaussstep = 8
    custom = 100


# --------------------------------------------------------------------------
# CVector (core/cvector.hpp:13-220, python/cmtj.cpp:100-127)
# --------------------------------------------------------------------------


class CVector:
    __slots__ = ("x", "y", "z")

    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.x = float(x)
        self.y = float(y)
        self.z = float(z)

    @staticmethod
    def _coerce(v):
        """Implicit list -> CVector conversion (python/cmtj.cpp:126-127)."""
        if isinstance(v, CVector):
            return v
        try:
            seq = list(v)
        except TypeError:
            raise TypeError("expected a CVector or a sequence of 3 floats, got %r" % (v,))
        if len(seq) != 3:
            raise RuntimeError("Failed to create vector -- passed list was not of len 3!")
        return CVector(*seq)

    def length(self):
        return math.sqrt(self.x * self.x + self.y * self.y + self.z * self.z)

    def normalize(self):
        mag = self.length()
        if mag != 0:
            self.x = self.x / mag
            self.y = self.y / mag
            self.z = self.z / mag

    def tolist(self):
        return [self.x, self.y, self.z]

    @staticmethod
    def fromSpherical(theta, phi, r=1.0):
        return CVector(r * math.sin(theta) * math.cos(phi), r * math.sin(theta) * math.sin(phi),
                       r * math.cos(theta))

    def copy(self):
        return CVector(self.x, self.y, self.z)

    def __add__(self, o):
        return CVector(self.x + o.x, self.y + o.y, self.z + o.z)

    def __iadd__(self, o):
        self.x += o.x
        self.y += o.y
        self.z += o.z
        return self

    def __sub__(self, o):
        return CVector(self.x - o.x, self.y - o.y, self.z - o.z)

    def __isub__(self, o):
        self.x -= o.x
        self.y -= o.y
        self.z -= o.z
        return self

    def __mul__(self, s):
        return CVector(self.x * s, self.y * s, self.z * s)

    def __rmul__(self, s):
        return CVector(s * self.x, s * self.y, s * self.z)

    def __imul__(self, s):
        self.x *= s
        self.y *= s
        self.z *= s
        return self

    def __eq__(self, o):
        if not isinstance(o, CVector):
            return NotImplemented
        return self.x == o.x and self.y == o.y and self.z == o.z

    def __ne__(self, o):
        r = self.__eq__(o)
        return r if r is NotImplemented else not r

    __hash__ = None

    def __getitem__(self, i):
        if i == 0:
            return self.x
        if i == 1:
            return self.y
        return self.z

    def __len__(self):
        return 3

    def __iter__(self):
        return iter((self.x, self.y, self.z))

    def __str__(self):
        return "[x:%g, y:%g, z:%g]" % (self.x, self.y, self.z)

    __repr__ = __str__


def c_dot(a, b):
    a, b = CVector._coerce(a), CVector._coerce(b)
    return a.x * b.x + a.y * b.y + a.z * b.z


# --------------------------------------------------------------------------
# Drivers (core/drivers.hpp)
# --------------------------------------------------------------------------


class ScalarDriver:
    """Time-dependent scalar (drivers.hpp:63-354).  The ten parameters and
    their defaults follow the ScalarDriver constructor (drivers.hpp:113-131)."""

    __slots__ = ("update", "constantValue", "amplitude", "frequency", "phase", "period", "cycle",
                 "timeStart", "timeStop", "edgeTime", "steadyTime", "callback")

    def __init__(self, update=UpdateType.constant, constantValue=0.0, amplitude=0.0, frequency=-1.0,
                 phase=0.0, period=-1.0, cycle=-1.0, timeStart=-1.0, timeStop=-1.0, edgeTime=-1.0,
                 steadyTime=-1.0, callback=None):
        self.update = UpdateType(int(update))
        self.constantValue = float(constantValue)
        self.amplitude = float(amplitude)
        self.frequency = float(frequency)
        self.phase = float(phase)
        self.period = float(period)
        self.cycle = float(cycle)
        self.timeStart = float(timeStart)
        self.timeStop = float(timeStop)
        self.edgeTime = float(edgeTime)
        self.steadyTime = float(steadyTime)
        self.callback = callback
        if self.update == UpdateType.pulse and (self.period == -1 or self.cycle == -1):
            raise RuntimeError("Selected pulse train driver type but either period or cycle were not set")
        if self.update == UpdateType.sine and self.frequency == -1:
            raise RuntimeError("Selected sine driver type but frequency was not set")

    # factories (drivers.hpp:133-260)
    @staticmethod
    def getConstantDriver(constantValue):
        return ScalarDriver(UpdateType.constant, constantValue)

    @staticmethod
    def getPulseDriver(constantValue, amplitude, period, cycle):
        return ScalarDriver(UpdateType.pulse, constantValue, amplitude, -1, -1, period, cycle)

    @staticmethod
    def getSineDriver(constantValue, amplitude, frequency, phase):
        return ScalarDriver(UpdateType.sine, constantValue, amplitude, frequency, phase)

    @staticmethod
    def getPosSineDriver(constantValue, amplitude, frequency, phase):
        return ScalarDriver(UpdateType.posine, constantValue, amplitude, frequency, phase)

    @staticmethod
    def getHalfSineDriver(constantValue, amplitude, frequency, phase):
        return ScalarDriver(UpdateType.halfsine, constantValue, amplitude, frequency, phase)

    @staticmethod
    def getStepDriver(constantValue, amplitude, timeStart, timeStop):
        if timeStop <= timeStart:
            raise RuntimeError("Start time cannot be later than stop time!")
        return ScalarDriver(UpdateType.step, constantValue, amplitude, -1, -1, -1, -1, timeStart, timeStop)

    @staticmethod
    def getTrapezoidDriver(constantValue, amplitude, timeStart, edgeTime, steadyTime):
        return ScalarDriver(UpdateType.trapezoid, constantValue, amplitude, -1, -1, -1, -1, timeStart, -1,
                            edgeTime, steadyTime)

    @staticmethod
    def getGaussianImpulseDriver(constantValue, amplitude, t0, sigma):
        return ScalarDriver(UpdateType.gaussimpulse, constantValue, amplitude, -1, -1, -1, -1, t0, -1, sigma)

    @staticmethod
    def getGaussianStepDriver(constantValue, amplitude, t0, sigma):
        # drivers.hpp:241-245 builds a gaussimpulse here as well.
        return ScalarDriver(UpdateType.gaussimpulse, constantValue, amplitude, -1, -1, -1, -1, t0, -1, sigma)

    @staticmethod
    def getCustomDriver(callback):
        if not callback:
            raise RuntimeError("Callback function is not set")
        code = getattr(callback, "__code__", None)
        if code is None or code.co_argcount != 1:
            raise RuntimeError("Callback function must have one argument")
        return ScalarDriver(UpdateType.custom, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, callback)

    def copy(self):
        d = ScalarDriver.__new__(ScalarDriver)
        for k in ScalarDriver.__slots__:
            setattr(d, k, getattr(self, k))
        return d

    def is_zero(self):
        """True when the driver is identically zero (constant 0)."""
        return self.update == UpdateType.constant and self.constantValue == 0.0

    # drivers.hpp:262-305
    def getCurrentScalarValue(self, time):
        t = float(time)
        rv = self.constantValue
        u = self.update
        if u == UpdateType.pulse:
            n = int(t / self.period)
            dT = self.cycle * self.period
            nT = n * self.period
            if nT <= t <= nT + dT:
                rv += self.amplitude
        elif u == UpdateType.sine:
            rv += self.amplitude * math.sin(2 * math.pi * t * self.frequency + self.phase)
        elif u == UpdateType.posine:
            rv += abs(self.amplitude * math.sin(2 * math.pi * t * self.frequency + self.phase))
        elif u == UpdateType.halfsine:
            tamp = self.amplitude * math.sin(2 * math.pi * t * self.frequency + self.phase)
            if tamp <= 0:
                rv += tamp
        elif u == UpdateType.step:
            if self.timeStart <= t <= self.timeStop:
                rv += self.amplitude
        elif u == UpdateType.trapezoid:
            ts, e, s, a = self.timeStart, self.edgeTime, self.steadyTime, self.amplitude
            if t < ts:
                add = 0.0
            elif t <= ts + e:
                add = (a / e) * (t - ts)
            elif t <= ts + e + s:
                add = a
            elif t <= ts + 2 * e + s:
                add = a - (a / e) * (t - (ts + e + s))
            else:
                add = 0.0
            rv += add
        elif u == UpdateType.gaussimpulse:
            rv += self.amplitude * math.exp(-((t - self.timeStart) ** 2) / (2 * self.edgeTime ** 2))
        elif u == UpdateType.gaussstep:
            rv += 0.5 * self.amplitude * (1 + math.erf((t - self.timeStart) / (math.sqrt(2) * self.edgeTime)))
        elif u == UpdateType.custom:
            return _call_custom(self.callback, t)
        return rv

    # operators (drivers.hpp:313-353): both the offset and the amplitude move
    def _scaled(self, c, a):
        d = ScalarDriver.__new__(ScalarDriver)
        for k in ScalarDriver.__slots__:
            setattr(d, k, getattr(self, k))
        d.constantValue, d.amplitude = c, a
        d.callback = None  # the reference's operators drop a custom callback
        return d

    def __mul__(self, val):
        return self._scaled(self.constantValue * val, self.amplitude * val)

    def __imul__(self, val):
        self.constantValue *= val
        self.amplitude *= val
        return self

    def __add__(self, val):
        return self._scaled(self.constantValue + val, self.amplitude + val)

    def __iadd__(self, val):
        self.constantValue += val
        self.amplitude += val
        return self

    def phaseShift(self, phase):
        self.phase += phase

    def __repr__(self):
        return "ScalarDriver(%s, c=%g, a=%g)" % (self.update.name, self.constantValue, self.amplitude)


def _call_custom(callback, t):
    if callback is None:
        raise RuntimeError("Error in Python callback")
    try:
        return float(callback(t))
    except Exception as e:  # drivers.hpp:296-302
        print("Error in Python callback: %s" % e, file=sys.stderr)
        raise RuntimeError("Error in Python callback") from e


# The driver of every Layer slot that has not been given one.  One shared
# object, never handed out: a Layer replaces a slot's driver with a copy of
# the one it is given and never changes a driver in place, and a Layer copy
# keeps this object in its unset slots (_keep_unset), so it stays the
# default ScalarDriver() and lowering recognises it by identity.
_UNSET_DRIVER = ScalarDriver()


def _keep_unset(d):
    """A layer copy's driver for a slot holding d."""
    return d if d is _UNSET_DRIVER else d.copy()


class NullDriver(ScalarDriver):
    """drivers.hpp:356-360: always zero."""

    __slots__ = ()

    def __init__(self):
        super().__init__()

    def getCurrentScalarValue(self, time):
        return 0.0


def _as_scalar_driver(d):
    if isinstance(d, ScalarDriver):
        return d.copy() if type(d) is ScalarDriver else ScalarDriver().copy()
    raise TypeError("expected a ScalarDriver, got %r" % (d,))


class AxialDriver:
    """Three scalar drivers (drivers.hpp:362-461)."""

    __slots__ = ("drivers",)

    def __init__(self, *args):
        if len(args) == 3 and all(isinstance(a, ScalarDriver) for a in args):
            self.drivers = [_as_scalar_driver(a) for a in args]
        elif len(args) == 1 and isinstance(args[0], (list, tuple)) and len(args[0]) > 0 and all(
                isinstance(a, ScalarDriver) for a in args[0]):
            if len(args[0]) != 3:
                raise RuntimeError("The axial driver can only have 3 axes!")
            self.drivers = [_as_scalar_driver(a) for a in args[0]]
        elif len(args) == 3:
            self.drivers = [ScalarDriver.getConstantDriver(float(a)) for a in args]
        elif len(args) == 1:
            v = CVector._coerce(args[0])
            self.drivers = [ScalarDriver.getConstantDriver(c) for c in (v.x, v.y, v.z)]
        elif len(args) == 0:
            self.drivers = [ScalarDriver(), ScalarDriver(), ScalarDriver()]
        else:
            raise TypeError("AxialDriver(): incompatible constructor arguments")

    @staticmethod
    def getVectorAxialDriver(x, y, z):
        return AxialDriver(CVector(x, y, z))

    def getCurrentAxialDrivers(self, time):
        return CVector(*(d.getCurrentScalarValue(time) for d in self.drivers))

    def getConstantValues(self):
        return CVector(*(d.constantValue for d in self.drivers))

    def applyMask(self, mask):
        m = list(mask)
        if len(m) != 3:
            raise RuntimeError("Invalid mask value, mask must be binary!")
        for i in range(3):
            v = int(m[i])
            if v == 0:
                self.drivers[i] = ScalarDriver()
            elif v != 1:
                raise RuntimeError("Invalid mask value, mask must be binary!")

    def copy(self):
        a = AxialDriver.__new__(AxialDriver)
        a.drivers = [d.copy() for d in self.drivers]
        return a

    def _layer_copy(self):
        """copy() for a Layer copy: unset slots keep the shared unset driver."""
        a = AxialDriver.__new__(AxialDriver)
        a.drivers = [_keep_unset(d) for d in self.drivers]
        return a

    @staticmethod
    def _unset():
        """The axial driver of a Layer slot that has not been given one."""
        a = AxialDriver.__new__(AxialDriver)
        a.drivers = [_UNSET_DRIVER, _UNSET_DRIVER, _UNSET_DRIVER]
        return a


def constantDriver(value):
    return ScalarDriver.getConstantDriver(value)


def pulseDriver(constantValue, amplitude, period, cycle):
    return ScalarDriver.getPulseDriver(constantValue, amplitude, period, cycle)


def sineDriver(constantValue, amplitude, frequency, phase):
    return ScalarDriver.getSineDriver(constantValue, amplitude, frequency, phase)


def posSineDriver(constantValue, amplitude, frequency, phase):
    return ScalarDriver.getPosSineDriver(constantValue, amplitude, frequency, phase)


def stepDriver(constantValue, amplitude, timeStart, timeStop):
    return ScalarDriver.getStepDriver(constantValue, amplitude, timeStart, timeStop)


def trapezoidDriver(constantValue, amplitude, timeStart, edgeTime, steadyTime):
    return ScalarDriver.getTrapezoidDriver(constantValue, amplitude, timeStart, edgeTime, steadyTime)


def gaussianImpulseDriver(constantValue, amplitude, t0, sigma):
    return ScalarDriver.getGaussianImpulseDriver(constantValue, amplitude, t0, sigma)


def gaussianStepDriver(constantValue, amplitude, t0, sigma):
    return ScalarDriver.getGaussianStepDriver(constantValue, amplitude, t0, sigma)


# --------------------------------------------------------------------------
# Layer (core/junction.hpp:145-1137, python/cmtj.cpp:226-287)
# --------------------------------------------------------------------------

# driver slot names -> index in cmtj_layer_t.drv (include/cmtj_gpu.h)
_SCALAR_SLOTS = ("temperature", "iec_top", "iec_bottom", "iecq_top", "iecq_bottom", "current", "anis",
                 "anis2", "fl", "dl", "fl2", "dl2")
_AXIAL_SLOTS = {"hext": 12, "hoe": 15, "hdmi": 18, "hres": 21, "idmi_top": 24, "idmi_bottom": 27}


class AdaptiveIntegrationParams:
    """junction.hpp:125-139 (Dormand-Prince step control)."""

    def __init__(self):
        self.abs_tol = 1e-6
        self.rel_tol = 1e-3
        self.max_factor = 5.0
        self.min_factor = 0.1
        self.safety_factor = 0.9
        self.use_pid_control = False
        self.ki = 0.0
        self.kp = 0.2
        self.kd = 0.0
        self.prev_error_ratio = 1.0
        self.integral_error = 0.0


def _tensor(t):
    rows = [CVector._coerce(r) for r in t]
    if len(rows) != 3:
        raise RuntimeError("Failed to create vector -- passed list was not of len 3!")
    return rows


def _new_seed():
    return int.from_bytes(os.urandom(8), "little")


class Layer:
    """One magnetic layer.  `mag` is stored as given: the reference's
    constructor normalises its argument copy, not the member
    (junction.hpp:195), so an unnormalised initial m reaches the first step."""

    def __init__(self, id, mag, anis, Ms, thickness, cellSurface, demagTensor, damping=0.011):
        self._init(id, mag, anis, Ms, thickness, cellSurface, demagTensor, damping, 0.0, 0.0, 0.0, 0.0, 0.0)

    def _init(self, id, mag, anis, Ms, thickness, cellSurface, demagTensor, damping, fieldLikeTorque,
              dampingLikeTorque, slonczewski, beta, spinPolarisation):
        mag = CVector._coerce(mag)
        anis = CVector._coerce(anis)
        self.id = str(id)
        self.mag = mag.copy()
        self.anis = anis.copy()
        self.Ms = float(Ms)
        self.thickness = float(thickness)
        self.cellSurface = float(cellSurface)
        self.demagTensor = [r.copy() for r in _tensor(demagTensor)]
        self.damping = float(damping)
        self.fieldLikeTorque = float(fieldLikeTorque)
        self.dampingLikeTorque = float(dampingLikeTorque)
        self.SlonczewskiSpacerLayerParameter = float(slonczewski)
        self.beta = float(beta)
        self.spinPolarisation = float(spinPolarisation)
        if mag.length() == 0:
            raise RuntimeError("Initial magnetisation was set to a zero vector!")
        if anis.length() == 0:
            raise RuntimeError("Anisotropy was set to a zero vector!")
        self.cellVolume = self.cellSurface * self.thickness
        self.kappa = 1.0
        self.includeSTT = False
        self.includeSOT = False
        self.dynamicSOT = True
        self.alternativeSTT = False
        self.temperatureSet = False
        self.referenceType = Reference.none
        self.referenceLayer = CVector()
        self.secondaryReferenceLayer = CVector()
        self.dipoleTop = [CVector(), CVector(), CVector()]
        self.dipoleBottom = [CVector(), CVector(), CVector()]
        self.scalar = {k: _UNSET_DRIVER for k in _SCALAR_SLOTS}
        self.axial = {k: AxialDriver._unset() for k in _AXIAL_SLOTS}
        # BufferedNoiseParameters defaults (junction.hpp:203-209)
        self.alphaNoise = 1.0
        self.alphaNoiseStd = 0.0
        self.alphaNoiseScale = 0.0
        self.alphaNoiseAxis = Axis.all
        self._alpha_source = None
        self.adaptiveParams = AdaptiveIntegrationParams()
        # Thermal noise stream: copies of a Layer share it, like the
        # reference's copied std::mt19937 state.
        self.noise_seed = _new_seed()
        self.noise_step = 0

    @staticmethod
    def createSOTLayer(id, mag, anis, Ms, thickness, cellSurface, demagTensor, damping=0.011,
                       fieldLikeTorque=0.0, dampingLikeTorque=0.0):
        l = Layer.__new__(Layer)
        l._init(id, mag, anis, Ms, thickness, cellSurface, demagTensor, damping, fieldLikeTorque,
                dampingLikeTorque, 0.0, 0.0, 0.0)
        l.includeSTT = False
        l.includeSOT = True
        l.dynamicSOT = False
        return l

    @staticmethod
    def createSTTLayer(id, mag, anis, Ms, thickness, cellSurface, demagTensor, damping=0.011,
                       SlonczewskiSpacerLayerParameter=1.0, beta=0.0, spinPolarisation=0.0):
        l = Layer.__new__(Layer)
        l._init(id, mag, anis, Ms, thickness, cellSurface, demagTensor, damping, 0.0, 0.0,
                SlonczewskiSpacerLayerParameter, beta, spinPolarisation)
        l.includeSTT = True
        l.includeSOT = False
        return l

    def copy(self):
        return copy.deepcopy(self)

    def __deepcopy__(self, memo):
        l = Layer.__new__(Layer)
        for k, v in self.__dict__.items():
            if k in ("scalar",):
                l.scalar = {s: _keep_unset(d) for s, d in v.items()}
            elif k in ("axial",):
                l.axial = {s: d._layer_copy() for s, d in v.items()}
            else:
                setattr(l, k, copy.deepcopy(v, memo))
        return l

    # --- getters
    def getId(self):
        return self.id

    def getReferenceLayer(self):
        return self.referenceLayer.copy()

    def getSecondaryReferenceLayer(self):
        return self.secondaryReferenceLayer.copy()

    def getReferenceType(self):
        return self.referenceType

    def hasTemperature(self):
        return self.temperatureSet

    # --- setters (junction.hpp:355-560)
    def setMagnetisation(self, mag):
        mag = CVector._coerce(mag)
        if mag.length() == 0:
            raise RuntimeError("Initial magnetisation was set to a zero vector!")
        self.mag = mag.copy()
        self.mag.normalize()

    def setAnisotropyDriver(self, driver):
        self.scalar["anis"] = _driver_copy(driver)

    def setSecondOrderAnisotropyDriver(self, driver):
        self.scalar["anis2"] = _driver_copy(driver)

    def setExternalFieldDriver(self, driver):
        self.axial["hext"] = _axial_copy(driver)

    def setOerstedFieldDriver(self, driver):
        self.axial["hoe"] = _axial_copy(driver)

    def setHdmiDriver(self, driver):
        self.axial["hdmi"] = _axial_copy(driver)

    def setReservedInteractionField(self, driver):
        self.axial["hres"] = _axial_copy(driver)

    def setCurrentDriver(self, driver):
        self.scalar["current"] = _driver_copy(driver)

    def setTemperatureDriver(self, driver):
        self.scalar["temperature"] = _driver_copy(driver)
        self.temperatureSet = True

    def setNonStochasticLangevinDriver(self, driver):
        self.scalar["temperature"] = _driver_copy(driver)
        self.temperatureSet = False

    def setIECDriverTop(self, driver):
        self.scalar["iec_top"] = _driver_copy(driver)

    def setIECDriverBottom(self, driver):
        self.scalar["iec_bottom"] = _driver_copy(driver)

    def setQuadIECDriverTop(self, driver):
        self.scalar["iecq_top"] = _driver_copy(driver)

    def setQuadIECDriverBottom(self, driver):
        self.scalar["iecq_bottom"] = _driver_copy(driver)

    def setIDMIDriverTop(self, driver):
        self.axial["idmi_top"] = _axial_copy(driver)

    def setIDMIDriverBottom(self, driver):
        self.axial["idmi_bottom"] = _axial_copy(driver)

    def _setTorqueParameters(self):
        self.includeSOT = True
        if self.includeSTT:
            raise RuntimeError("includeSTT was on and now setting SOT interaction!")
        if not self.dynamicSOT:
            raise RuntimeError("used a static SOT definition, now trying to set it dynamically!")

    def setFieldLikeTorqueDriver(self, driver):
        self._setTorqueParameters()
        self.scalar["fl"] = _driver_copy(driver)

    def setDampingLikeTorqueDriver(self, driver):
        self._setTorqueParameters()
        self.scalar["dl"] = _driver_copy(driver)

    def setSecondaryFieldLikeTorqueDriver(self, driver):
        self._setTorqueParameters()
        self.scalar["fl2"] = _driver_copy(driver)

    def setSecondaryDampingLikeTorqueDriver(self, driver):
        self._setTorqueParameters()
        self.scalar["dl2"] = _driver_copy(driver)

    def setPrimaryTorqueDrivers(self, fieldLikeTorque, dampingLikeTorque):
        self._setTorqueParameters()
        self.scalar["fl"] = _driver_copy(fieldLikeTorque)
        self.scalar["dl"] = _driver_copy(dampingLikeTorque)

    def setSecondaryTorqueDrivers(self, fieldLikeTorque, dampingLikeTorque):
        self._setTorqueParameters()
        self.scalar["fl2"] = _driver_copy(fieldLikeTorque)
        self.scalar["dl2"] = _driver_copy(dampingLikeTorque)

    def setReferenceLayer(self, ref):
        if isinstance(ref, Reference):
            if ref == Reference.fixed and not self.referenceLayer.length():
                raise RuntimeError("Cannot set fixed polarisation layer to 0! "
                                   "Set reference to NONE to disable reference.")
            self.referenceType = ref
        else:
            self.referenceLayer = CVector._coerce(ref).copy()
            self.referenceType = Reference.fixed

    def setSecondaryReferenceLayer(self, ref):
        self.secondaryReferenceLayer = CVector._coerce(ref).copy()
        self.referenceType = Reference.fixed

    def setTopDipoleTensor(self, tensor):
        self.dipoleTop = [r.copy() for r in _tensor(tensor)]

    def setBottomDipoleTensor(self, tensor):
        self.dipoleBottom = [r.copy() for r in _tensor(tensor)]

    def setKappa(self, kappa):
        self.kappa = float(kappa)

    def setAlternativeSTT(self, alternative):
        self.alternativeSTT = bool(alternative)

    def setAdaptiveParams(self, params):
        self.adaptiveParams = params

    # 1/f noise (OneFNoise, core/noise.hpp:72-135): the reference's solvers
    # never tick it (getStochasticOneFNoise has no caller), so setting it
    # changes no run, here as there.
    def setOneFNoise(self, sources, bias, scale):
        pass

    # Buffered 1/f^alpha noise (setAlphaNoise / createBufferedAlphaNoise /
    # getOneFVector, junction.hpp:406-424, 1130-1136): with a non-zero
    # scale, runSimulation forces Euler-Heun (unless Heun) and every run
    # gets fresh buffers of its iteration count, filled on the GPU
    # (cmtj_gb300.noise) from this layer's Philox key on the alpha-noise
    # stream, at counter noise_step.
    def setAlphaNoise(self, alpha, std, scale, axis=Axis.all):
        if alpha < 0 or alpha > 2:
            raise RuntimeError("alpha must be between 0 and 2")
        self.alphaNoise = float(alpha)
        self.alphaNoiseStd = float(std)
        self.alphaNoiseScale = float(scale)
        self.alphaNoiseAxis = Axis(int(axis))

    def createBufferedAlphaNoise(self, bufferSize):
        from .noise import VectorAlphaNoise
        self._alpha_source = VectorAlphaNoise(bufferSize, self.alphaNoise, self.alphaNoiseStd,
                                              self.alphaNoiseScale, self.alphaNoiseAxis)

    def getOneFVector(self):
        if self.alphaNoiseScale != 0:
            if self._alpha_source is None:
                raise RuntimeError("getOneFVector: createBufferedAlphaNoise(bufferSize) has not been called")
            return self._alpha_source.tickVector()
        return CVector()


def _driver_copy(d):
    if not isinstance(d, ScalarDriver):
        raise TypeError("expected a ScalarDriver, got %r" % (d,))
    c = d.copy()
    if type(d) is NullDriver:
        c = ScalarDriver()
    return c


def _axial_copy(d):
    if not isinstance(d, AxialDriver):
        raise TypeError("expected an AxialDriver, got %r" % (d,))
    return d.copy()


# --------------------------------------------------------------------------
# Junction (core/junction.hpp:1139-2057, python/cmtj.cpp:289-356)
# --------------------------------------------------------------------------

_STRIP_KEYS = ("Rx0", "Ry0", "AMR_X", "AMR_Y", "SMR_X", "SMR_Y", "AHE")
MR_NONE, MR_CLASSIC, MR_STRIP = 0, 1, 2


class Junction:
    """Stack of layers with its log.  The Layers are copied on construction
    (junction.hpp:1164-1166); getLayer returns the junction's own copy."""

    def __init__(self, layers, *args, **kwargs):
        strip = len(args) == 7 or any(k in kwargs for k in _STRIP_KEYS)
        classic = not strip and (len(args) > 0 or "Rp" in kwargs or "Rap" in kwargs)
        self.layers = [l.copy() for l in layers]
        self.layerNo = len(self.layers)
        self.MR_mode = MR_NONE
        self.Rp = 0.0
        self.Rap = 0.0
        self.Rtag = "R"
        self.strip = None
        if self.layerNo == 0:
            raise ValueError("Passed a zero length Layer vector!")
        if strip:
            vals = dict(zip(_STRIP_KEYS, args))
            vals.update({k: kwargs[k] for k in _STRIP_KEYS if k in kwargs})
            missing = [k for k in _STRIP_KEYS if k not in vals]
            if missing:
                raise TypeError("Junction(): missing strip resistance arguments %s" % missing)
            vals = {k: [float(x) for x in v] for k, v in vals.items()}
            if any(len(v) != self.layerNo for v in vals.values()):
                raise ValueError("Layers and Rx0, Ry, AMR, AMR and SMR must be of the same size!")
            self.strip = vals
            self.MR_mode = MR_STRIP
        else:
            ids = set()
            for l in self.layers:
                if l.id in ids:
                    raise ValueError("Layers must have unique ids!")
                ids.add(l.id)
            if classic:
                Rp = args[0] if len(args) > 0 else kwargs.get("Rp", 100)
                Rap = args[1] if len(args) > 1 else kwargs.get("Rap", 200)
                if self.layerNo == 1 and not self.layers[0].referenceLayer.length():
                    raise ValueError("MTJ with a single layer must have a pinning (referenceLayer) set!")
                if self.layerNo > 2:
                    raise ValueError("This constructor supports only bilayers! "
                                     "Choose the other one with the strip resistance!")
                self.Rp = float(Rp)
                self.Rap = float(Rap)
                self.MR_mode = MR_CLASSIC
                if self.layerNo == 2:
                    self.Rtag = "R_" + self.layers[0].id + "_" + self.layers[1].id
        self._log_chunks = {}
        self._log_order = []
        self.logLength = 0

    # ---------------------------------------------------------------- log
    def getLayerIds(self):
        return [l.id for l in self.layers]

    def clearLog(self):
        self._log_chunks = {}
        self._log_order = []
        self.logLength = 0

    def _append_log(self, cols, n_rows):
        """cols: ordered dict key -> 1-D float64 array (one log column)."""
        for k, v in cols.items():
            if k not in self._log_chunks:
                self._log_chunks[k] = []
                self._log_order.append(k)
            self._log_chunks[k].append(np.asarray(v, dtype=np.float64))
        self.logLength += n_rows

    def getLogArrays(self):
        """The log as numpy arrays (no list conversion)."""
        return {k: (np.concatenate(self._log_chunks[k]) if len(self._log_chunks[k]) > 1 else
                    self._log_chunks[k][0]) for k in self._log_order}

    def getLog(self):
        return {k: v.tolist() for k, v in self.getLogArrays().items()}

    def saveLogs(self, filename):
        if filename == "":
            raise RuntimeError("The filename may not be empty!")
        log = self.getLogArrays()
        keys = list(log.keys())
        with open(filename, "w") as f:
            f.write("".join(k + ";" for k in keys) + "\n")
            for i in range(self.logLength):
                f.write("".join("%g;" % log[k][i] for k in keys) + "\n")

    saveLog = saveLogs

    # ------------------------------------------------------------ setters
    def _layer_setter(self, layerID, fn):
        found = False
        for l in self.layers:
            if l.id == layerID or layerID == "all":
                fn(l)
                found = True
        if not found:
            raise RuntimeError("Failed to find a layer with a given id: " + layerID + "!")

    def getLayer(self, layerId):
        for l in self.layers:
            if l.id == layerId:
                return l
        raise RuntimeError("Failed to find a layer with a given id " + layerId + "!")

    def _coupling(self, bottomLayer, topLayer, set_top, set_bottom):
        for i in range(self.layerNo - 1):
            a, b = self.layers[i], self.layers[i + 1]
            if (a.id == bottomLayer and b.id == topLayer) or (a.id == topLayer and b.id == bottomLayer):
                set_top(a)
                set_bottom(b)
                return
        raise RuntimeError("Failed to match the layer order or find layer ids: " + bottomLayer + " and " +
                           topLayer + "!")

    def setLayerTemperatureDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setTemperatureDriver(driver))

    def setLayerNonStochasticLangevinDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setNonStochasticLangevinDriver(driver))

    def setLayerAnisotropyDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setAnisotropyDriver(driver))

    def setLayerSecondOrderAnisotropyDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setSecondOrderAnisotropyDriver(driver))

    def setLayerExternalFieldDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setExternalFieldDriver(driver))

    def setLayerOerstedFieldDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setOerstedFieldDriver(driver))

    def setLayerCurrentDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setCurrentDriver(driver))

    def setLayerDampingLikeTorqueDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setDampingLikeTorqueDriver(driver))

    def setLayerFieldLikeTorqueDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setFieldLikeTorqueDriver(driver))

    def setLayerSecondaryFieldLikeTorqueDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setSecondaryFieldLikeTorqueDriver(driver))

    def setLayerSecondaryDampingLikeTorqueDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setSecondaryDampingLikeTorqueDriver(driver))

    def setLayerPrimaryTorqueDrivers(self, layerId, fieldLikeTorque, dampingLikeTorque):
        self._layer_setter(layerId, lambda l: l.setFieldLikeTorqueDriver(fieldLikeTorque))
        self._layer_setter(layerId, lambda l: l.setDampingLikeTorqueDriver(dampingLikeTorque))

    def setLayerSecondaryTorqueDrivers(self, layerId, fieldLikeTorque, dampingLikeTorque):
        self._layer_setter(layerId, lambda l: l.setSecondaryFieldLikeTorqueDriver(fieldLikeTorque))
        self._layer_setter(layerId, lambda l: l.setSecondaryDampingLikeTorqueDriver(dampingLikeTorque))

    def setLayerReservedInteractionField(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setReservedInteractionField(driver))

    def setLayerHdmiDriver(self, layerId, driver):
        self._layer_setter(layerId, lambda l: l.setHdmiDriver(driver))

    def setLayerAlternativeSTT(self, layerId, alternative):
        if layerId == "all":
            for l in self.layers:
                l.setAlternativeSTT(alternative)
        else:
            self.getLayer(layerId).setAlternativeSTT(alternative)

    def setLayerOneFNoise(self, layerId, sources, bias, scale):
        if layerId == "all":
            for l in self.layers:
                l.setOneFNoise(sources, bias, scale)
        else:
            self.getLayer(layerId).setOneFNoise(sources, bias, scale)

    def setIDMIDriver(self, bottomLayer, topLayer, driver):
        self._coupling(bottomLayer, topLayer, lambda l: l.setIDMIDriverTop(driver),
                       lambda l: l.setIDMIDriverBottom(driver))

    def setQuadIECDriver(self, bottomLayer, topLayer, driver):
        self._coupling(bottomLayer, topLayer, lambda l: l.setQuadIECDriverTop(driver),
                       lambda l: l.setQuadIECDriverBottom(driver))

    def setIECDriver(self, bottomLayer, topLayer, driver):
        self._coupling(bottomLayer, topLayer, lambda l: l.setIECDriverTop(driver),
                       lambda l: l.setIECDriverBottom(driver))

    def setLayerMagnetisation(self, layerId, mag):
        self._layer_setter(layerId, lambda l: l.setMagnetisation(mag))

    def getLayerMagnetisation(self, layerId):
        return self.getLayer(layerId).mag.copy()

    def getLayerReferenceType(self, layerId):
        return self.getLayer(layerId).referenceType

    def setLayerReferenceLayer(self, layerId, referenceLayer):
        if layerId == "all":
            for l in self.layers:
                l.setReferenceLayer(CVector._coerce(referenceLayer))
        else:
            self.getLayer(layerId).setReferenceLayer(CVector._coerce(referenceLayer))

    def setLayerReferenceType(self, layerId, referenceType):
        if layerId == "all":
            for l in self.layers:
                l.setReferenceLayer(Reference(int(referenceType)))
        else:
            self.getLayer(layerId).setReferenceLayer(Reference(int(referenceType)))

    # ------------------------------------------------------------ resistance
    def calculateMagnetoresistance(self, cosTheta):
        return self.Rp + (((self.Rap - self.Rp) / 2.0) * (1.0 - cosTheta))

    def getMagnetoresistance(self):
        """junction.hpp:1869-1889."""
        if self.MR_mode == MR_CLASSIC and self.layerNo == 2:
            return [self.calculateMagnetoresistance(c_dot(self.layers[0].mag, self.layers[1].mag))]
        if self.MR_mode == MR_CLASSIC and self.layerNo == 1:
            return [self.calculateMagnetoresistance(c_dot(self.layers[0].mag, self.layers[0].referenceLayer))]
        if self.MR_mode == MR_STRIP:
            s = self.strip
            Rx_acc = 0.0
            Ry_acc = 0.0
            for i, l in enumerate(self.layers):
                m = l.mag
                Rx = s["Rx0"][i] + s["AMR_X"][i] * (m.x * m.x) + s["SMR_X"][i] * (m.y * m.y)
                Ry = s["Ry0"][i] + 0.5 * s["AHE"][i] * m.z + (s["AMR_Y"][i] + s["SMR_Y"][i]) * m.x * m.y
                Rx_acc += 1. / Rx
                Ry_acc += 1. / Ry
            return [1 / Rx_acc, 1 / Ry_acc, 0.]
        raise RuntimeError("Magnetisation calculation is not supported for this structure!")

    # ------------------------------------------------------------ solving
    def getSolver(self, mode):
        """junction.hpp:1891-1931: a temperature driver or alpha noise forces
        Euler-Heun unless Heun was asked for."""
        local = SolverMode(int(mode))
        for l in self.layers:
            if l.hasTemperature() and local not in (SolverMode.Heun, SolverMode.EulerHeun):
                print("[WARNING] Solver automatically changed to Euler Heun for stochastic calculation.")
                local = SolverMode.EulerHeun
            if l.alphaNoiseScale != 0 and local not in (SolverMode.Heun, SolverMode.EulerHeun):
                print("[WARNING] Solver automatically changed to Euler Heun for stochastic calculation.")
                local = SolverMode.EulerHeun
        return local

    def runSimulation(self, totalTime, timeStep=1e-13, writeFrequency=1e-11, verbose=False,
                      calculateEnergies=False, solverMode=SolverMode.RK4, *, arithmetic="reference"):
        """Junction::runSimulation (junction.hpp:1948-2056).  The keyword
        arithmetic has no counterpart in the reference: "fused" runs
        field-only RK4 layers in fused FP64 arithmetic (cmtj_arithmetic in
        include/cmtj_gpu.h), close to but not bit-identical with the
        default "reference"."""
        from . import engine
        begin = _time.perf_counter()
        plan = engine.plan_run(totalTime, timeStep, writeFrequency)
        solver = self.getSolver(solverMode)
        plan = plan.for_solver(solver)
        engine.run_junctions([self], plan, solver, bool(calculateEnergies), arithmetic)
        if verbose:
            print("Steps in simulation: %d" % plan.total_iterations)
            print("Write every: %d" % plan.write_every)
            print("Simulation time = %d[s]" % int(_time.perf_counter() - begin))
