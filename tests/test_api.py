"""Host API of cmtj_gb300 against the reference's API tests (tests/test_drivers.py,
test_sanity.py, test_basic.py, test_sot_torques.py, test_constants.py,
test_imports.py in the reference suite): construction, driver arithmetic,
error types and messages.  No simulation runs here."""
import math

import numpy as np

import pytest

import cmtj_gb300 as cmtj
from cmtj_gb300 import AxialDriver, CVector, Junction, Layer, ScalarDriver, constantDriver, sineDriver

DEMAG = [CVector(0, 0, 0), CVector(0, 0, 0), CVector(0, 0, 1)]


def _layer(id="free", **kw):
    args = dict(mag=CVector(0, 0, 1), anis=CVector(1, 0, 0), Ms=1.65, thickness=3e-9, cellSurface=0,
                demagTensor=DEMAG, damping=0.005)
    args.update(kw)
    return Layer(id, **args)


def test_cvector_operators():
    cvec1, cvec2, cvec3 = CVector(1.0, 2.0, 3.0), CVector(1.0, 2.0, 3.0), CVector(2, 4, 6)
    assert (1.0, 2.0, 3.0)[0] == cvec1[0] and cvec1[2] == 3.0
    assert cvec1 == cvec2 and cvec1 != cvec3
    assert (cvec1 + cvec2) == cvec3 and (cvec3 - cvec1) == cvec1
    assert 2 * cvec1 == cvec3 and cvec3 * 0.5 == cvec1
    cvec1 += CVector(1.0, 2.0, 3.0)
    assert cvec1 == cvec3
    cvec3 -= cvec2
    assert cvec3 == cvec2
    assert len(cvec1) == 3 and cvec1.tolist() == [2.0, 4.0, 6.0]
    v = CVector(3, 0, 4)
    assert v.length() == 5.0
    v.normalize()
    assert v == CVector(0.6, 0, 0.8)


def test_axial_definitions_and_aliases():
    cvec = CVector(1.0, 2.0, 3.0)
    assert AxialDriver(1.0, 2.0, 3.0).getCurrentAxialDrivers(0.0) == cvec
    assert AxialDriver(cvec).getCurrentAxialDrivers(0.0) == cvec
    d1 = AxialDriver(constantDriver(1.0), constantDriver(2.0), constantDriver(3.0))
    assert d1.getCurrentAxialDrivers(1e6) == cvec
    d2 = AxialDriver([constantDriver(1.0), constantDriver(2.0), constantDriver(3.0)])
    assert d2.getCurrentAxialDrivers(0.0) == cvec
    d2.applyMask([1, 0, 1])
    assert d2.getCurrentAxialDrivers(0.0) == CVector(1.0, 0.0, 3.0)
    with pytest.raises(RuntimeError, match="mask must be binary"):
        d2.applyMask([1, 2, 1])


def test_driver_ops():
    """Exact values of test_drivers.py:51-65: the operators shift or scale
    both the offset and the amplitude."""
    driver = sineDriver(10, 20, 1, 0)
    assert driver.getCurrentScalarValue(1 / 4) == 30
    driver *= 2
    assert driver.getCurrentScalarValue(1 / 4) == 60
    driver = sineDriver(10, 20, 1, 0)
    driver += 2
    assert driver.getCurrentScalarValue(1 / 4) == 34
    assert (sineDriver(10, 20, 1, 0) * 2).getCurrentScalarValue(1 / 4) == 60
    assert (sineDriver(10, 20, 1, 0) + 2).getCurrentScalarValue(1 / 4) == 34


def test_driver_waveforms():
    assert cmtj.stepDriver(1, 2, 1.0, 2.0).getCurrentScalarValue(1.0) == 3  # inclusive start
    assert cmtj.stepDriver(1, 2, 1.0, 2.0).getCurrentScalarValue(2.0) == 3  # inclusive stop
    assert cmtj.stepDriver(1, 2, 1.0, 2.0).getCurrentScalarValue(2.5) == 1
    assert cmtj.pulseDriver(0, 1, 1.0, 0.25).getCurrentScalarValue(3.1) == 1
    assert cmtj.pulseDriver(0, 1, 1.0, 0.25).getCurrentScalarValue(3.3) == 0
    tr = cmtj.trapezoidDriver(0, 10, 1.0, 1.0, 2.0)
    assert [tr.getCurrentScalarValue(t) for t in (0.5, 1.5, 2.5, 4.5, 6)] == [0, 5, 10, 5, 0]
    assert cmtj.gaussianImpulseDriver(0, 2, 1.0, 0.5).getCurrentScalarValue(1.0) == 2
    assert cmtj.posSineDriver(0, -2, 1, 0).getCurrentScalarValue(0.25) == 2
    assert cmtj.NullDriver().getCurrentScalarValue(1.0) == 0
    with pytest.raises(RuntimeError, match="Start time cannot be later than stop time"):
        cmtj.stepDriver(0, 1, 2.0, 1.0)


def test_custom_driver_contract():
    driver = ScalarDriver.getCustomDriver(lambda t: math.sqrt(t))
    assert driver.getCurrentScalarValue(1e-9) == math.sqrt(1e-9)

    def faulty(t):
        raise ValueError("Intentional exception")

    with pytest.raises(RuntimeError):
        ScalarDriver.getCustomDriver(faulty).getCurrentScalarValue(1e-9)

    def no_arg():
        return 0.0

    with pytest.raises(RuntimeError):
        ScalarDriver.getCustomDriver(no_arg)


def test_sanity_errors():
    with pytest.raises(ValueError, match="Layers must have unique ids!"):
        Junction([_layer("free"), _layer("free")])
    with pytest.raises(ValueError, match="Passed a zero length Layer vector!"):
        Junction([])
    with pytest.raises(ValueError, match="must have a pinning"):
        Junction([_layer()], 100, 200)
    with pytest.raises(ValueError, match="supports only bilayers"):
        Junction([_layer("a"), _layer("b"), _layer("c")], 100, 200)
    with pytest.raises(ValueError, match="must be of the same size"):
        Junction([_layer("a")], [1, 2], [1], [1], [1], [1], [1], [1])
    with pytest.raises(RuntimeError, match="zero vector"):
        _layer(mag=CVector(0, 0, 0))


def test_junction_setters_and_errors():
    l = _layer()
    l.setReferenceLayer(CVector(1, 0, 0))
    j = Junction([l], 100, 200)
    assert j.Rtag == "R"
    with pytest.raises(RuntimeError, match="Failed to find a layer with a given id: nope!"):
        j.setLayerAnisotropyDriver("nope", constantDriver(1))
    with pytest.raises(RuntimeError, match="Failed to find a layer with a given id nope!"):
        j.getLayer("nope")
    j2 = Junction([_layer("a"), _layer("b")], 100, 200)
    assert j2.Rtag == "R_a_b"
    j2.setIECDriver("b", "a", constantDriver(1e-3))  # order irrelevant
    with pytest.raises(RuntimeError, match="Failed to match the layer order"):
        j2.setIECDriver("a", "c", constantDriver(1e-3))
    j2.setLayerMagnetisation("a", CVector(0, 3, 4))
    assert j2.getLayerMagnetisation("a") == CVector(0, 0.6, 0.8)
    assert j2.getMagnetoresistance()[0] == 100 + ((200 - 100) / 2.0) * (1.0 - 0.8)
    assert Junction([_layer("a")]).getLayerIds() == ["a"]
    with pytest.raises(RuntimeError, match="not supported for this structure"):
        Junction([_layer("a")]).getMagnetoresistance()


def test_layer_copy_semantics():
    l = _layer()
    j = Junction([l])
    l.setMagnetisation(CVector(1, 0, 0))
    assert j.getLayerMagnetisation("free") == CVector(0, 0, 1)
    assert _layer(mag=CVector(0, 0, 0.5)).mag == CVector(0, 0, 0.5)  # ctor keeps |m| != 1


def test_sot_layer_misuse():
    layer = Layer.createSOTLayer(id="free", mag=CVector(0, 0, 1), anis=CVector(0, 0, 1), Ms=1, thickness=2e-9,
                                 cellSurface=1e-18, demagTensor=[CVector(0, 0, 0)] * 3, damping=0.01)
    with pytest.raises(RuntimeError):
        layer.setFieldLikeTorqueDriver(constantDriver(0.1))
    with pytest.raises(RuntimeError):
        layer.setDampingLikeTorqueDriver(constantDriver(0.1))
    stt = Layer.createSTTLayer(id="s", mag=CVector(0, 0, 1), anis=CVector(0, 0, 1), Ms=1, thickness=2e-9,
                               cellSurface=1e-18, demagTensor=[CVector(0, 0, 0)] * 3)
    with pytest.raises(RuntimeError, match="includeSTT"):
        stt.setFieldLikeTorqueDriver(constantDriver(0.1))


def test_reference_layers():
    layer = _layer()
    layer.setReferenceLayer(CVector(1, 0, 0))
    assert layer.getReferenceLayer() == CVector(1, 0, 0)
    layer.setSecondaryReferenceLayer(CVector(0, 1, 0))
    assert layer.getSecondaryReferenceLayer() == CVector(0, 1, 0)
    fresh = _layer()
    with pytest.raises(RuntimeError, match="Cannot set fixed polarisation layer to 0"):
        fresh.setReferenceLayer(cmtj.Reference.fixed)


def test_constants_runtime_change():
    pc = cmtj.constants.PhysicalConstants
    try:
        assert pc.gyromagnetic_ratio() == 220880.0
        pc.set_gyromagnetic_ratio(300000.0)
        assert pc.gyromagnetic_ratio() == 300000.0
        pc.set_boltzmann_constant(1.5e-23)
        assert pc.boltzmann_constant() == 1.5e-23
    finally:
        pc.resetToDefaults()
    assert pc.gyromagnetic_ratio() == 220880.0
    assert pc.hbar() == 6.62607015e-34 / (2.0 * math.pi)


def test_enums_exported():
    assert cmtj.RK4 == cmtj.SolverMode.RK4 and cmtj.EulerHeun == 0 and cmtj.Heun == 3
    assert cmtj.xaxis == cmtj.Axis.xaxis and cmtj.fixed == cmtj.Reference.fixed
    assert int(cmtj.custom) == 100


def test_run_plan_matches_reference_truncation():
    from cmtj_gb300.engine import plan_run
    p = plan_run(10e-9, 1e-13, 1e-13)
    assert p.total_iterations == int(10e-9 / 1e-13) and p.write_every == 1
    p = plan_run(4e-9, 1e-13, 1e-12)
    assert p.write_every == int(1e-12 / 1e-13)
    with pytest.raises(RuntimeError, match="cannot be larger than write frequency"):
        plan_run(1e-9, 1e-12, 1e-13)


def test_stack_validation():
    """stack.hpp:123-152 and test_stack.py's error contract."""
    from cmtj_gb300.stack import ParallelStack, SeriesStack
    l = _layer()
    l.setReferenceLayer(CVector(1, 0, 0))
    j = Junction([l], 100, 200)
    with pytest.raises(RuntimeError, match="must have at least 2 junctions"):
        ParallelStack([j])
    with pytest.raises(RuntimeError, match="must have at least 2 junctions"):
        SeriesStack([])
    with pytest.raises(RuntimeError, match="Asking for id of a non-existing junction!"):
        ParallelStack([j, j]).getLog(2)
    with pytest.raises(TypeError):
        SeriesStack([j, j]).getLog(-10)
    with pytest.raises(RuntimeError, match="non-classic"):
        SeriesStack([Junction([_layer("a")]), Junction([_layer("b")])])
    s = SeriesStack([j, j])
    with pytest.raises(RuntimeError, match="size of stack size - 1"):
        s.setCouplingStrength([0.1, 0.2])
    with pytest.raises(RuntimeError, match="only supported for 2 layer stacks"):
        s.setDelayed(False)


def test_lowpass_weights_reproduce_filtered_mean():
    """mean(lfilter(b, a, x)) = sum_k s[N-1-k] x_k / N for the step response
    s of the Butterworth low-pass used by compute_sd (resistance.py:12-22)."""
    from scipy.signal import butter, lfilter
    from cmtj_gb300 import batch
    rng = np.random.default_rng(3)
    n, dt = 4000, 1e-13
    x = rng.standard_normal(n) + 0.3 * np.sin(np.arange(n) * 0.01)
    s = batch.lowpass_step_response(n, 1.0 / dt)
    b, a = butter(3, 10e6 / (0.5 / dt), btype="low", analog=False)
    want = np.mean(lfilter(b, a, x))
    got = np.dot(s[::-1], x) / n
    assert abs(got - want) <= 1e-12 * max(1.0, abs(want)) + 1e-18


def test_reduction_sample_counts():
    from cmtj_gb300 import batch
    n_steps = np.array([0, 1, 10, 11, 100])
    win = np.array([0, 0, 3, 11, 5])
    for every in (1, 3, 7):
        got = batch.reduction_samples(n_steps, win, every)
        want = [len(range(w, n, every)) if n > w else 0 for n, w in zip(n_steps, win)]
        assert got.tolist() == want


def test_partitions_submit_longest_critical_path_first():
    from cmtj_gb300 import batch
    # (layers, longest junction's steps) in the order partitions are built
    parts = [(1, 500_000), (1, 400_000), (2, 500_000), (3, 200_000), (3, 500_000), (4, 500_000), (4, 100_000)]
    order = batch.submission_order(parts)
    assert sorted(order) == list(range(len(parts)))
    # 4 layers at 500k steps first (2 pairs, ties go to more layers), then
    # the 3-layer one; 1 and 2 layers at 500k cost one unit a step
    assert order[:2] == [5, 4]
    assert order[2:4] == [2, 0]
    costs = [parts[q][1] * ((parts[q][0] + 1) // 2) for q in order]
    assert costs == sorted(costs, reverse=True)
    assert batch.submission_order([]) == []
    assert batch.submission_order([(2, 10)]) == [0]


def test_layer_records_mark_identically_zero_terms():
    """The FP64 solver skips field terms the host marks identically zero
    (CMTJ_ZERO_*); the mask must be set exactly when the term is zero, and
    the derived constants are the reference's expressions evaluated once."""
    import cases
    from cmtj_gb300 import _abi, constants
    from cmtj_gb300._lower import lower, plan_run
    plain, _ = cases.mtj_rh_point(cmtj, total=1e-12)
    zoo, _ = cases.drivers_zoo(cmtj)
    k2, _ = cases.energies_k2(cmtj)
    plan = plan_run(1e-12, 1e-13, 1e-13)
    every = _abi.ZERO_DIPOLE | _abi.ZERO_IDMI | _abi.ZERO_K2 | _abi.ZERO_J2
    low = lower([plain], plan, cmtj.SolverMode.RK4, False)
    assert all(int(r["zero_terms"]) == every for r in low.layers)
    low = lower([zoo], plan, cmtj.SolverMode.RK4, False)
    masks = [int(r["zero_terms"]) for r in low.layers]
    assert all(not (m & _abi.ZERO_DIPOLE) for m in masks)  # both layers carry a dipole tensor
    assert all(not (m & _abi.ZERO_IDMI) and not (m & _abi.ZERO_J2) for m in masks)
    low = lower([k2], plan, cmtj.SolverMode.RK4, False)
    assert any(not (int(r["zero_terms"]) & _abi.ZERO_K2) for r in low.layers)
    c = constants.snapshot()
    for r in low.layers:
        d = float(r["damping"])
        assert r["conv_term"] == 1 / (1 + d * d)
        assert r["stoch_conv"] == -c["gyro"] / (1. + d * d)
        assert r["ms_over_mu0"] == float(r["Ms"]) / c["mu0"]


def test_unset_driver_slots_lower_like_default_drivers():
    """Slots a layer was never given a driver for lower to the record of a
    default ScalarDriver(), the same as slots given one explicitly; giving
    one layer a driver, or changing the given driver in place afterwards,
    leaves every other slot and layer as it was."""
    from cmtj_gb300 import _abi, _lower
    z = cmtj.CVector(0, 0, 0)

    def layer(i):
        return cmtj.Layer("L%d" % i, mag=cmtj.CVector(0, 0, 1), anis=cmtj.CVector(0, 0, 1), Ms=1.0, thickness=1e-9,
                        cellSurface=1e-16, demagTensor=[z, z, z])

    plan = _lower.plan_run(1e-12, 1e-13, 1e-13)
    unset, given = layer(0), layer(1)
    for name in ("anis", "current", "temperature", "iec_top", "fl"):
        given.scalar[name] = cmtj.ScalarDriver().copy()
    for name in ("hext", "hoe", "idmi_top"):
        given.axial[name] = cmtj.AxialDriver(cmtj.ScalarDriver(), cmtj.ScalarDriver(), cmtj.ScalarDriver())
    a = _lower.lower([cmtj.Junction([unset])], plan, cmtj.SolverMode.RK4, False).layers["drv"]
    b = _lower.lower([cmtj.Junction([given])], plan, cmtj.SolverMode.RK4, False).layers["drv"]
    assert a.tobytes() == b.tobytes()
    # a driver given to one layer is a copy: changing it later changes nothing
    d = cmtj.ScalarDriver.getSineDriver(1.0, 2.0, 3e9, 0.0)
    l2, l3 = layer(2), layer(3)
    l2.setAnisotropyDriver(d)
    d *= 5
    d.phaseShift(1.0)
    low = _lower.lower([cmtj.Junction([l2]), cmtj.Junction([l3])], plan, cmtj.SolverMode.RK4, False).layers["drv"]
    anis = low[0, _abi.SLOT_ANIS]
    assert (int(anis["update"]), float(anis["constantValue"]), float(anis["amplitude"]), float(anis["phase"])) == \
        (int(cmtj.UpdateType.sine), 1.0, 2.0, 0.0)
    assert low[1].tobytes() == a[0].tobytes()
    ref = cmtj.ScalarDriver()
    assert (ref.constantValue, ref.amplitude, ref.frequency) == (0.0, 0.0, -1.0)


def test_shared_unset_driver_is_never_changed():
    """Every layer slot without a driver of its own holds one shared unset
    driver; the API paths that set, combine, copy and lower drivers leave it
    equal to a fresh ScalarDriver()."""
    from cmtj_gb300 import _lower, core
    fields = core.ScalarDriver.__slots__

    def snapshot(d):
        return tuple(getattr(d, k) for k in fields)

    fresh = snapshot(core.ScalarDriver())
    z = cmtj.CVector(0, 0, 0)
    ls = [cmtj.Layer("L%d" % i, mag=cmtj.CVector(0, 0, 1), anis=cmtj.CVector(0, 0, 1), Ms=1.0, thickness=1e-9,
                     cellSurface=1e-16, demagTensor=[z, z, z]) for i in range(2)]
    j = cmtj.Junction(ls, 100, 200)
    j.setLayerAnisotropyDriver("all", cmtj.constantDriver(1e5))
    j.setLayerExternalFieldDriver("all", cmtj.AxialDriver(cmtj.sineDriver(0, 1e3, 1e9, 0), cmtj.NullDriver(),
                                                          cmtj.NullDriver()))
    j.setIECDriver("L0", "L1", cmtj.constantDriver(1e-4))
    for l in j.layers:
        for d in list(l.scalar.values()) + [d for a in l.axial.values() for d in a.drivers]:
            c = d.copy()
            c *= 3
            c += 1
            c.phaseShift(0.5)
    j2 = j.layers[0].copy()
    j2.axial["hoe"].applyMask([1, 0, 1])
    _lower.lower([j, cmtj.Junction([j2])], _lower.plan_run(1e-12, 1e-13, 1e-13), cmtj.SolverMode.RK4, True)
    assert snapshot(core._UNSET_DRIVER) == fresh
    assert j.layers[0].scalar["anis2"] is core._UNSET_DRIVER


def test_layer_count_limits_raise_before_any_launch():
    """Nine layers exceed the FP64 form's 8 (CMTJ_MAX_LAYERS), five the FP32
    form's 4: both raise ValueError at lowering, before a launch."""
    from cmtj_gb300 import SolverMode, _lower, batch, engine
    nine = Junction([_layer("l%d" % k) for k in range(9)])
    plan = engine.plan_run(1e-12, 1e-13, 1e-13)
    with pytest.raises(ValueError, match="at most 8 layers"):
        _lower.lower([nine], plan, SolverMode.RK4, False)
    five = Junction([_layer("l%d" % k) for k in range(5)])
    with pytest.raises(ValueError, match="1-4 layers"):
        batch.BatchSpec.from_junctions([five])
