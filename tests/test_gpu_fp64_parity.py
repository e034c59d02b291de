"""FP64 plain GPU form against the reference's own logs.

Tolerances (deterministic, T = 0): max|dm| <= 1e-9 on every logged
magnetisation component, relative 1e-9 on resistances and on the other
logged fields, time stamps identical (Dormand-Prince: relative 1e-9)."""
import numpy as np
import pytest

import cases
import cmtj_gb300
from test_oracle_pin import load_golden

TOL_M = 1e-9
TOL_REL = 1e-9


def _check(name, log, golden):
    assert set(log) == set(golden), set(log) ^ set(golden)
    for k, g in golden.items():
        a = log[k]
        assert a.shape == g.shape, (k, a.shape, g.shape)
        if k == "time" and not name.startswith("dp_"):
            assert np.array_equal(a, g)
        elif k == "time":
            # Dormand-Prince times are sums of adaptive steps whose factor
            # comes from pow(), which may differ from glibc's by an ulp
            assert np.max(np.abs(a - g)) <= TOL_REL * np.max(np.abs(g)), (name, k)
        elif k.endswith(("_mx", "_my", "_mz")):
            assert np.max(np.abs(a - g)) <= TOL_M, (name, k, np.max(np.abs(a - g)))
        else:
            scale = max(np.max(np.abs(g)), 1e-300)
            assert np.max(np.abs(a - g)) <= TOL_REL * scale, (name, k, np.max(np.abs(a - g)) / scale)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.DETERMINISTIC))
def test_fp64_plain_matches_reference(gpu_lib, name):
    golden, gmags = load_golden(name)
    _, log, mags = cases.run_case(cmtj_gb300, name)
    _check(name, log, golden)
    for lid, gm in gmags.items():
        assert np.max(np.abs(np.asarray(mags[lid]) - gm)) <= TOL_M


@pytest.mark.gpu
def test_fp64_plain_batch_equals_single(gpu_lib):
    """A junction gives the same log alone and inside a batch of others."""
    from cmtj_gb300 import engine
    js = [cases.mtj_rh_point(cmtj_gb300, hx=h, total=2e-10)[0] for h in (-5e5, -1e5, 2e5, 6e5)]
    solo = cases.mtj_rh_point(cmtj_gb300, hx=2e5, total=2e-10)[0]
    plan = engine.plan_run(2e-10, 1e-13, 1e-12)
    engine.run_junctions(js, plan, cmtj_gb300.SolverMode.RK4)
    engine.run_junctions([solo], plan, cmtj_gb300.SolverMode.RK4)
    a, b = js[2].getLog(), solo.getLog()
    for k in b:
        assert a[k] == b[k], k


def _force_lanes(monkeypatch, lanes):
    """Lower with cmtj_sim_params_t.lanes_per_layer = lanes (1: a layer per
    lane; 4: a layer's x, y, z on a quad of lanes)."""
    from cmtj_gb300 import _lower
    orig = _lower.make_params

    def make_params(*a, **k):
        p = orig(*a, **k)
        p["lanes_per_layer"] = lanes
        return p

    monkeypatch.setattr(_lower, "make_params", make_params)


@pytest.mark.gpu
@pytest.mark.parametrize("lanes", [1, 4])
@pytest.mark.parametrize("name", sorted(cases.DETERMINISTIC))
def test_fp64_plain_both_layouts_match_reference(gpu_lib, monkeypatch, name, lanes):
    """Fixed step: a layer per lane / a layer per quad.  Dormand-Prince: a
    junction per thread / a junction per quad."""
    _force_lanes(monkeypatch, lanes)
    golden, gmags = load_golden(name)
    _, log, mags = cases.run_case(cmtj_gb300, name)
    _check(name, log, golden)
    for lid, gm in gmags.items():
        assert np.max(np.abs(np.asarray(mags[lid]) - gm)) <= TOL_M


def _sine(cm, amplitude):
    return cm.sineDriver(0, amplitude, 3e9, 0)


def _rh_junction(oersted=False, iec_sine=False):
    """The R(H) MTJ (field-only layers, constant drivers); oersted adds a
    time-dependent Oersted field (still field-only), iec_sine a
    time-dependent IEC coupling (which sends its warp down the general
    loop)."""
    cm = cmtj_gb300
    j = cases.mtj_rh_point(cm, hx=2e5, total=2e-10)[0]
    if oersted:
        j.setLayerOerstedFieldDriver("all", cm.AxialDriver(_sine(cm, 1e3), cm.NullDriver(), cm.NullDriver()))
    if iec_sine:
        j.setIECDriver("free", "ref", cm.ScalarDriver.getSineDriver(-5e-5, 1e-5, 3e9, 0))
    return j


def test_field_only_selection():
    """The lowered R(H) MTJ is field-only (every CMTJ_ZERO_* term absent, no
    STT or SOT); a time-dependent Oersted driver keeps it so, a
    time-dependent IEC driver does not (its IEC slots are dynamic)."""
    from cmtj_gb300 import _abi, _lower
    plan = _lower.plan_run(2e-10, 1e-13, 1e-12)
    js = [_rh_junction(), _rh_junction(oersted=True), _rh_junction(iec_sine=True)]
    L = _lower.lower(js, plan, cmtj_gb300.SolverMode.RK4, False).layers
    assert np.all(L["zero_terms"] == 15)
    assert not np.any(L["includeSTT"]) and not np.any(L["includeSOT"])
    dyn = L["drv"]["update"] != _abi.DRV_CONSTANT
    assert not dyn[:2].any()
    assert dyn[2:4, _abi.SLOT_HOE].all() and not dyn[2:4, _abi.SLOT_IEC_TOP].any()
    assert dyn[4:6, _abi.SLOT_IEC_TOP].any() or dyn[4:6, _abi.SLOT_IEC_BOTTOM].any()


@pytest.mark.gpu
@pytest.mark.parametrize("oersted", [False, True], ids=["constant", "oersted_sine"])
@pytest.mark.parametrize("lanes", [1, 4])
def test_field_only_variant_gives_the_general_bits(gpu_lib, monkeypatch, lanes, oersted):
    """Alone, the R(H) MTJ runs the field-only RK4 loop (constant drivers, or
    a time-dependent Oersted field); in one warp with a junction whose IEC
    driver is time-dependent it runs the general loop.  Both give the same
    bits in every log column (with the energy log too) and in the final m."""
    from cmtj_gb300 import engine
    _force_lanes(monkeypatch, lanes)
    plan = engine.plan_run(2e-10, 1e-13, 1e-12)
    for energies in (False, True):
        solo = _rh_junction(oersted)
        mixed, other = _rh_junction(oersted), _rh_junction(iec_sine=True)
        engine.run_junctions([solo], plan, cmtj_gb300.SolverMode.RK4, calculate_energies=energies)
        engine.run_junctions([mixed, other], plan, cmtj_gb300.SolverMode.RK4, calculate_energies=energies)
        la, lb = solo.getLogArrays(), mixed.getLogArrays()
        assert set(la) == set(lb)
        for k in la:
            assert np.array_equal(la[k], lb[k]), (energies, k)
        for x, y in zip(solo.layers, mixed.layers):
            assert (x.mag.x, x.mag.y, x.mag.z) == (y.mag.x, y.mag.y, y.mag.z)


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["RK4", "EulerHeun", "Heun"])
def test_fp64_plain_layouts_give_identical_bits(gpu_lib, monkeypatch, solver):
    """One batch of 1- to 3-layer junctions (STT, SOT, strip and classic R,
    time-dependent drivers, the energy log; seeded thermal noise for the
    stochastic solvers): a layer per lane and a layer per quad of lanes give
    the same bits in every log column and final m."""
    from cmtj_gb300 import engine
    mode = getattr(cmtj_gb300.SolverMode, solver)
    names = ("mtj_rh_point", "sto", "sot_strip", "tri_layer", "energies_k2", "alt_stt_bottom", "drivers_zoo")
    plan = engine.plan_run(3e-11, 1e-13, 2e-13)
    runs = []
    for lanes in (1, 4):
        _force_lanes(monkeypatch, lanes)
        js = []
        for q, name in enumerate(names):
            j, _ = cases.DETERMINISTIC[name](cmtj_gb300)
            if solver != "RK4":
                j.setLayerTemperatureDriver("all", cmtj_gb300.constantDriver(300.0))
                for l, layer in enumerate(j.layers):
                    layer.noise_seed = 7000 + 10 * q + l
            js.append(j)
        engine.run_junctions(js, plan, mode, calculate_energies=True)
        runs.append(js)
    for a, b in zip(*runs):
        la, lb = a.getLogArrays(), b.getLogArrays()
        assert set(la) == set(lb)
        for k in la:
            assert np.array_equal(la[k], lb[k]), k
        for x, y in zip(a.layers, b.layers):
            assert (x.mag.x, x.mag.y, x.mag.z) == (y.mag.x, y.mag.y, y.mag.z)


@pytest.mark.gpu
def test_dormand_prince_layouts_give_identical_bits(gpu_lib, monkeypatch):
    """64 sine-driven free layers under Dormand-Prince: one thread per
    junction and one quad of lanes per junction take the same adaptive steps
    and give the same bits."""
    from cmtj_gb300 import engine
    V = cmtj_gb300.CVector

    def build():
        js = []
        for k in range(64):
            demag = [V(0.0024, 0, 0), V(0, 0.0024, 0), V(0, 0, 0.9952)]
            layer = cmtj_gb300.Layer("free", mag=V(0.1, 0, 0.995), anis=V(0, 0, 1), Ms=1.2, thickness=1.5e-9,
                                     cellSurface=1e-16, demagTensor=demag, damping=0.01)
            j = cmtj_gb300.Junction([layer])
            j.setLayerAnisotropyDriver("free", cmtj_gb300.constantDriver(3e5))
            j.setLayerOerstedFieldDriver("free", cmtj_gb300.AxialDriver(
                cmtj_gb300.sineDriver(0, 5e3, 2e9 + 1.5e8 * k, 0), cmtj_gb300.NullDriver(), cmtj_gb300.NullDriver()))
            js.append(j)
        return js

    runs = []
    for lanes in (1, 4):
        _force_lanes(monkeypatch, lanes)
        js = build()
        engine.run_junctions(js, engine.plan_run(1e-9, 1e-13, 1e-11), cmtj_gb300.SolverMode.DormandPrince)
        runs.append(js)
    for a, b in zip(*runs):
        la, lb = a.getLogArrays(), b.getLogArrays()
        for k in la:
            assert np.array_equal(la[k], lb[k]), k
        assert (a.layers[0].mag.x, a.layers[0].mag.y, a.layers[0].mag.z) == \
               (b.layers[0].mag.x, b.layers[0].mag.y, b.layers[0].mag.z)


@pytest.mark.gpu
def test_layer_bound_below_a_junctions_layers_is_an_error(gpu_lib, monkeypatch):
    """cmtj_sim_params_t.max_layers bounds every junction's layer count: a
    3-layer junction launched with max_layers = 2 gets
    CMTJ_STATUS_BAD_INPUT, which the host raises, and keeps its m."""
    from cmtj_gb300 import _lower, engine
    orig = _lower.make_params

    def make_params(*a, **k):
        p = orig(*a, **k)
        p["max_layers"] = 2
        return p

    monkeypatch.setattr(_lower, "make_params", make_params)
    j, _ = cases.tri_layer(cmtj_gb300)
    assert j.layerNo == 3
    m0 = [(l.mag.x, l.mag.y, l.mag.z) for l in j.layers]
    with pytest.raises(RuntimeError, match="status 3"):
        engine.run_junctions([j], engine.plan_run(1e-12, 1e-13, 1e-13), cmtj_gb300.SolverMode.RK4)
    assert [(l.mag.x, l.mag.y, l.mag.z) for l in j.layers] == m0
