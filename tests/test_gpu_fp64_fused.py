"""CMTJ_ARITH_FUSED: field-only RK4 layers in fused FP64 arithmetic.

The fused form is not bit-identical with the reference, so it is checked
against the reference-arithmetic run of the same junctions (whose bits
equal the reference's, test_gpu_fp64_parity.py) with stated bounds:
  * the R(H) MTJ sweep, 64 fields x 20,000 RK4 steps, every row logged:
    max|dm| <= 1e-9 and R relative <= 1e-9 (the FP64 plain tolerance);
  * the same sweep in full (100,000 steps): max|dm| <= 1e-9 on every field
    where the reference compiled with FMA contraction stays within 1e-10 of
    its x86-64 build (tests/golden/rh_fma_spread.npz: 60 of the 64), and
    <= 1e-7 on the others, where that build itself moves by up to 4.2e-9;
  * a time-dependent Oersted field (the PIMM step): max|dm| <= 1e-9.
Junctions the fused form does not cover (STT, calculateEnergies, a
time-dependent anisotropy) must keep the reference's bits under it, alone
and sharing a warp with fused ones, and both lane layouts give the same
fused bits."""
import numpy as np
import pytest

import cases
import cmtj_gb300
from cmtj_gb300 import engine

KEYS = ("free_mx", "free_my", "free_mz", "ref_mx", "ref_my", "ref_mz")
TOL_M = 1e-9
TOL_REL = 1e-9
DT = 1e-13


def _rh(n=64, total=2e-9):
    from cmtj_gb300 import tune
    return tune.rh_junctions(n, total)


def _run(js, total, arithmetic, write=DT, lanes=None, monkeypatch=None):
    if lanes is not None:
        from cmtj_gb300 import _lower
        orig = _lower.make_params

        def make_params(*a, **k):
            p = orig(*a, **k)
            p["lanes_per_layer"] = lanes
            return p

        monkeypatch.setattr(_lower, "make_params", make_params)
    plan = engine.plan_run(total, DT, write)
    engine.run_junctions(js, plan, cmtj_gb300.SolverMode.RK4, arithmetic=arithmetic)
    if lanes is not None:
        monkeypatch.undo()
    return js


def _m(js):
    return np.stack([np.stack([j.getLogArrays()[k] for k in KEYS], 1) for j in js])


def _r(js):
    return np.stack([j.getLogArrays()["R_free_ref"] for j in js])


@pytest.mark.gpu
def test_fused_rh_sweep_within_fp64_tolerance(gpu_lib):
    ref = _run(_rh(), 2e-9, "reference")
    fus = _run(_rh(), 2e-9, "fused")
    m0, m1 = _m(ref), _m(fus)
    assert m0.shape == m1.shape and m0.shape[1] == 20_000
    dm = float(np.max(np.abs(m1 - m0)))
    assert dm <= TOL_M, dm
    r0, r1 = _r(ref), _r(fus)
    assert float(np.max(np.abs(r1 - r0) / np.abs(r0))) <= TOL_REL
    # fused is a different rounding, not the same code path
    assert dm > 0.0
    assert np.array_equal(ref[0].getLogArrays()["time"], fus[0].getLogArrays()["time"])


@pytest.mark.gpu
def test_fused_full_rh_sweep_against_fma_built_reference(gpu_lib):
    import os
    spread = np.load(os.path.join(os.path.dirname(__file__), "golden", "rh_fma_spread.npz"))
    ref = _run(_rh(64, 1e-8), 1e-8, "reference")
    m0, r0 = _m(ref), _r(ref)
    del ref
    fus = _run(_rh(64, 1e-8), 1e-8, "fused")
    m1, r1 = _m(fus), _r(fus)
    del fus
    assert m1.shape == (64, 100_000, 6)
    dm = np.max(np.abs(m1 - m0), axis=(1, 2))
    rel = np.max(np.abs(r1 - r0) / np.abs(r0), axis=1)
    calm = spread["max_abs_dm"] <= 1e-10
    assert int(calm.sum()) == 60
    assert np.all(dm[calm] <= TOL_M), dm[calm].max()
    assert np.all(rel[calm] <= TOL_REL), rel[calm].max()
    assert np.all(dm[~calm] <= 1e-7), dm[~calm]


@pytest.mark.gpu
def test_fused_layouts_give_identical_bits(gpu_lib, monkeypatch):
    a = _run(_rh(8, 2e-10), 2e-10, "fused", lanes=1, monkeypatch=monkeypatch)
    b = _run(_rh(8, 2e-10), 2e-10, "fused", lanes=4, monkeypatch=monkeypatch)
    assert np.array_equal(_m(a), _m(b))


def _pimm_junctions(n=16, total=1e-9):
    js = []
    for h in np.linspace(-600e3, 600e3, n):
        j = cases.mtj_rh_point(cmtj_gb300, hx=float(h), total=total)[0]
        j.setLayerOerstedFieldDriver("all", cmtj_gb300.AxialDriver(
            cmtj_gb300.stepDriver(0, 1000, 0, 1e-12), cmtj_gb300.NullDriver(), cmtj_gb300.NullDriver()))
        js.append(j)
    return js


@pytest.mark.gpu
def test_fused_time_dependent_field(gpu_lib):
    ref = _run(_pimm_junctions(), 1e-9, "reference", write=1e-12)
    fus = _run(_pimm_junctions(), 1e-9, "fused", write=1e-12)
    dm = float(np.max(np.abs(_m(fus) - _m(ref))))
    assert 0.0 < dm <= TOL_M, dm


def _stt_junction():
    return cases.sto(cmtj_gb300, 2e-10)[0]


def _log_arrays_equal(a, b):
    la, lb = a.getLogArrays(), b.getLogArrays()
    assert set(la) == set(lb)
    return all(np.array_equal(la[k], lb[k]) for k in la)


@pytest.mark.gpu
def test_uncovered_junctions_keep_reference_bits(gpu_lib):
    """STT, a time-dependent anisotropy and calculateEnergies run the
    reference arithmetic under CMTJ_ARITH_FUSED."""
    plan = engine.plan_run(2e-10, DT, 1e-12)
    for make, energies in ((_stt_junction, False), (lambda: _rh(1, 2e-10)[0], True)):
        a, b = make(), make()
        engine.run_junctions([a], plan, cmtj_gb300.SolverMode.RK4, energies, arithmetic="reference")
        engine.run_junctions([b], plan, cmtj_gb300.SolverMode.RK4, energies, arithmetic="fused")
        assert _log_arrays_equal(a, b)
    a, b = _rh(1, 2e-10)[0], _rh(1, 2e-10)[0]
    for j in (a, b):
        j.setLayerAnisotropyDriver("free", cmtj_gb300.sineDriver(3e5, 1e4, 5e9, 0))
    engine.run_junctions([a], plan, cmtj_gb300.SolverMode.RK4, arithmetic="reference")
    engine.run_junctions([b], plan, cmtj_gb300.SolverMode.RK4, arithmetic="fused")
    assert _log_arrays_equal(a, b)


@pytest.mark.gpu
def test_fused_choice_is_per_warp(gpu_lib):
    """Junctions that share a warp with an uncovered one run the reference
    arithmetic (the choice is made per warp); junctions of all-covered warps
    run fused.  A 2-layer junction takes 8 lanes in the quad layout (4 per
    warp): the STT single-layer junction first puts junctions 0-3 in warp 0."""
    plan = engine.plan_run(2e-10, DT, 1e-12)
    mixed = [_stt_junction()] + _rh(7, 2e-10)
    ref = [_stt_junction()] + _rh(7, 2e-10)
    engine.run_junctions(mixed, plan, cmtj_gb300.SolverMode.RK4, arithmetic="fused")
    engine.run_junctions(ref, plan, cmtj_gb300.SolverMode.RK4, arithmetic="reference")
    for k in range(4):
        assert _log_arrays_equal(mixed[k], ref[k]), k
    dms = []
    for a, b in zip(mixed[4:], ref[4:]):
        la, lb = a.getLogArrays(), b.getLogArrays()
        dms.append(max(float(np.max(np.abs(la[k] - lb[k]))) for k in KEYS))
    assert 0.0 < max(dms) <= TOL_M, dms


@pytest.mark.gpu
@pytest.mark.parametrize("arithmetic", ["reference", "fused"])
def test_blow_up_raises_like_the_reference(gpu_lib, arithmetic):
    """A field large enough to overflow the torque makes m NaN within the
    first steps.  Either arithmetic stops the junction there and raises the
    RuntimeError of the reference's rk4_step ("NAN magnetisation"), keeping
    the rows logged before it."""
    j = _rh(1, 2e-12)[0]
    j.setLayerExternalFieldDriver("all", cmtj_gb300.AxialDriver(1e308, 0, 0))
    with pytest.raises(RuntimeError, match="NAN magnetisation"):
        _run([j], 2e-12, arithmetic)
    assert len(j.getLogArrays().get("time", [])) < 20
