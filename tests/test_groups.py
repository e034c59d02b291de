"""Dipole-coupled groups (cmtj_gb300.reservoir.GroupInteraction) against the
reference's own logs (tests/golden/groups.npz, tests/golden/make_groups.py):
the oracle bit for bit on CPU, the FP64 plain GPU form within 1e-9.  Plus
the reference's API checks (tests/test_group_interaction.py in its suite)."""
import os

import numpy as np
import pytest

import cmtj_gb300 as cm
import group_cases
import oracle_harness

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "groups.npz"))


def _golden(name):
    out = {}
    for key in GOLDEN.files:
        case, k, col = key.split("__", 2)
        if case == name:
            out.setdefault(int(k), {})[col] = GOLDEN[key]
    return out


@pytest.mark.parametrize("name", sorted(group_cases.CASES))
def test_group_oracle_matches_reference_bitwise(name):
    got = group_cases.run_case(oracle_harness.oracle_module(), name)
    want = _golden(name)
    assert sorted(got) == sorted(want)
    for k in want:
        assert set(got[k]) == set(want[k]), (k, set(got[k]) ^ set(want[k]))
        for col, v in want[k].items():
            assert got[k][col].shape == v.shape, (name, k, col)
            assert np.array_equal(got[k][col], v), (name, k, col, np.max(np.abs(got[k][col] - v)))


def test_group_api_checks():
    z = cm.CVector(0, 0, 0)

    def junction():
        l = cm.Layer("free", mag=cm.CVector(0, 0, 1), anis=cm.CVector(0, 0, 1), Ms=1.0, thickness=2e-9,
                     cellSurface=1e-16, demagTensor=[z, z, z])
        return cm.Junction([l])

    p1, p2 = cm.CVector(0, 0, 0), cm.CVector(100e-9, 0, 0)
    cm.reservoir.GroupInteraction([p1, p2], [junction(), junction()])
    with pytest.raises(RuntimeError):
        cm.reservoir.GroupInteraction([p1], [junction(), junction()])
    with pytest.raises(RuntimeError):
        cm.reservoir.GroupInteraction([], [])
    with pytest.raises(RuntimeError):
        cm.reservoir.GroupInteraction([p1, p1], [junction(), junction()])
    g = cm.reservoir.GroupInteraction([p1, p2], [junction(), junction()])
    with pytest.raises(RuntimeError, match="non-existing"):
        g.getLog(5)
    j1, j2 = junction(), junction()
    h = cm.reservoir.nullDipoleInteraction(p1, p2, j1.getLayer("free"), j2.getLayer("free"))
    assert (h.x, h.y, h.z) == (0, 0, 0)
    assert isinstance(cm.reservoir.computeDipoleInteraction(p1, p2, j1.getLayer("free"), j2.getLayer("free")),
                      cm.CVector)
    assert isinstance(cm.reservoir.computeDipoleInteractionNoumra(p1, p2, j1.getLayer("free"),
                                                                  j2.getLayer("free")), cm.CVector)
    with pytest.raises(RuntimeError, match="too close"):
        cm.reservoir.computeDipoleInteraction(p1, cm.CVector(1e-12, 0, 0), j1.getLayer("free"), j2.getLayer("free"))


def test_group_pair_table():
    """The device pair table of a group: for every ordered pair (i, k != i)
    the fixed geometry of reservoir.hpp:82-90 (dipole) or the tensor of
    37-57 (Nomura) and the source junction's Ms V / mu0 factor; zero rows on
    the diagonal; too-close points raise when the table is formed."""
    from cmtj_gb300 import reservoir
    z = cm.CVector(0, 0, 0)

    def junction(ms, t):
        l = cm.Layer("free", mag=cm.CVector(0, 0, 1), anis=cm.CVector(0, 0, 1), Ms=ms, thickness=t,
                     cellSurface=1e-16, demagTensor=[z, z, z])
        return cm.Junction([l])

    pos = [cm.CVector(0, 0, 0), cm.CVector(60e-9, 0, 0), cm.CVector(0, 45e-9, 5e-9)]
    js = [junction(1.0 + 0.1 * k, (1 + k) * 1e-9) for k in range(3)]
    g = reservoir.GroupInteraction(pos, js)
    mu0 = reservoir._mu0()
    P = [reservoir._v(p) for p in pos]
    dip = g._pairs(reservoir.INTERACTION_DIPOLE)
    nom = g._pairs(reservoir.INTERACTION_NOUMRA)
    for i in range(3):
        for k in range(3):
            a, b = dip[3 * i + k], nom[3 * i + k]
            if i == k:
                assert not a["g"].any() and a["scale"] == 0 and not b["g"].any() and b["scale"] == 0
                continue
            ms, t = 1.0 + 0.1 * k, (1 + k) * 1e-9
            rij, r3, r5 = reservoir._dipole_geometry(P[i], P[k])
            assert list(a["g"][:5]) == [rij[0], rij[1], rij[2], r3, r5] and not a["g"][5:].any()
            assert a["scale"] == (ms / mu0) * (t * 1e-16)
            assert list(b["g"]) == reservoir._dipole_tensor(P[i], P[k])
            assert b["scale"] == (ms * (t * 1e-16)) / mu0
    close = reservoir.GroupInteraction([cm.CVector(0, 0, 0), cm.CVector(1e-12, 0, 0)],
                                       [junction(1.0, 1e-9), junction(1.0, 1e-9)])
    with pytest.raises(RuntimeError, match="too close"):
        close._pairs(reservoir.INTERACTION_DIPOLE)


def test_group_interaction_functions_match_reference_formula():
    """The host forms of the two dipole fields against their formulas
    written with numpy (reservoir.hpp:77-97 and 37-57, 99-122)."""
    z = cm.CVector(0, 0, 0)
    l1 = cm.Layer("free", mag=cm.CVector(0, 0, 1), anis=cm.CVector(0, 0, 1), Ms=1.1, thickness=2e-9,
                  cellSurface=1e-16, demagTensor=[z, z, z])
    l2 = cm.Layer("free", mag=cm.CVector(0.6, 0.0, 0.8), anis=cm.CVector(0, 0, 1), Ms=1.3, thickness=3e-9,
                  cellSurface=2e-16, demagTensor=[z, z, z])
    r1, r2 = np.array([10e-9, 5e-9, 0.0]), np.array([-40e-9, 20e-9, 3e-9])
    mu0 = cm.constants.snapshot()["mu0"] if hasattr(cm.constants, "snapshot") else 12.566e-7
    rij = r1 - r2
    n = np.linalg.norm(rij)
    m = np.array([0.6, 0.0, 0.8])
    V = 3e-9 * 2e-16
    want = (1.3 / mu0) * V * (3 * np.dot(m, rij) * rij / n ** 5 - m / n ** 3)
    got = cm.reservoir.computeDipoleInteraction(cm.CVector(*r1), cm.CVector(*r2), l1, l2)
    assert np.allclose([got.x, got.y, got.z], want, rtol=1e-12, atol=0)
    T = 3 / (4 * np.pi * n ** 5) * (np.outer(rij, rij) - np.eye(3) * n * n / 3)
    want = T @ m * (1.3 * V / mu0)
    got = cm.reservoir.computeDipoleInteractionNoumra(cm.CVector(*r1), cm.CVector(*r2), l1, l2)
    assert np.allclose([got.x, got.y, got.z], want, rtol=1e-12, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(group_cases.CASES))
def test_group_fp64_gpu_matches_reference(gpu_lib, name):
    got = group_cases.run_case(cm, name)
    want = _golden(name)
    for k in want:
        for col, v in want[k].items():
            a = got[k][col]
            assert a.shape == v.shape
            if col == "time":
                assert np.array_equal(a, v)
            elif col.endswith(("_mx", "_my", "_mz")):
                assert np.max(np.abs(a - v)) <= 1e-9, (name, k, col)
            else:
                assert np.max(np.abs(a - v)) <= 1e-9 * max(np.max(np.abs(v)), 1e-300), (name, k, col)


def _force_params(monkeypatch, **fields):
    """Lower with the given cmtj_sim_params_t fields overridden."""
    from cmtj_gb300 import _lower
    orig = _lower.make_params

    def make_params(*a, **k):
        p = orig(*a, **k)
        for f, v in fields.items():
            p[f] = v
        return p

    monkeypatch.setattr(_lower, "make_params", make_params)


@pytest.mark.gpu
@pytest.mark.parametrize("lanes", [1, 4])
@pytest.mark.parametrize("name", sorted(group_cases.CASES))
def test_group_both_layouts_match_reference(gpu_lib, monkeypatch, name, lanes):
    """The group kernel with a layer per lane and with a layer's x, y, z on a
    quad of lanes, against the reference's logs."""
    _force_params(monkeypatch, lanes_per_layer=lanes)
    got = group_cases.run_case(cm, name)
    for k, cols in _golden(name).items():
        for col, v in cols.items():
            a = got[k][col]
            if col == "time":
                assert np.array_equal(a, v)
            elif col.endswith(("_mx", "_my", "_mz")):
                assert np.max(np.abs(a - v)) <= 1e-9, (name, k, col)
            else:
                assert np.max(np.abs(a - v)) <= 1e-9 * max(np.max(np.abs(v)), 1e-300), (name, k, col)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["dipole", "noumra_thermal"])
def test_wide_group_thread_per_junction_equals_lanes(gpu_lib, monkeypatch, mode):
    """40 bilayer junctions on a 4 x 10 grid.  Told that a junction may hold
    8 layers, the group no longer fits a CTA of lanes and runs one thread
    per junction (k_group_f64); otherwise its layers run on lanes
    (k_group_lanes).  Both give the same bits in every log and leave the
    same reserved interaction field on every top layer."""
    def build():
        js = [group_cases._bilayer(cm, (0.3 - 0.01 * k, 0.05 * (k % 3), 0.95)) for k in range(40)]
        if mode == "noumra_thermal":
            for q, j in enumerate(js):
                j.setLayerTemperatureDriver("all", cm.constantDriver(300.0))
                for l, layer in enumerate(j.layers):
                    layer.noise_seed = 5000 + 10 * q + l
        pos = [cm.CVector(70e-9 * (k % 4), 70e-9 * (k // 4), 0) for k in range(40)]
        g = cm.reservoir.GroupInteraction(pos, js)
        if mode == "noumra_thermal":
            g.setInteractionFunction(cm.reservoir.computeDipoleInteractionNoumra)
        g.runSimulation(3e-11, 1e-13, 1e-12)
        return g

    on_lanes = build()
    _force_params(monkeypatch, max_layers=8, lanes_per_layer=1)
    per_thread = build()
    for q in range(40):
        la, lb = on_lanes.getLog(q), per_thread.getLog(q)
        assert la.keys() == lb.keys()
        for k in la:
            assert np.array_equal(np.asarray(la[k]), np.asarray(lb[k])), (q, k)
        a = on_lanes.junctionList[q].getLayer("free")
        b = per_thread.junctionList[q].getLayer("free")
        assert (a.mag.x, a.mag.y, a.mag.z) == (b.mag.x, b.mag.y, b.mag.z)
        ha, hb = a.axial["hres"], b.axial["hres"]
        assert [d.getCurrentScalarValue(0.0) for d in ha.drivers] == [d.getCurrentScalarValue(0.0) for d in hb.drivers]
