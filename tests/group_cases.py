"""GroupInteraction cases (core/reservoir.hpp:122-245) written against the
`cmtj` API (reference, cmtj_gb300 or the oracle module), shared by
tests/golden/make_groups.py and tests/test_groups.py.  Each case returns
(group, run keyword arguments)."""
import math

SURFACE = math.pi * (20e-9) ** 2


def _free(cm, mag, Ms=1.0, K=3e5, hx=0.0, layer_id="free"):
    z = cm.CVector(0, 0, 0)
    l = cm.Layer(layer_id, mag=cm.CVector(*mag), anis=cm.CVector(0, 0, 1), Ms=Ms, thickness=2e-9,
                 cellSurface=SURFACE, demagTensor=[z, z, cm.CVector(0, 0, 0.9)], damping=0.02)
    l.setAnisotropyDriver(cm.constantDriver(K))
    l.setExternalFieldDriver(cm.AxialDriver(hx, 0, 0))
    return l


def _single(cm, mag, **kw):
    return cm.Junction([_free(cm, mag, **kw)])


def _bilayer(cm, mag):
    free = _free(cm, mag)
    ref = _free(cm, (0, 0, 1), Ms=1.4, K=1e6, layer_id="ref")
    j = cm.Junction([free, ref], 100, 200)
    j.setIECDriver("free", "ref", cm.constantDriver(-2e-5))
    return j


def grp_dipole_pair(cm):
    js = [_single(cm, (0.3, 0.1, 0.95)), _single(cm, (-0.2, 0.2, 0.96), hx=2e4)]
    g = cm.reservoir.GroupInteraction([cm.CVector(0, 0, 0), cm.CVector(60e-9, 0, 0)], js)
    return g, dict(totalTime=2e-10, timeStep=1e-13, writeFrequency=1e-12)


def grp_noumra_quad(cm):
    js = [_single(cm, (0.1 * k, 0.2, 0.97)) for k in range(4)]
    pos = [cm.CVector(x, y, 0) for x in (0.0, 50e-9) for y in (0.0, 50e-9)]
    g = cm.reservoir.GroupInteraction(pos, js)
    g.setInteractionFunction(cm.reservoir.computeDipoleInteractionNoumra)
    return g, dict(totalTime=2e-10, timeStep=1e-13, writeFrequency=1e-12)


def grp_bilayers_single_runner(cm):
    """Two 2-layer junctions, then a 1-layer one: the reference takes the
    runner from the last junction, so every junction steps only layer 0."""
    js = [_bilayer(cm, (0.3, 0.0, 0.95)), _bilayer(cm, (0.0, 0.3, 0.95)), _single(cm, (0.2, 0.2, 0.96))]
    pos = [cm.CVector(0, 0, 0), cm.CVector(70e-9, 0, 0), cm.CVector(0, 70e-9, 0)]
    g = cm.reservoir.GroupInteraction(pos, js)
    return g, dict(totalTime=1e-10, timeStep=1e-13, writeFrequency=1e-12)


def grp_bilayers(cm):
    js = [_bilayer(cm, (0.3, 0.0, 0.95)), _bilayer(cm, (0.0, 0.3, 0.95))]
    g = cm.reservoir.GroupInteraction([cm.CVector(0, 0, 0), cm.CVector(0, 80e-9, 0)], js)
    return g, dict(totalTime=1e-10, timeStep=1e-13, writeFrequency=1e-12)


def grp_null(cm):
    js = [_single(cm, (0.3, 0.1, 0.95)), _single(cm, (-0.2, 0.2, 0.96))]
    g = cm.reservoir.GroupInteraction([cm.CVector(0, 0, 0), cm.CVector(60e-9, 0, 0)], js)
    g.setInteractionFunction(cm.reservoir.nullDipoleInteraction)
    return g, dict(totalTime=1e-10, timeStep=1e-13, writeFrequency=1e-12)


CASES = {
    "grp_dipole_pair": grp_dipole_pair,
    "grp_noumra_quad": grp_noumra_quad,
    "grp_bilayers_single_runner": grp_bilayers_single_runner,
    "grp_bilayers": grp_bilayers,
    "grp_null": grp_null,
}


def run_case(cm, name):
    """Build and run; returns {junction index: log dict of numpy arrays}."""
    import numpy as np
    g, kw = CASES[name](cm)
    g.runSimulation(**kw)
    return {k: {key: np.asarray(v, dtype=np.float64) for key, v in g.getLog(k).items()} for k in range(_count(g))}


def _count(g):
    n = 0
    while True:
        try:
            g.getLog(n)
        except RuntimeError:
            return n
        n += 1
