"""Junction cases written once against the `cmtj` API and built with either
module: the reference (`cmtj` from the reference build, only where the
golden fixtures are generated) or `cmtj_gb300`.

Each case returns (junction, runs) where runs is a list of runSimulation
keyword dicts applied in order (state and log carry over, as in the
reference).  Sizes are kept small so the oracle and the reference finish in
well under a second per case.
"""
import math

# demag of tests/conftest.py:12 in the reference suite
DEMAG_Z = ((0, 0, 0), (0, 0, 0), (0, 0, 1))
SURFACE = 150e-9 * 150e-9 * math.pi


def _v(cm, t):
    return cm.CVector(*t)


def _demag(cm, rows):
    return [cm.CVector(*r) for r in rows]


def mtj_rh_point(cm, hx=-300e3, total=1e-9):
    """One field point of the 2-layer R(H) sweep (free Ms 1.2 T, Ku 3e5 z,
    t 1.5 nm; reference Ms 1.5 T, Ku 1e6 z, t 2 nm; alpha 0.01; demag
    diag(0.0024, 0.0024, 0.9952); surface 1e-16; IEC -5e-5)."""
    demag = [(0.0024, 0, 0), (0, 0.0024, 0), (0, 0, 0.9952)]
    free = cm.Layer("free", mag=_v(cm, (0, 0, 1)), anis=_v(cm, (0, 0, 1)), Ms=1.2, thickness=1.5e-9,
                    cellSurface=1e-16, demagTensor=_demag(cm, demag), damping=0.01)
    ref = cm.Layer("ref", mag=_v(cm, (0, 0, 1)), anis=_v(cm, (0, 0, 1)), Ms=1.5, thickness=2e-9,
                   cellSurface=1e-16, demagTensor=_demag(cm, demag), damping=0.01)
    j = cm.Junction([free, ref], 100, 200)
    j.setLayerAnisotropyDriver("free", cm.constantDriver(3e5))
    j.setLayerAnisotropyDriver("ref", cm.constantDriver(1e6))
    j.setIECDriver("free", "ref", cm.constantDriver(-5e-5))
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(hx, 0, 0))
    return j, [dict(totalTime=total, timeStep=1e-13, writeFrequency=1e-12)]


def sto(cm, total=2e-9):
    """STT oscillator (curated test_sto, shortened)."""
    l1 = cm.Layer.createSTTLayer(id="free", mag=_v(cm, (0, 0, 1)), anis=_v(cm, (0, 0, 1)), Ms=1.0,
                                 thickness=1.4e-9, cellSurface=7e-10 * 7e-10, demagTensor=_demag(cm, DEMAG_Z),
                                 damping=0.3, SlonczewskiSpacerLayerParameter=1.0, spinPolarisation=1.0, beta=1)
    l1.setReferenceLayer(_v(cm, (0, 1.0, 1.0)))
    j = cm.Junction([l1], 100, 200)
    j.setLayerAnisotropyDriver("free", cm.constantDriver(350e3))
    j.setLayerCurrentDriver("free", cm.constantDriver(-6e9))
    return j, [dict(totalTime=total, timeStep=1e-13, writeFrequency=1e-12)]


def sot_strip(cm):
    """Two static-SOT layers with strip resistance (curated test_ahe_loops)."""
    demag = [(0, 0, 0), (0, 0, 0), (0, 0, 1)]
    OetoAm = 79.57747
    jden = 4.24e10
    HDL, HFL = 90 * OetoAm * 0.45 / jden, 90 * OetoAm / jden
    k1 = (math.sin(math.radians(1)), 0.0, math.cos(math.radians(1)))
    k2 = (math.sin(math.radians(0.01)), 0.0, math.cos(math.radians(0.01)))
    area = 10e-6 * 80e-6
    layers = []
    for name, k in (("free", k1), ("bottom", k2)):
        layers.append(cm.Layer.createSOTLayer(id=name, mag=_v(cm, k), anis=_v(cm, k), Ms=1.1, thickness=1e-9,
                                              cellSurface=area, demagTensor=_demag(cm, demag), damping=5e-2,
                                              dampingLikeTorque=HDL, fieldLikeTorque=HFL))
    j = cm.Junction(layers, [100, 100], [0, 0], [0.41, 0.41], [0.41, 0.41], [5.11, 5.11], [5.11, 5.11], [5, 5])
    j.setLayerAnisotropyDriver("free", cm.constantDriver(0.55e6))
    j.setLayerAnisotropyDriver("bottom", cm.constantDriver(0.3e6))
    j.setLayerReferenceLayer("free", _v(cm, (0, 1.0, 0)))
    j.setLayerReferenceLayer("bottom", _v(cm, (0, 1.0, 0)))
    j.setIECDriver("free", "bottom", cm.constantDriver(3e-3))
    j.setLayerCurrentDriver("all", cm.stepDriver(0, 5e10, 1e-10, 6e-10))
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(0, 0, -50e3))
    return j, [dict(totalTime=1e-9, timeStep=1e-13, writeFrequency=1e-12)]


def tri_layer(cm, solver=None):
    """3-layer strip junction with IEC + quadratic IEC (conftest tri_layer_mtj)."""
    mk = lambda i, m, a, Ms, t: cm.Layer(i, mag=_v(cm, m), anis=_v(cm, a), Ms=Ms, thickness=t,
                                         cellSurface=SURFACE, demagTensor=_demag(cm, DEMAG_Z), damping=0.005)
    l1 = mk("free", (0, 0, 1), (1, 0, 0), 1.65, 3e-9)
    l2 = mk("middle", (0, 0, 1), (1, 0, 0), 1.45, 4e-9)
    l3 = mk("bottom", (0, 0, 1.0), (0, 0, 1.0), 0.7, 1e-9)
    j = cm.Junction([l1, l2, l3], [100] * 3, [1] * 3, [-0.24] * 3, [-0.24] * 3, [-0.46] * 3, [-0.46] * 3,
                    [-2.7] * 3)
    for l, k in zip(["free", "middle", "bottom"], [1.05e3, 50e3, 1e4]):
        j.setLayerAnisotropyDriver(l, cm.constantDriver(k))
    j.setIECDriver("free", "middle", cm.constantDriver(-1.78e-3))
    j.setQuadIECDriver("free", "middle", cm.constantDriver(-1.69e-4))
    j.setIECDriver("middle", "bottom", cm.constantDriver(3e-4))
    j.setQuadIECDriver("middle", "bottom", cm.constantDriver(2e-6))
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(cm.constantDriver(20e3), cm.sineDriver(0, 5e3, 3e9, 0.1),
                                                         cm.constantDriver(-10e3)))
    run = dict(totalTime=1e-9, timeStep=1e-13, writeFrequency=1e-12)
    if solver is not None:
        run["solverMode"] = getattr(cm.SolverMode, solver)
    return j, [run]


def vsd_sine(cm):
    """Single strip layer under a sine Oersted field (curated VSD scans)."""
    l1 = cm.Layer(id="free", mag=_v(cm, (0.0, 0.0, 1.0)), anis=_v(cm, (0, 0.0, 1.0)), Ms=0.525, thickness=1.45e-9,
                  cellSurface=0, demagTensor=_demag(cm, DEMAG_Z), damping=30e-3)
    j = cm.Junction([l1], [304.306], [1.008], [-0.053], [-0.053], [-0.464], [-0.464], [-5.71])
    j.setLayerAnisotropyDriver("free", cm.constantDriver(1.54e5))
    th, ph = math.radians(91), 0.0
    H = 500e3
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(cm.constantDriver(H * math.sin(th) * math.cos(ph)),
                                                         cm.constantDriver(H * math.sin(th) * math.sin(ph)),
                                                         cm.constantDriver(H * math.cos(th))))
    j.setLayerOerstedFieldDriver("all", cm.AxialDriver(cm.NullDriver(), cm.NullDriver(),
                                                       cm.sineDriver(0, -5000, 14e9, 0)))
    return j, [dict(totalTime=2e-9, timeStep=1e-13, writeFrequency=5e-13)]


def energies_k2(cm):
    """Second-order anisotropy with the energy log (test_basic.py:55-102)."""
    l1 = cm.Layer("free", mag=_v(cm, (0.1, 0.2, 1)), anis=_v(cm, (0, 0.3, 1)), Ms=0.5, thickness=1e-9,
                  cellSurface=70e-9, demagTensor=_demag(cm, ((0, 0, 0), (0, 0, 0), (0, 0, 0))), damping=0.03)
    l1.setAnisotropyDriver(cm.ScalarDriver.getConstantDriver(1e6))
    l1.setSecondOrderAnisotropyDriver(cm.ScalarDriver.getConstantDriver(-2e5))
    j = cm.Junction([l1])
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(30e3, -20e3, 5e3))
    return j, [dict(totalTime=5e-10, timeStep=1e-13, writeFrequency=1e-12, calculateEnergies=True)]


def harmonic_hall(cm):
    """Full 3x3 demag tensor, step Oersted pulse, warm restart between two
    fields (curated test_harmonic_hall)."""
    demag = [(0.00024164288391924, 2.71396011566517e-10, 5.95503928124313e-14),
             (2.71396011566517e-10, 0.000160046006320031, 1.32504057070646e-14),
             (5.95503928124313e-14, 1.32504057070646e-14, 0.999598310229469)]
    l1 = cm.Layer(id="free", mag=_v(cm, (0, 0, 1)), anis=_v(cm, (0.0, 0, 1)), Ms=0.525, thickness=1.45e-9,
                  cellSurface=3e-5 * 2e-5, damping=0.03, demagTensor=_demag(cm, demag))
    j = cm.Junction([l1])
    j.setLayerOerstedFieldDriver("all", cm.AxialDriver(cm.NullDriver(), cm.NullDriver(),
                                                       cm.ScalarDriver.getStepDriver(0, 50, 0.0, 1e-11)))
    j.setLayerAnisotropyDriver("all", cm.ScalarDriver.getConstantDriver(1.54e5))
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(-200e3 * math.sin(math.radians(92)), 0,
                                                         -200e3 * math.cos(math.radians(92))))
    r = dict(totalTime=1e-9, timeStep=1e-12, writeFrequency=1e-12)
    return j, [r, r]


def drivers_zoo(cm):
    """Every waveform on some slot, dipole tensors, IDMI, Hdmi, kappa,
    alternative STT and a TOP reference in a 2-layer STT junction."""
    d1 = [(0.01, 0.002, 0), (0.002, 0.02, 0), (0, 0, 0.97)]
    l1 = cm.Layer.createSTTLayer("free", mag=_v(cm, (0.3, 0.1, 0.9)), anis=_v(cm, (0.1, 0, 1)), Ms=1.1,
                                 thickness=1.2e-9, cellSurface=2e-16, demagTensor=_demag(cm, d1), damping=0.02,
                                 SlonczewskiSpacerLayerParameter=1.5, beta=0.1, spinPolarisation=0.6)
    l2 = cm.Layer("pinned", mag=_v(cm, (0, 0.2, 1)), anis=_v(cm, (0, 0, 1)), Ms=1.4, thickness=2e-9,
                  cellSurface=2e-16, demagTensor=_demag(cm, d1), damping=0.015)
    l1.setTopDipoleTensor(_demag(cm, [(0.001, 0, 0), (0, 0.001, 0), (0, 0, -0.002)]))
    l2.setBottomDipoleTensor(_demag(cm, [(0.002, 0, 0), (0, 0.002, 0), (0, 0, -0.004)]))
    l1.setReferenceLayer(cm.Reference.top)
    l1.setKappa(0.8)
    j = cm.Junction([l1, l2], 120, 260)
    j.setLayerAnisotropyDriver("free", cm.trapezoidDriver(4e5, 5e4, 1e-10, 5e-11, 1e-10))
    j.setLayerAnisotropyDriver("pinned", cm.constantDriver(9e5))
    j.setLayerCurrentDriver("free", cm.pulseDriver(1e10, 4e10, 2e-10, 0.3))
    j.setIECDriver("free", "pinned", cm.gaussianImpulseDriver(-2e-4, 1e-4, 2e-10, 5e-11))
    j.setQuadIECDriver("free", "pinned", cm.constantDriver(1e-5))
    j.setIDMIDriver("free", "pinned", cm.AxialDriver(1e-5, 0, 2e-5))
    j.setLayerHdmiDriver("free", cm.AxialDriver(cm.posSineDriver(0, 2e3, 5e9, 0.3), cm.constantDriver(0),
                                                cm.constantDriver(100)))
    j.setLayerOerstedFieldDriver("pinned", cm.AxialDriver(cm.gaussianStepDriver(0, 3e3, 2e-10, 4e-11),
                                                          cm.constantDriver(0), cm.constantDriver(0)))
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(cm.sineDriver(1e4, 2e3, 2e9, 0.5), cm.constantDriver(-5e3),
                                                         cm.stepDriver(0, 2e4, 1e-10, 3e-10)))
    return j, [dict(totalTime=5e-10, timeStep=1e-13, writeFrequency=5e-13)]


def alt_stt_bottom(cm):
    """Alternative STT with a BOTTOM reference and a secondary SOT layer."""
    dz = _demag(cm, DEMAG_Z)
    l1 = cm.Layer("bottomL", mag=_v(cm, (1, 0, 0)), anis=_v(cm, (1, 0, 0)), Ms=1.2, thickness=2e-9,
                  cellSurface=1e-16, demagTensor=dz, damping=0.02)
    l2 = cm.Layer.createSTTLayer("topL", mag=_v(cm, (0, 0, 1)), anis=_v(cm, (0, 0, 1)), Ms=1.0, thickness=1e-9,
                                 cellSurface=1e-16, demagTensor=dz, damping=0.01,
                                 SlonczewskiSpacerLayerParameter=1.2, beta=0.05, spinPolarisation=0.5)
    l2.setReferenceLayer(cm.Reference.bottom)
    l2.setAlternativeSTT(True)
    j = cm.Junction([l1, l2])
    j.setLayerAnisotropyDriver("bottomL", cm.constantDriver(2e5))
    j.setLayerAnisotropyDriver("topL", cm.constantDriver(6e5))
    j.setLayerCurrentDriver("topL", cm.constantDriver(3e11))
    j.setLayerFieldLikeTorqueDriver("bottomL", cm.constantDriver(500))
    j.setLayerDampingLikeTorqueDriver("bottomL", cm.sineDriver(0, 800, 3e9, 0))
    j.setLayerSecondaryTorqueDrivers("bottomL", cm.constantDriver(100), cm.constantDriver(-200))
    j.setLayerReferenceLayer("bottomL", _v(cm, (0, 1, 0)))
    l = j.getLayer("bottomL")
    l.setSecondaryReferenceLayer(_v(cm, (0, 0, 1)))
    j.setIECDriver("bottomL", "topL", cm.constantDriver(1e-4))
    return j, [dict(totalTime=5e-10, timeStep=1e-13, writeFrequency=1e-12, calculateEnergies=True)]


def custom_driver(cm):
    """A Python-callback anisotropy driver (test_drivers.py:128-136 form)."""
    l1 = cm.Layer("free", mag=_v(cm, (0, 0, 1)), anis=_v(cm, (1, 0, 0)), Ms=1.65, thickness=3e-9,
                  cellSurface=SURFACE, demagTensor=_demag(cm, DEMAG_Z), damping=0.005)
    l1.setReferenceLayer(_v(cm, (1, 0, 0)))
    j = cm.Junction([l1], 100, 200)
    j.setLayerAnisotropyDriver("free", cm.ScalarDriver.getCustomDriver(lambda t: 1.05e3 + 5e12 * t))
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(cm.constantDriver(0), cm.constantDriver(0),
                                                         cm.ScalarDriver.getCustomDriver(lambda t: 1e4 * math.cos(3e9 * t))))
    return j, [dict(totalTime=3e-10, timeStep=1e-13, writeFrequency=1e-12)]


def fmr_unnormalised(cm):
    """3 layers, initial |m| = 0.99 (curated test_fmr_basic), warm restart."""
    dz = _demag(cm, DEMAG_Z)
    l1 = cm.Layer("free", mag=_v(cm, (0, 0, 0.99)), anis=_v(cm, (0, 0, 1)), Ms=1.03, thickness=1.0e-9,
                  damping=0.01, demagTensor=dz, cellSurface=1e-9)
    l2 = cm.Layer("perpendicular", mag=_v(cm, (0, 0, 0.99)), anis=_v(cm, (0, 0, 1)), Ms=1.03, thickness=1.0e-9,
                  damping=0.01, cellSurface=1e-9, demagTensor=dz)
    l3 = cm.Layer("buffer", mag=_v(cm, (1, 0, 0)), anis=_v(cm, (1, 0, 0)), Ms=0.12, thickness=1.0e-9,
                  damping=0.015, cellSurface=1e-9, demagTensor=dz)
    l1.setAnisotropyDriver(cm.constantDriver(489e3))
    l2.setAnisotropyDriver(cm.constantDriver(514e3))
    l3.setAnisotropyDriver(cm.constantDriver(17e3))
    j = cm.Junction([l1, l2, l3])
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(0, 0, 500e3))
    j.setLayerOerstedFieldDriver("all", cm.AxialDriver(cm.NullDriver(), cm.stepDriver(0, 500, 0, 2e-11),
                                                       cm.NullDriver()))
    r = dict(totalTime=5e-10, timeStep=5e-13, writeFrequency=5e-13)
    return j, [r, r]


def heun_det(cm):
    return tri_layer(cm, solver="Heun")


def euler_heun_det(cm):
    return tri_layer(cm, solver="EulerHeun")


def _dormand_prince(fn, total=None):
    """Case `fn` run with SolverMode.DormandPrince (junction.hpp:866-1002,
    1982-2045), optionally over a shorter horizon."""
    def case(cm):
        j, runs = fn(cm)
        out = []
        for r in runs:
            r = dict(r)
            r["solverMode"] = cm.SolverMode.DormandPrince
            if total is not None:
                r["totalTime"] = total
            out.append(r)
        return j, out
    case.__doc__ = "%s with the Dormand-Prince solver" % fn.__name__
    return case


# Multi-layer Dormand-Prince runs only while no layer rejects a step (the
# reference's rejection path for several layers does not terminate), so the
# multi-layer cases are short.
DORMAND_PRINCE = {
    "dp_sto": _dormand_prince(sto),
    "dp_vsd_sine": _dormand_prince(vsd_sine),
    "dp_harmonic_hall": _dormand_prince(harmonic_hall),
    "dp_energies_k2": _dormand_prince(energies_k2),
    "dp_mtj_rh_point": _dormand_prince(mtj_rh_point, total=2e-11),
    "dp_tri_layer": _dormand_prince(tri_layer, total=2e-12),
}

DETERMINISTIC = {
    "mtj_rh_point": mtj_rh_point,
    "sto": sto,
    "sot_strip": sot_strip,
    "tri_layer": tri_layer,
    "vsd_sine": vsd_sine,
    "energies_k2": energies_k2,
    "harmonic_hall": harmonic_hall,
    "drivers_zoo": drivers_zoo,
    "alt_stt_bottom": alt_stt_bottom,
    "custom_driver": custom_driver,
    "fmr_unnormalised": fmr_unnormalised,
    "heun_det": heun_det,
    "euler_heun_det": euler_heun_det,
    **DORMAND_PRINCE,
}


def run_case(cm, name):
    """Build and run a case with module cm; returns (junction, log dict of
    numpy arrays, final magnetisations {id: (x, y, z)})."""
    import numpy as np
    j, runs = DETERMINISTIC[name](cm)
    for r in runs:
        j.runSimulation(**r)
    log = {k: np.asarray(v, dtype=np.float64) for k, v in j.getLog().items()}
    mags = {}
    for lid in j.getLayerIds():
        m = j.getLayerMagnetisation(lid)
        mags[lid] = (m.x, m.y, m.z)
    return j, log, mags


# --------------------------------------------------------------------------
# Stacks (core/stack.hpp): STT junctions so that the coupled current moves m.
# --------------------------------------------------------------------------
def _stt_junction(cm, Ms, K, mag, anis, P=0.5):
    l1 = cm.Layer.createSTTLayer("free", mag=_v(cm, mag), anis=_v(cm, anis), Ms=Ms, thickness=2e-9,
                                 cellSurface=SURFACE, demagTensor=_demag(cm, DEMAG_Z), damping=0.02,
                                 SlonczewskiSpacerLayerParameter=1.0, beta=0.1, spinPolarisation=P)
    l1.setReferenceLayer(_v(cm, (1, 0, 0)))
    j = cm.Junction([l1], 100, 200)
    j.setLayerAnisotropyDriver("free", cm.constantDriver(K))
    j.setLayerExternalFieldDriver("all", cm.AxialDriver(5e3, 1e3, 0))
    return j


def _stt_bilayer(cm, Ms, K, mag):
    l1 = cm.Layer.createSTTLayer("free", mag=_v(cm, mag), anis=_v(cm, (1, 0, 0)), Ms=Ms, thickness=2e-9,
                                 cellSurface=SURFACE, demagTensor=_demag(cm, DEMAG_Z), damping=0.02,
                                 SlonczewskiSpacerLayerParameter=1.0, beta=0.0, spinPolarisation=0.4)
    l1.setReferenceLayer(cm.Reference.bottom)
    l2 = cm.Layer("bottom", mag=_v(cm, (1, 0, 0)), anis=_v(cm, (1, 0, 0)), Ms=1.4, thickness=3e-9,
                  cellSurface=SURFACE, demagTensor=_demag(cm, DEMAG_Z), damping=0.02)
    j = cm.Junction([l1, l2], 100, 200)
    j.setLayerAnisotropyDriver("free", cm.constantDriver(K))
    j.setLayerAnisotropyDriver("bottom", cm.constantDriver(5e4))
    j.setIECDriver("free", "bottom", cm.constantDriver(-1e-4))
    return j


def stack_series_kcl(cm):
    js = [_stt_junction(cm, 1.2, 1e3, (0.1, 0.2, 1), (1, 0, 0)),
          _stt_junction(cm, 1.0, 2e3, (0.3, 0.2, 0.9), (1, 0.1, 0.3))]
    s = cm.stack.SeriesStack(js)
    s.setCouplingStrength(0.3)
    s.setCoupledCurrentDriver(cm.constantDriver(5e10))
    return s, dict(totalTime=2e-10, timeStep=1e-13, writeFrequency=1e-12)


def stack_parallel_nonkcl(cm):
    js = [_stt_junction(cm, 1.2, 1e3, (0.1, 0.2, 1), (1, 0, 0)),
          _stt_junction(cm, 1.1, 1.5e3, (0.2, 0.1, 1), (1, 0, 0)),
          _stt_junction(cm, 1.0, 2e3, (0.3, 0.2, 0.9), (1, 0.1, 0.3))]
    s = cm.stack.ParallelStack(js, useKCL=False, phaseOffset=0.3)
    s.setCouplingStrength([0.1, 0.25])
    s.setCoupledCurrentDriver(cm.sineDriver(2e10, 3e10, 2e9, 0.1))
    return s, dict(totalTime=2e-10, timeStep=1e-13, writeFrequency=1e-12)


def stack_series_nondelayed(cm):
    js = [_stt_bilayer(cm, 1.2, 1e3, (0.1, 0.2, 1)), _stt_bilayer(cm, 1.0, 2e3, (0.3, 0.1, 0.9))]
    s = cm.stack.SeriesStack(js, useKCL=False, phaseOffset=0.2)
    s.setDelayed(False)
    s.setCouplingStrength(0.2)
    s.setCoupledCurrentDriver(cm.sineDriver(0, 8e10, 3e9, 0))
    return s, dict(totalTime=2e-10, timeStep=1e-13, writeFrequency=1e-12)


def stack_parallel_kcl_bilayer(cm):
    js = [_stt_bilayer(cm, 1.2, 1e3, (0.1, 0.2, 1)), _stt_bilayer(cm, 1.0, 2e3, (0.3, 0.1, 0.9))]
    s = cm.stack.ParallelStack(js)
    s.setCouplingStrength(0.4)
    s.setCoupledCurrentDriver(cm.stepDriver(0, 6e10, 2e-11, 1.5e-10))
    return s, dict(totalTime=2e-10, timeStep=1e-13, writeFrequency=2e-12)


STACKS = {
    "stack_series_kcl": stack_series_kcl,
    "stack_parallel_nonkcl": stack_parallel_nonkcl,
    "stack_series_nondelayed": stack_series_nondelayed,
    "stack_parallel_kcl_bilayer": stack_parallel_kcl_bilayer,
}


def run_stack_case(cm, name):
    """Build and run a stack case; returns (stack log, [junction logs]) as
    dicts of numpy arrays."""
    import numpy as np
    s, r = STACKS[name](cm)
    s.runSimulation(**r)
    slog = {k: np.asarray(v, dtype=np.float64) for k, v in s.getLog().items()}
    jlogs = []
    for q in range(len(s.junctionList) if hasattr(s, "junctionList") else 0):
        jlogs.append({k: np.asarray(v, dtype=np.float64) for k, v in s.getLog(q).items()})
    if not jlogs:
        q = 0
        while True:
            try:
                jlogs.append({k: np.asarray(v, dtype=np.float64) for k, v in s.getLog(q).items()})
            except RuntimeError:
                break
            q += 1
    return slog, jlogs


def junctions_from_spec(spec, rows, oersted=None):
    """Junction objects for rows of a sweeps.* spec (constant parts only;
    `oersted(k)` returns the AxialDriver of row k's time-dependent field)."""
    import cmtj_gb300 as cm
    out = []
    for k in rows:
        L = int(spec.n_layers[k])
        layers = []
        for l in range(L):
            d = [cm.CVector(*spec.demag[k, l, 3 * r:3 * r + 3]) for r in range(3)]
            ly = cm.Layer("L%d" % l, cm.CVector(*spec.m0[k, l]), cm.CVector(*spec.anis[k, l]), float(spec.Ms[k, l]),
                          float(spec.thickness[k, l]), float(spec.surface[k, l]), d, float(spec.alpha[k, l]))
            ly.setAnisotropyDriver(cm.constantDriver(float(spec.K[k, l])))
            ly.setExternalFieldDriver(cm.AxialDriver(*[float(x) for x in spec.Hc[k, l]]))
            if oersted is not None:
                ly.setOerstedFieldDriver(oersted(k))
            ly.mag = cm.CVector(*spec.m0[k, l])  # exact start, no renormalisation
            layers.append(ly)
        if spec.mr_mode[k] == 1:
            if L == 1:
                layers[0].setReferenceLayer(cm.CVector(*spec.ref[k, 0]))
            j = cm.Junction(layers, float(spec.Rp[k]), float(spec.Rap[k]))
        else:
            j = cm.Junction(layers)
        for l in range(L - 1):
            j.setIECDriver("L%d" % l, "L%d" % (l + 1), cm.constantDriver(float(spec.Jt[k, l])))
        out.append(j)
    return out
