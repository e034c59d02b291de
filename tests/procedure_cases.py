"""Small PIMM and spin-diode sweeps written against the `cmtj` API
(reference or cmtj_gb300), shared by tests/golden/make_procedures.py and
tests/test_procedures.py.  Each case returns (junction, keyword arguments of
the procedure, with "kind" naming it)."""
import numpy as np

SEED = 1234


def _bilayer(cm):
    import cases
    j, _ = cases.mtj_rh_point(cm, hx=0.0)
    return j


def _res(RP, n):
    return [RP(Rxx0=100, Rxy0=5, Ramr=-0.24, Rahe=-0.3, Rsmr=-0.46, w=3e-5, l=2e-5) for _ in range(n)]


def pimm_bilayer(cm, RP):
    Hspan = np.linspace(-300e3, 300e3, 5)
    Hvecs = np.stack([Hspan, 0 * Hspan, 0 * Hspan], 1)
    return _bilayer(cm), dict(kind="pimm", Hvecs=Hvecs, int_step=1e-13, resistance_params=_res(RP, 2),
                              Hoe_excitation=1e3, simulation_duration=2e-10, disturbance=0.0, take_last_n=50,
                              max_frequency=80e9, disable_tqdm=True)


def pimm_bilayer_disturbed(cm, RP):
    j, kw = pimm_bilayer(cm, RP)
    kw["disturbance"] = 1e-3
    kw["wait_time"] = 5e-11
    return j, kw


def vsd_bilayer(cm, RP):
    Hspan = np.linspace(-200e3, 200e3, 3)
    Hvecs = np.stack([Hspan, 0 * Hspan, 0 * Hspan], 1)
    return _bilayer(cm), dict(kind="vsd", Hvecs=Hvecs, frequencies=np.array([3e9, 7e9]), int_step=1e-13,
                              resistance_params=_res(RP, 2), Hoe_excitation=2e3, simulation_duration=2e-10,
                              disturbance=0.0, Rtype="Rz", disable_tqdm=True)


def vsd_bilayer_rx(cm, RP):
    j, kw = vsd_bilayer(cm, RP)
    kw["Rtype"] = "Rx"
    return j, kw


CASES = {
    "pimm_bilayer": pimm_bilayer,
    "pimm_bilayer_disturbed": pimm_bilayer_disturbed,
    "vsd_bilayer": vsd_bilayer,
    "vsd_bilayer_rx": vsd_bilayer_rx,
}


def pimm_bilayer_saturated(cm, RP):
    """The same junction swept from saturation downwards along +x (no
    switching on the way): a well-conditioned chain."""
    j, kw = pimm_bilayer(cm, RP)
    Hspan = np.linspace(600e3, 350e3, 5)
    kw["Hvecs"] = np.stack([Hspan, 0 * Hspan, 0 * Hspan], 1)
    j.setLayerMagnetisation("free", cm.CVector(1, 0, 0.1))
    j.setLayerMagnetisation("ref", cm.CVector(1, 0, 0.2))
    return j, kw


CASES["pimm_bilayer_saturated"] = pimm_bilayer_saturated
