"""The simulation-running tests of the reference suite (tests/test_basic.py,
test_solvers.py, test_procedures.py and the fixtures of its conftest.py),
imported as the reference's users import it (`import cmtj`, the alias
package of cmtj_gb300) and run on the GPU solver unchanged in
substance: the same junctions, solvers, calls and assertions.  The
procedure sweeps are shortened (5 field points, 1 ns) so the file runs in
seconds; the full-size numerical parity is pinned elsewhere."""
from math import pi

import numpy as np
import pytest

import cmtj
from cmtj import AxialDriver, CVector, Junction, Layer, ScalarDriver, SolverMode
from cmtj.utils import FieldScan
from cmtj.utils.procedures import PIMM_procedure, ResistanceParameters, VSD_procedure
from cmtj.utils.resistance import calculate_resistance_parallel, calculate_resistance_series

rp = ResistanceParameters(Rxx0=100, Rxy0=1, Rsmr=-0.46, Rahe=-2.7, Ramr=-0.24, l=30, w=20)
demag = [CVector(0, 0, 0), CVector(0, 0, 0), CVector(0, 0, 1)]
alpha = 0.005
surface = 150e-9 * 150e-9 * pi


def single_layer_mtj():
    l1 = Layer("free", mag=CVector(0, 0, 1), anis=CVector(1, 0, 0), Ms=1.65, thickness=3e-9, cellSurface=surface,
               demagTensor=demag, damping=alpha)
    junction = Junction([l1])
    junction.setLayerAnisotropyDriver("free", ScalarDriver.getConstantDriver(1.05e3))
    return junction, [rp]


def two_layer_mtj():
    l1 = Layer("free", mag=CVector(0, 0, 1), anis=CVector(1, 0, 0), Ms=1.65, thickness=3e-9, cellSurface=surface,
               demagTensor=demag, damping=alpha)
    l2 = Layer("bottom", mag=CVector(0, 0, 1), anis=CVector(1, 0, 0), Ms=1.45, thickness=4e-9,
               cellSurface=surface, demagTensor=demag, damping=alpha)
    junction = Junction([l1, l2], 100, 200)
    junction.setLayerAnisotropyDriver("free", ScalarDriver.getConstantDriver(1.05e3))
    junction.setLayerAnisotropyDriver("bottom", ScalarDriver.getConstantDriver(50e3))
    junction.setIECDriver("free", "bottom", ScalarDriver.getConstantDriver(-1.78e-3))
    junction.setQuadIECDriver("free", "bottom", ScalarDriver.getConstantDriver(-1.69e-4))
    return junction, [rp, rp]


def tri_layer_mtj():
    l1 = Layer("free", mag=CVector(0, 0, 1), anis=CVector(1, 0, 0), Ms=1.65, thickness=3e-9, cellSurface=surface,
               demagTensor=demag, damping=alpha)
    l2 = Layer("middle", mag=CVector(0, 0, 1), anis=CVector(1, 0, 0), Ms=1.45, thickness=4e-9,
               cellSurface=surface, demagTensor=demag, damping=alpha)
    l3 = Layer("bottom", mag=CVector(0.0, 0, 1.0), anis=CVector(0, 0, 1.0), Ms=0.7, thickness=1e-9,
               cellSurface=surface, demagTensor=demag, damping=alpha)
    junction = Junction([l1, l2, l3])
    for l, k in zip(["free", "middle", "bottom"], [1.05e3, 50e3, 1e4]):
        junction.setLayerAnisotropyDriver(l, ScalarDriver.getConstantDriver(k))
    junction.setIECDriver("free", "middle", ScalarDriver.getConstantDriver(-1.78e-3))
    junction.setQuadIECDriver("free", "middle", ScalarDriver.getConstantDriver(-1.69e-4))
    junction.setIECDriver("middle", "bottom", ScalarDriver.getConstantDriver(3e-4))
    junction.setQuadIECDriver("middle", "bottom", ScalarDriver.getConstantDriver(2e-6))
    return junction, [rp, rp, rp]


FIXTURES = {"single_layer_mtj": single_layer_mtj, "two_layer_mtj": two_layer_mtj, "tri_layer_mtj": tri_layer_mtj}


def _unit_norm(junction):
    for lid in junction.getLayerIds():
        m = junction.getLayerMagnetisation(lid)
        assert abs(np.sqrt(m.x ** 2 + m.y ** 2 + m.z ** 2) - 1) < 1e-9


@pytest.mark.gpu
def test_basic_mtj(gpu_lib):
    """test_basic.py::test_basic_mtj."""
    l1 = Layer("free", mag=CVector(0, 0, 1), anis=CVector(1, 0, 0), Ms=1.65, thickness=3e-9, cellSurface=0,
               demagTensor=demag, damping=alpha)
    l1.setReferenceLayer(CVector(1, 0, 0))
    junction = Junction([l1], 100, 200)
    junction.setLayerAnisotropyDriver("free", ScalarDriver.getConstantDriver(1.05e3))
    junction.setLayerExternalFieldDriver("all", AxialDriver(CVector(300e3, 10e3, 0)))
    junction.runSimulation(10e-9, 1e-12, 1e-12)
    log = junction.getLog()
    assert "R" in log.keys()
    assert np.all(np.asarray(log["R"]))
    assert len(log["time"]) == 10000


@pytest.mark.gpu
def test_second_order_anisotropy(gpu_lib):
    """test_basic.py::test_second_order_anisotropy."""
    z = CVector(0, 0, 0)
    l1 = Layer("free", mag=CVector(0, 0, 1), anis=CVector(0, 0, 1), Ms=0.5, thickness=1e-9, cellSurface=70e-9,
               demagTensor=[z, z, z], damping=0.03)
    l1.setAnisotropyDriver(ScalarDriver.getConstantDriver(1e6))
    l1.setSecondOrderAnisotropyDriver(ScalarDriver.getConstantDriver(1e6))
    j = Junction([l1])
    j.runSimulation(1e-9, 1e-12, 1e-12, calculateEnergies=True)
    assert "free_K2" in j.getLog().keys()


@pytest.mark.gpu
@pytest.mark.parametrize("arg", sorted(FIXTURES))
def test_base_solver(gpu_lib, arg):
    """test_solvers.py::test_base_solver (both definitions): every solver,
    deterministic and at 300 K, back to back on the same junction."""
    junction, _ = FIXTURES[arg]()
    junction.runSimulation(10e-9, 1e-12, 1e-12)
    junction.runSimulation(10e-9, 1e-12, 1e-12, solverMode=SolverMode.EulerHeun)
    junction.runSimulation(10e-9, 1e-12, 1e-12, solverMode=SolverMode.Heun)
    _unit_norm(junction)
    junction.setLayerTemperatureDriver("all", ScalarDriver.getConstantDriver(300))
    junction.runSimulation(10e-9, 1e-12, 1e-12)
    junction.runSimulation(10e-9, 1e-12, 1e-12, solverMode=SolverMode.EulerHeun)
    junction.runSimulation(10e-9, 1e-12, 1e-12, solverMode=SolverMode.Heun)
    _unit_norm(junction)
    assert len(junction.getLog()["time"]) == 6 * 10000


def _hvecs():
    _, Hvecs = FieldScan.amplitude_scan(-500e3, 500e3, steps=5, theta=90, phi=0)
    return Hvecs


@pytest.mark.gpu
def test_base_pimm(gpu_lib):
    """test_procedures.py::test_base_pimm, every parameter variant."""
    from itertools import product
    junction, res = single_layer_mtj()
    variants = {"static_only": [True, False], "full_output": [True, False],
                "resistance_fn": [calculate_resistance_series, calculate_resistance_parallel],
                "Hoe_direction": [cmtj.Axis.xaxis, cmtj.Axis.yaxis]}
    for values in product(*variants.values()):
        kw = dict(zip(variants.keys(), values))
        spec, f, out = PIMM_procedure(junction, Hvecs=_hvecs(), resistance_params=res, int_step=1e-12,
                                      simulation_duration=1e-9, disable_tqdm=True, **kw)
        if kw["static_only"]:
            assert f is None
            assert len(spec) == 0
        elif kw["full_output"]:
            assert "m_traj" in out


@pytest.mark.gpu
@pytest.mark.parametrize("arg", sorted(FIXTURES))
def test_pimm_and_vsd(gpu_lib, arg):
    """test_procedures.py::test_pimm and ::test_vsd (Rx)."""
    junction, res = FIXTURES[arg]()
    spec, freqs, out = PIMM_procedure(junction, Hvecs=_hvecs(), int_step=1e-12, resistance_params=res,
                                      simulation_duration=1e-9, disable_tqdm=True)
    assert spec.shape[0] == 5 and np.all(np.isfinite(spec))
    vsd = VSD_procedure(junction, Hvecs=_hvecs(), resistance_params=res, frequencies=np.arange(1e9, 4e9, 1e9),
                        int_step=1e-12, simulation_duration=1e-9, Rtype="Rx", disable_tqdm=True)
    assert vsd.shape == (5, 3) and np.all(np.isfinite(vsd))
