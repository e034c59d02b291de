"""Stochastic cases written against the `cmtj` API (reference or
cmtj_gb300).

p-bit: one STT free layer (Ms 1.0 T, t 1.2 nm, surface 7e-17 m^2, alpha
0.02, zero demag, Slonczewski polarisation 0.6, reference -z), Ku chosen so
the barrier is about 3 kT at 300 K, m from +z, a 1 ns current step, 2 ns in
total at dt = 1e-13 with Euler-Heun.  The observable is P(m_z < 0 at the
end) per current density."""
import math

PBIT_CURRENTS = [0.0, 2e10, 4e10, 6e10, 8e10, 1e11, 1.5e11, 3e11]
PBIT_KU = 1.5e5
PBIT_T = 300.0


def pbit_junction(cm, j_density, Ku=PBIT_KU, T=PBIT_T):
    """The p-bit junction; T = None sets no temperature driver."""
    z = cm.CVector(0, 0, 0)
    l = cm.Layer.createSTTLayer("free", mag=cm.CVector(0, 0, 1), anis=cm.CVector(0, 0, 1), Ms=1.0,
                                thickness=1.2e-9, cellSurface=7e-17, demagTensor=[z, z, z], damping=0.02,
                                SlonczewskiSpacerLayerParameter=1.0, beta=0.0, spinPolarisation=0.6)
    l.setReferenceLayer(cm.CVector(0, 0, -1))
    j = cm.Junction([l])
    j.setLayerAnisotropyDriver("free", cm.constantDriver(Ku))
    j.setLayerCurrentDriver("free", cm.stepDriver(0, j_density, 0, 1e-9))
    if T is not None:
        j.setLayerTemperatureDriver("free", cm.constantDriver(T))
    return j, dict(totalTime=2e-9, timeStep=1e-13, writeFrequency=1e-10,
                   solverMode=cm.SolverMode.EulerHeun)


def boltzmann_mz_density(mz, Ku, V, T, kB=1.380649e-23):
    """Equilibrium density of m_z for a uniaxial macrospin with zero demag
    and no field: p(m_z) proportional to exp(Ku V m_z^2 / kB T) on [-1, 1]
    (the sin(theta) of the solid angle is absorbed by d m_z)."""
    import numpy as np
    d = Ku * V / (kB * T)
    x = np.linspace(-1, 1, 20001)
    Z = np.trapezoid(np.exp(d * x * x), x)
    return np.exp(d * np.asarray(mz) ** 2) / Z


# The p-bit sweep at its full parameters (1,048,576 junctions in the bench:
# 64 current densities over [0, 5e11] A/m^2 x 16,384): Ku 2.5e5 J/m^3, a
# barrier of about 5 kT at 300 K, the same STT layer as above, a 1 ns
# current step, and a duration drawn per run from U[5, 20] ns.  The
# reference fixture uses every 4th current of the 64 plus the last one.
SWEEP_KU = 2.5e5
SWEEP_T_MIN, SWEEP_T_MAX = 5e-9, 20e-9
SWEEP_ALL_CURRENTS = [float(x) for x in __import__("numpy").linspace(0, 5e11, 64)]
SWEEP_CURRENTS = SWEEP_ALL_CURRENTS[0:64:4] + [SWEEP_ALL_CURRENTS[63]]


def sweep_durations(n, seed):
    """Per-run durations U[5, 20] ns (seeded)."""
    import numpy as np
    return np.random.default_rng(seed).uniform(SWEEP_T_MIN, SWEEP_T_MAX, size=n)


def pbit_sweep_junction(cm, j_density, duration):
    """One junction of the full p-bit sweep and its run arguments (logging
    once per ns: the observable is the final m_z)."""
    j, run = pbit_junction(cm, j_density, Ku=SWEEP_KU)
    run = dict(run)
    run.update(totalTime=float(duration), writeFrequency=1e-9)
    return j, run


# The p-bit layer above with buffered 1/f^alpha noise (setAlphaNoise(alpha,
# std 1, scale, axis)), 2 ns Euler-Heun: (current A/m^2, temperature K,
# alpha, scale, axis: 3 all, 0 x only).  Without alpha noise the T = 0
# cases never switch; with it most switch a good part of the time, and the
# 300 K case switches about three times as often as thermal noise alone.
ALPHA_CASES = [(1e11, 0.0, 1.0, 0.01, 3), (6e10, 0.0, 1.0, 0.03, 3), (0.0, 300.0, 1.0, 0.01, 3),
               (1e11, 0.0, 0.5, 0.01, 3), (1e11, 0.0, 1.5, 0.01, 3), (1e11, 0.0, 1.0, 0.03, 0)]


def alpha_pbit_junction(cm, j_density, T, alpha, scale, axis):
    """The p-bit junction with alpha noise on its layer; T = 0 sets no
    temperature."""
    j, run = pbit_junction(cm, j_density, T=T if T else None)
    j.getLayer("free").setAlphaNoise(alpha, 1.0, scale, cm.Axis(int(axis)))
    return j, run
