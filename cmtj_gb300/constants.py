"""Runtime-mutable physical constants (core/constants.hpp:6-55, bound in
python/cmtj.cpp:496-511).  The solver reads them at every launch, so a
change applies to the next runSimulation, as in the reference."""
import math

_DEFAULTS = {
    "mu0": 12.566e-7,
    "gyro": 220880.0,
    "TtoAm": 795774.715459,
    "hbar": 6.62607015e-34 / (2.0 * math.pi),
    "echarge": 1.60217662e-19,
    "kB": 1.380649e-23,
}
_values = dict(_DEFAULTS)


def snapshot():
    """Current constants as a dict (mu0, gyro, TtoAm, hbar, echarge, kB)."""
    return dict(_values)


class PhysicalConstants:
    @staticmethod
    def set_magnetic_permeability(value):
        _values["mu0"] = float(value)

    @staticmethod
    def set_gyromagnetic_ratio(value):
        _values["gyro"] = float(value)

    @staticmethod
    def set_TtoAm(value):
        _values["TtoAm"] = float(value)

    @staticmethod
    def set_hbar(value):
        _values["hbar"] = float(value)

    @staticmethod
    def set_elementary_charge(value):
        _values["echarge"] = float(value)

    @staticmethod
    def set_boltzmann_constant(value):
        _values["kB"] = float(value)

    @staticmethod
    def magnetic_permeability():
        return _values["mu0"]

    @staticmethod
    def gyromagnetic_ratio():
        return _values["gyro"]

    @staticmethod
    def TtoAm():
        return _values["TtoAm"]

    @staticmethod
    def hbar():
        return _values["hbar"]

    @staticmethod
    def elementary_charge():
        return _values["echarge"]

    @staticmethod
    def boltzmann_constant():
        return _values["kB"]

    @staticmethod
    def resetToDefaults():
        _values.update(_DEFAULTS)
