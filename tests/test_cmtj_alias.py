"""`import cmtj` (the reference's import name, cmtj/__init__.py:10-18)
resolves to cmtj_gb300: the module's names and every submodule path the
reference's users import, as the same module objects."""
import importlib
import sys

import pytest


def test_cmtj_names_are_cmtj_gb300_names():
    import cmtj
    import cmtj_gb300
    for name in cmtj_gb300.__all__:
        assert getattr(cmtj, name) is getattr(cmtj_gb300, name), name
    assert cmtj.Junction is cmtj_gb300.Junction and cmtj.RK4 == cmtj_gb300.SolverMode.RK4


@pytest.mark.parametrize("sub", ["stack", "reservoir", "noise", "constants", "utils", "utils.procedures",
                                 "utils.resistance", "utils.filters", "utils.linear", "utils.parallel"])
def test_cmtj_submodules_alias_cmtj_gb300(sub):
    a = importlib.import_module("cmtj." + sub)
    b = importlib.import_module("cmtj_gb300." + sub)
    assert a is b and sys.modules["cmtj." + sub] is b


def test_reference_style_imports():
    from cmtj import AxialDriver, CVector, Junction, Layer, ScalarDriver  # noqa: F401
    from cmtj.stack import ParallelStack, SeriesStack  # noqa: F401
    from cmtj.noise import BufferedAlphaNoise, VectorAlphaNoise  # noqa: F401
    from cmtj.utils import FieldScan, Filters, compute_sd  # noqa: F401
    from cmtj.utils.procedures import PIMM_procedure, ResistanceParameters, VSD_procedure  # noqa: F401
    import cmtj.stack
    assert cmtj.stack.SeriesStack is SeriesStack


def test_unknown_submodule_is_an_import_error():
    with pytest.raises(ImportError):
        importlib.import_module("cmtj.no_such_module")
