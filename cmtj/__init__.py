"""`import cmtj`: the reference's import name (cmtj/__init__.py:10-18,
python/cmtj.cpp:35) for cmtj_gb300.

`cmtj` holds every name of cmtj_gb300 (the names the reference's `_cmtj`
exports), and `cmtj.<sub>` for any submodule path resolves to
`cmtj_gb300.<sub>`: cmtj.stack, cmtj.reservoir, cmtj.noise,
cmtj.constants, cmtj.utils, cmtj.utils.procedures, cmtj.utils.resistance,
cmtj.utils.filters, cmtj.utils.linear, cmtj.utils.parallel.  The modules are
the same objects under both names, imported on first use.
"""
import importlib as _importlib
import importlib.abc as _abc
import importlib.util as _util
import sys as _sys

import cmtj_gb300 as _impl
from cmtj_gb300 import *  # noqa: F401,F403
from cmtj_gb300 import __all__, __version__  # noqa: F401

_PREFIX = __name__ + "."
_TARGET = _impl.__name__ + "."


class _SubmoduleAlias(_abc.MetaPathFinder, _abc.Loader):
    """Resolves cmtj.<sub> to the module cmtj_gb300.<sub>.  The import
    machinery stamps the alias spec on the module it loads; exec_module puts
    the module's own spec back, so its relative imports and reloads keep
    working under its real name."""

    def __init__(self):
        self._own_specs = {}

    def find_spec(self, fullname, path=None, target=None):
        if not fullname.startswith(_PREFIX):
            return None
        if _util.find_spec(_TARGET + fullname[len(_PREFIX):]) is None:
            return None
        return _util.spec_from_loader(fullname, self, is_package=True)

    def create_module(self, spec):
        module = _importlib.import_module(_TARGET + spec.name[len(_PREFIX):])
        self._own_specs[spec.name] = module.__spec__
        return module

    def exec_module(self, module):
        own = self._own_specs.pop(module.__spec__.name, None)
        if own is not None:
            module.__spec__ = own


if not any(isinstance(f, _SubmoduleAlias) for f in _sys.meta_path):
    _sys.meta_path.insert(0, _SubmoduleAlias())


def __getattr__(name):
    # cmtj.stack, cmtj.noise, ... as attributes, imported on first use
    try:
        return _importlib.import_module(_PREFIX + name)
    except ImportError:
        raise AttributeError(name) from None
