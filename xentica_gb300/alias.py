"""Run programs written for ``xentica`` unchanged.

:func:`install` makes ``import xentica`` (and every ``xentica.*`` submodule)
resolve to this package, so a model file written against the reference --
``from xentica import core, seeds``, ``from xentica.tools.rules import
LifeLike``, ... -- runs on the GB300 kernels without editing a line::

    import xentica_gb300.alias
    xentica_gb300.alias.install()
    import my_reference_model          # its "from xentica import core" is ours
"""
import importlib
import importlib.abc
import importlib.util
import sys

__all__ = ['install', 'uninstall']

_PREFIX = "xentica"
_TARGET = "xentica_gb300"


class _Loader(importlib.abc.Loader):
    def __init__(self, target):
        self.target = target

    def create_module(self, spec):
        return importlib.import_module(self.target)

    def exec_module(self, module):
        """The target module is already executed."""


class _Finder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path=None, target=None):
        if fullname != _PREFIX and not fullname.startswith(_PREFIX + "."):
            return None
        real = _TARGET + fullname[len(_PREFIX):]
        if importlib.util.find_spec(real) is None:
            return None
        return importlib.util.spec_from_loader(fullname, _Loader(real))


_FINDER = _Finder()


def install():
    """Make ``xentica.*`` imports load ``xentica_gb300.*`` (first in the import
    path, ahead of any installed reference package)."""
    if _FINDER not in sys.meta_path:
        sys.meta_path.insert(0, _FINDER)


def uninstall():
    """Undo :func:`install` (modules already imported stay imported)."""
    if _FINDER in sys.meta_path:
        sys.meta_path.remove(_FINDER)
