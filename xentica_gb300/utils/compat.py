"""Saved states that this package and the reference read alike.

``CellularAutomaton.save`` of the reference pickles ``{"cells", "colors",
"random"}`` (``xentica/core/base.py:755-771``), where ``random`` is its
``xentica.seeds.random.LocalRandom``.  :func:`dump_state` writes the same
layout with the ``random`` entry under the reference's class path, so the
reference can load it; :func:`load_state` reads both its pickles and the
reference's, mapping the reference's ``xentica.*`` classes onto this
package's.  Only ``standard`` and ``numpy`` of the random holder are used by
either side's ``load``.
"""
import pickle
import sys
import types

__all__ = ['dump_state', 'load_state']

_REF_PACKAGE = "xentica"
_REF_MODULE = "xentica.seeds.random"


class _RefLocalRandom:
    """Pickled as the reference's ``LocalRandom`` (same two attributes)."""


_RefLocalRandom.__module__ = _REF_MODULE
_RefLocalRandom.__name__ = "LocalRandom"
_RefLocalRandom.__qualname__ = "LocalRandom"


def _holder(rng):
    ref = sys.modules.get(_REF_MODULE)
    cls = getattr(ref, "LocalRandom", None) if ref is not None else None
    cls = cls or _RefLocalRandom
    obj = cls.__new__(cls)
    obj.standard = rng.standard
    obj.numpy = rng.numpy
    return obj


def dump_state(state, fh):
    """Pickle ``state`` (cells, colors, random) in the reference's layout."""
    state = dict(state, random=_holder(state["random"]))
    if isinstance(state["random"], _RefLocalRandom):
        # pickle checks that the class is importable under its path: make the
        # path resolve to the stand-in while dumping, without touching a
        # module that is really there
        added = []
        for name in ("xentica", "xentica.seeds", _REF_MODULE):
            if name not in sys.modules:
                sys.modules[name] = types.ModuleType(name)
                added.append(name)
        sys.modules[_REF_MODULE].LocalRandom = _RefLocalRandom
        try:
            pickle.dump(state, fh)
        finally:
            for name in added:
                del sys.modules[name]
    else:
        pickle.dump(state, fh)


class _Unpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if module == _REF_PACKAGE or module.startswith(_REF_PACKAGE + "."):
            module = "xentica_gb300" + module[len(_REF_PACKAGE):]
        return super().find_class(module, name)


def load_state(fh):
    """Unpickle a state saved by this package or by the reference."""
    return _Unpickler(fh).load()
