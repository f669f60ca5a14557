"""Mixins shared by the core classes (reference ``xentica/core/mixins.py``).

``BscaDetectorMixin.bsca`` finds the model a DSL object belongs to.  While a
model is being traced the translator publishes itself on a module-level stack,
so the lookup is a list access; outside tracing it falls back to the
reference's behaviour of scanning the caller frames for a
``CellularAutomaton`` instance (``mixins.py:16-40``).
"""
import inspect
import os

from xentica_gb300.core.exceptions import XenticaException

__all__ = ['BscaDetectorMixin', 'DimensionsMixin', ]

#: models currently being traced (innermost last)
ACTIVE = []

_CORE_DIR = os.path.dirname(os.path.abspath(__file__))
# modules whose frames are DSL machinery, never the code that names a variable
_MACHINERY = {os.path.join(_CORE_DIR, name + ".py") for name in (
    "base", "expressions", "variables", "properties", "parameters", "mixins",
    "color_effects", "renderers", "ir")}


def _is_core_frame(frame):
    return os.path.abspath(frame.f_code.co_filename) in _MACHINERY


class BscaDetectorMixin:
    """Adds ``bsca``: the ``CellularAutomaton`` instance holding this object."""

    @property
    def bsca(self):
        """The model being traced, else the first one found up the stack."""
        if ACTIVE:
            return ACTIVE[-1]
        from xentica_gb300.core.base import CellularAutomaton
        frame = inspect.currentframe()
        while frame is not None:
            for local in frame.f_locals.values():
                if hasattr(local, "__get__"):
                    continue
                if isinstance(local, CellularAutomaton):
                    return local
            frame = frame.f_back
        raise XenticaException("BSCA not detected")

    @property
    def _holder_frame(self):
        """First frame outside the core package: where user code runs."""
        frame = inspect.currentframe().f_back
        while frame is not None and _is_core_frame(frame):
            frame = frame.f_back
        return frame


class DimensionsMixin:
    """Adds a validated ``dimensions`` property (``mixins.py:59-101``)."""

    #: dimensionalities the class supports; set it in every subclass
    supported_dimensions = []

    def __init__(self):
        self._dimensions = None

    def allowed_dimension(self, num_dim):
        """Test if ``num_dim`` dimensions are supported."""
        return num_dim in self.supported_dimensions

    @property
    def dimensions(self):
        """Number of dimensions."""
        return self._dimensions

    @dimensions.setter
    def dimensions(self, num_dim):
        if not self.allowed_dimension(num_dim):
            msg = "%d-D %s is not supported." % (num_dim, self.__class__.__name__)
            raise XenticaException(msg)
        self._dimensions = num_dim
