"""Model meta-parameters (reference ``xentica/core/parameters.py:64-145``).

Non-interactive
    constant for a run; read as a plain Python value while the model is traced,
    so it is folded into the traced program.

Interactive
    may change between steps; read as a symbolic kernel argument, and its
    current value is passed to the kernel at every step.
"""
import numpy as np

from xentica_gb300.core import ir
from xentica_gb300.core.variables import Constant
from xentica_gb300.core.mixins import BscaDetectorMixin
from xentica_gb300.core.expressions import DeferredExpression

__all__ = ['Parameter']

_CTYPES = {int: 'int', float: 'float', bool: 'bool'}
_DTYPES = {int: np.int32, float: np.float32, bool: bool}


class Parameter(BscaDetectorMixin):
    """A model meta-parameter.

    :param default: value used when the experiment does not set one.
    :param interactive: ``True`` if it can change at runtime.
    """

    def __init__(self, default=0, interactive=False):
        self._value = default
        self._default = default
        self._interactive = interactive
        self._declared = False
        self._name = "param" + str(id(self))

    @property
    def value(self):
        """Current value."""
        return self._value

    @property
    def default(self):
        """Value the parameter was declared with."""
        return self._default

    @property
    def interactive(self):
        """Whether the value is a runtime kernel argument."""
        return self._interactive

    @property
    def name(self):
        """Parameter's name."""
        return self._name

    @name.setter
    def name(self, val):
        self._name = val

    @property
    def ctype(self):
        """C type of the kernel argument."""
        return _CTYPES.get(type(self._value), 'int32')

    @property
    def dtype(self):
        """NumPy type of the kernel argument."""
        return _DTYPES.get(type(self._value), np.int32)

    def _declare_interactive(self):
        if self.bsca.is_parameter(self.name):
            return
        self.bsca.define_parameter(self)

    def _declare_once(self):
        if self._interactive:
            self._declare_interactive()
            return
        if self._declared:
            return
        self._declared = True
        self.bsca.define_constant(Constant(self.name, self._value))

    def __get__(self, obj, objtype):
        self._declare_once()
        if self._interactive:
            return DeferredExpression(self._name, ir.ParamRef(self._name, ir.ctype_of(self.ctype)))
        return self._value

    def __set__(self, obj, value):
        self._value = value
