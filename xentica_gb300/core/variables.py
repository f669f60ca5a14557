"""Kernel-local variables and ``#define`` constants.

Same API as the reference (``xentica/core/variables.py:38-173``)::

    myvar = core.IntegerVariable()
    myvar += self.neighbors[i].buffer.state
    self.main.state = myvar & 1

A variable is declared (with its initial value) on first use.  Its C name is
the Python name it is bound to in the code that uses it, else the name of the
model class attribute holding it, else ``name=`` (default ``"var"``).
"""
from xentica_gb300.core import ir
from xentica_gb300.core.mixins import BscaDetectorMixin
from xentica_gb300.core.exceptions import XenticaException
from xentica_gb300.core.expressions import DeferredExpression

__all__ = ['Constant', 'Variable', 'IntegerVariable', 'FloatVariable', ]

_BAD_NAMES = ("self_var", "obj", "cls")


class Constant(BscaDetectorMixin):
    """A named constant (a ``#define`` in the reference's kernels).

    Register it with ``self.bsca.define_constant(Constant("NAME", value))``.
    """

    def __init__(self, name, value):
        self._name = name
        self._value = value
        self.base_class = Constant

    def get_define_code(self):
        """``#define`` line for this constant."""
        return "#define %s %s\n" % (self._name, str(self._value))

    @property
    def name(self):
        """Constant's name."""
        return self._name

    @property
    def value(self):
        """Constant's value."""
        return self._value


class Variable(DeferredExpression, BscaDetectorMixin):
    """Base class of kernel-local variables.

    :param val: initial value (mandatory).
    :param name: fallback C name.
    """

    var_type = "int"

    def __init__(self, val=None, name="var"):
        super().__init__()
        self.fallback_name = name
        self.base_class = Variable
        if val is None:
            raise XenticaException("Variable should have an initial value.")
        node = ir.parse_literal(val) if isinstance(val, str) else ir.to_node(val)
        self._init_val = DeferredExpression(str(val), node)

    @property
    def var_name(self):
        """C name of the variable (resolved once, on first use)."""
        cached = self.__dict__.get("_var_name")
        if cached is not None:
            return cached
        name = self._resolve_name()
        self.__dict__["_var_name"] = name
        return name

    def _resolve_name(self):
        from xentica_gb300.core.base import CellularAutomaton
        frame = self._holder_frame
        model = None
        if frame is not None:
            for key, var in frame.f_locals.items():
                if isinstance(var, CellularAutomaton):
                    model = var
                if var is self and key not in _BAD_NAMES and key.isidentifier():
                    return key
        if model is not None and self.fallback_name == "var":
            for key, var in model.__class__.__dict__.items():
                if var is self and key not in _BAD_NAMES:
                    return key
        return self.fallback_name

    @property
    def ctype(self):
        """IR type of the variable."""
        return ir.ctype_of(self.var_type)

    def ir_node(self):
        return ir.VarRef(self.var_name, self.ctype)

    def declare_once(self):
        """Declare the variable with its initial value, once per kernel."""
        bsca = self.bsca
        if not bsca.is_declared(self):
            name = self.var_name
            code = "%s %s = %s;\n" % (self.var_type, name, self._init_val)
            bsca._record(ir.Stmt("decl", var=name, ctype=self.ctype,
                              expr=self._init_val.ir_node()), code)
            bsca.declare(self)
            setattr(bsca, name, self)

    def __str__(self):
        return self.var_name

    def __get__(self, obj, objtype):
        self.declare_once()
        return self

    def __set__(self, obj, value):
        self.declare_once()
        if str(self.var_name) == str(value):
            return
        code = "%s = %s;\n" % (self.var_name, value)
        self.bsca._record(ir.Stmt("assign", var=self.var_name, expr=ir.to_node(value)), code)

    @property
    def code(self):
        """The variable's name as C code."""
        return self.var_name

    @code.setter
    def code(self, val):
        """The code of a variable is its name; assignments are ignored."""


class IntegerVariable(Variable):
    """A variable holding an ``unsigned int``."""

    var_type = "unsigned int"

    def __init__(self, val="0", **kwargs):
        super().__init__(val, **kwargs)


class FloatVariable(Variable):
    """A variable holding a 32-bit ``float``."""

    var_type = "float"

    def __init__(self, val="0.0f", **kwargs):
        super().__init__(val, **kwargs)
