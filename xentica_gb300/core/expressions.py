"""Deferred expressions: operator overloading that records typed IR.

Mirrors the reference's ``DeferredExpression`` / ``PatternExpression``
(``xentica/core/expressions.py:9-204``): the same operators are overloaded and
``str()`` gives the same parenthesised C text, but every result also carries
an IR node (:mod:`xentica_gb300.core.ir`) so the translator can analyse the
model instead of pasting text into a kernel.

Allowed binary ops: ``+ - * / % >> << & ^ | < <= == != > >=``.
Allowed unary ops: ``- + ~ abs``.
Allowed augmented assigns: ``+= -= *= /= %= <<= >>= &= ^= |=`` (only on
variables and properties, never on a bare expression).
"""
import operator

from xentica_gb300.core import ir
from xentica_gb300.core.exceptions import XenticaException

__all__ = ['DeferredExpression', 'PatternExpression']

_BINARY = (
    ('+', 'add'), ('-', 'sub'), ('*', 'mul'), ('/', 'truediv'), ('%', 'mod'),
    ('>>', 'rshift'), ('<<', 'lshift'), ('&', 'and'), ('^', 'xor'),
    ('|', 'or'), ('<', 'lt'), ('<=', 'le'), ('==', 'eq'), ('!=', 'ne'),
    ('>', 'gt'), ('>=', 'ge'),
)
_UNARY = (('-', 'neg'), ('+', 'pos'), ('abs', 'abs'), ('~', 'invert'))
_REFLECT = {'<': '>', '<=': '>=', '>': '<', '>=': '<=', '==': '==', '!=': '!='}


class DeferredExpression:
    """An expression whose value is only known inside the kernel.

    ``code`` is its C text; :meth:`ir_node` its typed IR.
    """

    def __init__(self, code='', node=None):
        self.code = code
        self._node = node

    def ir_node(self):
        """The IR node this expression stands for."""
        node = object.__getattribute__(self, "_node")
        if node is None:
            return ir.Raw(str(self))
        return node

    __hash__ = object.__hash__

    def __str__(self):
        return self.code


def _make_binary(c_op):
    def direct(self_var, value):
        code = "(%s %s %s)" % (self_var, c_op, value)
        return DeferredExpression(code, ir.Bin(c_op, ir.to_node(self_var), ir.to_node(value), code))

    def reflected(self_var, value):
        code = "(%s %s %s)" % (value, c_op, self_var)
        return DeferredExpression(code, ir.Bin(c_op, ir.to_node(value), ir.to_node(self_var), code))

    def augmented(self_var, value):
        if type(self_var).__name__ == "DeferredExpression":
            raise XenticaException("Can't assign to DeferredExpression")
        self_var.declare_once()
        name = self_var.var_name
        code = "%s %s= %s;\n" % (name, c_op, value)
        self_var.bsca._record(ir.Stmt("aug", var=name, aug=c_op, expr=ir.to_node(value)), code)
        return self_var
    return direct, reflected, augmented


def _make_unary(c_op):
    def unary(self_var):
        code = "(%s(%s))" % (c_op, self_var)
        return DeferredExpression(code, ir.Un(c_op, ir.to_node(self_var), code))
    return unary


for _c_op, _name in _BINARY:
    _d, _r, _a = _make_binary(_c_op)
    setattr(DeferredExpression, "__%s__" % _name, _d)
    setattr(DeferredExpression, "__i%s__" % _name, _a)
    if _name in ('lt', 'le', 'gt', 'ge', 'eq', 'ne'):
        continue
    setattr(DeferredExpression, "__r%s__" % _name, _r)
for _c_op, _name in _UNARY:
    setattr(DeferredExpression, "__%s__" % _name, _make_unary(_c_op))


class PatternExpression:
    """Seed-time arithmetic over random values (``expressions.py:123-204``).

    Operators build a small expression tree; reading it as a descriptor
    (``__get__``) draws the random operands and applies the operators.
    """

    def __init__(self, arg1=None, arg2=None, cur_oper=None):
        self.arg1 = arg1
        self.arg2 = arg2
        self.cur_oper = cur_oper

    def __get__(self, instance, owner):
        res1 = self.arg1.__get__(instance, owner) \
            if isinstance(self.arg1, PatternExpression) else self.arg1
        res2 = self.arg2.__get__(instance, owner) \
            if isinstance(self.arg2, PatternExpression) else self.arg2
        oper = getattr(operator, "__%s__" % self.cur_oper)
        if self.arg2 is None:
            return oper(res1)
        return oper(res1, res2)


def _pattern_binary(op_name):
    def direct(self_var, value):
        return PatternExpression(self_var, value, op_name)

    def reflected(self_var, value):
        return PatternExpression(value, self_var, op_name)
    return direct, reflected


for _name in ('add', 'sub', 'mul', 'truediv', 'mod', 'rshift', 'lshift', 'and', 'xor', 'or'):
    _d, _r = _pattern_binary(_name)
    setattr(PatternExpression, "__%s__" % _name, _d)
    setattr(PatternExpression, "__r%s__" % _name, _r)
for _name in ('neg', 'pos', 'invert'):
    setattr(PatternExpression, "__%s__" % _name,
            (lambda op_name: lambda self_var: PatternExpression(self_var, None, op_name))(_name))
