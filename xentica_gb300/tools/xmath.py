"""Math helpers for model code (reference ``xentica/tools/xmath.py:6-43``).

Each helper returns a :class:`DeferredExpression` with the same C text as the
reference and the matching IR node.
"""
from xentica_gb300.core import ir
from xentica_gb300.core.expressions import DeferredExpression


def _fold(args, cmp_op):
    text = str(args[0])
    node = ir.to_node(args[0])
    for arg in args[1:]:
        a_text, b_text = text, str(arg)
        text = "(({a}) {op} ({b})) ? ({a}) : ({b})".format(a=a_text, b=b_text, op=cmp_op)
        b_node = ir.to_node(arg)
        node = ir.Cond(ir.Bin(cmp_op, node, b_node), node, b_node, "(%s)" % text)
    return DeferredExpression("(%s)" % text, ir.Cond(node.c, node.a, node.b, "(%s)" % text)
                              if isinstance(node, ir.Cond) else node)


class Xmath:
    """Static collection of math functions usable in ``emit/absorb/color``."""

    @staticmethod
    def min(*args):
        """Minimum of the arguments (nested conditional expressions)."""
        return _fold(args, "<")

    @staticmethod
    def max(*args):
        """Maximum of the arguments (nested conditional expressions)."""
        return _fold(args, ">")

    @staticmethod
    def float(val):
        """Cast to ``float``."""
        text = "((float) (%s))" % val
        return DeferredExpression(text, ir.Cast(ir.F32, ir.to_node(val), text))

    @staticmethod
    def int(val):
        """Cast to ``unsigned int``."""
        text = "((unsigned int) (%s))" % val
        return DeferredExpression(text, ir.Cast(ir.U32, ir.to_node(val), text))

    @staticmethod
    def popc(val):
        """Number of set bits of a 32-bit integer."""
        text = "(__popc(%s))" % val
        return DeferredExpression(text, ir.Call("__popc", [ir.to_node(val)], ir.I32, text))

    @staticmethod
    def exp(val):
        """Exponent (not supported by the GB300 templates)."""
        text = "(exp(%s))" % val
        return DeferredExpression(text, ir.Call("exp", [ir.to_node(val)], ir.F64, text))
