"""Colour effects: decorators for a model's ``color()`` method.

Reference ``xentica/core/color_effects.py:36-130``.  ``color()`` returns an
``(r, g, b)`` triple of expressions of the new state; the effect decides how it
is combined with the cell's previous colour:

``ColorEffect``
    stores the triple as is.
``MovingAverage``
    multiplies by ``smooth_factor`` and limits the change per step to
    ``+fade_in`` / ``-fade_out`` (experiment attributes, default 255, 255, 1).

The traced colour becomes one IR ``color`` statement that the kernels
implement; a subclass with its own C ``effect`` text is not supported by the
GB300 templates.
"""
from xentica_gb300.core import ir
from xentica_gb300.core.variables import Constant
from xentica_gb300.core.mixins import BscaDetectorMixin

__all__ = ['ColorEffect', 'MovingAverage', ]


class ColorEffect(BscaDetectorMixin):
    """Plain colour: the computed RGB is stored directly."""

    #: effect kind recorded in the traced program
    kind = "plain"

    def __init__(self, func):
        self.func = func
        self.effect = ""

    def _effect_info(self):
        kind = self.kind
        if kind == "plain" and self.effect.strip():
            kind = "custom"
        return {"kind": kind}

    def __call__(self):
        bsca = self.bsca
        red, green, blue = self.func(bsca)
        code = """
            int new_r = %s;
            int new_g = %s;
            int new_b = %s;
            %s
            col[i] = make_int3(new_r, new_g, new_b);
        """ % (red, green, blue, self.effect)
        info = self._effect_info()
        info["rgb"] = [ir.to_node(red), ir.to_node(green), ir.to_node(blue)]
        bsca._record(ir.Stmt("color", extra=info), code)


class MovingAverage(ColorEffect):
    """Per-channel moving average with bounded fade in/out."""

    kind = "moving_average"

    def __call__(self):
        bsca = self.bsca
        if not hasattr(bsca, "fade_in"):
            bsca.fade_in = 255
        if not hasattr(bsca, "fade_out"):
            bsca.fade_out = 255
        if not hasattr(bsca, "smooth_factor"):
            bsca.smooth_factor = 1
        bsca.define_constant(Constant("FADE_IN", bsca.fade_in))
        bsca.define_constant(Constant("FADE_OUT", bsca.fade_out))
        bsca.define_constant(Constant("SMOOTH_FACTOR", bsca.smooth_factor))
        self.effect = """
            new_r *= SMOOTH_FACTOR;
            new_g *= SMOOTH_FACTOR;
            new_b *= SMOOTH_FACTOR;
            int3 old_col = col[i];
            new_r = max(min(new_r, old_col.x + FADE_IN),
                        old_col.x - FADE_OUT);
            new_g = max(min(new_g, old_col.y + FADE_IN),
                        old_col.y - FADE_OUT);
            new_b = max(min(new_b, old_col.z + FADE_IN),
                        old_col.z - FADE_OUT);
        """
        return super().__call__()

    def _effect_info(self):
        bsca = self.bsca
        return {"kind": "moving_average", "fade_in": int(bsca.fade_in),
                "fade_out": int(bsca.fade_out), "smooth": int(bsca.smooth_factor)}
