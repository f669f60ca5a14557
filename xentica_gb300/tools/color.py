"""Colour helpers (reference ``xentica/tools/color.py``)."""
from xentica_gb300 import core
from xentica_gb300.core.expressions import DeferredExpression
from xentica_gb300.tools import xmath


def hsv2rgb(hue, saturation, value):
    """HSV (each in ``[0, 1]``) to an ``(r, g, b)`` triple.

    With a deferred ``hue`` the intermediates are float/int kernel variables;
    with plain numbers it is evaluated in Python.
    """
    if isinstance(hue, DeferredExpression):
        hue_f = core.FloatVariable()
        hue_f += hue * 6
        hue_i = core.IntegerVariable()
        hue_i += xmath.int(hue_f)
        hue_f -= hue_i
        sat = core.FloatVariable()
        sat += saturation
        val = core.FloatVariable()
        val += value
        grad_p = core.FloatVariable()
        grad_p += val * (1 - sat)
        grad_q = core.FloatVariable()
        grad_q += val * (1 - sat * hue_f)
        grad_t = core.FloatVariable()
        grad_t += val * (1 - sat * (1 - hue_f))
    else:
        hue_f = hue * 6
        hue_i = int(hue_f)
        hue_f -= hue_i
        sat = saturation
        val = value
        grad_p = val * (1 - sat)
        grad_q = val * (1 - sat * hue_f)
        grad_t = val * (1 - sat * (1 - hue_f))

    red = ((hue_i == 0) | (hue_i >= 5)) * val
    red = red + (hue_i == 1) * grad_q
    red = red + ((hue_i == 2) | (hue_i == 3)) * grad_p
    red = red + (hue_i == 4) * grad_t

    green = ((hue_i == 0) | (hue_i >= 6)) * grad_t
    green = green + ((hue_i == 1) | (hue_i == 2)) * val
    green = green + (hue_i == 3) * grad_q
    green = green + ((hue_i == 4) | (hue_i == 5)) * grad_p

    blue = ((hue_i == 0) | (hue_i == 1) | (hue_i >= 6)) * grad_p
    blue = blue + (hue_i == 2) * grad_t
    blue = blue + ((hue_i == 3) | (hue_i == 4)) * val
    blue = blue + (hue_i == 5) * grad_q

    return (red, green, blue)


class GenomeColor:
    """Ways to colour a bit-string genome."""

    @staticmethod
    def positional(genome, num_genes):
        """Blend one hue per set gene (by position), normalised to max 1."""
        red = core.FloatVariable()
        green = core.FloatVariable()
        blue = core.FloatVariable()
        for i in range(num_genes):
            d_red, d_green, d_blue = hsv2rgb(i / num_genes, 1, 1 / num_genes)
            val = (genome >> i) & 1
            red += d_red * val
            green += d_green * val
            blue += d_blue * val
        maxval = core.FloatVariable()
        maxval += xmath.max(red, green, blue)
        red /= maxval
        green /= maxval
        blue /= maxval
        return (red, green, blue)

    @staticmethod
    def modular(genome, divider):
        """Hue from ``genome % divider``."""
        return hsv2rgb(genome % divider / xmath.float(divider), 1, 1)
