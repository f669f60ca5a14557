"""Renderers (reference ``xentica/core/renderers.py:32-270``).

``RendererPlain`` maps viewport pixel ``i`` to lattice coordinates
``x = (int)((float)(i % width) / (float)zoom) + pos[0]`` (same for ``y`` with
``i / width`` and ``pos[1]``), wraps them onto the board, averages the colours
of all cells along the non-projected axes and divides by ``SMOOTH_FACTOR``
when the model's colour effect defines one.  The GB300 render kernel computes
exactly that; this class keeps the API (projection axes, bridge actions,
kernel-argument values).
"""
import abc

import numpy as np

from xentica_gb300.core.mixins import BscaDetectorMixin

__all__ = ['Renderer', 'RendererPlain', ]


class Renderer(BscaDetectorMixin):
    """Base class of renderers."""

    def __init__(self):
        self.args = [
            ("int3", "*col"),
            ("int", "*img"),
        ]

    def get_args_vals(self, bsca):
        """Values of ``self.args`` for the given model."""
        return [bsca.gpu.arrays.colors, bsca.gpu.arrays.img]

    @abc.abstractmethod
    def render_code(self):
        """Text of the render kernel body (empty for the base class)."""
        return ""

    def setup_actions(self, bridge):
        """Add renderer-specific actions to ``bridge.key_actions``."""


class RendererPlain(Renderer):
    """Renders the board as a 2-D plane, projecting over ``projection_axes``."""

    def __init__(self, projection_axes=None):
        super().__init__()
        self.args += [
            ("int", "zoom"),
            ("int", "dx"),
            ("int", "dy"),
            ("int", "width"),
        ]
        self.projection_axes = projection_axes
        if self.projection_axes is None:
            self.projection_axes = (0, 1)

    def get_args_vals(self, bsca):
        vals = super().get_args_vals(bsca)
        vals += [np.int32(bsca.zoom), np.int32(bsca.pos[0]), np.int32(bsca.pos[1]),
                 np.int32(bsca.width)]
        return vals

    def setup_actions(self, bridge):
        bridge.key_actions.update({
            "up": self.move(0, 1),
            "down": self.move(0, -1),
            "left": self.move(-1, 0),
            "right": self.move(1, 0),
            "=": self.zoom(1),
            "-": self.zoom(-1),
        })

    @staticmethod
    def move(delta_x, delta_y):
        """Bridge action moving the view by ``(delta_x, delta_y)``."""
        def func(model, _gui):
            model.renderer.apply_move(model, delta_x, delta_y)
        return func

    @staticmethod
    def zoom(dzoom):
        """Bridge action changing the zoom by ``dzoom``."""
        def func(model, _gui):
            model.renderer.apply_zoom(model, dzoom)
        return func

    @staticmethod
    def apply_move(bsca, *args):
        """Shift ``bsca.pos`` by the deltas, wrapping around the board."""
        for i, delta in enumerate(args):
            bsca.pos[i] = (bsca.pos[i] + delta) % bsca.size[i]

    @staticmethod
    def apply_zoom(bsca, dval):
        """Change ``bsca.zoom`` by ``dval`` (minimum 1)."""
        bsca.zoom = max(1, (bsca.zoom + dval))

    def render_code(self):
        """Description of the render kernel the model runs."""
        return "xk_render projection_axes=%s" % (tuple(self.projection_axes),)
