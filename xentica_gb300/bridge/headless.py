"""A viewer loop without a window.

The reference drives a model from its Moire GUI: each frame applies the
pressed keys' bridge actions (``xentica/bridge/moire.py:10-34``, the
renderer's move and zoom keys, ``renderers.py:181-215``), advances the model
``speed`` generations unless it is paused (``base.py:671-728``) and draws
``render()``.  There is no graphics stack here, so :class:`HeadlessViewer`
runs the same loop and hands every frame to a sink (a callback, or PPM files
through :func:`ppm_sink`) instead of a window.
"""
import os

import numpy as np

__all__ = ['HeadlessViewer', 'ppm_sink', 'write_ppm']


class _Toggle:
    """The GUI's system-info panel (shown or hidden)."""

    def __init__(self):
        self.shown = False

    def toggle(self):
        self.shown = not self.shown


class HeadlessViewer:
    """Frame loop of a GUI front-end, without a window.

    :param model: a ``CellularAutomaton``.
    :param viewport: ``(width, height)`` of the frames (default: the first two
        lattice sides).
    """

    def __init__(self, model, viewport=None):
        self.model = model
        self.viewport = tuple(viewport or model.size[:2])
        model.set_viewport(self.viewport)
        self.running = True
        self.sysinfo = _Toggle()
        self.frames = 0

    # the GUI interface bridge actions call
    def exit_app(self):
        """Stop the loop after the current frame."""
        self.running = False

    def press(self, key):
        """Apply the bridge action bound to ``key`` (unknown keys are ignored)."""
        action = self.model.bridge.key_actions.get(key)
        if action is not None:
            action(self.model, self)

    def frame(self):
        """Advance ``speed`` generations (none while paused) and render.

        :returns: ``uint8`` array of shape ``(height, width, 3)``.
        """
        for _ in range(self.model.speed):
            self.model.step()
        self.frames += 1
        width, height = self.viewport
        return self.model.render().reshape(height, width, 3)

    def run(self, frames, keys=None, sink=None):
        """Run up to ``frames`` frames.

        :param keys: ``{frame_index: [key, ...]}`` pressed before that frame.
        :param sink: ``sink(frame_index, image)`` called with every frame.
        :returns: the number of frames drawn (fewer if a key exits).
        """
        keys = keys or {}
        drawn = 0
        for index in range(frames):
            for key in keys.get(index, ()):
                self.press(key)
            if not self.running:
                break
            image = self.frame()
            if sink is not None:
                sink(index, image)
            drawn += 1
        return drawn


def write_ppm(path, image):
    """Write an ``(height, width, 3)`` uint8 image as binary PPM."""
    image = np.ascontiguousarray(image, dtype=np.uint8)
    height, width = image.shape[:2]
    with open(path, "wb") as fh:
        fh.write(b"P6\n%d %d\n255\n" % (width, height))
        fh.write(image.tobytes())


def ppm_sink(directory, prefix="frame"):
    """A sink writing ``<directory>/<prefix>_00000.ppm`` etc."""
    os.makedirs(directory, exist_ok=True)

    def sink(index, image):
        write_ppm(os.path.join(directory, "%s_%05d.ppm" % (prefix, index)), image)
    return sink
