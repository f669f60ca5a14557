"""Models written against the reference's public API for the oracle harness.

Test fixtures: executed by ``oracle/ref_harness.py`` with the reference package
on ``sys.path`` (never by the product).  Each exercises a reference code path
its own examples do not reach directly; ``tests/models.py`` has the same
models written against xentica_gb300.
"""
from xentica import core
from xentica.core import color_effects
from examples.game_of_life import GameOfLife


class GameOfLifeInt(GameOfLife):
    """16-bit state variant used by the reference's cell-width test."""
    state = core.IntegerProperty(max_val=2 ** 16 - 1)


class GameOfLifeFade(GameOfLife):
    """History-dependent MovingAverage colour (small fades, smooth factor 2)."""

    @color_effects.MovingAverage
    def color(self):
        red = self.main.state * 200
        green = self.main.state * 100 + 10
        blue = 250 - self.main.state * 250
        return (red, green, blue)


class FadeExperiment(core.Experiment):
    word = "FADE AWAY"
    size = (50, 30)
    zoom = 1
    pos = [0, 0]
    fade_in = 40
    fade_out = 15
    smooth_factor = 2
    from xentica import seeds as _seeds
    seed = _seeds.patterns.PrimordialSoup(vals={"state": _seeds.random.RandInt(0, 1)})


class GameOfLifePlainColor(GameOfLife):
    """Plain ColorEffect (no SMOOTH_FACTOR in the render)."""

    @color_effects.ColorEffect
    def color(self):
        return (self.main.state * 255, self.main.state * 3, 7)


class GameOfLife3DStatic(GameOfLife):
    """3-D Moore neighbourhood (with the reference's d != 2 delta list) and a
    static border of dead cells."""

    class Topology(GameOfLife.Topology):
        dimensions = 3
        border = core.StaticBorder(0)


class LifelikeFixed(GameOfLife):
    """Life-like rule from an interactive parameter, never switched."""

    rule = core.Parameter(default=6152, interactive=True)

    def absorb(self):
        neighbors_alive = core.IntegerVariable()
        for i in range(len(self.buffers)):
            neighbors_alive += self.neighbors[i].buffer.state
        is_born = (self.rule >> neighbors_alive) & 1
        is_sustain = (self.rule >> 9 >> neighbors_alive) & 1
        self.main.state = is_born | is_sustain & self.main.state
