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


import functools as _functools
import operator as _operator

from xentica import seeds as _seeds
from xentica.core.expressions import PatternExpression
from xentica.tools import xmath


class RandPoisson(PatternExpression):
    """Poisson(lam) per cell from the pattern's NumPy stream (the seed
    expression xentica_gb300.seeds.random.RandPoisson adds)."""

    def __init__(self, lam):
        super().__init__()
        self.lam = lam

    def __get__(self, instance, owner):
        n = _functools.reduce(_operator.mul, instance.size)
        return instance.random.numpy.poisson(self.lam, n).astype("int64")


WALL = 2 ** 32 - 1


class MassTransfer(core.CellularAutomaton):
    """Mass-conserving sand transfer on a 3-D von Neumann lattice whose
    border is a wall: every cell sends mass // 7 to each neighbour that is
    not a wall and absorbs what its neighbours send."""

    mass = core.IntegerProperty(max_val=2 ** 32 - 2)

    class Topology:
        dimensions = 3
        lattice = core.OrthogonalLattice()
        neighborhood = core.VonNeumannNeighborhood()
        border = core.StaticBorder(WALL)

    def emit(self):
        share = core.IntegerVariable()
        share += self.main.mass / 7
        for i in range(len(self.buffers)):
            self.buffers[i].mass = share * (self.neighbors[i].main.mass != WALL)

    def absorb(self):
        total = core.IntegerVariable()
        total += self.main.mass
        for i in range(len(self.buffers)):
            total -= self.buffers[i].mass
        for i in range(len(self.buffers)):
            incoming = self.neighbors[i].buffer.mass
            total += incoming * (incoming != WALL)
        self.main.mass = total

    @color_effects.ColorEffect
    def color(self):
        v = xmath.min(self.main.mass * 32, 255)
        return (v, v, v)


class MassExperiment(core.Experiment):
    word = "SAND PILES 3D"
    size = (24, 20, 12)
    zoom = 1
    pos = [0, 0]
    seed = _seeds.patterns.PrimordialSoup(vals={"mass": RandPoisson(4)})


from examples.shifting_sands import ShiftingSands as _ShiftingSands  # noqa: E402


class ShiftingSandsStatic(_ShiftingSands):
    """ShiftingSands with a static border of dead cells: edge cells lose the
    state that would wrap in."""

    class Topology(_ShiftingSands.Topology):
        border = core.StaticBorder(0)


class ShiftingSands3D(_ShiftingSands):
    """ShiftingSands on a 3-D von Neumann torus (emit into buffer 2)."""

    class Topology(_ShiftingSands.Topology):
        dimensions = 3
        neighborhood = core.VonNeumannNeighborhood()

    def emit(self):
        for i, buf in enumerate(self.buffers):
            if i == 2:
                buf.state = self.main.state
            else:
                buf.state = 0


class ShiftingSandsFade(_ShiftingSands):
    """ShiftingSands with history-dependent colours (FadeExperiment's fades)."""

    @color_effects.MovingAverage
    def color(self):
        red = self.main.state * 200
        green = self.main.state * 100 + 10
        blue = 250 - self.main.state * 250
        return (red, green, blue)
