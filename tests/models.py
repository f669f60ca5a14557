"""Fixture models written against the xentica_gb300 API.

They restate the reference's example models (``examples/game_of_life.py``,
``examples/evolife.py``, ``examples/shifting_sands.py``) statement for
statement, because parity with the reference's golden checksums depends on the
exact operation order (the random stream of EvoLife advances once per read).
Experiments carry the same words, sizes and seed patterns.
"""
from xentica_gb300 import core, seeds
from xentica_gb300.core import color_effects
from xentica_gb300.tools import xmath
from xentica_gb300.tools.color import GenomeColor
from xentica_gb300.tools.genetics import genome_crossover
from xentica_gb300.tools.rules import LifeLike
from xentica_gb300.seeds.random import RandInt


class GameOfLife(core.CellularAutomaton):
    """Conway's Life: one bit of state, B3/S23 literal rule."""

    state = core.IntegerProperty(max_val=1)

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()

    def emit(self):
        for buf in self.buffers:
            buf.state = self.main.state

    def absorb(self):
        neighbors_alive = core.IntegerVariable()
        for i in range(len(self.buffers)):
            neighbors_alive += self.neighbors[i].buffer.state
        is_born = (8 >> neighbors_alive) & 1
        is_sustain = (12 >> neighbors_alive) & 1
        self.main.state = is_born | is_sustain & self.main.state

    @color_effects.MovingAverage
    def color(self):
        red = self.main.state * 255
        green = self.main.state * 255
        blue = self.main.state * 255
        return (red, green, blue)


class GameOfLifeStatic(GameOfLife):
    """Life surrounded by live cells."""

    class Topology(GameOfLife.Topology):
        border = core.StaticBorder(1)


class GameOfLife6D(GameOfLife):
    """Life on a 6-D von Neumann lattice."""

    class Topology(GameOfLife.Topology):
        dimensions = 6
        neighborhood = core.VonNeumannNeighborhood()


class GameOfLifeInt(GameOfLife):
    """16-bit state holding 0/1."""

    state = core.IntegerProperty(max_val=2 ** 16 - 1)


class LifelikeCA(GameOfLife):
    """Life-like rule as an interactive parameter, switched at timestep 23."""

    rule = core.Parameter(default=LifeLike.golly2int("B3/S23"), interactive=True)

    def absorb(self):
        neighbors_alive = core.IntegerVariable()
        for i in range(len(self.buffers)):
            neighbors_alive += self.neighbors[i].buffer.state
        is_born = (self.rule >> neighbors_alive) & 1
        is_sustain = (self.rule >> 9 >> neighbors_alive) & 1
        self.main.state = is_born | is_sustain & self.main.state

    def step(self):
        if self.timestep == 23:
            self.rule = LifeLike.golly2int("B3/S23")
        super().step()


class GOLExperiment(core.Experiment):
    word = "OBEY XENTICA"
    size = (640, 360, )
    zoom = 3
    pos = [0, 0]
    seed = seeds.patterns.BigBang(
        pos=(320, 180),
        size=(100, 100),
        vals={"state": seeds.random.RandInt(0, 1)},
    )


class GOLExperiment2(GOLExperiment):
    word = "XENTICA IS YOUR GODDESS"
    seed = seeds.patterns.PrimordialSoup(vals={"state": seeds.random.RandInt(0, 1)})


class DiamoebaExperiment(GOLExperiment):
    rule = LifeLike.golly2int("B35678/S5678")


class ShiftingSands(core.CellularAutomaton):
    """Directional emit: not a Life-like model (no GB300 template yet)."""

    state = core.IntegerProperty(max_val=1)

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()

    def emit(self):
        for i, buf in enumerate(self.buffers):
            if i == 0:
                buf.state = self.main.state
            else:
                buf.state = 0

    def absorb(self):
        new_val = core.IntegerVariable()
        for i in range(len(self.buffers)):
            new_val += self.neighbors[i].buffer.state
        self.main.state = new_val

    @color_effects.MovingAverage
    def color(self):
        return (self.main.state * 255, self.main.state * 255, self.main.state * 255)


class ShiftingSandsExperiment(core.Experiment):
    word = "LET IT SHIFT"
    size = (640, 360, )
    zoom = 3
    pos = [0, 0]
    seed = seeds.patterns.BigBang(pos=(320, 180), size=(100, 100),
                                  vals={"state": seeds.random.RandInt(0, 1)})


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
    seed = seeds.patterns.PrimordialSoup(vals={"state": seeds.random.RandInt(0, 1)})


class GameOfLifePlainColor(GameOfLife):
    """Plain ColorEffect (no SMOOTH_FACTOR in the render)."""

    @color_effects.ColorEffect
    def color(self):
        return (self.main.state * 255, self.main.state * 3, 7)


class GameOfLife3DStatic(GameOfLife):
    """3-D Moore neighbourhood and a static border of dead cells."""

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


MODELS = {
    "GameOfLife": GameOfLife, "GameOfLifeStatic": GameOfLifeStatic,
    "GameOfLife6D": GameOfLife6D, "GameOfLifeInt": GameOfLifeInt, "LifelikeCA": LifelikeCA,
    "GameOfLifeFade": GameOfLifeFade, "GameOfLifePlainColor": GameOfLifePlainColor,
    "GameOfLife3DStatic": GameOfLife3DStatic, "LifelikeFixed": LifelikeFixed,
}
EXPERIMENTS = {
    "GOLExperiment": GOLExperiment, "GOLExperiment2": GOLExperiment2,
    "DiamoebaExperiment": DiamoebaExperiment, "FadeExperiment": FadeExperiment,
}


def from_job(job):
    """Our model and experiment for a golden-fixture job (see make_golden.py)."""
    model = MODELS[job["model"].rsplit(":", 1)[1]]
    exp = EXPERIMENTS[job["experiment"].rsplit(":", 1)[1]]
    overrides = dict(job.get("exp_overrides", {}))
    if "size" in overrides:
        overrides["size"] = tuple(overrides["size"])
    if "pos" in overrides:
        overrides["pos"] = list(overrides["pos"])
    if overrides:
        exp = type("GoldenExperiment", (exp,), overrides)
    return model, exp
