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


class GameOfLifeColor(GameOfLife):
    """Life whose live cells carry three colour channels, each the sum over
    the neighbours of (channel + 1) (examples/game_of_life.py:112-159)."""

    state = core.IntegerProperty(max_val=1)
    red = core.IntegerProperty(max_val=255)
    green = core.IntegerProperty(max_val=255)
    blue = core.IntegerProperty(max_val=255)

    def emit(self):
        for buf in self.buffers:
            buf.state = self.main.state
            buf.red = self.main.red
            buf.green = self.main.green
            buf.blue = self.main.blue

    def absorb(self):
        GameOfLife.absorb(self)
        red_sum = core.IntegerVariable()
        green_sum = core.IntegerVariable()
        blue_sum = core.IntegerVariable()
        for i in range(len(self.buffers)):
            red_sum += self.neighbors[i].buffer.red + 1
            green_sum += self.neighbors[i].buffer.green + 1
            blue_sum += self.neighbors[i].buffer.blue + 1
        self.main.red = red_sum * self.main.state
        self.main.green = green_sum * self.main.state
        self.main.blue = blue_sum * self.main.state

    @color_effects.MovingAverage
    def color(self):
        red = self.main.state * self.main.red
        green = self.main.state * self.main.green
        blue = self.main.state * self.main.blue
        return (red, green, blue)


class GameOfLifeColorStatic(GameOfLifeColor):
    """The same on a lattice surrounded by one fixed container value (a live
    cell with colour channels 1, 2 and 3)."""

    class Topology(GameOfLife.Topology):
        border = core.StaticBorder(1 | 1 << 1 | 2 << 9 | 3 << 17)


class GameOfLifeColorPlus2(GameOfLifeColor):
    """Not the colour-Life program (each neighbour adds channel + 2): runs on
    the interpreter."""

    def absorb(self):
        GameOfLife.absorb(self)
        red_sum = core.IntegerVariable()
        green_sum = core.IntegerVariable()
        blue_sum = core.IntegerVariable()
        for i in range(len(self.buffers)):
            red_sum += self.neighbors[i].buffer.red + 2
            green_sum += self.neighbors[i].buffer.green + 1
            blue_sum += self.neighbors[i].buffer.blue + 1
        self.main.red = red_sum * self.main.state
        self.main.green = green_sum * self.main.state
        self.main.blue = blue_sum * self.main.state


class NoiseTV(core.CellularAutomaton):
    """Per-cell pseudo-random noise (examples/noisetv.py:13-31)."""

    rng = core.RandomProperty()

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()

    def emit(self):
        """Nothing is sent."""

    def absorb(self):
        return self.main.rng

    @color_effects.MovingAverage
    def color(self):
        val = xmath.int(self.main.rng.uniform * 255)
        return (val, val, val)


class NoiseTV3D(NoiseTV):
    """The same noise on a 3-D von Neumann lattice with a static border."""

    class Topology:
        dimensions = 3
        lattice = core.OrthogonalLattice()
        neighborhood = core.VonNeumannNeighborhood()
        border = core.StaticBorder(7)


class GraviCowboys(core.CellularAutomaton):
    """Energy units rolling down a gravity field that the energy itself
    raises (examples/gravicowboys.py:20-71)."""

    energy = core.IntegerProperty(max_val=2 ** 12 - 1)
    new_energy = core.IntegerProperty(max_val=2 ** 12 - 1)
    gravity = core.FloatProperty()

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()

    def emit(self):
        self.main.new_energy = 1 * self.main.energy
        max_gravity = core.FloatVariable()
        max_gravity += xmath.min(*[nbr.main.gravity for nbr in self.neighbors])
        energy_passed = core.IntegerVariable()
        energy_passed *= 0
        denergy = core.IntegerVariable()
        for i, buf in enumerate(self.buffers):
            fit_dir = max_gravity == self.neighbors[i].main.gravity
            has_energy = (self.main.energy - energy_passed) > 0
            denergy *= 0
            denergy += fit_dir * has_energy * 1
            energy_passed += denergy
            buf.energy = denergy
            buf.gravity = self.main.gravity + self.main.energy
        self.main.new_energy -= energy_passed

    def absorb(self):
        energy_passed = core.IntegerVariable()
        for i in range(len(self.buffers)):
            energy_passed += self.neighbors[i].buffer.energy
        self.main.energy = self.main.new_energy + energy_passed
        new_gravity = core.FloatVariable()
        for i in range(len(self.buffers)):
            new_gravity += self.neighbors[i].buffer.gravity
        self.main.gravity = new_gravity / (len(self.buffers) * 1.001)

    @color_effects.MovingAverage
    def color(self):
        red = self.main.energy * 255
        green = xmath.int(self.main.gravity * 108)
        blue = xmath.int(self.main.gravity * 108)
        return (red, green, blue)


class GraviCowboysStatic(GraviCowboys):
    """The same inside a fixed border container: energy 3 at gravity 0.5."""

    class Topology(GraviCowboys.Topology):
        border = core.StaticBorder(3 | 0x3F000000 << 24)


class GraviCowboysHalf(GraviCowboys):
    """Not the GraviCowboys program (gravity averaged over 4.004): runs on the
    interpreter."""

    def absorb(self):
        energy_passed = core.IntegerVariable()
        for i in range(len(self.buffers)):
            energy_passed += self.neighbors[i].buffer.energy
        self.main.energy = self.main.new_energy + energy_passed
        new_gravity = core.FloatVariable()
        for i in range(len(self.buffers)):
            new_gravity += self.neighbors[i].buffer.gravity
        self.main.gravity = new_gravity / (len(self.buffers) * 0.5005)


class GraviExperiment(core.Experiment):
    word = "LET IT GROOVE"
    size = (64, 48)
    zoom = 1
    pos = [0, 0]
    seed = seeds.patterns.PrimordialSoup(vals={"energy": seeds.random.RandInt(0, 1) * 1, "gravity": 0})


class NoiseExperiment(core.Experiment):
    word = "PSHSHSHSH!"
    size = (64, 48)
    zoom = 1
    pos = [0, 0]
    fade_in = 40
    fade_out = 25
    smooth_factor = 1
    seed = seeds.patterns.PrimordialSoup(vals={"rng": seeds.random.RandInt(0, 2 ** 16 - 1)})


class GOLColorExperiment(core.Experiment):
    word = "XENTICA IN COLOR"
    size = (96, 64)
    zoom = 1
    pos = [0, 0]
    fade_in = 255
    fade_out = 10
    smooth_factor = 1
    seed = seeds.patterns.PrimordialSoup(vals={
        "state": seeds.random.RandInt(0, 1), "red": seeds.random.RandInt(0, 255),
        "green": seeds.random.RandInt(0, 255), "blue": seeds.random.RandInt(0, 255)})


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
    """Directional emit (examples/shifting_sands.py:15-47): the shifting
    family's template."""

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


class ShiftingSandsStatic(ShiftingSands):
    """ShiftingSands with a static border of dead cells."""

    class Topology(ShiftingSands.Topology):
        border = core.StaticBorder(0)


class ShiftingSands3D(ShiftingSands):
    """ShiftingSands on a 3-D von Neumann torus (emit into buffer 2)."""

    class Topology(ShiftingSands.Topology):
        dimensions = 3
        neighborhood = core.VonNeumannNeighborhood()

    def emit(self):
        for i, buf in enumerate(self.buffers):
            if i == 2:
                buf.state = self.main.state
            else:
                buf.state = 0


class ShiftingSandsFade(ShiftingSands):
    """ShiftingSands with history-dependent colours."""

    @color_effects.MovingAverage
    def color(self):
        red = self.main.state * 200
        green = self.main.state * 100 + 10
        blue = 250 - self.main.state * 250
        return (red, green, blue)


MODELS = {
    "ShiftingSands": ShiftingSands, "ShiftingSandsStatic": ShiftingSandsStatic,
    "ShiftingSands3D": ShiftingSands3D, "ShiftingSandsFade": ShiftingSandsFade,
    "GameOfLife": GameOfLife, "GameOfLifeStatic": GameOfLifeStatic,
    "GameOfLife6D": GameOfLife6D, "GameOfLifeInt": GameOfLifeInt, "LifelikeCA": LifelikeCA,
    "GameOfLifeFade": GameOfLifeFade, "GameOfLifePlainColor": GameOfLifePlainColor,
    "GameOfLife3DStatic": GameOfLife3DStatic, "LifelikeFixed": LifelikeFixed,
}
EXPERIMENTS = {
    "GOLExperiment": GOLExperiment, "GOLExperiment2": GOLExperiment2,
    "DiamoebaExperiment": DiamoebaExperiment, "FadeExperiment": FadeExperiment,
    "ShiftingSandsExperiment": ShiftingSandsExperiment,
}


def from_job(job):
    """Our model and experiment for a golden-fixture job (see make_golden.py);
    model keyword arguments are in ``job["model_kwargs"]``."""
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


def build_from_job(job):
    """Construct the model of a fixture job as a fresh reference process
    would: meta-parameters are class-level and keep the last experiment's
    values, so they start from their declared defaults here."""
    model_cls, exp = from_job(job)
    for param in model_cls.meta.__dict__.values():
        if hasattr(param, "default"):
            param.__set__(None, param.default)
    return model_cls(exp, **job.get("model_kwargs", {}))


class RegularCA(core.CellularAutomaton):
    """2-D Moore torus template without logic (examples/base.py:11-37)."""

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()


class RegularExperiment(core.Experiment):
    word = "I AM MUNDANE"
    size = (640, 360, )
    zoom = 3
    pos = [0, 0]


class EvoLife(RegularCA):
    """Life-like CA whose every cell carries its own rule, energy and RNG."""

    energy = core.IntegerProperty(max_val=255 * 2)
    rule = core.TotalisticRuleProperty(outer=True)
    rng = core.RandomProperty()
    death_speed = core.Parameter(default=15)
    max_genes = core.Parameter(default=9)
    mutation_prob = core.Parameter(default=.0)

    def __init__(self, *args, legacy_coloring=True):
        self._legacy_coloring = legacy_coloring
        super().__init__(*args)

    def emit(self):
        for buf in self.buffers:
            buf.energy = self.main.energy
            buf.rule = self.main.rule

    def absorb(self):
        num_neighbors = core.IntegerVariable()
        for i in range(len(self.buffers)):
            nbr_energy = self.neighbors[i].buffer.energy
            nbr_rule = self.neighbors[i].buffer.rule
            num_neighbors += xmath.min(1, (nbr_energy + nbr_rule))
        is_sustained = core.IntegerVariable()
        is_sustained += self.main.rule.is_sustained(num_neighbors)
        fitnesses = []
        for i in range(len(self.buffers)):
            fitnesses.append(core.IntegerVariable(name="fit%d" % i))
        num_parents = core.IntegerVariable()
        for gene in range(len(self.buffers)):
            num_parents *= 0
            for i in range(len(self.buffers)):
                nbr_energy = self.neighbors[i].buffer.energy
                nbr_rule = self.neighbors[i].buffer.rule
                is_alive = xmath.min(1, (nbr_energy + nbr_rule))
                is_fit = self.neighbors[i].buffer.rule.is_born(gene + 1)
                num_parents += is_alive * is_fit
            fitnesses[gene] += num_parents * (num_parents == (gene + 1))
        num_fit = core.IntegerVariable()
        num_fit += xmath.max(*fitnesses)
        genomes = []
        for i in range(len(self.buffers)):
            genomes.append(core.IntegerVariable(name="genome%d" % i))
        for i in range(len(self.buffers)):
            is_fit = self.neighbors[i].buffer.rule.is_born(num_fit)
            genomes[i] += self.neighbors[i].buffer.rule * is_fit
        num_genes = self.main.rule.bit_width
        old_rule = core.IntegerVariable()
        old_rule += self.main.rule
        old_energy = core.IntegerVariable()
        old_energy += self.main.energy
        new_genome = genome_crossover(
            self.main, num_genes, *genomes,
            max_genes=self.meta.max_genes,
            mutation_prob=self.meta.mutation_prob
        )
        self.main.rule = new_genome + self.main.rule * (new_genome == 0)
        self.main.energy *= 0
        is_live = core.IntegerVariable()
        old_live = (old_energy + old_rule) == 0
        is_live += (old_energy < 0xff) & (old_live | is_sustained)
        old_dead = (old_energy + old_rule) != 0
        new_energy = old_energy + self.meta.death_speed * old_dead
        self.main.energy = new_energy * (self.main.rule == old_rule) + \
            self.main.energy * (self.main.rule != old_rule)
        self.main.rule = old_rule * (self.main.rule == old_rule) + \
            self.main.rule * (self.main.rule != old_rule)
        self.main.energy *= is_live
        self.main.rule *= is_live

    @color_effects.MovingAverage
    def color(self):
        if self._legacy_coloring:
            red, green, blue = GenomeColor.modular(self.main.rule >> 1, 360)
        else:
            red, green, blue = GenomeColor.positional(self.main.rule,
                                                      self.main.rule.bit_width)
        is_live = (self.main.rule > 0) * (self.main.energy < 255)
        energy = (255 - self.main.energy) * is_live
        red = xmath.int(red * energy)
        green = xmath.int(green * energy)
        blue = xmath.int(blue * energy)
        return (red, green, blue, )


class CrossbreedingExperiment(RegularExperiment):
    word = "FUTURE BREEDING MACHINE 2041"
    size = (1920, 1080)
    zoom = 1
    fade_in = 18
    fade_out = 3
    seed_diamoeba = seeds.patterns.BigBang(
        pos=(380, 280), size=(440, 340),
        vals={"energy": 0, "rule": LifeLike.golly2int("B35678/S5678") * RandInt(0, 1),
              "rng": RandInt(0, 2 ** 16 - 1)})
    seed_conway = seeds.patterns.BigBang(
        pos=(0, 0), size=(1280, 720),
        vals={"energy": 0, "rule": +RandInt(0, 1) * LifeLike.golly2int("B3/S23"),
              "rng": 0 + RandInt(0, 2 ** 16 - 1)})
    seed_rng = seeds.patterns.PrimordialSoup(vals={"rng": RandInt(0, 2 ** 16 - 1)})
    seed = seed_rng + seed_conway + seed_diamoeba


class CrossbreedingExperiment2(CrossbreedingExperiment):
    death_speed = 25
    max_genes = 9
    mutation_prob = 0.0001


class PrimordialSoupExperiment(RegularExperiment):
    """Every cell of a 1920x1080 torus seeded with a uniform random energy,
    genome and random state; EvoLife's default meta-parameters (death_speed 15,
    max_genes 9, no mutation) and CrossbreedingExperiment's fades 18/3."""
    word = "EVOLIFE PRIMORDIAL SOUP 1920X1080"
    size = (1920, 1080)
    zoom = 1
    pos = [0, 0]
    fade_in = 18
    fade_out = 3
    death_speed = 15
    max_genes = 9
    mutation_prob = 0.0
    seed = seeds.patterns.PrimordialSoup(vals={
        "energy": RandInt(0, 255), "rule": RandInt(0, 2 ** 18 - 1),
        "rng": RandInt(0, 2 ** 16 - 1)})


class BigBangExperiment(RegularExperiment):
    death_speed = 0
    max_genes = 9
    seed_bang = seeds.patterns.BigBang(
        pos=(0, 0), size=(100, 100),
        vals={"energy": RandInt(0, 255), "rule": RandInt(0, 2 ** 18 - 1) & 0b111111110111111110,
              "rng": RandInt(0, 2 ** 16 - 1)})
    seed_rng = seeds.patterns.PrimordialSoup(vals={"rng": RandInt(0, 2 ** 16 - 1)})
    seed = seed_rng + seed_bang


MODELS["EvoLife"] = EvoLife
EXPERIMENTS.update({"CrossbreedingExperiment": CrossbreedingExperiment,
                    "CrossbreedingExperiment2": CrossbreedingExperiment2,
                    "BigBangExperiment": BigBangExperiment})


WALL = 2 ** 32 - 1


class MassTransfer(core.CellularAutomaton):
    """Mass-conserving sand transfer, 3-D von Neumann, wall border."""

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
    seed = seeds.patterns.PrimordialSoup(vals={"mass": seeds.random.RandPoisson(4)})


MODELS["MassTransfer"] = MassTransfer
EXPERIMENTS["MassExperiment"] = MassExperiment
