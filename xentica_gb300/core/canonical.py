"""Reference programs of the kernel families matched by fingerprint.

A family whose kernel restates one specific model (rather than a rule table
read off by evaluation) is defined here by that model, written in the DSL.
A user model matches when its traced programs are identical to the
reference program traced with the user's parameter values (variables may be
named differently).  The EvoLife kernel (``csrc/evolife.cu``) implements
exactly the program below -- the EvoLife example of the reference
(``examples/evolife.py:20-128``), whose operation order fixes the random
stream and the float rounding, so it is kept statement for statement.
"""
import threading

from xentica_gb300 import core
from xentica_gb300.core import color_effects
from xentica_gb300.core.base import Translator
from xentica_gb300.tools import xmath
from xentica_gb300.tools.color import GenomeColor
from xentica_gb300.tools.genetics import genome_crossover

_LOCK = threading.Lock()


class EvoLifeProgram(core.CellularAutomaton):
    """EvoLife: per-cell outer-totalistic genome, energy and random stream."""

    energy = core.IntegerProperty(max_val=255 * 2)
    rule = core.TotalisticRuleProperty(outer=True)
    rng = core.RandomProperty()
    _legacy_coloring = True          # GenomeColor.modular; False: .positional
    death_speed = core.Parameter(default=15)
    max_genes = core.Parameter(default=9)
    mutation_prob = core.Parameter(default=.0)

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()

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
        new_genome = genome_crossover(self.main, num_genes, *genomes,
                                      max_genes=self.meta.max_genes,
                                      mutation_prob=self.meta.mutation_prob)
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
            red, green, blue = GenomeColor.positional(self.main.rule, self.main.rule.bit_width)
        is_live = (self.main.rule > 0) * (self.main.energy < 255)
        energy = (255 - self.main.energy) * is_live
        red = xmath.int(red * energy)
        green = xmath.int(green * energy)
        blue = xmath.int(blue * energy)
        return (red, green, blue, )


def trace(program_cls, size, params, attrs):
    """Traced ``{"emit", "absorb"}`` programs of ``program_cls`` with the given
    meta-parameter values and model attributes."""
    with _LOCK:
        inst = program_cls.__new__(program_cls)
        Translator.__init__(inst)
        inst.size = tuple(size)
        for name, value in attrs.items():
            setattr(inst, name, value)
        for name, value in params.items():
            inst.meta.__dict__[name].__set__(inst, value)
        inst.cells_num = 1
        for s in inst.size:
            inst.cells_num *= s
        inst.build_emit()
        inst.build_absorb()
        return inst.programs


#: off-board (and wall) mass of the mass-transfer family
MASS_WALL = 2 ** 32 - 1


class MassTransferProgram(core.CellularAutomaton):
    """Mass-conserving sand transfer: each cell sends mass / 7 to every
    neighbour that is not the wall and absorbs what it is sent."""

    mass = core.IntegerProperty(max_val=2 ** 32 - 2)

    class Topology:
        dimensions = 3
        lattice = core.OrthogonalLattice()
        neighborhood = core.VonNeumannNeighborhood()
        border = core.StaticBorder(MASS_WALL)

    def emit(self):
        share = core.IntegerVariable()
        share += self.main.mass / 7
        for i in range(len(self.buffers)):
            self.buffers[i].mass = share * (self.neighbors[i].main.mass != MASS_WALL)

    def absorb(self):
        total = core.IntegerVariable()
        total += self.main.mass
        for i in range(len(self.buffers)):
            total -= self.buffers[i].mass
        for i in range(len(self.buffers)):
            incoming = self.neighbors[i].buffer.mass
            total += incoming * (incoming != MASS_WALL)
        self.main.mass = total

    @color_effects.ColorEffect
    def color(self):
        v = xmath.min(self.main.mass * 32, 255)
        return (v, v, v)


class LifeColorProgram(core.CellularAutomaton):
    """Conway's Life whose live cells carry a colour: each 8-bit channel of
    a cell becomes the sum over its eight neighbours of (channel + 1), kept
    only while the cell lives (the reference's GameOfLifeColor,
    ``examples/game_of_life.py:112-159``; the statement order fixes the
    traced program the matcher compares with)."""

    state = core.IntegerProperty(max_val=1)
    red = core.IntegerProperty(max_val=255)
    green = core.IntegerProperty(max_val=255)
    blue = core.IntegerProperty(max_val=255)

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()

    def emit(self):
        for buf in self.buffers:
            buf.state = self.main.state
            buf.red = self.main.red
            buf.green = self.main.green
            buf.blue = self.main.blue

    def absorb(self):
        alive = core.IntegerVariable()
        for k in range(len(self.buffers)):
            alive += self.neighbors[k].buffer.state
        self.main.state = (8 >> alive) & 1 | (12 >> alive) & 1 & self.main.state
        # (each accumulator bound to its own local name: a variable's C name
        # is the Python name it is used under)
        acc_r = core.IntegerVariable()
        acc_g = core.IntegerVariable()
        acc_b = core.IntegerVariable()
        for k in range(len(self.buffers)):
            nbr = self.neighbors[k].buffer
            acc_r += nbr.red + 1
            acc_g += nbr.green + 1
            acc_b += nbr.blue + 1
        self.main.red = acc_r * self.main.state
        self.main.green = acc_g * self.main.state
        self.main.blue = acc_b * self.main.state

    @color_effects.MovingAverage
    def color(self):
        return (self.main.state * self.main.red, self.main.state * self.main.green,
                self.main.state * self.main.blue)


class NoiseProgram(core.CellularAutomaton):
    """Per-cell noise (the reference's NoiseTV, ``examples/noisetv.py:13-31``):
    no buffer is written; each generation reads the cell's RandomProperty
    once in absorb and once more for the colour's uniform draw, each read
    one advance of its stream."""

    rng = core.RandomProperty()

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()

    def emit(self):
        """Nothing: a cell depends on no neighbour."""

    def absorb(self):
        return self.main.rng      # the read advances the stream

    @color_effects.MovingAverage
    def color(self):
        grey = xmath.int(self.main.rng.uniform * 255)
        return (grey, grey, grey)


class GravityProgram(core.CellularAutomaton):
    """Energy drifting down a diffusing field (the reference's GraviCowboys,
    ``examples/gravicowboys.py``): a cell sends one unit of its energy to
    each neighbour, in neighbour order and while it has energy left, whose
    field value equals the smallest around it; every buffer carries the
    cell's field plus its energy, and the new field is the neighbours' sum
    divided by 8.008.  The statement order fixes the float rounding."""

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
        lowest = core.FloatVariable()
        lowest += xmath.min(*[nbr.main.gravity for nbr in self.neighbors])
        sent = core.IntegerVariable()
        sent *= 0
        unit = core.IntegerVariable()
        for k, buf in enumerate(self.buffers):
            towards = lowest == self.neighbors[k].main.gravity
            left = (self.main.energy - sent) > 0
            unit *= 0
            unit += towards * left * 1
            sent += unit
            buf.energy = unit
            buf.gravity = self.main.gravity + self.main.energy
        self.main.new_energy -= sent

    def absorb(self):
        received = core.IntegerVariable()
        for k in range(len(self.buffers)):
            received += self.neighbors[k].buffer.energy
        self.main.energy = self.main.new_energy + received
        field = core.FloatVariable()
        for k in range(len(self.buffers)):
            field += self.neighbors[k].buffer.gravity
        self.main.gravity = field / (len(self.buffers) * 1.001)

    @color_effects.MovingAverage
    def color(self):
        return (self.main.energy * 255, xmath.int(self.main.gravity * 108),
                xmath.int(self.main.gravity * 108))
