"""Small experiments for the reference's own example models (fixtures).

Written against the ``xentica`` names, so the reference's oracle harness
imports this file as it is, and this package runs it through
``xentica_gb300.alias``.  Each experiment keeps the example's parameters and
replaces the seed with a soup over a small lattice (the examples' BigBang
areas need lattices of hundreds of cells a side).
"""
from xentica import seeds
from xentica.seeds.random import RandInt

from examples import game_of_life, shifting_sands, noisetv, conserved_life, gravicowboys, evolife

SOUP = seeds.patterns.PrimordialSoup


class ColorSmall(game_of_life.GOLExperimentColor):
    size = (64, 48)
    seed = SOUP(vals={"state": RandInt(0, 1), "red": RandInt(0, 255),
                      "green": RandInt(0, 255), "blue": RandInt(0, 255)})


class SandsSmall(shifting_sands.ShiftingSandsExperiment):
    size = (64, 48)
    seed = SOUP(vals={"state": RandInt(0, 1)})


class NoiseSmall(noisetv.NoiseTVExperiment):
    size = (64, 48)


class ConservedSmall(conserved_life.BigBangExperiment):
    size = (64, 48)
    seed = SOUP(vals={"energy": 16 * RandInt(0, 1), "new_energy": 16 * RandInt(0, 1),
                      "rule": RandInt(0, 2 ** 18 - 1), "rng": RandInt(0, 2 ** 16 - 1)})


class GraviSmall(gravicowboys.GraviCowboysExperiment):
    size = (64, 48)
    seed = SOUP(vals={"energy": RandInt(0, 1), "gravity": 0})


class EvoLife6DSmall(evolife.EvoLife6DExperiment):
    size = (24, 20, 3, 2, 2, 2)
    seed = SOUP(vals={"energy": RandInt(0, 1) * 255, "rule": RandInt(0, 2 ** 26 - 1),
                      "rng": RandInt(0, 2 ** 16 - 1)})

