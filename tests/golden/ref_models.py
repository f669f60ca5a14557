"""Models written against the reference's public API for the oracle harness.

These are test fixtures: they are executed by ``oracle/ref_harness.py`` with the
reference package on ``sys.path`` (never by the product).  Each one exercises a
reference code path that its own examples do not reach directly.
"""
from xentica import core, seeds
from xentica.core import color_effects
from examples.game_of_life import GameOfLife


class GameOfLifeInt(GameOfLife):
    """16-bit state variant used by the reference's cell-width test."""
    state = core.IntegerProperty(max_val=2 ** 16 - 1)
