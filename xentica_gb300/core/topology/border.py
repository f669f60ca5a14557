"""Borders (reference ``xentica/core/topology/border.py``).

``TorusBorder`` wraps every axis; ``StaticBorder(value)`` makes every off-board
neighbour read as the packed container ``value`` (all of its properties).
"""
import abc

from xentica_gb300.core.mixins import DimensionsMixin

__all__ = ['Border', 'WrappedBorder', 'GeneratedBorder', 'TorusBorder', 'StaticBorder', ]


class Border(DimensionsMixin):
    """Base class of borders."""

    def __init__(self):
        self.topology = None
        super().__init__()


class WrappedBorder(Border):
    """Borders that map off-board coordinates back onto the board."""

    @abc.abstractmethod
    def wrap_coords(self, coord_prefix):
        """C code wrapping coordinates."""


class GeneratedBorder(Border):
    """Borders that generate the state of off-board cells."""

    @abc.abstractmethod
    def off_board_state(self, coord_prefix):
        """C expression of an off-board cell's packed state."""


class TorusBorder(WrappedBorder):
    """Wraps the field into an N-torus."""

    supported_dimensions = list(range(1, 100))

    def wrap_coords(self, coord_prefix):
        return "".join("{x}{i} = ({x}{i} + {w}{i}) % {w}{i};\n".format(
            x=coord_prefix, i=i, w=self.topology.lattice.width_prefix)
            for i in range(self.dimensions))


class StaticBorder(GeneratedBorder):
    """Every off-board cell holds the same packed ``value`` (default 0)."""

    supported_dimensions = list(range(1, 100))

    def __init__(self, value=0):
        self._value = value
        super().__init__()

    @property
    def value(self):
        """Packed off-board state."""
        return self._value

    def off_board_state(self, coord_prefix):
        return str(self._value)
