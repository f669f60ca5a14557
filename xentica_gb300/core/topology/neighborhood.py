"""Neighbourhoods (reference ``xentica/core/topology/neighborhood.py``).

Neighbour ``k`` of a cell is at ``coords + deltas[k]``; the cell's
``buffers[k]`` is stored in plane ``rev_index_map[k] + 1`` and neighbour ``k``'s
emitted value is read from plane ``k + 1``, so ``rev_index_map`` pairs every
direction with its opposite.

* Moore: deltas are ``itertools.product([-1, 0, 1], repeat=d)`` without the
  2-D zero vector, the first ``3**d - 1`` of them (for d != 2 this keeps the
  zero vector and drops the last delta, exactly as the reference does);
  ``rev_index_map`` is the reversed index list.
* von Neumann: ``+e_i, -e_i`` per axis; ``rev_index_map`` swaps each pair.
"""
import abc
import itertools

from xentica_gb300.core.mixins import DimensionsMixin

__all__ = ['Neighborhood', 'OrthogonalNeighborhood', 'MooreNeighborhood',
           'VonNeumannNeighborhood', ]


class Neighborhood(DimensionsMixin):
    """Base class of neighbourhoods."""

    def __init__(self):
        self.num_neighbors = None
        self.topology = None
        self._delta2str = {-1: " - 1", 0: "", 1: " + 1"}
        self._neighbor_deltas = []
        self.rev_index_map = []
        super().__init__()

    def __len__(self):
        return self.num_neighbors or 0

    @property
    def deltas(self):
        """Offsets of the neighbours actually used (``num_neighbors`` of them)."""
        return [tuple(d) for d in self._neighbor_deltas[:len(self)]]

    @abc.abstractmethod
    def neighbor_coords(self, index, coord_prefix, neighbor_prefix):
        """C code computing the coordinates of neighbour ``index``."""

    @abc.abstractmethod
    def neighbor_state(self, neighbor_index, state_index, coord_prefix):
        """C expression reading a neighbour's state plane."""


class OrthogonalNeighborhood(Neighborhood):
    """Neighbourhoods on an orthogonal lattice."""

    supported_dimensions = list(range(1, 100))

    def neighbor_coords(self, index, coord_prefix, neighbor_prefix):
        return "".join("{n}{i} = {c}{i}{d};\n".format(
            n=neighbor_prefix, i=i, c=coord_prefix,
            d=self._delta2str[self._neighbor_deltas[index][i]]) for i in range(self.dimensions))

    def neighbor_state(self, neighbor_index, state_index, coord_prefix):
        cell_index = self.topology.lattice.coord_to_index_code(coord_prefix)
        return "fld[{}]".format(cell_index + " + n * " + str(state_index))


class MooreNeighborhood(OrthogonalNeighborhood):
    """All cells sharing at least one vertex."""

    @OrthogonalNeighborhood.dimensions.setter
    def dimensions(self, num_dim):
        OrthogonalNeighborhood.dimensions.fset(self, num_dim)
        self.num_neighbors = 3 ** num_dim - 1
        self._neighbor_deltas = [d for d in itertools.product([-1, 0, 1], repeat=num_dim)
                                 if d != (0, 0)]
        self.rev_index_map = list(range(self.num_neighbors))[::-1]


class VonNeumannNeighborhood(OrthogonalNeighborhood):
    """Adjacent cells along every axis."""

    @OrthogonalNeighborhood.dimensions.setter
    def dimensions(self, num_dim):
        OrthogonalNeighborhood.dimensions.fset(self, num_dim)
        self.num_neighbors = 2 * num_dim
        self._neighbor_deltas = []
        self.rev_index_map = []
        for i in range(num_dim):
            self._neighbor_deltas.append(tuple(1 if i == j else 0 for j in range(num_dim)))
            self._neighbor_deltas.append(tuple(-1 if i == j else 0 for j in range(num_dim)))
            self.rev_index_map += [i * 2 + 1, i * 2]
