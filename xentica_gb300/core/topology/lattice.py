"""Lattices (reference ``xentica/core/topology/lattice.py:26-221``).

``OrthogonalLattice`` is an N-dimensional grid with axis 0 fastest:
``index = x0 + w0 * x1 + w0 * w1 * x2 + ...``.  The ``*_code`` methods give
the reference's C spelling of the same arithmetic (used for the traced-program
listing); the kernels implement it directly.
"""
import abc

from xentica_gb300.core.mixins import DimensionsMixin, BscaDetectorMixin
from xentica_gb300.core.variables import Constant
from xentica_gb300.core.exceptions import XenticaException

__all__ = ['Lattice', 'OrthogonalLattice', ]


class Lattice(DimensionsMixin, BscaDetectorMixin, metaclass=abc.ABCMeta):
    """Base class of lattices."""

    #: prefix of the per-axis size constants
    width_prefix = "_w"

    def _define_constants_once(self):
        bsca = self.bsca
        num_dimensions = bsca.topology.dimensions
        for i in range(num_dimensions):
            if not hasattr(bsca, "size") or i >= len(bsca.size):
                msg = "Wrong field's dimensionality ({} instead of {})."
                raise XenticaException(msg.format(len(bsca.size), num_dimensions))
            bsca.define_constant(Constant("%s%d" % (self.width_prefix, i), bsca.size[i]))

    @abc.abstractmethod
    def index_to_coord_code(self, index_name, coord_prefix):
        """C code turning a cell index into coordinates."""

    @abc.abstractmethod
    def index_to_coord(self, idx, bsca):
        """Coordinates of index ``idx`` (int or NumPy array), per axis."""

    @abc.abstractmethod
    def coord_to_index_code(self, coord_prefix):
        """C expression of the index at the given coordinates."""

    @abc.abstractmethod
    def is_off_board_code(self, coord_prefix):
        """C condition testing whether coordinates are off the board."""


class OrthogonalLattice(Lattice):
    """N-dimensional orthogonal lattice."""

    supported_dimensions = list(range(1, 100))

    def index_to_coord_code(self, index_name, coord_prefix):
        self._define_constants_once()
        code = "int _{idx} = {idx};\n".format(idx=index_name)
        index_name = "_" + index_name
        for i in range(self.dimensions):
            if i < self.dimensions - 1:
                code += "int {x}{i} = {idx} % {w}{i};\n".format(
                    x=coord_prefix, i=i, idx=index_name, w=self.width_prefix)
                code += "{idx} /= {w}{i};\n".format(idx=index_name, w=self.width_prefix, i=i)
            else:
                code += "int {x}{i} = {idx};\n".format(x=coord_prefix, i=i, idx=index_name)
        return code

    def index_to_coord(self, idx, bsca):
        coord = []
        for i in range(bsca.topology.dimensions):
            if i < self.dimensions - 1:
                x_i = idx % bsca.size[i]
                idx //= bsca.size[i]
            else:
                x_i = idx
            coord.append(x_i)
        return coord

    def coord_to_index_code(self, coord_prefix):
        self._define_constants_once()
        summands = []
        for i in range(self.dimensions):
            summand = coord_prefix + str(i)
            for j in range(i):
                summand = self.width_prefix + str(j) + " * " + summand
            summands.append(summand)
        return " + ".join(summands)

    def is_off_board_code(self, coord_prefix):
        self._define_constants_once()
        return " || ".join("{x}{i} < 0 || {x}{i} >= {w}{i}".format(
            x=coord_prefix, i=i, w=self.width_prefix) for i in range(self.dimensions))
