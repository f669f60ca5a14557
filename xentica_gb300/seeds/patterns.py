"""Seed patterns (reference ``xentica/seeds/patterns.py:28-274``).

A pattern's ``generate(cells, model)`` fills the main plane of the initial
state.  Values are drawn per property in *sorted property-name order* and
packed with ``model.pack_state``, exactly as the reference does, so the same
experiment produces the same initial state.
"""
import abc

import numpy as np

from xentica_gb300.seeds.random import LocalRandom

__all__ = ['RandomPattern', 'BigBang', 'PrimordialSoup', 'ValDict', 'ChainedPattern', ]


class ValDictMeta(type):
    """Metaclass placeholder of :class:`ValDict`."""


class ValDict(metaclass=ValDictMeta):
    """Read-only dict whose descriptor values are resolved on access.

    :param dct: mapping of names to plain values or descriptors (``RandInt``...).
    :param parent: object the descriptors are resolved against (default: self).
    """

    def __init__(self, dct, parent=None):
        self._d = dct
        self.parent = parent
        if parent is None:
            self.parent = self
            self.random = LocalRandom()

    def items(self):
        """Iterate over ``(key, resolved value)``."""
        for key in self._d.keys():
            yield key, self[key]

    def keys(self):
        """Iterate over keys."""
        for key in self._d.keys():
            yield key

    def __getitem__(self, key):
        if key in self._d:
            val = self._d[key]
            if hasattr(val, '__get__'):
                return val.__get__(self.parent, self.parent.__class__)
            return val
        raise KeyError(key)

    def __setitem__(self, key, val):
        raise NotImplementedError


class RandomPattern:
    """Base class of random patterns."""

    def __init__(self, vals):
        self._random = LocalRandom()
        self.vals = ValDict(vals, self)

    @property
    def random(self):
        """The pattern's random stream (the model's, once attached)."""
        return self._random

    @random.setter
    def random(self, val):
        self._random = val

    def __add__(self, other):
        return ChainedPattern(self, other)

    @abc.abstractmethod
    def generate(self, cells, bsca):
        """Fill ``cells`` (main plane) for model ``bsca``."""


class ChainedPattern(RandomPattern):
    """Two patterns applied in order."""

    def __init__(self, pattern1, pattern2):
        self._pattern1 = pattern1
        self._pattern2 = pattern2
        super().__init__({})

    @RandomPattern.random.setter
    def random(self, val):
        self._pattern1.random = val
        self._pattern2.random = val

    def generate(self, cells, bsca):
        self._pattern1.generate(cells, bsca)
        self._pattern2.generate(cells, bsca)


class BigBang(RandomPattern):
    """Random values inside an N-box; cells outside keep their value.

    :param vals: property values (plain or random).
    :param pos: lowest corner of the box (random if omitted).
    :param size: box size per axis (random if omitted).
    """

    def __init__(self, vals, pos=None, size=None):
        self.pos = np.asarray(pos) if pos else None
        self.size = np.asarray(size) if size else None
        super().__init__(vals)

    def _prepare_area(self, bsca_size):
        dims = range(len(bsca_size))
        randint = self.random.standard.randint
        if self.size is None:
            self.size = np.asarray([randint(1, bsca_size[i]) for i in dims])
        if self.pos is None:
            self.pos = np.asarray([randint(0, bsca_size[i]) for i in dims])
        for i, coord in enumerate(self.pos):
            width, side = self.size[i], bsca_size[i]
            if coord + width >= side:
                self.pos[i] = side - width
            self.pos[i] = max(0, self.pos[i])

    def generate(self, cells, bsca):
        self._prepare_area(bsca.size)
        coords = bsca.index_to_coord(np.arange(0, bsca.cells_num))
        area = None
        for i in range(len(bsca.size)):
            cond = (coords[i] >= self.pos[i]) & (coords[i] < self.pos[i] + self.size[i])
            area = cond if area is None else (area & cond)
        state = {name: self.vals[name] for name in sorted(self.vals.keys())}
        cells[np.where(area)] = bsca.pack_state(state)


class PrimordialSoup(RandomPattern):
    """Random values in every cell."""

    def __init__(self, vals):
        self.size = None
        super().__init__(vals)

    def generate(self, cells, bsca):
        self.size = bsca.size
        state = {name: self.vals[name] for name in sorted(self.vals.keys())}
        cells[:bsca.cells_num] = bsca.pack_state(state)
