"""Per-model random streams and random seed values.

Reference ``xentica/seeds/random.py:22-96``: a model's ``LocalRandom(word)``
holds a ``random.Random(word)`` stream and a NumPy ``RandomState`` seeded with
that stream's first ``getrandbits(32)``, so seeds are bit-identical to the
reference's for the same ``word``.

``RandBernoulli`` and ``RandPoisson`` have no counterpart in the reference;
they draw from the same NumPy stream (``random_sample(n) < p`` and
``poisson(lam, n)``) for the Bernoulli and Poisson initial states of the
benchmark configurations.
"""
import functools
import operator
import random

import numpy as np

from xentica_gb300.core.expressions import PatternExpression

__all__ = ['LocalRandom', 'RandInt', 'RandBernoulli', 'RandPoisson', ]


class LocalRandom:
    """Holder of a standard-library and a NumPy random stream."""

    def __init__(self, seed=None):
        self.standard = random.Random(seed)
        np_seed = self.standard.getrandbits(32)
        self.numpy = np.random.RandomState(np_seed)

    def load(self, rng):
        """Adopt the streams of another :class:`LocalRandom`."""
        self.standard = rng.standard
        self.numpy = rng.numpy


def _num_values(instance):
    return functools.reduce(operator.mul, instance.size)


class RandInt(PatternExpression):
    """Random integers in ``[min_val, max_val]``.

    Read through a pattern with a ``size`` it gives one value per cell from
    the NumPy stream; otherwise (or with ``constant=True``) one value from the
    standard stream.
    """

    def __init__(self, min_val, max_val, constant=False):
        super().__init__()
        self.min_val = min_val
        self.max_val = max_val
        self._constant = constant

    def __get__(self, instance, owner):
        if hasattr(instance, "size") and not self._constant:
            return instance.random.numpy.randint(self.min_val, self.max_val + 1,
                                                 _num_values(instance))
        instance = instance or owner
        return instance.random.standard.randint(self.min_val, self.max_val)


class RandBernoulli(PatternExpression):
    """1 with probability ``p``, else 0 (``random_sample(n) < p``)."""

    def __init__(self, p):
        super().__init__()
        self.p = p

    def __get__(self, instance, owner):
        if hasattr(instance, "size"):
            n = _num_values(instance)
            return (instance.random.numpy.random_sample(n) < self.p).astype(np.int64)
        instance = instance or owner
        return int(instance.random.standard.random() < self.p)


class RandPoisson(PatternExpression):
    """Poisson(``lam``) integers (``poisson(lam, n)``)."""

    def __init__(self, lam):
        super().__init__()
        self.lam = lam

    def __get__(self, instance, owner):
        if hasattr(instance, "size"):
            return instance.random.numpy.poisson(self.lam, _num_values(instance)).astype(np.int64)
        instance = instance or owner
        return int(instance.random.numpy.poisson(self.lam))
