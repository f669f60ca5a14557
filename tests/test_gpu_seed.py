"""Bernoulli seeds drawn on the device (``xk_batch_seed_bernoulli``) against
NumPy's own ``RandomState.random_sample`` stream: bit-exact per lattice,
across MT19937 twist boundaries (312 cells per twist), for the extreme
densities, and for the seeded ensemble workload the benchmark uses."""
import numpy as np
import pytest

from xentica_gb300.batch import Ensemble, ensemble_seeds, ensemble_workload

pytestmark = pytest.mark.gpu


def _host(seed, n, p):
    return (np.random.RandomState(int(seed)).random_sample(n) < p).astype(np.uint8)


def test_stream_boundaries_and_densities():
    # sizes around the 312-cell twist boundary and one many-twist lattice
    sizes = [(1, 1), (311, 1), (312, 1), (313, 1), (624, 1), (625, 1), (37, 23), (64, 64),
             (1024, 17), (100, 100)]
    seeds = [0, 1, 5489, 2 ** 32 - 1, 123456789, 42, 7, 2 ** 31, 99991, 3]
    dens = [0.5, 0.0, 1.0, 0.3, 0.999, 0.001, 0.5, 0.25, 0.75, 0.6]
    ens = Ensemble([w for w, _ in sizes], [h for _, h in sizes], [6152] * len(sizes))
    ms = ens.seed_bernoulli(seeds, dens)
    assert ms >= 0.0
    got = ens.download()
    for i, (w, h) in enumerate(sizes):
        want = _host(seeds[i], w * h, dens[i])
        assert np.array_equal(ens.lattice(got, i).ravel(), want), "lattice %d (%dx%d)" % (i, w, h)


def test_matches_the_host_workload():
    widths, heights, rules, dens, cells = ensemble_workload(count=24, base_seed=11,
                                                            sides=(64, 128, 256))
    w2, h2, r2, d2, seeds = ensemble_seeds(count=24, base_seed=11, sides=(64, 128, 256))
    assert np.array_equal(widths, w2) and np.array_equal(dens, d2)
    ens = Ensemble(widths, heights, rules)
    ens.seed_bernoulli(seeds, dens)
    assert np.array_equal(ens.download(), cells)
    ens.step(3)                       # seeded cells step like uploaded ones
    ref = Ensemble(widths, heights, rules)
    ref.upload(cells)
    ref.step(3)
    assert np.array_equal(ens.download(), ref.download())


def test_rejects_wrong_lengths():
    from xentica_gb300.core.exceptions import XenticaException
    ens = Ensemble([8, 8], [8, 8], [6152, 6152])
    with pytest.raises(XenticaException):
        ens.seed_bernoulli([1], [0.5, 0.5])
