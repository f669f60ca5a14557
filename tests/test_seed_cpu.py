"""The ensemble's seed definition on the host: ``ensemble_seeds`` gives the
per-lattice RandomState seeds whose ``random_sample(n) < p`` draws are
exactly the cells ``ensemble_workload`` makes (the draw the device seeding,
``Ensemble.seed_bernoulli``, reproduces bit for bit on the GPU)."""
import numpy as np

from xentica_gb300.batch import ensemble_seeds, ensemble_workload, hash64


def test_seeds_reproduce_the_workload_cells():
    w, h, r, d, cells = ensemble_workload(count=12, base_seed=99, sides=(64, 128))
    w2, h2, r2, d2, seeds = ensemble_seeds(count=12, base_seed=99, sides=(64, 128))
    assert np.array_equal(w, w2) and np.array_equal(h, h2) and np.array_equal(r, r2)
    assert np.array_equal(d, d2)
    assert seeds.dtype == np.uint32
    off = 0
    for i in range(12):
        n = int(w[i]) * int(h[i])
        want = np.random.RandomState(int(seeds[i])).random_sample(n) < d[i]
        assert np.array_equal(cells[off:off + n], want.astype(np.uint8)), i
        assert int(seeds[i]) == hash64(99, i + 1) & 0xFFFFFFFF
        off += n
    assert off == cells.size
