"""GPU parity of the cluster path for single Life-like lattices.

``XK_CLUSTER=n`` makes a model's multi-generation steps run on a cluster of
(up to) n CTAs, whatever the tuner would pick, and ``XK_CLUSTER_BAND=b`` sets
the rows each lane group walks (b = 1 .. 4 or 8, and 5 for bands that do not
divide a CTA's rows); every lattice is compared cell by cell with the oracle,
torus and static border (value 1), widths around the word size and up to
1024, heights from a few rows to more than one CTA holds.
"""
import numpy as np
import pytest

import oracle as O
from xentica_gb300 import core, seeds
from tests.models import GameOfLife, GameOfLifeStatic


class SoupExperiment(core.Experiment):
    word = "CLUSTER SOUP"
    size = (64, 64)
    zoom = 1
    pos = [0, 0]
    seed = seeds.patterns.PrimordialSoup(vals={"state": seeds.random.RandInt(0, 1)})

pytestmark = pytest.mark.gpu

SIZES = [(512, 512), (33, 17), (1024, 40), (1, 9), (100, 301), (1000, 700), (32, 2), (7, 1024)]


def _run(cls, size, forced, gens, monkeypatch, seed, band=2, sync="barrier"):
    monkeypatch.setenv("XK_CLUSTER", str(forced))
    monkeypatch.setenv("XK_CLUSTER_BAND", str(band))
    monkeypatch.setenv("XK_CLUSTER_SYNC", sync)
    exp = type("E", (SoupExperiment, ), {"size": size})
    model = cls(exp)
    n = model.cells_num
    rng = np.random.RandomState(seed)
    cells = (rng.random_sample(n) < 0.45).astype(np.uint8)
    model.gpu.load(cells, np.zeros(3 * n, dtype=np.int32))
    model.gpu.step(gens)
    border = 1 if cls is GameOfLifeStatic else None
    topo = O.Topology(size, "moore", border)
    fld = topo.field(cells, np.uint8)
    O.life_run(topo, fld, np.zeros(3 * n, np.int32), gens)
    return model.gpu.arrays.cells.get()[:n], fld[:n]


@pytest.mark.parametrize("band", [1, 2, 4, 5])
@pytest.mark.parametrize("forced", [2, 4, 8, 16])
@pytest.mark.parametrize("cls", [GameOfLife, GameOfLifeStatic])
def test_cluster_sizes_vs_oracle(cls, forced, band, monkeypatch):
    for k, size in enumerate(SIZES):
        got, want = _run(cls, size, forced, 37, monkeypatch, 10 * forced + k, band)
        assert np.array_equal(got, want), (cls.__name__, size, forced, band)


@pytest.mark.parametrize("band", [1, 2, 4])
@pytest.mark.parametrize("forced", [2, 3, 4, 8, 16])
@pytest.mark.parametrize("cls", [GameOfLife, GameOfLifeStatic])
def test_neighbour_sync_vs_oracle(cls, forced, band, monkeypatch):
    """The neighbour form (each CTA waits on mbarriers for its two
    neighbours' rows only, CTAs run at their own pace) for every cluster size
    and band length it has, against the oracle; odd generation counts leave
    the last generation's slots unsent."""
    for k, size in enumerate(SIZES):
        got, want = _run(cls, size, forced, 37 + k % 2, monkeypatch, 10 * forced + k, band, "p2p")
        assert np.array_equal(got, want), (cls.__name__, size, forced, band)


@pytest.mark.parametrize("band", [4, 8])
@pytest.mark.parametrize("size,forced", [((512, 512), 16), ((512, 512), 8), ((1024, 64), 16),
                                         ((100, 256), 8), ((64, 512), 4), ((1000, 48), 2)])
@pytest.mark.parametrize("cls", [GameOfLife, GameOfLifeStatic])
def test_split_sync_vs_oracle(cls, size, forced, band, monkeypatch):
    """The split form (the cluster barrier's arrive before the bands' inner
    rows, its wait after them; bands of exactly 4 or 8 rows in every CTA)
    against the oracle, and over 3000 generations on the 512 x 512 torus."""
    got, want = _run(cls, size, forced, 41, monkeypatch, 3 * forced + band, band, "split")
    assert np.array_equal(got, want), (cls.__name__, size, forced, band)
    if size == (512, 512) and cls is GameOfLife:
        got, want = _run(cls, size, forced, 3000, monkeypatch, 11 + band, band, "split")
        assert np.array_equal(got, want)


@pytest.mark.parametrize("band", [1, 2, 4, 8])
@pytest.mark.parametrize("forced", [2, 3, 4, 8, 16])
@pytest.mark.parametrize("cls", [GameOfLife, GameOfLifeStatic])
def test_async_sync_vs_oracle(cls, forced, band, monkeypatch):
    """The async form (rows sent by asynchronous remote stores, each counted
    in bytes on the receiving CTA's mbarrier, which that CTA arms once per
    phase) for every cluster size and band length, against the oracle; bands
    of 2, 4 or 8 rows only where every CTA's bands have that length, the
    cluster barrier elsewhere; odd generation counts leave the last
    generation's rows unsent."""
    for k, size in enumerate(SIZES):
        got, want = _run(cls, size, forced, 37 + k % 2, monkeypatch, 10 * forced + k + band, band,
                         "async")
        assert np.array_equal(got, want), (cls.__name__, size, forced, band)


@pytest.mark.parametrize("band", [1, 2, 4, 8])
def test_async_sync_long_run(band, monkeypatch):
    """3000 generations in one launch of the async form on 16 CTAs (a store
    landing in the wrong phase, or overwriting a slot before it was read,
    would show here)."""
    got, want = _run(GameOfLife, (512, 512), 16, 3000, monkeypatch, 21 + band, band, "async")
    assert np.array_equal(got, want)


@pytest.mark.parametrize("band", [1, 2, 4])
def test_neighbour_sync_long_run(band, monkeypatch):
    """3000 generations in one launch of the neighbour form on 16 CTAs (a
    race between a slot's reader and its next writer would show here)."""
    got, want = _run(GameOfLife, (512, 512), 16, 3000, monkeypatch, 5 + band, band, "p2p")
    assert np.array_equal(got, want)


def test_long_run_and_tuner_choice(monkeypatch):
    # 1000 generations (one launch) with the tuner's own choice
    monkeypatch.delenv("XK_CLUSTER", raising=False)
    monkeypatch.delenv("XK_CLUSTER_BAND", raising=False)
    monkeypatch.delenv("XK_CLUSTER_SYNC", raising=False)
    exp = type("E", (SoupExperiment, ), {"size": (512, 512)})
    model = GameOfLife(exp)
    n = model.cells_num
    cells = (np.random.RandomState(3).random_sample(n) < 0.5).astype(np.uint8)
    model.gpu.load(cells, np.zeros(3 * n, dtype=np.int32))
    model.gpu.step(1000)
    topo = O.Topology((512, 512))
    fld = topo.field(cells, np.uint8)
    O.life_run(topo, fld, np.zeros(3 * n, np.int32), 1000)
    assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n])
