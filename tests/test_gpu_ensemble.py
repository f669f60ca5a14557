"""GPU parity of the ensemble (``xk_batch_*``): every lattice, bit-exact.

Mixed sizes exercise every kernel path: resident in shared memory with one or
many row groups per warp, partial last words, the in-place 1024-wide case, and
lattices too wide for a CTA (plain per-generation launches).
"""
import json

import numpy as np
import pytest

import oracle as O
from xentica_gb300 import _native as nat
from xentica_gb300.batch import Ensemble, ensemble_workload
from xentica_gb300.core.exceptions import XenticaException

pytestmark = pytest.mark.gpu

SIZES = [(1, 1), (1, 9), (9, 1), (37, 23), (64, 64), (33, 200), (1024, 1024), (1000, 3),
         (2000, 10), (128, 1024), (1024, 64), (95, 95)]


def _ensemble(seed=7):
    rng = np.random.RandomState(seed)
    widths = [w for w, _ in SIZES]
    heights = [h for _, h in SIZES]
    rules = [int(r) for r in rng.randint(0, 2 ** 18, len(SIZES))]
    rules[4] = 6152     # B3/S23
    ens = Ensemble(widths, heights, rules)
    cells = (rng.random_sample(ens.total_cells) < 0.4).astype(np.uint8)
    return ens, cells


def _oracle(ens, cells, generations):
    out = cells.copy()
    for i in range(ens.count):
        w, h, rule = int(ens.widths[i]), int(ens.heights[i]), int(ens.rules[i])
        topo = O.Topology((w, h))
        fld = topo.field(ens.lattice(cells, i).ravel(), np.uint8)
        col = np.zeros(topo.cells * 3, dtype=np.int32)
        O.life_run(topo, fld, col, generations, born=rule & 511, sustain=rule >> 9)
        ens.lattice(out, i)[...] = fld[:topo.cells].reshape(h, w)
    return out


@pytest.mark.parametrize("generations", [1, 2, 17])
def test_batched_matches_oracle(generations):
    ens, cells = _ensemble()
    ens.upload(cells)
    ens.step(generations)
    got = ens.download()
    want = _oracle(ens, cells, generations)
    for i in range(ens.count):
        assert np.array_equal(ens.lattice(got, i), ens.lattice(want, i)), "lattice %d %s" % (i, SIZES[i])


_ORACLE_CACHE = {}


def _oracle_cached(ens, cells, generations, key):
    if (key, generations) not in _ORACLE_CACHE:
        _ORACLE_CACHE[(key, generations)] = _oracle(ens, cells, generations)
    return _ORACLE_CACHE[(key, generations)]


@pytest.mark.parametrize("generations", [1, 17, 256])
@pytest.mark.parametrize("band", [2, 4, 8, 16, 32])
def test_every_band_matches_oracle(band, generations):
    """Every band length the tuner may choose (rows per lane group, set as
    the tuning cache applies it) against the oracle, up to the benchmark's
    256 generations per launch."""
    ens, cells = _ensemble()
    ens.band = band
    assert ens.band == band
    ens.upload(cells)
    ens.step(generations)
    got = ens.download()
    want = _oracle_cached(ens, cells, generations, "mixed")
    for i in range(ens.count):
        assert np.array_equal(ens.lattice(got, i), ens.lattice(want, i)), \
            "band %d, lattice %d %s" % (band, i, SIZES[i])


def test_per_size_bands_match_oracle():
    """Per-size band lengths (as the tuner's second phase sets them, mixed
    with a common band) against the oracle; clearing them restores the
    common band."""
    ens, cells = _ensemble()
    ens.band = 8
    ens.size_bands = [[1024, 1024, 32], [128, 1024, 2], [33, 200, 4], [95, 95, 16], [64, 64, 1]]
    assert sorted(map(tuple, ens.size_bands)) == sorted(
        [(1024, 1024, 32), (128, 1024, 2), (33, 200, 4), (95, 95, 16), (64, 64, 1)])
    ens.upload(cells)
    ens.step(17)
    got = ens.download()
    want = _oracle_cached(ens, cells, 17, "mixed")
    for i in range(ens.count):
        assert np.array_equal(ens.lattice(got, i), ens.lattice(want, i)), "lattice %d %s" % (i, SIZES[i])
    ens.band = 8
    assert ens.size_bands == []


def _size_classes(count=4096, base_seed=2041):
    """One lattice of each of the 25 size classes of the seeded 4096-lattice
    ensemble (its first member of that class): widths, heights, rules and
    cells exactly as the full ensemble draws them."""
    from xentica_gb300.batch import ensemble_seeds
    widths, heights, rules, dens, seeds = ensemble_seeds(count, base_seed)
    picks, seen = [], set()
    for i in range(count):
        key = (int(widths[i]), int(heights[i]))
        if key not in seen:
            seen.add(key)
            picks.append(i)
    assert len(picks) == 25
    cells = np.concatenate([
        (np.random.RandomState(int(seeds[i])).random_sample(int(widths[i]) * int(heights[i]))
         < dens[i]).astype(np.uint8) for i in picks])
    return widths[picks], heights[picks], rules[picks], cells


@pytest.mark.parametrize("band", ["tuned", 16])
def test_benchmark_size_classes_256_generations(band):
    """The benchmarked configuration: one lattice of every size class of the
    4096-lattice ensemble (sides 64..1024, their own random rules and
    densities), 256 generations in one captured launch, at the band the tuner
    picks for this workload and at 16 rows, lattice by lattice against the
    oracle."""
    widths, heights, rules, cells = _size_classes()
    ens = Ensemble(widths, heights, rules)
    ens.upload(cells)
    if band == "tuned":
        ens.tune(256)
    else:
        ens.band = band
    ens.upload(cells)
    ens.step(256)
    got = ens.download()
    want = _oracle_cached(ens, cells, 256, "classes")
    for i in range(ens.count):
        assert np.array_equal(ens.lattice(got, i), ens.lattice(want, i)), \
            "band %s (%d), lattice %dx%d" % (band, ens.band, widths[i], heights[i])
    # a second launch from the first one's result: the graph replays
    ens.step(256)
    again = ens.download()
    want2 = _oracle(ens, want, 256)
    assert np.array_equal(again, want2)


def test_plain_run_and_tune_agree():
    ens, cells = _ensemble(3)
    ens.upload(cells)
    ens.step_plain(9)
    plain = ens.download()
    ens.upload(cells)
    ens.step(4)
    ens.step(5)
    assert np.array_equal(ens.download(), plain)
    out = np.zeros_like(cells)
    ens.run(cells, out, 9)
    assert np.array_equal(out, plain)
    ens.upload(cells)
    ens.tune(3)
    assert np.array_equal(ens.download(), cells)   # tuning leaves the state alone
    ens.step(9)
    assert np.array_equal(ens.download(), plain)


def test_tuning_cache_applies_the_stored_band(monkeypatch, tmp_path):
    # the first tune times and stores its choices (the common band and the
    # per-size ones); a second ensemble of the same sizes takes them from the
    # cache (xk_batch_set_band, xk_batch_set_size_bands) and steps to the same
    # cells as the plain form
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "tune.json"))
    ens, cells = _ensemble(3)
    ens.upload(cells)
    ens.step_plain(9)
    plain = ens.download()
    chosen = ens.tune(9)
    assert ens.band == chosen
    sizes = ens.size_bands
    assert list(json.loads((tmp_path / "tune.json").read_text()).values()) == \
        [{"band": chosen, "sizes": sizes}]
    again, _ = _ensemble(3)
    for band in (2, 32):
        nat.check(again._lib.xk_batch_set_band(again._handle, band), "xk_batch_set_band")
        assert again.band == band
    assert again.tune(9) == chosen and again.band == chosen and again.size_bands == sizes
    again.upload(cells)
    again.step(9)
    assert np.array_equal(again.download(), plain)


def test_rejects_non_binary_cells():
    ens, cells = _ensemble()
    cells[5] = 3
    ens.upload(cells)
    with pytest.raises(XenticaException, match="0 or 1"):
        ens.step(1)


def test_workload_generator_subsample():
    widths, heights, rules, dens, cells = ensemble_workload(count=24, base_seed=11,
                                                            sides=(64, 128))
    ens = Ensemble(widths, heights, rules)
    ens.upload(cells)
    ens.step(5)
    got = ens.download()
    want = _oracle(ens, cells, 5)
    assert np.array_equal(got, want)


def _resident_ensemble(seed=5):
    """Every lattice fits a CTA (no plain-path member), so ``run`` takes the
    mapped or the pipelined form."""
    sizes = [s for s in SIZES if s[0] <= 1024]
    rng = np.random.RandomState(seed)
    ens = Ensemble([w for w, _ in sizes], [h for _, h in sizes],
                   [int(r) for r in rng.randint(0, 2 ** 18, len(sizes))])
    cells = (rng.random_sample(ens.total_cells) < 0.35).astype(np.uint8)
    return ens, cells


@pytest.mark.parametrize("form", ["default", "chunks"])
@pytest.mark.parametrize("buffers", ["pinned", "pinned-unaligned", "pinned-inplace", "pageable"])
def test_end_to_end_forms(form, buffers, monkeypatch):
    """Both forms of ``run`` (on page-locked buffers: the largest lattices
    copied around their launches, the others read and written by the kernels
    through the mapping; XK_E2E=chunks or pageable buffers: index-order
    chunks) on page-locked buffers (also at an odd offset inside a registered
    block, and in place) and on pageable ones give the oracle's cells and
    leave them on the device."""
    from xentica_gb300 import _native as nat
    monkeypatch.setenv("XK_E2E", form)
    ens, cells = _resident_ensemble()
    want = _oracle(ens, cells, 13)
    n = ens.total_cells
    bufs = []
    if buffers == "pageable":
        src, dst = cells.copy(), np.zeros(n, dtype=np.uint8)
    else:
        skew = 17 if buffers == "pinned-unaligned" else 0
        bufs = [nat.PinnedBuffer(n + 64), nat.PinnedBuffer(n + 64)]
        src = bufs[0].array[skew:skew + n]
        dst = src if buffers == "pinned-inplace" else bufs[1].array[skew:skew + n]
        src[:] = cells
        if dst is not src:
            dst[:] = 0
    ens.upload(cells)
    ens.step(2)          # a captured step first, as a caller may do
    ens.run(src, dst, 13)
    for i in range(ens.count):
        assert np.array_equal(ens.lattice(dst, i), ens.lattice(want, i)), "lattice %d" % i
    assert np.array_equal(ens.download(), want)
    out0 = np.zeros(n, dtype=np.uint8)
    ens.run(want, out0, 0)
    assert np.array_equal(out0, want)
    for b in bufs:
        b.release()


@pytest.mark.parametrize("form", ["default", "chunks"])
def test_end_to_end_rejects_non_binary_cells(form, monkeypatch):
    from xentica_gb300 import _native as nat
    monkeypatch.setenv("XK_E2E", form)
    ens, cells = _resident_ensemble()
    cells[3] = 2
    pin_in, pin_out = nat.PinnedBuffer(ens.total_cells), nat.PinnedBuffer(ens.total_cells)
    pin_in.array[:] = cells
    with pytest.raises(XenticaException, match="0 or 1"):
        ens.run(pin_in.array, pin_out.array, 3)
    pin_in.array[3] = 1
    ens.run(pin_in.array, pin_out.array, 3)   # the flag was cleared


def test_add_and_remove_between_steps():
    """Lattices added and removed between steps (xk_batch_add/remove): every
    lattice keeps its own history, compared with the oracle run for exactly
    the generations it has been a member."""
    ens, cells = _ensemble(9)
    lattices = [ens.lattice(cells, i).copy() for i in range(ens.count)]
    rules = [int(r) for r in ens.rules]
    ages = [0] * ens.count

    def check():
        got = ens.download()
        for i in range(ens.count):
            h, w = lattices[i].shape
            topo = O.Topology((w, h))
            fld = topo.field(lattices[i].ravel(), np.uint8)
            O.life_run(topo, fld, np.zeros(topo.cells * 3, np.int32), ages[i],
                       born=rules[i] & 511, sustain=rules[i] >> 9)
            assert np.array_equal(ens.lattice(got, i).ravel(), fld[:topo.cells]), \
                "lattice %d (%dx%d) after %d generations" % (i, w, h, ages[i])

    ens.upload(cells)
    ens.step(5)
    ages = [a + 5 for a in ages]
    rng = np.random.RandomState(4)
    new = (rng.random_sample((70, 301)) < 0.4).astype(np.uint8)
    idx = ens.add(301, 70, "B36/S23", new)
    assert idx == ens.count - 1 == len(SIZES)
    lattices.append(new)
    rules.append(int(ens.rules[idx]))
    ages.append(0)
    check()
    ens.step(7)
    ages = [a + 7 for a in ages]
    check()
    for drop in (4, 0):
        ens.remove(drop)
        del lattices[drop], rules[drop], ages[drop]
    assert ens._lib.xk_batch_count(ens._handle) == ens.count == len(SIZES) - 1
    ens.step(3)
    ages = [a + 3 for a in ages]
    check()
    ens.add(64, 64, 6152)                      # no cells: all dead
    lattices.append(np.zeros((64, 64), np.uint8))
    rules.append(6152)
    ages.append(0)
    ens.step(2)
    ages = [a + 2 for a in ages]
    check()
