"""Ensembles: thousands of independent Life-like lattices advanced together.

The reference has no batch API -- its equivalent is one ``LifelikeCA``
(``examples/game_of_life.py:183-203``) per lattice, each stepped in a Python
loop.  :class:`Ensemble` holds many such lattices (2-D Moore tori, one rule per
lattice) on the device and advances all of them with one CUDA graph launch of
the resident kernel (``xk_batch_step``); :meth:`Ensemble.step_plain` is the
one-launch-per-lattice-per-generation form for comparison.

Cells are one byte each (0/1), row-major (x fastest) per lattice, lattices
concatenated in order -- the main plane of the reference's layout.
"""
import ctypes

import numpy as np

from xentica_gb300 import _native as nat
from xentica_gb300 import tuning
from xentica_gb300.core.exceptions import XenticaException
from xentica_gb300.tools.rules import LifeLike

__all__ = ['Ensemble', 'ensemble_workload', 'ensemble_seeds', 'hash64']


def hash64(base_seed, index):
    """SplitMix64 of ``base_seed`` and ``index``: a 64-bit per-lattice seed."""
    mask = (1 << 64) - 1
    z = (base_seed * 0x9E3779B97F4A7C15 + index + 1) & mask
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
    return z ^ (z >> 31)


def _seed_state(args):
    seed, n, p = args
    rng = np.random.RandomState(seed & 0xFFFFFFFF)
    return (rng.random_sample(n) < p).astype(np.uint8)


def ensemble_seeds(count=4096, base_seed=2041, sides=(64, 128, 256, 512, 1024)):
    """The seeded ensemble without its cells: ``(widths, heights, rules,
    densities, seeds)``, ``seeds[i]`` the 32-bit RandomState seed of lattice
    ``i``'s cells (see :func:`ensemble_workload`; :meth:`Ensemble.seed_bernoulli`
    draws the same cells on the device)."""
    rng = np.random.RandomState(hash64(base_seed, 0) & 0xFFFFFFFF)
    widths = rng.choice(sides, count).astype(np.int32)
    heights = rng.choice(sides, count).astype(np.int32)
    rules = rng.randint(0, 2 ** 18, count).astype(np.uint32)
    dens = rng.uniform(0.1, 0.6, count)
    seeds = np.array([hash64(base_seed, i + 1) & 0xFFFFFFFF for i in range(count)], dtype=np.uint32)
    return widths, heights, rules, dens, seeds


def ensemble_workload(count=4096, base_seed=2041, sides=(64, 128, 256, 512, 1024), pool=None):
    """Seeded ensemble: sizes, rules, densities and initial states.

    Lattice ``i`` draws width and height uniformly from ``sides``, a rule
    uniformly from the 2**18 B/S rules and a density ``p ~ U[0.1, 0.6]`` from
    ``RandomState(hash64(base_seed, 0))``; its cells are
    ``RandomState(hash64(base_seed, i + 1)).random_sample(n) < p``.
    ``pool`` (a ``multiprocessing`` pool) parallelises the cell draws.
    """
    widths, heights, rules, dens, seeds = ensemble_seeds(count, base_seed, sides)
    jobs = [(int(seeds[i]), int(widths[i]) * int(heights[i]), float(dens[i]))
            for i in range(count)]
    parts = pool.map(_seed_state, jobs, chunksize=16) if pool else [_seed_state(j) for j in jobs]
    return widths, heights, rules, dens, np.concatenate(parts)


class Ensemble:
    """Independent Life-like lattices on the device.

    :param widths, heights: lattice sizes.
    :param rules: golly rule integers (``LifeLike.golly2int``) or strings.
    """

    def __init__(self, widths, heights, rules):
        self.widths = np.ascontiguousarray(widths, dtype=np.int32)
        self.heights = np.ascontiguousarray(heights, dtype=np.int32)
        rules = [LifeLike.golly2int(r) if isinstance(r, str) else int(r) for r in rules]
        self.rules = np.ascontiguousarray(rules, dtype=np.uint32)
        if not len(self.widths) == len(self.heights) == len(self.rules):
            raise XenticaException("widths, heights and rules differ in length")
        self._sync_layout()
        self._lib = nat.load()
        handle = ctypes.c_void_p()
        nat.check(self._lib.xk_batch_create(self.count, nat.ptr(self.widths), nat.ptr(self.heights),
                                            nat.ptr(self.rules), ctypes.byref(handle)),
                  "xk_batch_create")
        self._handle = handle

    def __del__(self):
        if getattr(self, "_handle", None) is not None:
            try:
                self._lib.xk_batch_destroy(self._handle)
            except Exception:
                pass
            self._handle = None

    def _sync_layout(self):
        self.count = len(self.widths)
        self.sizes = self.widths.astype(np.int64) * self.heights.astype(np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)[:-1]]).astype(np.int64)
        self.total_cells = int(self.sizes.sum())

    def add(self, width, height, rule, cells=None):
        """Append a lattice (cells: ``height x width`` bytes, 0/1; zeros when
        omitted) without disturbing the others; returns its index."""
        rule = LifeLike.golly2int(rule) if isinstance(rule, str) else int(rule)
        buf = None
        if cells is not None:
            buf = np.ascontiguousarray(cells, dtype=np.uint8).ravel()
            if buf.size != int(width) * int(height):
                raise XenticaException("expected %d cells, got %d" % (int(width) * int(height),
                                                                       buf.size))
        rc = self._lib.xk_batch_add(self._handle, int(width), int(height), rule,
                                    None if buf is None else nat.ptr(buf))
        if rc < 0:
            nat.check(rc, "xk_batch_add")
        self.widths = np.append(self.widths, np.int32(width))
        self.heights = np.append(self.heights, np.int32(height))
        self.rules = np.append(self.rules, np.uint32(rule))
        self._sync_layout()
        return int(rc)

    def remove(self, index):
        """Drop lattice ``index``; the lattices after it move down by one."""
        index = int(index)
        nat.check(self._lib.xk_batch_remove(self._handle, index), "xk_batch_remove")
        self.widths = np.delete(self.widths, index)
        self.heights = np.delete(self.heights, index)
        self.rules = np.delete(self.rules, index)
        self._sync_layout()

    def _cells(self, cells):
        cells = np.ascontiguousarray(cells, dtype=np.uint8)
        if cells.size != self.total_cells:
            raise XenticaException("expected %d cells, got %d" % (self.total_cells, cells.size))
        return cells

    def upload(self, cells):
        """Set every lattice's cells (concatenated bytes)."""
        cells = self._cells(cells)
        nat.check(self._lib.xk_batch_upload(self._handle, nat.ptr(cells), self.total_cells),
                  "xk_batch_upload")

    def download(self, out=None):
        """All cells, concatenated."""
        out = np.empty(self.total_cells, dtype=np.uint8) if out is None else out
        nat.check(self._lib.xk_batch_download(self._handle, nat.ptr(out), self.total_cells),
                  "xk_batch_download")
        return out

    def lattice(self, cells, i):
        """View of lattice ``i`` (height x width) inside concatenated ``cells``."""
        off, n = int(self.offsets[i]), int(self.sizes[i])
        return cells[off:off + n].reshape(int(self.heights[i]), int(self.widths[i]))

    def step(self, generations=1):
        """Advance every lattice (batched resident kernel, one graph launch)."""
        nat.check(self._lib.xk_batch_step(self._handle, int(generations)), "xk_batch_step")
        return self._lib.xk_last_step_ms()

    def step_plain(self, generations=1):
        """Advance with one launch per lattice per generation (comparison form)."""
        nat.check(self._lib.xk_batch_step_plain(self._handle, int(generations)),
                  "xk_batch_step_plain")
        return self._lib.xk_last_step_ms()

    def run(self, cells_in, cells_out, generations):
        """Upload ``cells_in``, advance, download into ``cells_out`` (one call)."""
        cells_in = self._cells(cells_in)
        if cells_out.size != self.total_cells or cells_out.dtype != np.uint8:
            raise XenticaException("cells_out must be uint8 of the ensemble's size")
        nat.check(self._lib.xk_batch_run(self._handle, nat.ptr(cells_in), nat.ptr(cells_out),
                                         self.total_cells, int(generations)), "xk_batch_run")
        return self._lib.xk_last_step_ms()

    def launches(self, generations):
        """Kernel launches one :meth:`step` of ``generations`` makes."""
        return int(self._lib.xk_batch_launches(self._handle, int(generations)))

    def seed_bernoulli(self, seeds, densities):
        """Draw every lattice's cells on the device: cell ``j`` of lattice
        ``i`` is ``RandomState(seeds[i]).random_sample(n_i)[j] < densities[i]``,
        bit for bit (the cells :func:`ensemble_workload` makes on the host
        when given the seeds of :func:`ensemble_seeds`).  Returns the device
        time in ms."""
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
        dens = np.ascontiguousarray(densities, dtype=np.float64)
        if seeds.size != self.count or dens.size != self.count:
            raise XenticaException("one seed and one density per lattice")
        nat.check(self._lib.xk_batch_seed_bernoulli(self._handle, nat.ptr(seeds), nat.ptr(dens)),
                  "xk_batch_seed_bernoulli")
        return self._lib.xk_last_step_ms()

    def tune(self, generations, cache=True):
        """Pick the resident kernel's band lengths by timing (one for every
        lattice, then per lattice size where that is faster: :attr:`band`,
        :attr:`size_bands`); returns the common one.  With
        ``cache`` the choice is kept in the tuning cache
        (:mod:`xentica_gb300.tuning`, keyed by device, library build, lattice
        sizes and ``generations``) and a later tune of the same workload
        applies it without timing."""
        return tuning.tuned_band(self._lib, self._handle, self.widths, self.heights,
                                 int(generations), cache=cache)

    @property
    def band(self):
        """Rows per lane group of the resident kernel's bands (the tuned choice)."""
        return int(self._lib.xk_batch_band(self._handle))

    @band.setter
    def band(self, rows_per_band):
        nat.check(self._lib.xk_batch_set_band(self._handle, int(rows_per_band)),
                  "xk_batch_set_band")

    @property
    def size_bands(self):
        """Per-size band lengths ``[[W, H, band], ...]`` overriding :attr:`band`
        for the lattices of those sizes (the tuner's per-size choices)."""
        return tuning.size_bands(self._lib, self._handle)

    @size_bands.setter
    def size_bands(self, triples):
        tuning.apply_bands(self._lib, self._handle, self.band, [list(t) for t in triples])
