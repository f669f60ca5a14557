"""GPU parity of the mass-transfer kernel (3-D von Neumann, wall border).

Fixture cases (reference checksums) replay through ``test_gpu_life``'s
fixture test; here: random states with large masses (unsigned wrap-around of
the reference's arithmetic, cells equal to the wall value) compared with the
oracle cell by cell, image parity, conservation of the total mass over a
long run read from the kernel's own per-generation totals, and step
transitions after long runs checked against the oracle.
"""
import numpy as np
import pytest

import oracle as O
from tests.models import MassTransfer, MassExperiment, WALL

pytestmark = pytest.mark.gpu


def _model(size):
    exp = type("E", (MassExperiment, ), {"size": size})
    return MassTransfer(exp)


def _topo(size):
    return O.Topology(size, "von_neumann", border=WALL)


@pytest.fixture(params=["tma", "tma-general", "rows"])
def kernel_form(request, monkeypatch):
    """Widths that are multiples of 4: the TMA form (default; its fast-only
    instantiation when the uploaded total is below 2^30, its general one
    otherwise or with XK_MASS_GENERAL=1) and the register-queue form
    (XK_MASS_KERNEL=rows)."""
    if request.param == "rows":
        monkeypatch.setenv("XK_MASS_KERNEL", "rows")
    if request.param == "tma-general":
        monkeypatch.setenv("XK_MASS_GENERAL", "1")
    return request.param


@pytest.mark.parametrize("size,high", [((33, 17, 9), 2 ** 32 - 1), ((64, 8, 31), 2 ** 20),
                                       ((7, 129, 5), 100), ((64, 24, 12), 2 ** 32 - 1),
                                       ((128, 40, 20), "mixed")])
def test_random_states_vs_oracle(size, high, kernel_form):
    # widths that are multiples of 4 take the tiled kernels: small values
    # their fast path, large ones (and the wall value) their exact path,
    # "mixed" both in one launch, with values next to the 2^30 and
    # 1431655765 boundaries
    model = _model(size)
    n = model.cells_num
    rng = np.random.RandomState(size[0])
    if high == "mixed":
        cells = rng.poisson(4, n).astype(np.uint32)
        edges = [2 ** 30 - 2, 2 ** 30 - 1, 2 ** 30, 2 ** 30 + 1, 1431655764, 1431655765,
                 1431655766, WALL - 1, WALL]
        where = rng.randint(0, n // 8, 24)          # the first z-slabs only
        cells[where] = rng.choice(edges, where.size)
    else:
        cells = rng.randint(0, high, n, dtype=np.uint64).astype(np.uint32)
    if high != "mixed" and high > 2 ** 31:
        cells[rng.randint(0, n, 20)] = WALL
    colors = np.zeros(3 * n, dtype=np.int32)
    model.gpu.load(cells, colors)
    topo = _topo(size)
    fld = topo.field(cells, np.uint32)
    col = colors.copy()
    for step in range(5):
        model.step()
        O.mass_run(topo, fld, col, 1)
        assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n]), "step %d" % step
        assert np.array_equal(model.gpu.arrays.colors.get(), col), "colours step %d" % step
    w, h = size[0] + 5, size[1] + 3
    img = O.render(topo, col, w, h, zoom=1, dx=-2, dy=3, smooth=0).astype(np.uint8)
    model.set_viewport((w, h))
    model.pos = [-2, 3]
    assert np.array_equal(model.render(), img)


def test_mass_conserved_long_run(kernel_form):
    model = _model((96, 80, 40))
    before = int(model.gpu.arrays.cells.get()[:model.cells_num].astype(np.uint64).sum())
    model.gpu.step(500)
    totals = model.gpu.mass_totals(500)
    assert totals.tolist() == [before] * 500
    after = int(model.gpu.arrays.cells.get()[:model.cells_num].astype(np.uint64).sum())
    assert after == before


@pytest.mark.parametrize("size,gens", [((256, 256, 256), 2000), ((171, 205, 43), 3000)])
def test_long_run_step_transitions(size, gens):
    # after a long GPU run, one and then two more generations agree with the
    # oracle started from the GPU state: the 256^3 lattice of the mass
    # benchmark, and a width that is not a multiple of 4 (pitched rows)
    model = _model(size)
    model.gpu.step(gens)
    n = model.cells_num
    topo = _topo(size)
    fld = topo.field(model.gpu.main_plane(), np.uint32)
    col = np.zeros(3 * n, dtype=np.int32)
    model.gpu.step(1)
    O.mass_run(topo, fld, col, 1)
    assert np.array_equal(model.gpu.main_plane(), fld[:n])
    model.gpu.step(2)
    O.mass_run(topo, fld, col, 2)
    assert np.array_equal(model.gpu.main_plane(), fld[:n])


def test_multi_generation_call_equals_single_steps():
    a, b = _model((40, 24, 16)), _model((40, 24, 16))
    a.gpu.step(7)
    for _ in range(7):
        b.step()
    assert np.array_equal(a.gpu.arrays.cells.get(), b.gpu.arrays.cells.get())
    assert np.array_equal(a.gpu.arrays.colors.get(), b.gpu.arrays.colors.get())


@pytest.mark.parametrize("zc", ["1", "3", "8", "20"])
def test_z_chunks_vs_oracle(zc, monkeypatch, kernel_form):
    # planes per CTA forced (the automatic choice gives small lattices one);
    # a few large cells put some CTAs on the exact path
    monkeypatch.setenv("XK_MASS_ZC", zc)
    size = (64, 24, 20)
    model = _model(size)
    n = model.cells_num
    rng = np.random.RandomState(int(zc))
    cells = rng.poisson(5, n).astype(np.uint32)
    cells[rng.randint(0, n, 6)] = rng.choice([2 ** 30, 1431655766, WALL], 6)
    model.gpu.load(cells, np.zeros(3 * n, dtype=np.int32))
    topo = _topo(size)
    fld = topo.field(cells, np.uint32)
    col = np.zeros(3 * n, dtype=np.int32)
    model.gpu.step(4)
    totals = []
    O.mass_run(topo, fld, col, 4, totals=totals)
    assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n])
    assert model.gpu.mass_totals(4).tolist() == totals


@pytest.mark.parametrize("size", [(4, 3, 1), (132, 9, 2), (256, 17, 3), (8, 1, 5), (260, 8, 7)])
def test_tile_edges_vs_oracle(size, kernel_form):
    # partial tiles in x (a second 128-cell tile mostly off the lattice), y
    # (heights not a multiple of the tile's 8 rows) and z (one to seven
    # planes), with a few cells at or above 2^30 in some runs
    model = _model(size)
    n = model.cells_num
    rng = np.random.RandomState(sum(size))
    cells = rng.poisson(6, n).astype(np.uint32)
    if size[0] > 8:
        cells[rng.randint(0, n, 3)] = rng.choice([2 ** 30, WALL], 3)
    model.gpu.load(cells, np.zeros(3 * n, dtype=np.int32))
    topo = _topo(size)
    fld = topo.field(cells, np.uint32)
    col = np.zeros(3 * n, dtype=np.int32)
    model.gpu.step(3)
    totals = []
    O.mass_run(topo, fld, col, 3, totals=totals)
    assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n])
    assert model.gpu.mass_totals(3).tolist() == totals


@pytest.mark.parametrize("form", ["tma", "tma-general", "generic", "generic-exact"])
@pytest.mark.parametrize("size", [(33, 17, 9), (171, 20, 9), (5, 3, 2), (1, 1, 1), (97, 1, 4), (63, 65, 3)])
def test_odd_widths_vs_oracle(size, form, monkeypatch):
    # widths that are not a multiple of 4: rows at a pitch padded to 4 cells;
    # the TMA kernel (its fast-only form for small totals, XK_MASS_GENERAL=1
    # the general one) or, with XK_MASS_KERNEL=rows, the generic one-cell
    # kernels; results, colours and totals against the oracle
    if form.endswith("general") or form.endswith("exact"):
        monkeypatch.setenv("XK_MASS_GENERAL", "1")
    if form.startswith("generic"):
        monkeypatch.setenv("XK_MASS_KERNEL", "rows")
    model = _model(size)
    n = model.cells_num
    rng = np.random.RandomState(sum(size) + len(form))
    cells = rng.poisson(5, n).astype(np.uint32)
    model.gpu.load(cells, np.zeros(3 * n, dtype=np.int32))
    topo = _topo(size)
    fld = topo.field(cells, np.uint32)
    col = np.zeros(3 * n, dtype=np.int32)
    model.gpu.step(4)
    totals = []
    O.mass_run(topo, fld, col, 4, totals=totals)
    assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n])
    assert model.gpu.mass_totals(4).tolist() == totals
    assert np.array_equal(model.gpu.arrays.colors.get(), col)
    model.gpu.load(cells, np.zeros(3 * n, dtype=np.int32))   # a second upload over the stepped state
    model.gpu.step(1)
    fld = topo.field(cells, np.uint32)
    O.mass_run(topo, fld, np.zeros(3 * n, dtype=np.int32), 1)
    assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n])
