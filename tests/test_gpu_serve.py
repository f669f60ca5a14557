"""GPU tests of the serving loop (``xentica_gb300.serve`` over ``xk_serve_*``).

Every request's result must equal the oracle's and be the same alone and in
a mix with others arriving while it runs (bit-exact: integer state), through
admission waits under a tight budget and next to a cancelled request.
"""
import os
import time

import numpy as np
import pytest

import oracle as O
from xentica_gb300 import serve
from xentica_gb300.core.exceptions import XenticaException

pytestmark = pytest.mark.gpu

WALL = 2 ** 32 - 1
BIG_MASS_SHAPE = (16, 12, 10)      # mass requests of this shape get cells at and above 2^30


def oracle_result(kind, cells, rule, generations):
    shape = cells.shape
    size = tuple(reversed(shape))
    if kind == "life2d":
        topo = O.Topology(size)
        fld = topo.field(cells.ravel(), np.uint8)
        col = np.zeros(3 * topo.cells, dtype=np.int32)
        O.life_run(topo, fld, col, generations, born=rule & 511, sustain=rule >> 9)
    elif kind == "life3d":
        topo = O.Topology(size, "von_neumann")
        fld = topo.field(cells.ravel(), np.uint8)
        col = np.zeros(3 * topo.cells, dtype=np.int32)
        O.life_run(topo, fld, col, generations, born=rule & 127, sustain=rule >> 7)
    else:
        topo = O.Topology(size, "von_neumann", border=WALL)
        fld = topo.field(cells.ravel(), np.uint32)
        col = np.zeros(3 * topo.cells, dtype=np.int32)
        O.mass_run(topo, fld, col, generations)
    return fld[:topo.cells].reshape(shape)


SPECS = [  # kind, shape, rule, generations
    ("life2d", (30, 40), 6152, 37),          # resident
    ("life2d", (97, 61), 0o1234 * 7, 50),    # resident, ragged width
    ("life2d", (420, 700), 6152, 70),        # > 2^18 cells: bit-packed global path
    ("life2d", (5, 33), 3 | (12 << 9), 9),
    ("life3d", (13, 17, 20), 0b0001100_0000100, 40),
    ("life3d", (7, 5, 9), 0b0011000_0001010, 3),
    ("mass", (12, 20, 24), 0, 45),           # W % 4 == 0: TMA kernel, fast-only (small total)
    ("mass", BIG_MASS_SHAPE, 0, 20),         # large masses and walls: TMA kernel, general form
    ("mass", (7, 9, 23), 0, 30),             # generic kernel
    ("life2d", (64, 64), 6152, 0),           # zero generations: the input back
]


def _cells(kind, shape, seed):
    rng = np.random.RandomState(seed)
    if kind == "mass":
        cells = rng.poisson(6, shape).astype(np.uint32)
        if shape == BIG_MASS_SHAPE:
            flat = cells.reshape(-1)
            flat[rng.randint(0, flat.size, 12)] = rng.choice([2 ** 30, 1431655766, WALL], 12)
        return cells
    return (rng.random_sample(shape) < 0.4).astype(np.uint8)


def _budget(specs):
    return sum(serve.request_bytes(k, s, r, g) for k, s, r, g in specs) + (1 << 20)


@pytest.mark.parametrize("quantum", [16, 7])
def test_each_kind_matches_oracle(quantum):
    # full rounds replay captured graphs (an odd quantum alternates two)
    with serve.Server(_budget(SPECS), quantum=quantum) as srv:
        for i, (kind, shape, rule, gens) in enumerate(SPECS):
            cells = _cells(kind, shape, i)
            got = srv.submit(kind, cells, rule, gens).result(timeout=120)
            want = oracle_result(kind, cells, rule, gens)
            assert np.array_equal(got, want), (kind, shape)


def _alone(specs, cells):
    out = []
    with serve.Server(_budget(specs), quantum=64) as srv:
        for (kind, shape, rule, gens), c in zip(specs, cells):
            out.append(srv.submit(kind, c, rule, gens).result(timeout=120))
    return out


def test_same_result_alone_and_in_the_mix():
    rng = np.random.RandomState(11)
    specs = []
    for i in range(24):
        kind = ["life2d", "life3d", "mass"][i % 3]
        if kind == "life2d":
            shape = (int(rng.randint(20, 300)), int(rng.randint(20, 900)))
            rule = int(rng.randint(0, 2 ** 18))
        else:
            shape = tuple(int(v) for v in rng.randint(8, 40, 3))
            rule = int(rng.randint(0, 2 ** 14)) if kind == "life3d" else 0
        specs.append((kind, shape, rule, int(rng.randint(10, 300))))
    cells = [_cells(k, s, 100 + i) for i, (k, s, _, _) in enumerate(specs)]
    alone = _alone(specs, cells)
    # mix: a budget for about a third of the requests, so later ones wait for
    # memory; submissions staggered so requests join while others run
    budget = _budget(specs) // 3
    with serve.Server(budget, max_active=64, quantum=8) as srv:
        handles = []
        for i, ((kind, shape, rule, gens), c) in enumerate(zip(specs, cells)):
            handles.append(srv.submit(kind, c, rule, gens))
            if i % 4 == 3:
                time.sleep(0.002)
        results = [h.result(timeout=300) for h in handles]
        st = srv.stats()
        infos = [h.info() for h in handles]
    for i, (got, want) in enumerate(zip(results, alone)):
        assert np.array_equal(got, want), "request %d %s" % (i, specs[i][:2])
    assert st["completed"] == len(specs)
    assert st["device_bytes_peak"] <= st["budget_bytes"]
    assert any(inf["admit_s"] - inf["submit_s"] > 0 for inf in infos)
    # spot-check the mix against the oracle as well
    for i in (0, 1, 2, 5):
        kind, shape, rule, gens = specs[i]
        assert np.array_equal(results[i], oracle_result(kind, cells[i], rule, gens))


def test_cancel_leaves_the_others_unchanged():
    specs = [("life2d", (300, 800), 6152, 4000), ("life3d", (30, 30, 30), 0b0001100_0000100, 200),
             ("mass", (16, 16, 32), 0, 150), ("life2d", (64, 100), 6152, 300)]
    cells = [_cells(k, s, 7 + i) for i, (k, s, _, _) in enumerate(specs)]
    alone = _alone(specs[1:], cells[1:])
    with serve.Server(_budget(specs), quantum=4) as srv:
        handles = [srv.submit(k, c, r, g) for (k, _, r, g), c in zip(specs, cells)]
        while handles[0].status() == "pending":
            time.sleep(0.001)
        handles[0].cancel()
        results = [h.result(timeout=120) for h in handles[1:]]
        assert handles[0].wait(timeout=60)["status"] == "cancelled"
        with pytest.raises(XenticaException):
            handles[0].result()
        assert srv.stats()["cancelled"] == 1
    for got, want in zip(results, alone):
        assert np.array_equal(got, want)


def test_rejections_and_mass_total():
    cells = _cells("mass", (10, 12, 16), 3)
    with serve.Server(serve.request_bytes("mass", cells.shape) + 4096) as srv:
        req = srv.submit("mass", cells, 0, 25)
        assert np.array_equal(req.result(timeout=60), oracle_result("mass", cells, 0, 25))
        assert req.info()["mass_total"] == int(cells.astype(np.uint64).sum())
        with pytest.raises(XenticaException, match="status -3"):
            srv.submit("mass", np.zeros((64, 64, 64), np.uint32), 0, 1)   # over the budget
        bad = np.zeros((8, 8), np.uint8)
        bad[3, 3] = 2
        with pytest.raises(XenticaException, match="0 or 1"):
            srv.submit("life2d", bad, 6152, 1)
        assert srv.stats()["rejected"] == 2


def test_pending_request_can_be_cancelled():
    specs = [("life2d", (512, 512), 6152, 3000), ("life2d", (512, 512), 6152, 10)]
    cells = [_cells(k, s, i) for i, (k, s, _, _) in enumerate(specs)]
    # room for one request at a time: the second waits in the queue
    with serve.Server(max(serve.request_bytes(*s) for s in specs) + 256, quantum=64) as srv:
        first = srv.submit(specs[0][0], cells[0], specs[0][2], specs[0][3])
        second = srv.submit(specs[1][0], cells[1], specs[1][2], specs[1][3])
        assert second.status() == "pending"
        second.cancel()
        assert second.status() == "cancelled"
        first.result(timeout=120)
