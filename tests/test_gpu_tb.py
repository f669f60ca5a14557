"""GPU parity of the temporally blocked 2-D Life-like kernel (``life_tb.cu``).

Lattices of many shapes -- widths not a multiple of 32, heights below one
tile, several tiles across and down -- on a torus and with static borders of
either state, stepped with every depth (generations per launch, forced with
``XK_TB``) for generation counts that are not multiples of the depth, against
the oracle; the tuned choice (no override) as well; and large requests of the
serving loop at its default depth.
"""
import numpy as np
import pytest

import oracle as O
from tests.models import GameOfLife, GameOfLifeStatic, GOLExperiment2, LifelikeFixed
from xentica_gb300 import core
from xentica_gb300.tools.rules import LifeLike

pytestmark = pytest.mark.gpu

SHAPES = [(64, 64), (70, 9), (100, 75), (1000, 70), (1030, 130), (2049, 131), (97, 600)]


def _model(shape, border, rule=None):
    if rule is not None:
        # a rule read from a table at run time (Conway's B3/S23 has its own
        # compiled rule form)
        exp = type("E", (GOLExperiment2, ), {"size": shape, "zoom": 1, "rule": rule})
        return LifelikeFixed(exp)
    if border == "torus":
        cls = GameOfLife
    else:
        state = 1 if border == "static1" else 0

        class Static(GameOfLife):
            class Topology(GameOfLife.Topology):
                border = core.StaticBorder(state)
        cls = Static
    exp = type("E", (GOLExperiment2, ), {"size": shape, "zoom": 1})
    return cls(exp)


def _run(shape, border, generations, seed):
    model = _model(shape, border)
    n = model.cells_num
    rng = np.random.RandomState(seed)
    cells = (rng.random_sample(n) < 0.4).astype(np.uint8)
    model.gpu.load(cells, np.zeros(3 * n, np.int32))
    model.gpu.step(generations)
    got = model.gpu.arrays.cells.get()[:n]
    kw = {} if border == "torus" else {"border": 1 if border == "static1" else 0}
    topo = O.Topology(shape, **kw)
    fld = topo.field(cells, np.uint8)
    O.life_run(topo, fld, np.zeros(3 * n, np.int32), generations)
    return got, fld[:n]


@pytest.mark.parametrize("depth", [2, 3, 5, 8])
@pytest.mark.parametrize("border", ["torus", "static0", "static1"])
@pytest.mark.parametrize("shape", SHAPES, ids=["%dx%d" % s for s in SHAPES])
def test_depth_matches_oracle(shape, border, depth, monkeypatch):
    monkeypatch.setenv("XK_TB", str(depth))
    got, want = _run(shape, border, 17, hash((shape, border, depth)) % 1000)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("shape", [(1500, 700), (4000, 300), (100, 75)])
def test_tuned_choice_matches_oracle(shape):
    got, want = _run(shape, "torus", 41, 7)
    assert np.array_equal(got, want)


def test_serving_large_requests_at_default_depth():
    from xentica_gb300 import serve
    rng = np.random.RandomState(3)
    shapes = [(700, 1500), (130, 2049), (1100, 300)]
    rules = [6152, int(rng.randint(0, 2 ** 18)), int(rng.randint(0, 2 ** 18))]
    with serve.Server(1 << 30, host_bytes=64 << 20, quantum=20) as srv:
        cells = [(rng.random_sample(s) < 0.35).astype(np.uint8) for s in shapes]
        hs = [srv.submit("life2d", c, r, 53) for c, r in zip(cells, rules)]
        for c, r, h, (hh, ww) in zip(cells, rules, hs, shapes):
            topo = O.Topology((ww, hh))
            fld = topo.field(c.ravel(), np.uint8)
            O.life_run(topo, fld, np.zeros(topo.cells * 3, np.int32), 53, born=r & 511,
                       sustain=r >> 9)
            assert np.array_equal(h.result(timeout=120).ravel(), fld[:topo.cells])


PLANS = {(512, 512): [[1, 0, 0, 0], [2, 16, 2, 0], [2, 4, 1, 0], [2, 8, 4, 0], [2, 16, 2, 1],
                      [2, 3, 4, 1], [2, 16, 4, 1], [2, 8, 1, 1], [2, 16, 4, 2], [2, 8, 4, 2],
                      [2, 16, 8, 0], [2, 16, 8, 2], [2, 8, 8, 2], [2, 16, 1, 3], [2, 4, 2, 3],
                      [2, 16, 4, 3], [2, 8, 8, 3], [3, 0, 0, 2], [3, 0, 0, 8]],
         (2049, 131): [[0, 0, 0, 0], [3, 0, 0, 4], [3, 0, 0, 7]]}


@pytest.mark.parametrize("rule", ["B3/S23", "B35678/S5678", "B36/S23"])
@pytest.mark.parametrize("shape", list(PLANS), ids=["%dx%d" % s for s in PLANS])
def test_every_plan_kind_matches_oracle(shape, rule):
    """Each launch plan the tuner can choose or the cache can re-apply
    (xk_model_set_plan): resident CTA, clusters of several sizes and bands,
    temporal blocking of several depths, the per-generation kernel -- the same
    cells as the oracle; plans that do not fit the lattice are refused.
    Conway's Life (the kernels with B3/S23 compiled in) and two rules read
    from a table at run time."""
    import ctypes
    from xentica_gb300 import _native as nat
    code = LifeLike.golly2int(rule)
    for plan in PLANS[shape]:
        model = _model(shape, "torus") if rule == "B3/S23" else _model(shape, "torus", code)
        n = model.cells_num
        cells = (np.random.RandomState(sum(plan)).random_sample(n) < 0.4).astype(np.uint8)
        model.gpu.load(cells, np.zeros(3 * n, np.int32))
        model.gpu._ensure()
        model.gpu._planned = True          # no tuning: the plan under test
        arr = (ctypes.c_int32 * 4)(*plan)
        nat.check(model.gpu._lib.xk_model_set_plan(model.gpu._handle, arr), "xk_model_set_plan")
        out = (ctypes.c_int32 * 4)()
        nat.check(model.gpu._lib.xk_model_plan(model.gpu._handle, out), "xk_model_plan")
        assert list(out) == plan
        assert model.gpu._lib.xk_model_rule_form(model.gpu._handle) == (rule == "B3/S23")
        model.gpu.step(29)
        topo = O.Topology(shape)
        fld = topo.field(cells, np.uint8)
        O.life_run(topo, fld, np.zeros(3 * n, np.int32), 29, born=code & 511, sustain=code >> 9)
        assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n]), "plan %s" % plan
    bad = {(512, 512): [[0, 0, 0, 0], [3, 0, 0, 9], [2, 17, 1, 0], [5, 0, 0, 0], [2, 16, 2, 2],
                        [2, 16, 3, 1], [2, 3, 1, 1], [2, 3, 4, 2], [2, 16, 4, 4], [2, 16, 8, 1],
                        [2, 3, 8, 2], [2, 3, 4, 3], [2, 3, 2, 3], [2, 16, 3, 3]],
           (2049, 131): [[1, 0, 0, 0], [2, 4, 1, 0], [3, 0, 0, 1]]}[shape]
    model = _model(shape, "torus")
    model.gpu._ensure()
    for plan in bad:
        arr = (ctypes.c_int32 * 4)(*plan)
        assert model.gpu._lib.xk_model_set_plan(model.gpu._handle, arr) != 0, plan


def test_plan_cache_round_trip(monkeypatch, tmp_path):
    """A model's tuned plan is stored; a second model of the same lattice
    takes it from the cache and steps to the oracle's cells."""
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "tune.json"))
    shape = (1500, 700)
    first = _model(shape, "torus")
    first.gpu.step(1)
    import json
    stored = list(json.loads((tmp_path / "tune.json").read_text()).values())
    assert stored == [first.gpu.plan]
    got, want = _run(shape, "torus", 23, 5)
    assert np.array_equal(got, want)
