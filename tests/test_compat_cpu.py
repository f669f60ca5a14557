"""``save``/``load`` interoperate with the reference's pickles.

The reference pickles ``{"cells", "colors", "random"}`` with its own
``LocalRandom`` (``xentica/core/base.py:755-771``).  Our states must load in
the reference and the reference's in ours, cells, colours and both random
streams intact.  The cross checks run the reference itself through the oracle
harness when its source is present (they are skipped elsewhere).
"""
import os
import tempfile

import numpy as np
import pytest

import oracle as O
from tests.models import GameOfLife, GOLExperiment


def _draws(model):
    return int(model.random.standard.getrandbits(32)), model.random.numpy.randint(0, 2 ** 31 - 1, 4)


def test_round_trip_and_reference_class_path(tmp_path):
    a = GameOfLife(GOLExperiment)
    path = str(tmp_path / "state.pkl")
    a.save(path)
    raw = open(path, "rb").read()
    assert b"xentica.seeds.random" in raw and b"LocalRandom" in raw
    assert b"xentica_gb300" not in raw           # the reference can resolve every class
    want = _draws(a)
    b = GameOfLife(GOLExperiment)
    b.random.standard.getrandbits(64)            # move b's streams away first
    b.load(path)
    assert np.array_equal(b.gpu.arrays.cells.get(), a.gpu.arrays.cells.get())
    assert np.array_equal(b.gpu.arrays.colors.get(), a.gpu.arrays.colors.get())
    got = _draws(b)
    assert got[0] == want[0] and np.array_equal(got[1], want[1])


def _reference_root():
    import ref_build
    root = ref_build.reference_root()
    if root is None or not os.path.isdir(os.path.join(root, "xentica")):
        pytest.skip("reference source not available (set XK_REFERENCE_SRC)")
    return root


GOL = {"model": "examples.game_of_life:GameOfLife",
       "experiment": "examples.game_of_life:GOLExperiment", "threads": 4}


def test_reference_loads_our_state():
    root = _reference_root()
    from ref_harness import run_reference
    ours = GameOfLife(GOLExperiment)
    n = ours.cells_num
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "ours.pkl")
        ours.save(path)
        want = _draws(ours)
        res = run_reference(dict(GOL, load_pickle=path, checkpoints=[5], workdir=tmp), root)
    assert np.array_equal(res["loaded_cells"], ours.gpu.arrays.cells.get()[:n])
    assert np.array_equal(res["loaded_colors"], ours.gpu.arrays.colors.get())
    assert int(res["rng_standard"]) == want[0] and np.array_equal(res["rng_numpy"], want[1])
    # and continues from it exactly as the oracle does
    topo = O.Topology(ours.size)
    fld = topo.field(ours.gpu.arrays.cells.get()[:n], np.uint8)
    O.life_run(topo, fld, np.zeros(3 * n, np.int32), 5)
    assert np.array_equal(res["cells_5"], fld[:n])


def test_we_load_the_references_state():
    root = _reference_root()
    from ref_harness import run_reference
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "ref.pkl")
        res = run_reference(dict(GOL, checkpoints=[3], save_pickle=path, workdir=tmp), root)
        model = GameOfLife(GOLExperiment)
        model.load(path)
    n = model.cells_num
    assert np.array_equal(model.gpu.arrays.cells.get()[:n], res["cells_3"])
    assert np.array_equal(model.gpu.arrays.colors.get(), res["colors_3"])
    got = _draws(model)
    assert got[0] == int(res["rng_standard"]) and np.array_equal(got[1], res["rng_numpy"])
