"""GPU parity of the Life-like family through the public API.

Every fixture case (``tests/golden/golden.json``, produced by the reference's
own kernels) is replayed on the GPU: main-plane, colour and image checksums
must match at every checkpoint.  Random lattices are compared cell by cell
with the oracle after every step.  Bit-exact throughout.
"""
import binascii
import os

import numpy as np
import pytest

import oracle as O
from tests.models import (GameOfLife, GOLExperiment, LifelikeFixed, GOLExperiment2,
                          GameOfLifeStatic, build_from_job)
from tests.test_oracle import crc

pytestmark = pytest.mark.gpu


def _run_case(golden, case):
    entry = golden[case]
    job = entry["job"]
    model = build_from_job(job)
    viewport = job.get("render", {}).get("viewport")
    if viewport:
        model.set_viewport(tuple(viewport))
    assert crc(model.gpu.arrays.cells.get()[:model.cells_num]) == entry["init"]
    done = 0
    for cp in sorted(int(c) for c in entry["steps"]):
        while done < cp:
            model.step()
            done += 1
        exp_cp = entry["steps"][str(cp)]
        assert crc(model.gpu.arrays.cells.get()[:model.cells_num]) == exp_cp["cells"], \
            "%s: cells at step %d" % (case, cp)
        assert crc(model.gpu.arrays.colors.get()) == exp_cp["colors"], \
            "%s: colours at step %d" % (case, cp)
        if "img" in exp_cp:
            assert crc(model.render()) == exp_cp["img"], "%s: image at step %d" % (case, cp)


def _cases():
    import json
    with open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")) as fh:
        return sorted(json.load(fh))


@pytest.mark.parametrize("case", _cases())
def test_fixture_case(golden, case):
    _run_case(golden, case)


def test_reference_single_and_multiple():
    # reference tests/core/test_base.py:28-53
    m1, m2 = GameOfLife(GOLExperiment), GameOfLife(GOLExperiment)
    for _ in range(1000):
        m1.step()
        m2.step()
    for m in (m1, m2):
        assert binascii.crc32(m.gpu.arrays.cells.get()[:m.cells_num]) == 2981695958


def test_render_reference_golden():
    # reference tests/core/test_base.py:55-70
    exp = type("E", (GOLExperiment, ), {"zoom": 1})
    model = GameOfLife(exp)
    model.set_viewport(exp.size)
    for _ in range(1000):
        model.step()
    assert binascii.crc32(model.render() / 255) == 1955702083


def test_pause_and_save_load(tmp_path):
    # reference tests/core/test_base.py:72-118
    model = GameOfLife(GOLExperiment)
    before = crc(model.gpu.arrays.cells.get()[:model.cells_num])
    model.step()
    after = crc(model.gpu.arrays.cells.get()[:model.cells_num])
    assert before != after
    model.paused = True
    model.step()
    assert crc(model.gpu.arrays.cells.get()[:model.cells_num]) == after
    ca1 = GameOfLife(GOLExperiment)
    for _ in range(500):
        ca1.step()
    path = str(tmp_path / "test.ca")
    ca1.save(path)
    ca2 = GameOfLife(GOLExperiment)
    ca2.load(path)
    for _ in range(500):
        ca2.step()
    assert binascii.crc32(ca2.gpu.arrays.cells.get()[:ca2.cells_num]) == 2981695958
    from xentica_gb300.utils import compat
    with open(path, "rb") as fh:
        state = compat.load_state(fh)     # the pickle names the reference's classes
    assert set(state) == {"cells", "colors", "random"}


@pytest.mark.parametrize("seed", range(6))
def test_random_lattices_vs_oracle(seed):
    rng = np.random.RandomState(seed)
    w, h = int(rng.randint(1, 300)), int(rng.randint(1, 120))
    if seed == 5:
        w, h = 1100, 37          # wider than one CTA: global-memory kernel
    static = bool(seed % 2)
    rule = int(rng.randint(0, 2 ** 18))
    base = GameOfLifeStatic if static else LifelikeFixed
    if static:
        model_cls = base
        exp = type("E", (GOLExperiment2, ), {"size": (w, h), "word": "r%d" % seed})
        born, sustain = 8, 12
    else:
        model_cls = base
        exp = type("E", (GOLExperiment2, ), {"size": (w, h), "word": "r%d" % seed, "rule": rule})
        born, sustain = rule & 511, (rule >> 9) & 511
    model = model_cls(exp)
    topo = O.Topology((w, h), "moore", 1 if static else None)
    fld = topo.field(model.gpu.arrays.cells.get()[:model.cells_num], np.uint8)
    col = np.zeros(topo.cells * 3, dtype=np.int32)
    for step in range(12):
        model.step()
        O.life_run(topo, fld, col, 1, born=born, sustain=sustain)
        got = model.gpu.arrays.cells.get()[:model.cells_num]
        assert np.array_equal(got, fld[:topo.cells]), "step %d (%dx%d)" % (step + 1, w, h)
    assert np.array_equal(model.gpu.arrays.colors.get(), col)


def test_multi_step_equals_single_steps():
    exp = type("E", (GOLExperiment2, ), {"size": (200, 150)})
    a, b = GameOfLife(exp), GameOfLife(exp)
    for _ in range(64):
        a.step()
    b.gpu.step(64)
    assert np.array_equal(a.gpu.arrays.cells.get(), b.gpu.arrays.cells.get())


def test_headless_viewer_frames_vs_oracle(tmp_path):
    # the GUI loop of the reference without a window: key actions between
    # frames, speed generations per frame, nothing while paused
    from xentica_gb300.bridge.headless import HeadlessViewer, ppm_sink
    # its own experiment: moving the view edits ``pos`` in place, which is the
    # experiment class's list (as in the reference)
    model = GameOfLife(type("E", (GOLExperiment, ), {"pos": [0, 0]}))
    n = model.cells_num
    init = model.gpu.arrays.cells.get()[:n].copy()
    viewer = HeadlessViewer(model, (160, 90))
    frames = []
    keys = {2: ["]"], 4: ["="], 5: ["right", "up"], 7: ["spacebar"], 9: ["spacebar"],
            11: ["escape"]}
    sink = ppm_sink(str(tmp_path))
    drawn = viewer.run(20, keys, lambda i, img: (frames.append(img), sink(i, img)))
    assert drawn == 11 and model.timestep == 2 + 5 * 2 + 2 * 2
    topo = O.Topology(model.size)
    fld = topo.field(init, np.uint8)
    col = np.zeros(3 * n, np.int32)
    O.life_run(topo, fld, col, model.timestep)
    smooth = model.constants["SMOOTH_FACTOR"].value if model.is_constant("SMOOTH_FACTOR") else 0
    want = O.render(topo, col, 160, 90, zoom=model.zoom, dx=model.pos[0], dy=model.pos[1],
                    smooth=smooth)
    assert np.array_equal(frames[-1].ravel(), want.astype(np.uint8))
    assert len(os.listdir(str(tmp_path))) == 11


def test_shifting_sands_reference_golden():
    """Reference tests/core/test_base.py:182-189: ShiftingSands (the shifting
    family's template, every generation of the run in one gather) after 1000
    steps of model.step() and as one step(1000)."""
    from tests.models import ShiftingSands, ShiftingSandsExperiment
    a, b = ShiftingSands(ShiftingSandsExperiment), ShiftingSands(ShiftingSandsExperiment)
    assert type(a.gpu.template).__name__ == "ShiftTemplate"
    for _ in range(1000):
        a.step()
    b.gpu.step(1000)
    assert crc(a.gpu.arrays.cells.get()[:a.cells_num]) == 1639048270
    assert crc(b.gpu.arrays.cells.get()[:b.cells_num]) == 1639048270
    assert np.array_equal(a.gpu.arrays.colors.get(), b.gpu.arrays.colors.get())
