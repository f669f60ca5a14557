"""GPU parity of ``step_frames`` (``xk_step_frames``): generations each
followed by a rendered frame, as the reference's viewer loop calls ``step()``
then ``render()`` (``xentica/core/base.py:703-753``).

Every frame equals the ``render()`` of a twin model stepped one generation at
a time, for each kernel family (Life-like with history-free and with fading
colours, EvoLife, mass transfer, the shifting family, the interpreter) and
for host frames
(page-locked and pageable) and device frames; EvoLife frames are also checked
against the oracle's render after every generation.
"""
import numpy as np
import pytest

import oracle as O
from tests.models import (EvoLife, BigBangExperiment, FadeExperiment, GameOfLife,
                          GameOfLifeFade, GOLExperiment2, MassTransfer, MassExperiment,
                          ShiftingSands, ShiftingSandsExperiment)
from xentica_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _evolife(size):
    exp = type("E", (BigBangExperiment, ), {"size": size, "zoom": 1, "death_speed": 9,
                                            "max_genes": 7, "fade_in": 30, "fade_out": 7})
    for p in EvoLife.meta.__dict__.values():
        if hasattr(p, "default"):
            p.__set__(None, p.default)
    return EvoLife(exp, legacy_coloring=True)


def _random_evolife(model, seed):
    rng = np.random.RandomState(seed)
    n = model.cells_num
    energy = rng.randint(0, 300, n).astype(np.uint64)
    rule = rng.randint(0, 2 ** 18, n).astype(np.uint64) * (rng.random_sample(n) < 0.5)
    rnd = rng.randint(0, 2 ** 16, n).astype(np.uint64)
    cells = energy + (rule << np.uint64(9)) + (rnd << np.uint64(27))
    colors = rng.randint(0, 256, 3 * n).astype(np.int32)
    model.gpu.load(cells, colors)
    return cells, colors


def _on_interpreter(model_cls, exp):
    import os
    os.environ["XENTICA_GB300_TEMPLATE"] = "vm"
    try:
        return model_cls(exp)
    finally:
        del os.environ["XENTICA_GB300_TEMPLATE"]


def _twins(make, viewport, zoom, pos, load=None):
    a, b = make(), make()
    for m in (a, b):
        m.set_viewport(viewport)
        m.zoom = zoom
        m.pos = list(pos)
    if load:
        state = load(a)
        b.gpu.load(*state)
    return a, b


def _frames_by_step(model, nsteps):
    out = []
    for _ in range(nsteps):
        model.step()
        out.append(model.render())
    return np.stack(out)


CASES = {
    "life-history-free": (lambda: GameOfLife(GOLExperiment2), (200, 120), 2, (17, 5), None),
    "life-fading": (lambda: GameOfLifeFade(FadeExperiment), (61, 40), 1, (3, 2), None),
    "evolife": (lambda: _evolife((131, 103)), (131, 103), 1, (0, 0),
                lambda m: _random_evolife(m, 5)),
    "mass": (lambda: MassTransfer(type("E", (MassExperiment, ), {"size": (36, 20, 12)})),
             (36, 20), 1, (0, 0), None),
    # the whole lattice at zoom 1: the step kernel sums the column colours
    # itself (one atomic per column and run of planes); an odd width, and a
    # deep lattice whose columns are cut into many runs
    "mass-odd": (lambda: MassTransfer(type("E", (MassExperiment, ), {"size": (37, 21, 13)})),
                 (37, 21), 1, (0, 0), None),
    "mass-deep": (lambda: MassTransfer(type("E", (MassExperiment, ), {"size": (64, 48, 100)})),
                  (64, 48), 1, (0, 0), None),
    "mass-offset": (lambda: MassTransfer(type("E", (MassExperiment, ), {"size": (36, 20, 12)})),
                    (30, 20), 1, (2, 3), None),
    "shift": (lambda: ShiftingSands(ShiftingSandsExperiment), (160, 90), 3, (0, 0), None),
    "interpreter": (lambda: _on_interpreter(ShiftingSands, ShiftingSandsExperiment), (160, 90), 3,
                    (0, 0), None),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("where", ["pinned", "pageable", "device"])
def test_frames_equal_step_then_render(case, where):
    make, viewport, zoom, pos, load = CASES[case]
    a, b = _twins(make, viewport, zoom, pos, load)
    nsteps = 7       # more than the 4-frame ring
    want = _frames_by_step(b, nsteps)
    size = viewport[0] * viewport[1] * 3
    if where == "device":
        torch = pytest.importorskip("torch")
        dev = torch.zeros(nsteps * size, dtype=torch.uint8, device="cuda")
        a.gpu.step_frames(nsteps, viewport[0], viewport[1], zoom, pos[0], pos[1],
                          dev.data_ptr(), on_device=True)
        got = dev.cpu().numpy().reshape(nsteps, size)
    elif where == "pinned":
        buf = nat.PinnedBuffer(nsteps * size)
        got = a.step_frames(nsteps, out=buf.array[:nsteps * size].reshape(nsteps, size)).copy()
        buf.release()
    else:
        got = a.step_frames(nsteps)
    for g in range(nsteps):
        assert np.array_equal(got[g], want[g]), "%s frame %d" % (case, g)
    # the state continues from the same place
    assert np.array_equal(a.gpu.arrays.cells.get(), b.gpu.arrays.cells.get())
    assert np.array_equal(a.gpu.arrays.colors.get(), b.gpu.arrays.colors.get())
    if where != "device":           # the model-level call counts the generations
        assert a.timestep == b.timestep


def test_evolife_frames_match_oracle_render():
    model = _evolife((131, 103))
    model.set_viewport((131, 103))
    cells, colors = _random_evolife(model, 11)
    frames = model.step_frames(5)
    tpl = model.gpu.template
    info = tpl.color.extra
    topo = O.Topology(model.size)
    fld = topo.field(cells, np.uint64)
    col = colors.copy()
    for g in range(5):
        O.evolife_run(topo, fld, col, 1, death_speed=tpl.params["death_speed"],
                      max_genes=tpl.params["max_genes"], mutation_prob=tpl.params["mutation_prob"],
                      fade_in=info["fade_in"], fade_out=info["fade_out"], smooth=info["smooth"])
        smooth = model.constants["SMOOTH_FACTOR"].value \
            if model.is_constant("SMOOTH_FACTOR") else 0
        img = O.render(topo, col, 131, 103, smooth=smooth).astype(np.uint8)
        assert np.array_equal(frames[g], img), "frame %d" % g
