"""GPU parity of the colour Life kernel (GameOfLifeColor): the reference's
own checksums through the C-ABI, and random states, colours and frames
against the oracle (torus and static border, widths around the warp size)."""
import binascii
import ctypes

import numpy as np
import pytest

import oracle as O
from tests.models import GameOfLifeColor, GameOfLifeColorStatic, GOLColorExperiment
from tests.test_vm_examples_cpu import load_case
from xentica_gb300 import _native as nat

pytestmark = pytest.mark.gpu

STATIC = 1 | 1 << 1 | 2 << 9 | 3 << 17


def test_reference_checksums_through_the_c_abi():
    """The seeded GameOfLifeColor case of the reference's examples on the
    colour Life kernel (its descriptor with the family swapped): the cells
    and colours its own generated kernels reach."""
    desc, _, c = load_case("GameOfLifeColor")
    desc.family = nat.XK_FAMILY_LIFECOLOR
    lib = nat.load()
    h = ctypes.c_void_p()
    nat.check(lib.xk_model_create(ctypes.byref(desc), ctypes.byref(h)), "xk_model_create")
    try:
        init = np.ascontiguousarray(c["init"])
        n = init.size
        nat.check(lib.xk_upload(h, nat.ptr(init), n), "xk_upload")
        col0 = np.ascontiguousarray(c["init_col"], dtype=np.int32)
        nat.check(lib.xk_upload_colors(h, nat.ptr(col0), n), "xk_upload_colors")
        nat.check(lib.xk_step(h, int(c["steps"])), "xk_step")
        cells = np.empty_like(init)
        nat.check(lib.xk_download(h, nat.ptr(cells), n), "xk_download")
        col = np.empty(3 * n, dtype=np.int32)
        nat.check(lib.xk_download_colors(h, nat.ptr(col), n), "xk_download_colors")
    finally:
        lib.xk_model_destroy(h)
    assert binascii.crc32(cells.tobytes()) == int(c["cells_crc"])
    assert binascii.crc32(col.tobytes()) == int(c["colors_crc"])


def _random_model(cls, size, seed):
    exp = type("E", (GOLColorExperiment, ), {"size": size})
    model = cls(exp)
    assert type(model.gpu.template).__name__ == "LifeColorTemplate"
    n = model.cells_num
    rng = np.random.RandomState(seed)
    cells = ((rng.random_sample(n) < 0.4).astype(np.uint32) |
             rng.randint(0, 1 << 24, n).astype(np.uint32) << np.uint32(1))
    colors = rng.randint(-400, 400, 3 * n).astype(np.int32)
    model.gpu.load(cells, colors)
    return model, cells, colors


@pytest.mark.parametrize("size", [(96, 64), (33, 17), (1, 9), (200, 3), (31, 33), (1920, 1080)])
@pytest.mark.parametrize("cls,border", [(GameOfLifeColor, None), (GameOfLifeColorStatic, STATIC)])
def test_random_states_vs_oracle(cls, border, size):
    model, cells, colors = _random_model(cls, size, size[0] * 31 + size[1] + (border is None))
    n = model.cells_num
    topo = O.Topology(size, "moore", border)
    fld = topo.field(cells, np.uint32)
    col = colors.copy()
    done = 0
    for steps in (1, 4, 12):
        model.gpu.step(steps)
        O.lifecolor_run(topo, fld, col, steps, color=O._color(True, 255, 10, 1))
        done += steps
        assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n]), (size, done)
        assert np.array_equal(model.gpu.arrays.colors.get(), col), (size, done)


def test_frames_vs_oracle_render():
    """step_frames on the whole lattice at zoom 1 (the step kernel writes the
    frame) against the oracle's render of each generation's colours."""
    size = (160, 90)
    model, cells, colors = _random_model(GameOfLifeColor, size, 5)
    model.set_viewport(size)
    topo = O.Topology(size, "moore", None)
    fld = topo.field(cells, np.uint32)
    col = colors.copy()
    frames = model.step_frames(7)
    for g in range(7):
        O.lifecolor_run(topo, fld, col, 1, color=O._color(True, 255, 10, 1))
        img = O.render(topo, col, size[0], size[1], smooth=1).astype(np.uint8)
        assert np.array_equal(frames[g], img), g
