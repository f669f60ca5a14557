"""GPU parity of the GraviCowboys kernel: the reference's own checksums
through the C-ABI, and random states (ties of gravity, energies near the
12-bit limit, gravities over most of the float range), colours and frames
against the oracle, on a torus and inside a static border."""
import binascii
import ctypes

import numpy as np
import pytest

import oracle as O
from tests.models import GraviCowboys, GraviCowboysStatic, GraviExperiment
from tests.test_gravity_cpu import STATIC, random_cells
from tests.test_vm_examples_cpu import load_case
from xentica_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def test_reference_checksums_through_the_c_abi():
    """The seeded GraviCowboys case of the reference's examples on the
    GraviCowboys kernel (its descriptor with the family swapped): the cells
    and colours its own generated kernels reach."""
    desc, _, c = load_case("GraviCowboys")
    desc.family = nat.XK_FAMILY_GRAVITY
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


def _model(cls, size, cells, seed):
    exp = type("E", (GraviExperiment, ), {"size": size})
    model = cls(exp)
    assert type(model.gpu.template).__name__ == "GravityTemplate"
    colors = np.random.RandomState(seed).randint(-400, 400, 3 * model.cells_num).astype(np.int32)
    model.gpu.load(cells, colors)
    return model, colors


def _run(cls, border, size, cells, seed, steps=(1, 4, 12)):
    model, colors = _model(cls, size, cells, seed)
    n = model.cells_num
    topo = O.Topology(size, "moore", border)
    fld = topo.field(cells, np.uint64)
    col = colors.copy()
    done = 0
    for k in steps:
        model.gpu.step(k)
        O.gravity_run(topo, fld, col, k, color=O._color(True, 255, 255, 1))
        done += k
        assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n]), (size, done)
        assert np.array_equal(model.gpu.arrays.colors.get(), col), (size, done)


@pytest.mark.parametrize("size", [(96, 64), (33, 17), (1, 9), (200, 3), (31, 33), (2, 2), (1920, 1080)])
@pytest.mark.parametrize("cls,border", [(GraviCowboys, None), (GraviCowboysStatic, STATIC)])
def test_random_states_vs_oracle(cls, border, size):
    seed = size[0] * 31 + size[1] + (border is None)
    _run(cls, border, size, random_cells(size[0] * size[1], seed), seed)


@pytest.mark.parametrize("cls,border", [(GraviCowboys, None), (GraviCowboysStatic, STATIC)])
def test_wide_float_range_vs_oracle(cls, border):
    """Gravities of random sign and exponent (|g| below 2^100, so no sum of
    eight overflows): the division by 8.008, the float sums and the colour
    conversion (negative, huge and subnormal values) exact."""
    size = (257, 121)
    n = size[0] * size[1]
    rng = np.random.RandomState(11)
    mant = rng.randint(0, 1 << 23, n).astype(np.uint32)
    expo = rng.randint(0, 127 + 100, n).astype(np.uint32)
    sign = rng.randint(0, 2, n).astype(np.uint32)
    bits = (sign << np.uint32(31) | expo << np.uint32(23) | mant).astype(np.uint64)
    cells = (rng.randint(0, 4096, n).astype(np.uint64) | rng.randint(0, 4096, n).astype(np.uint64) << np.uint64(12) |
             bits << np.uint64(24))
    _run(cls, border, size, cells, 12, steps=(1, 3))


def test_frames_vs_oracle_render():
    """step_frames on the whole lattice at zoom 1 (the step kernel writes the
    frame) against the oracle's render of each generation's colours."""
    size = (160, 90)
    cells = random_cells(size[0] * size[1], 5, energies=8)
    model, colors = _model(GraviCowboys, size, cells, 5)
    model.set_viewport(size)
    topo = O.Topology(size, "moore", None)
    fld = topo.field(cells, np.uint64)
    col = colors.copy()
    frames = model.step_frames(7)
    for g in range(7):
        O.gravity_run(topo, fld, col, 1, color=O._color(True, 255, 255, 1))
        img = O.render(topo, col, size[0], size[1], smooth=1).astype(np.uint8)
        assert np.array_equal(frames[g], img), g
