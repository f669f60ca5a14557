"""GPU parity of the noise kernel (NoiseTV): the reference's own checksums
through the C-ABI, and random states and colours against the oracle, one
generation per launch (frames) and many (up to 1024 per launch)."""
import binascii
import ctypes

import numpy as np
import pytest

import oracle as O
from tests.models import NoiseTV, NoiseTV3D, NoiseExperiment
from tests.test_vm_examples_cpu import load_case
from xentica_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def test_reference_checksums_through_the_c_abi():
    desc, _, c = load_case("NoiseTV")
    desc.family = nat.XK_FAMILY_NOISE
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


@pytest.mark.parametrize("cls,size", [(NoiseTV, (64, 48)), (NoiseTV, (333, 7)), (NoiseTV3D, (20, 9, 5))])
def test_random_states_vs_oracle(cls, size):
    exp = type("E", (NoiseExperiment, ), {"size": size})
    model = cls(exp)
    assert type(model.gpu.template).__name__ == "NoiseTemplate"
    n = model.cells_num
    rng = np.random.RandomState(n)
    cells = rng.randint(0, 65536, n).astype(np.uint16)          # 65535 (the seed's maximum) included
    cells[:3] = 65535
    colors = rng.randint(-600, 600, 3 * n).astype(np.int32)
    model.gpu.load(cells, colors)
    topo = O.Topology(size, "moore" if len(size) == 2 else "von_neumann", None if len(size) == 2 else 7)
    fld = topo.field(cells, np.uint16)
    col = colors.copy()
    for steps in (1, 3, 1500):
        model.gpu.step(steps)
        O.noise_run(topo, fld, col, steps, color=O._color(True, 40, 25, 1))
        assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n]), steps
        assert np.array_equal(model.gpu.arrays.colors.get(), col), steps


def test_frames_vs_oracle_render():
    size = (96, 40)
    exp = type("E", (NoiseExperiment, ), {"size": size})
    model = NoiseTV(exp)
    n = model.cells_num
    rng = np.random.RandomState(9)
    cells = rng.randint(0, 65535, n).astype(np.uint16)
    colors = rng.randint(0, 256, 3 * n).astype(np.int32)
    model.gpu.load(cells, colors)
    model.set_viewport(size)
    topo = O.Topology(size)
    fld = topo.field(cells, np.uint16)
    col = colors.copy()
    frames = model.step_frames(5)
    for g in range(5):
        O.noise_run(topo, fld, col, 1, color=O._color(True, 40, 25, 1))
        img = O.render(topo, col, size[0], size[1], smooth=1).astype(np.uint8)
        assert np.array_equal(frames[g], img), g
