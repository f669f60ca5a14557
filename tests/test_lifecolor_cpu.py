"""Colour Life (GameOfLifeColor) on the CPU: the oracle pinned to the
reference's own kernels, the template choice, and the oracle's static border
against the interpreter's CPU executor."""
import binascii

import numpy as np

import oracle as O
from tests import vm_cpu
from tests.models import (GameOfLifeColor, GameOfLifeColorStatic, GameOfLifeColorPlus2,
                          GOLColorExperiment)
from tests.test_vm_examples_cpu import load_case
from xentica_gb300 import _native as nat


def test_oracle_reproduces_the_reference_kernels():
    """GameOfLifeColor of the reference's examples, seeded, run by its own
    generated kernels (checksums in tests/golden/vm_examples.npz) and by the
    oracle's restatement: the same cells and colours."""
    desc, _, c = load_case("GameOfLifeColor")
    size = [desc.size[i] for i in range(desc.ndim)]
    topo = O.Topology(size, "moore", None if desc.torus else desc.border_value)
    n = c["init"].size
    fld = topo.field(c["init"], np.uint32)
    col = np.ascontiguousarray(c["init_col"], dtype=np.int32).copy()
    O.lifecolor_run(topo, fld, col, int(c["steps"]),
                    color=O._color(True, desc.fade_in, desc.fade_out, desc.smooth))
    assert binascii.crc32(fld[:n].tobytes()) == int(c["cells_crc"])
    assert binascii.crc32(col.tobytes()) == int(c["colors_crc"])


def test_template_choice():
    for cls, family, torus in [(GameOfLifeColor, nat.XK_FAMILY_LIFECOLOR, 1),
                               (GameOfLifeColorStatic, nat.XK_FAMILY_LIFECOLOR, 0),
                               (GameOfLifeColorPlus2, nat.XK_FAMILY_VM, 1)]:
        d = cls(GOLColorExperiment).gpu.template.descriptor()
        assert d.family == family, cls.__name__
        assert d.torus == torus
        assert (d.fade_in, d.fade_out, d.smooth) == (255, 10, 1)
        assert d.color_kind == nat.XK_COLOR_MOVING_AVERAGE
    d = GameOfLifeColorStatic(GOLColorExperiment).gpu.template.descriptor()
    assert d.border_value == 1 | 1 << 1 | 2 << 9 | 3 << 17


def test_oracle_static_border_matches_the_interpreter_semantics():
    """The oracle's off-board container (a live cell with colours 1, 2, 3)
    against the CPU executor of the traced programs, cell for cell."""
    for cls, border in [(GameOfLifeColorStatic, 1 | 1 << 1 | 2 << 9 | 3 << 17), (GameOfLifeColor, None)]:
        for size in [(13, 7), (1, 5), (40, 3)]:
            exp = type("E", (GOLColorExperiment, ), {"size": size})
            model = cls(exp)
            n = model.cells_num
            rng = np.random.RandomState(n + (border or 0) % 97)
            cells = ((rng.random_sample(n) < 0.5).astype(np.uint32) |
                     rng.randint(0, 1 << 24, n).astype(np.uint32) << np.uint32(1))
            colors = rng.randint(-300, 300, 3 * n).astype(np.int32)
            topo = O.Topology(size, "moore", border)
            a = topo.field(cells, np.uint32)
            ca = colors.copy()
            O.lifecolor_run(topo, a, ca, 6, color=O._color(True, 255, 10, 1))
            b = np.zeros(n * 9 + 1, dtype=np.uint32)
            b[:n] = cells
            cb = colors.copy()
            vm_cpu.step(model, b, cb, 6)
            assert np.array_equal(a[:n], b[:n]), (cls.__name__, size)
            assert np.array_equal(ca, cb), (cls.__name__, size)
