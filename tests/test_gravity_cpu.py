"""GraviCowboys on the CPU: the oracle pinned to the reference's own
kernels, the template choice, and the oracle against the interpreter's CPU
executor on random states (ties of gravity, energies near the 12-bit limit,
a static border)."""
import binascii

import numpy as np

import oracle as O
from tests import vm_cpu
from tests.models import GraviCowboys, GraviCowboysHalf, GraviCowboysStatic, GraviExperiment
from tests.test_vm_examples_cpu import load_case
from xentica_gb300 import _native as nat

STATIC = 3 | 0x3F000000 << 24


def test_oracle_reproduces_the_reference_kernels():
    """GraviCowboys of the reference's examples, seeded, run by its own
    generated kernels (checksums in tests/golden/vm_examples.npz) and by the
    oracle's restatement: the same cells and colours."""
    desc, _, c = load_case("GraviCowboys")
    size = [desc.size[i] for i in range(desc.ndim)]
    topo = O.Topology(size, "moore", None if desc.torus else desc.border_value)
    n = c["init"].size
    fld = topo.field(c["init"], np.uint64)
    col = np.ascontiguousarray(c["init_col"], dtype=np.int32).copy()
    O.gravity_run(topo, fld, col, int(c["steps"]),
                  color=O._color(True, desc.fade_in, desc.fade_out, desc.smooth))
    assert binascii.crc32(fld[:n].tobytes()) == int(c["cells_crc"])
    assert binascii.crc32(col.tobytes()) == int(c["colors_crc"])


def test_template_choice():
    for cls, family, torus in [(GraviCowboys, nat.XK_FAMILY_GRAVITY, 1),
                               (GraviCowboysStatic, nat.XK_FAMILY_GRAVITY, 0),
                               (GraviCowboysHalf, nat.XK_FAMILY_VM, 1)]:
        d = cls(GraviExperiment).gpu.template.descriptor()
        assert d.family == family, cls.__name__
        assert d.torus == torus
        assert d.state_bytes == 8
        assert d.color_kind == nat.XK_COLOR_MOVING_AVERAGE
    d = GraviCowboysStatic(GraviExperiment).gpu.template.descriptor()
    assert d.border_value == STATIC


def random_cells(n, seed, energies=4096):
    """Random energies and new energies, and gravities drawn from a few
    values so that ties between neighbours are common."""
    rng = np.random.RandomState(seed)
    grav = rng.choice(np.array([0.0, 0.5, 1.0, 1.5, 2.75, 1e-3], dtype=np.float32), n)
    grav = np.where(rng.random_sample(n) < 0.3, rng.random_sample(n).astype(np.float32) * 9, grav)
    bits = grav.astype(np.float32).view(np.uint32).astype(np.uint64)
    return (rng.randint(0, energies, n).astype(np.uint64) |
            rng.randint(0, 4096, n).astype(np.uint64) << np.uint64(12) | bits << np.uint64(24))


def test_oracle_matches_the_interpreter_semantics():
    """The oracle against the CPU executor of the traced programs, cell for
    cell, on a torus and inside a static border."""
    for cls, border in [(GraviCowboysStatic, STATIC), (GraviCowboys, None)]:
        for size in [(13, 7), (1, 5), (40, 3), (2, 2)]:
            exp = type("E", (GraviExperiment, ), {"size": size})
            model = cls(exp)
            n = model.cells_num
            cells = random_cells(n, n + (border is None))
            rng = np.random.RandomState(n)
            colors = rng.randint(-300, 300, 3 * n).astype(np.int32)
            topo = O.Topology(size, "moore", border)
            a = topo.field(cells, np.uint64)
            ca = colors.copy()
            O.gravity_run(topo, a, ca, 6, color=O._color(True, 255, 255, 1))
            b = np.zeros(n * 9 + 1, dtype=np.uint64)
            b[:n] = cells
            cb = colors.copy()
            vm_cpu.step(model, b, cb, 6)
            assert np.array_equal(a[:n], b[:n]), (cls.__name__, size)
            assert np.array_equal(ca, cb), (cls.__name__, size)
