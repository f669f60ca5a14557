"""Per-cell noise (NoiseTV) on the CPU: the oracle pinned to the reference's
own kernels, and the template choice."""
import binascii

import numpy as np

import oracle as O
from tests.models import NoiseTV, NoiseTV3D, NoiseExperiment
from tests.test_vm_examples_cpu import load_case
from xentica_gb300 import _native as nat


def test_oracle_reproduces_the_reference_kernels():
    """NoiseTV of the reference's examples, seeded, run by its own generated
    kernels (checksums in tests/golden/vm_examples.npz) and by the oracle's
    restatement: the same cells and colours."""
    desc, _, c = load_case("NoiseTV")
    size = [desc.size[i] for i in range(desc.ndim)]
    topo = O.Topology(size, "moore", None if desc.torus else desc.border_value)
    n = c["init"].size
    fld = topo.field(c["init"], np.uint16)
    col = np.ascontiguousarray(c["init_col"], dtype=np.int32).copy()
    O.noise_run(topo, fld, col, int(c["steps"]),
                color=O._color(True, desc.fade_in, desc.fade_out, desc.smooth))
    assert binascii.crc32(fld[:n].tobytes()) == int(c["cells_crc"])
    assert binascii.crc32(col.tobytes()) == int(c["colors_crc"])


def test_template_choice():
    for cls, ndim in [(NoiseTV, 2), (NoiseTV3D, 3)]:
        exp = type("E", (NoiseExperiment, ), {"size": (20, 10, 6)[:ndim]})
        d = cls(exp).gpu.template.descriptor()
        assert d.family == nat.XK_FAMILY_NOISE, cls.__name__
        assert d.ndim == ndim and d.state_bytes == 2
        assert (d.fade_in, d.fade_out, d.smooth) == (40, 25, 1)
        assert d.color_kind == nat.XK_COLOR_MOVING_AVERAGE
