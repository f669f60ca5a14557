"""The reference's own example models on the GPU interpreter kernel.

``tests/golden/vm_examples.npz`` (made by ``make_vm_fixtures.py``) holds, for
GameOfLifeColor, ShiftingSands, NoiseTV, ConservedLife, GraviCowboys and
EvoLife6D of the reference's ``examples`` package: our translator's compiled
emit/absorb programs of the unmodified example, the model descriptor, a
seeded initial state and the checksums the reference's own generated kernels
reach after some generations.  Here the stored bytecode alone is replayed by
the NumPy executor; ``test_gpu_vm_examples`` replays it on the GPU kernel.
"""
import binascii
import os

import numpy as np
from xentica_gb300 import _native as nat

HERE = os.path.dirname(os.path.abspath(__file__))
ARCHIVE = os.path.join(HERE, "golden", "vm_examples.npz")


def _cases():
    with np.load(ARCHIVE) as data:
        return sorted({k.split("__")[0] for k in data.files})


def load_case(name):
    with np.load(ARCHIVE) as data:
        c = {k.split("__")[1]: data[k] for k in data.files if k.startswith(name + "__")}
    desc = nat.XkDesc.from_buffer_copy(c["desc"].tobytes())
    programs = [(c[w + "_code"], c[w + "_consts"], int(c[w + "_nregs"])) for w in ("emit", "absorb")]
    return desc, programs, c


def test_archive_replays_on_the_cpu_executor():
    # the stored bytecode alone (no example source) reproduces the
    # reference's checksums with the NumPy executor
    from tests import vm_cpu
    for name in _cases():
        desc, programs, c = load_case(name)
        n = c["init"].size
        fld = np.zeros(n * (desc.nbr + 1) + 1, dtype=c["init"].dtype)
        fld[:n] = c["init"]
        col = c["init_col"].copy()
        vm_cpu.replay(desc, programs, c["params"], fld, col, int(c["steps"]))
        assert binascii.crc32(fld[:n].tobytes()) == int(c["cells_crc"]), name
        assert binascii.crc32(col.tobytes()) == int(c["colors_crc"]), name


def test_optimised_archive_replays_on_the_cpu_executor():
    """The stored bytecode after the compiler's straight-line optimisation
    (value numbering, constant conversions folded, dead values dropped,
    registers re-allocated): fewer instructions, the same checksums."""
    from tests import vm_cpu
    from xentica_gb300.core import vm
    for name in _cases():
        desc, programs, c = load_case(name)
        opt = []
        for code, consts, nregs in programs:
            o_code, o_consts, o_nregs = vm.optimize(code, consts)
            assert len(o_code) <= len(code) and o_nregs <= max(nregs, 1)
            opt.append((o_code, o_consts, o_nregs))
        n = c["init"].size
        fld = np.zeros(n * (desc.nbr + 1) + 1, dtype=c["init"].dtype)
        fld[:n] = c["init"]
        col = c["init_col"].copy()
        vm_cpu.replay(desc, opt, c["params"], fld, col, int(c["steps"]))
        assert binascii.crc32(fld[:n].tobytes()) == int(c["cells_crc"]), name
        assert binascii.crc32(col.tobytes()) == int(c["colors_crc"]), name
