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


def test_folding_matches_the_executor_on_edge_values():
    """Every integer binary operation and type, on constant operands chosen at
    the edges (0, 1, -1, the extremes, shift counts at and past the width,
    division by zero), folded by the optimiser and run unfolded by the CPU
    executor: the same stored register images.  Identities are checked with
    one operand loaded from the lattice, so they cannot fold away."""
    from tests import vm_cpu
    from xentica_gb300.core import vm
    OP, INS = vm.OP, vm.INS_DTYPE
    edges = {3: [0, 1, -1, 2, -7, 31, 32, 33, 2 ** 31 - 1, -2 ** 31],
             4: [0, 1, 2, 7, 31, 32, 33, 2 ** 32 - 1, 2 ** 31],
             5: [0, 1, -1, -7, 63, 64, 65, 2 ** 63 - 1, -2 ** 63],
             6: [0, 1, 7, 63, 64, 65, 2 ** 64 - 1, 2 ** 63]}
    ops = [OP[k] for k in ("+", "-", "*", "/", "%", "&", "|", "^", "<<", ">>",
                           "<", "<=", ">", ">=", "==", "!=")]
    lat = vm_cpu.Lattice(size=(2, ), deltas=[], torus=True)
    for ty, vals in edges.items():
        ctype = vm.ir.ctype_of(vm._CODE_TYPES[ty])
        images = [vm.pack_value(v, ctype) for v in vals]
        code, consts = [], list(images)
        out = 0
        for op in ops:
            for i in range(len(images)):
                for j in range(len(images)):
                    # r0 = const i, r1 = const j, r2 = r0 op r1, stored to plane out + 1
                    code += [(OP["const"], ty, 0, i, 0, 0, 0), (OP["const"], ty, 1, j, 0, 0, 0),
                             (op, ty, 2, 0, 1, 0, 0), (OP["store"], 6, 0, 2, out + 1, 0, 0)]
                    out += 1
            # identities: the lattice value (plane 0) with 0 and 1
            for k, c in enumerate((0, 1)):
                for left in (False, True):
                    code += [(OP["load"], 6, 0, 0, 0, 0, 0), (OP["cvt"], ty, 1, 0, 6, 0, 0),
                             (OP["const"], ty, 2, images.index(vm.pack_value(c, ctype)), 0, 0, 0)]
                    code += [(op, ty, 3, 2, 1, 0, 0) if left else (op, ty, 3, 1, 2, 0, 0),
                             (OP["store"], 6, 0, 3, out + 1, 0, 0)]
                    out += 1
        code = np.array(code, dtype=INS)
        consts = np.array(consts, dtype=np.uint64)
        results = []
        for prog in ((code, consts, 4), vm.optimize(code, consts)):
            fld = np.zeros(lat.n * (out + 1), dtype=np.uint64)
            fld[:lat.n] = [vm.pack_value(-3, ctype), vm.pack_value(5, ctype)]
            vm_cpu.run(vm.VmProgram(prog[0], prog[1], prog[2], [], False), fld,
                       np.zeros(3 * lat.n, dtype=np.int32), lat, 8, [], None)
            results.append(fld)
        assert len(vm.optimize(code, consts)[0]) < len(code)
        assert np.array_equal(results[0], results[1]), ty
