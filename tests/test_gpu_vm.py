"""GPU parity of the generic interpreter kernel.

Every fixture of ``tests/golden/golden.json`` (checksums of the reference's own
kernels) is replayed with ``XENTICA_GB300_TEMPLATE=vm``, i.e. on the
interpreter instead of the hand-written family kernels: cells, colours and
images at every checkpoint, bit-exact.
"""
import numpy as np
import pytest

from tests.test_gpu_life import _cases, _run_case
from tests.models import GameOfLife, GOLExperiment

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", _cases())
def test_fixture_case_on_the_interpreter(golden, case, monkeypatch):
    monkeypatch.setenv("XENTICA_GB300_TEMPLATE", "vm")
    _run_case(golden, case)


def test_interpreter_is_chosen(monkeypatch):
    monkeypatch.setenv("XENTICA_GB300_TEMPLATE", "vm")
    model = GameOfLife(GOLExperiment)
    assert type(model.gpu.template).__name__ == "VMTemplate"
    monkeypatch.delenv("XENTICA_GB300_TEMPLATE")
    assert type(GameOfLife(GOLExperiment).gpu.template).__name__ == "LifeTemplate"


def test_malformed_bytecode_is_rejected():
    # every instruction is checked before it reaches the GPU: registers,
    # constant and parameter slots, planes, neighbours, opcodes
    import ctypes
    from xentica_gb300 import _native as nat
    from xentica_gb300.core import vm
    from xentica_gb300.core.exceptions import XenticaException
    import os
    os.environ["XENTICA_GB300_TEMPLATE"] = "vm"
    try:
        model = GameOfLife(GOLExperiment)
        model.gpu.step(1)                        # creates the device model
    finally:
        del os.environ["XENTICA_GB300_TEMPLATE"]
    lib, h = model.gpu._lib, model.gpu._handle
    good = model.gpu.template.programs[1]
    consts = good.consts

    def load(code, nregs=good.nregs):
        code = np.ascontiguousarray(code, dtype=vm.INS_DTYPE)
        return lib.xk_vm_load(h, 1, nat.ptr(code), len(code), nat.ptr(consts), len(consts), nregs)

    def ins(op, ty=3, dst=0, a=0, b=0, c=0):
        return np.array([(op, ty, dst, a, b, c, 0)], dtype=vm.INS_DTYPE)

    assert load(good.code) == 0
    bad = [ins(vm.OP["const"], dst=good.nregs),            # register past the file
           ins(vm.OP["const"], a=len(consts)),             # constant slot
           ins(vm.OP["param"], a=64),                      # parameter slot
           ins(vm.OP["load"], a=3, b=8, c=1),              # neighbour 8 of 0..7
           ins(vm.OP["load"], a=0, c=10),                  # plane 10 of 9
           ins(vm.OP["store"], a=0, b=10),                 # plane 10 of 9
           ins(vm.OP["cvt"], b=9),                         # unknown source type
           ins(99)]                                        # unknown opcode
    for code in bad:
        assert load(code) == nat.XK_ERR_ARG
    assert load(good.code, nregs=257) == nat.XK_ERR_ARG
    # the model still steps with its own programs
    assert load(good.code) == 0
    model.step()
