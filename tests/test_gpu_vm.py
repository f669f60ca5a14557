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
