"""Run one of the reference's example models, unmodified, on xentica_gb300.

Test infrastructure: ``python examples_ours.py <reference root> <module:Class>
<module:Experiment> <json overrides> <steps> <python random seed>`` imports the example module
from the reference's ``examples`` package with ``xentica`` aliased to this
package (``xentica_gb300.alias``), builds the model, runs ``steps``
generations of its compiled interpreter programs with the NumPy executor
(``tests/vm_cpu.py``, the GPU interpreter's semantics) and prints the CRC-32
of the initial and final main plane and colours as JSON.
"""
import binascii
import importlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    ref_root, model_path, exp_path, overrides, steps, py_seed = sys.argv[1:7]
    import random
    random.seed(int(py_seed))             # as the harness does before importing
    sys.path.insert(0, ROOT)
    import xentica_gb300.alias
    xentica_gb300.alias.install()
    sys.path.insert(1, ref_root)          # for the reference's "examples" package only
    import numpy as np
    from tests import vm_cpu

    def load(path):
        mod, name = path.split(":")
        return getattr(importlib.import_module(mod), name)

    model_cls, exp_cls = load(model_path), load(exp_path)
    over = json.loads(overrides)
    if "size" in over:
        over["size"] = tuple(over["size"])
    if over:
        exp_cls = type("Overridden", (exp_cls, ), over)
    os.environ["XENTICA_GB300_TEMPLATE"] = "vm"
    model = model_cls(exp_cls)
    n = model.cells_num
    fld = np.zeros(n * (len(model.buffers) + 1) + 1, dtype=model.main.dtype)
    fld[:n] = model.gpu.arrays.cells.get()[:n]
    col = model.gpu.arrays.colors.get().astype(np.int32)
    init = binascii.crc32(fld[:n].tobytes())
    vm_cpu.step(model, fld, col, int(steps))
    print(json.dumps({"init": init, "cells": binascii.crc32(fld[:n].tobytes()),
                      "colors": binascii.crc32(col.tobytes()),
                      "module": type(sys.modules["xentica.core"]).__name__,
                      "template": type(model.gpu.template).__name__}))


if __name__ == "__main__":
    main()
