"""Make ``tests/golden/vm_examples.npz``: the reference's example models as
interpreter bytecode, with the reference's own results.

Test infrastructure.  ``python tests/golden/make_vm_fixtures.py <reference
root>`` runs each case of ``ref_examples.py`` twice:

* through the oracle harness (``oracle/ref_harness.py``): the reference's
  translator and its generated kernels, compiled for the CPU -- the initial
  state and the state and colours after the case's generations;
* in a child process with ``xentica`` aliased to xentica_gb300: our translator
  traces the same unmodified example model, ``core/vm.py`` compiles it, and
  the NumPy executor (``tests/vm_cpu.py``) must reproduce the reference.

The archive keeps, per case, the model descriptor, both programs, the initial
cells and colours and the reference's checksums; the GPU test replays the
bytecode on the interpreter kernel without needing the example sources.
"""
import binascii
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CHILD = r'''
import importlib, json, os, sys, random
a = json.loads(sys.argv[1])
sys.path.insert(0, a["root"])
import xentica_gb300.alias
xentica_gb300.alias.install()
sys.path.insert(1, a["ref"])
sys.path.insert(1, a["here"])
import numpy as np
from xentica_gb300.core import vm
from tests import vm_cpu
random.seed(2041)
import ref_examples
mod, cls = a["model"].split(":")
model_cls = getattr(importlib.import_module(mod), cls)
os.environ["XENTICA_GB300_TEMPLATE"] = "vm"
model = model_cls(getattr(ref_examples, a["exp"]))
tpl = model.gpu.template
n = model.cells_num
fld = np.zeros(n * (len(model.buffers) + 1) + 1, dtype=model.main.dtype)
fld[:n] = model.gpu.arrays.cells.get()[:n]
col = model.gpu.arrays.colors.get().astype(np.int32)
init, init_col = fld[:n].copy(), col.copy()
vm_cpu.step(model, fld, col, a["steps"])
desc = tpl.descriptor()
vals = [vm.pack_value(model.meta.__dict__[nm].value, vm.ir.ctype_of(model.meta.__dict__[nm].ctype))
        for nm in tpl.param_names]
out = {"desc": np.frombuffer(bytes(desc), dtype=np.uint8),
       "init": init, "init_col": init_col, "cells": fld[:n].copy(), "colors": col,
       "params": np.array(vals, dtype=np.uint64)}
for which, prog in zip(("emit", "absorb"), tpl.programs):
    out[which + "_code"] = prog.code
    out[which + "_consts"] = prog.consts
    out[which + "_nregs"] = np.int64(prog.nregs)
np.savez(a["out"], **out)
'''


def main():
    ref = sys.argv[1]
    sys.path.insert(0, HERE)
    from ref_harness import run_reference
    import ref_examples_cases
    archive = {}
    for name, model, exp, steps in ref_examples_cases.CASES:
        with tempfile.TemporaryDirectory() as tmp:
            res = run_reference({"model": model, "experiment": "ref_examples:" + exp,
                                 "checkpoints": [steps], "workdir": tmp, "threads": 4,
                                 "py_random_seed": 2041, "sys_path": [HERE]}, ref)
            out = os.path.join(tmp, "ours.npz")
            args = {"root": ROOT, "ref": ref, "here": HERE, "model": model, "exp": exp,
                    "steps": steps, "out": out}
            subprocess.run([sys.executable, "-c", CHILD, json.dumps(args)], check=True, cwd=tmp)
            with np.load(out) as ours:
                ours = {k: ours[k] for k in ours.files}
        assert np.array_equal(ours["init"], res["init_cells"]), "%s: seeded state" % name
        assert np.array_equal(ours["cells"], res["cells_%d" % steps]), "%s: cells" % name
        assert np.array_equal(ours["colors"], res["colors_%d" % steps]), "%s: colours" % name
        for key in ("desc", "init", "init_col", "params", "emit_code", "emit_consts",
                    "emit_nregs", "absorb_code", "absorb_consts", "absorb_nregs"):
            archive["%s__%s" % (name, key)] = ours[key]
        archive["%s__steps" % name] = np.int64(steps)
        archive["%s__cells_crc" % name] = np.int64(binascii.crc32(res["cells_%d" % steps].tobytes()))
        archive["%s__colors_crc" % name] = np.int64(binascii.crc32(res["colors_%d" % steps].tobytes()))
        print(name, "ok", ours["init"].size, "cells")
    np.savez_compressed(os.path.join(HERE, "vm_examples.npz"), **archive)


if __name__ == "__main__":
    main()
