"""The reference's own example models, unmodified, on this package.

Each example module of the reference is imported with ``xentica`` aliased to
``xentica_gb300`` (``xentica_gb300.alias``) -- exactly the file a reference
user has -- traced by our translator, compiled for the interpreter and run by
the NumPy executor of the GPU interpreter's semantics; its cells and colours
must equal what the reference's own generated kernels produce for the same
experiment (run through the oracle harness).  Needs the reference source, so
it is skipped where that is absent.
"""
import binascii
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

EXAMPLES = [  # model, experiment, overrides (smaller lattices that hold the seed areas), generations
    ("examples.game_of_life:GameOfLifeColor", "examples.game_of_life:GOLExperimentColor",
     {"size": [96, 64]}, 12),
    ("examples.shifting_sands:ShiftingSands", "examples.shifting_sands:ShiftingSandsExperiment",
     {"size": [424, 284]}, 10),
    ("examples.noisetv:NoiseTV", "examples.noisetv:NoiseTVExperiment", {"size": [64, 48]}, 5),
    ("examples.conserved_life:ConservedLife", "examples.conserved_life:BigBangExperiment", {}, 4),
    ("examples.gravicowboys:GraviCowboys", "examples.gravicowboys:GraviCowboysExperiment",
     {"size": [416, 196]}, 6),
    ("examples.evolife:EvoLife6D", "examples.evolife:EvoLife6DExperiment",
     {"size": [100, 100, 2, 2, 1, 1]}, 2),
]


def _reference_root():
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import ref_build
    root = ref_build.reference_root()
    if root is None or not os.path.isdir(os.path.join(root, "examples")):
        pytest.skip("reference source not available (set XK_REFERENCE_SRC)")
    return root


@pytest.mark.parametrize("model,exp,over,steps", EXAMPLES,
                         ids=[e[0].split(":")[1] for e in EXAMPLES])
def test_reference_example_runs_unmodified(model, exp, over, steps, tmp_path):
    root = _reference_root()
    from ref_harness import run_reference
    res = run_reference({"model": model, "experiment": exp, "exp_overrides": over,
                         "checkpoints": [steps], "workdir": str(tmp_path), "threads": 4,
                         "py_random_seed": 2041}, root)
    out = subprocess.run([sys.executable, os.path.join(HERE, "golden", "examples_ours.py"), root,
                          model, exp, json.dumps(over), str(steps), "2041"],
                         capture_output=True, text=True, timeout=900, cwd=str(tmp_path))
    assert out.returncode == 0, out.stderr[-3000:]
    ours = json.loads(out.stdout.strip().splitlines()[-1])
    assert ours["template"] == "VMTemplate"
    assert ours["init"] == binascii.crc32(res["init_cells"].tobytes()), "seeded state"
    assert ours["cells"] == binascii.crc32(res["cells_%d" % steps].tobytes()), "cells"
    assert ours["colors"] == binascii.crc32(res["colors_%d" % steps].tobytes()), "colours"
