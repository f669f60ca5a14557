"""Generate ``tests/golden/golden.json`` from the reference implementation.

Run in a checkout where the reference source is available::

    python tests/golden/make_golden.py /path/to/xentica-reference

Every case runs the reference's own ``CellularAutomaton.step()`` /
``render()`` with its translator-generated kernels compiled for the CPU
(``oracle/ref_harness.py``) and records CRC32 checksums: the initial main
plane (pins the seed streams), the main plane and colours at checkpoints, and
rendered images.  The fixtures are what the GPU tests compare against; they do
not need the reference at test time.
"""
import binascii
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ref_harness import run_reference  # noqa: E402

GOL = "examples.game_of_life"
REF_MODELS = "tests/golden/ref_models.py"   # relative to the repository root

# name -> job (see ref_harness.py for the keys)
CASES = {
    "gol_640x360": dict(model=GOL + ":GameOfLife", experiment=GOL + ":GOLExperiment",
                        exp_overrides={"zoom": 1}, checkpoints=[1, 10, 1000],
                        render={"viewport": [640, 360]}),
    "gol_zoom3_pos": dict(model=GOL + ":GameOfLife", experiment=GOL + ":GOLExperiment",
                          exp_overrides={"zoom": 3, "pos": [-7, 13]}, checkpoints=[40],
                          render={"viewport": [700, 300]}),
    "gol_static_640x360": dict(model=GOL + ":GameOfLifeStatic", experiment=GOL + ":GOLExperiment",
                               checkpoints=[1000]),
    "lifelike_diamoeba": dict(model=GOL + ":LifelikeCA", experiment=GOL + ":DiamoebaExperiment",
                              checkpoints=[1, 23, 24, 1000]),
    "gol6d_64x36": dict(model=GOL + ":GameOfLife6D", experiment=GOL + ":GOLExperiment2",
                        exp_overrides={"size": [64, 36, 3, 3, 3, 3], "zoom": 2},
                        checkpoints=[1, 1000], render={"viewport": [100, 50]}),
    "gol_int16": dict(model=REF_MODELS + ":GameOfLifeInt", experiment=GOL + ":GOLExperiment",
                      checkpoints=[1000]),
    "gol_color_fade": dict(model=REF_MODELS + ":GameOfLifeFade", experiment=REF_MODELS + ":FadeExperiment",
                           checkpoints=[1, 5, 60], render={"viewport": [50, 30]}),
    "gol_plain_color": dict(model=REF_MODELS + ":GameOfLifePlainColor",
                            experiment=GOL + ":GOLExperiment2",
                            exp_overrides={"size": [45, 29], "zoom": 1}, checkpoints=[3, 30],
                            render={"viewport": [45, 29]}),
    "gol3d_moore_static": dict(model=REF_MODELS + ":GameOfLife3DStatic",
                               experiment=GOL + ":GOLExperiment2",
                               exp_overrides={"size": [12, 10, 7]}, checkpoints=[1, 25],
                               render={"viewport": [12, 10]}),
}

EVO = "examples.evolife"
CASES.update({
    # reference tests/core/test_base.py:197-216 (colours compared as stored)
    "evolife_cross1_positional": dict(model=EVO + ":EvoLife", experiment=EVO + ":CrossbreedingExperiment",
                                      model_kwargs={"legacy_coloring": False}, checkpoints=[1, 100]),
    "evolife_cross2": dict(model=EVO + ":EvoLife", experiment=EVO + ":CrossbreedingExperiment2",
                           checkpoints=[1, 100], render={"viewport": [480, 270]},
                           exp_overrides={"zoom": 4, "pos": [100, 50]}),
    "evolife_bigbang_160x120": dict(model=EVO + ":EvoLife", experiment=EVO + ":BigBangExperiment",
                                    exp_overrides={"size": [160, 120], "zoom": 1},
                                    checkpoints=[1, 2, 10, 60], render={"viewport": [160, 120]}),
    "evolife_bigbang_mut_131x101": dict(model=EVO + ":EvoLife", experiment=EVO + ":BigBangExperiment",
                                        exp_overrides={"size": [131, 101], "mutation_prob": 0.05,
                                                       "death_speed": 7, "max_genes": 5,
                                                       "fade_in": 40, "fade_out": 11},
                                        model_kwargs={"legacy_coloring": False},
                                        checkpoints=[1, 5, 40]),
})

CASES.update({
    "mass_24x20x12": dict(model=REF_MODELS + ":MassTransfer", experiment=REF_MODELS + ":MassExperiment",
                          checkpoints=[1, 2, 10, 50], render={"viewport": [24, 20]}),
    "mass_37x5x64": dict(model=REF_MODELS + ":MassTransfer", experiment=REF_MODELS + ":MassExperiment",
                         exp_overrides={"size": [37, 5, 64], "word": "tall"}, checkpoints=[1, 7, 40],
                         render={"viewport": [40, 9]}),
    "mass_64cube": dict(model=REF_MODELS + ":MassTransfer", experiment=REF_MODELS + ":MassExperiment",
                        exp_overrides={"size": [64, 64, 64], "word": "cube", "zoom": 2, "pos": [3, -5]},
                        checkpoints=[1, 30], render={"viewport": [100, 90]}),
})

SANDS = "examples.shifting_sands"
CASES.update({
    "sands_640x360": dict(model=SANDS + ":ShiftingSands", experiment=SANDS + ":ShiftingSandsExperiment",
                          checkpoints=[1, 7, 100, 1000], render={"viewport": [640, 360]},
                          exp_overrides={"zoom": 1}),
    "sands_static_97x61": dict(model=REF_MODELS + ":ShiftingSandsStatic",
                               experiment=GOL + ":GOLExperiment2",
                               exp_overrides={"size": [97, 61], "word": "static sands"},
                               checkpoints=[1, 2, 30, 100]),
    "sands3d_vn_20x17x9": dict(model=REF_MODELS + ":ShiftingSands3D",
                               experiment=GOL + ":GOLExperiment2",
                               exp_overrides={"size": [20, 17, 9], "word": "sands 3d", "zoom": 1},
                               checkpoints=[1, 5, 64], render={"viewport": [20, 17]}),
    "sands_fade_80x50": dict(model=REF_MODELS + ":ShiftingSandsFade",
                             experiment=REF_MODELS + ":FadeExperiment",
                             exp_overrides={"size": [80, 50], "word": "fading sands"},
                             checkpoints=[1, 4, 33], render={"viewport": [80, 50]}),
})

# odd sizes, both borders: pins word-boundary and wrap handling
for w, h in [(1, 1), (1, 17), (17, 1), (2, 2), (31, 5), (32, 7), (33, 9), (63, 64), (64, 63),
             (65, 3), (100, 100), (1023, 5), (1024, 3), (1025, 4), (2000, 11), (3, 1200)]:
    for model in ("GameOfLife", "GameOfLifeStatic"):
        name = "%s_%dx%d" % ("gol" if model == "GameOfLife" else "static", w, h)
        CASES[name] = dict(model=GOL + ":" + model, experiment=GOL + ":GOLExperiment2",
                           exp_overrides={"size": [w, h], "word": "ODD %d %d" % (w, h)},
                           checkpoints=[1, 2, 7, 50])

for name, rule in [("highlife", "B36/S23"), ("seeds", "B2/S"), ("life_without_death", "B3/S012345678"),
                   ("b0_rule", "B0123/S45"), ("b8_rule", "B8/S8")]:
    CASES["rule_" + name] = dict(model=REF_MODELS + ":LifelikeFixed", experiment=GOL + ":GOLExperiment2",
                                 exp_overrides={"size": [77, 51], "word": name, "rule": rule},
                                 checkpoints=[1, 3, 20])


def crc(a):
    return binascii.crc32(a) & 0xFFFFFFFF


def main(ref_root):
    only = set(sys.argv[2:])
    out = {}
    path = os.path.join(HERE, "golden.json")
    if only and os.path.exists(path):
        with open(path) as fh:
            out = json.load(fh)
    for name, job in CASES.items():
        if only and name not in only:
            continue
        job = dict(job)
        job.setdefault("threads", os.cpu_count())
        job["workdir"] = os.path.join(ROOT, "oracle", "_ref")
        job["sys_path"] = [HERE]
        overrides = dict(job.get("exp_overrides", {}))
        if "rule" in overrides:
            sys.path.insert(0, os.path.join(ROOT))
            from xentica_gb300.tools.rules import LifeLike
            overrides["rule"] = LifeLike.golly2int(overrides["rule"])
            job["exp_overrides"] = overrides
        res = run_reference(job, ref_root)
        case = {"job": {k: v for k, v in job.items() if k not in ("workdir", "threads", "sys_path")},
                "cells_num": int(res["cells_num"]),
                "init": crc(res["init_cells"]), "steps": {}}
        for cp in job["checkpoints"]:
            entry = {"cells": crc(res["cells_%d" % cp]), "colors": crc(res["colors_%d" % cp])}
            if "img_%d" % cp in res:
                entry["img"] = crc(res["img_%d" % cp])
            case["steps"][str(cp)] = entry
        out[name] = case
        print(name, case["init"], json.dumps(case["steps"]), flush=True)
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    # usage: make_golden.py [reference checkout] [case ...]; without the
    # argument the checkout is $XK_REFERENCE_SRC or one named "reference"
    # beside this repository
    if len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import ref_build
        main(ref_build.reference_root(required=True))
