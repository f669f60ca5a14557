"""Pins the CPU oracle (``oracle/oracle.c``) to the reference.

The reference's own golden checksums (its ``tests/core/test_base.py``) and the
fixtures in ``tests/golden/golden.json`` (made by running the reference's
generated kernels, see ``make_golden.py``) are reproduced by the oracle from
initial states seeded by xentica_gb300 -- which also pins the seed streams.
"""
import binascii

import numpy as np
import pytest

import oracle as O
from tests.models import build_from_job
from xentica_gb300.core.topology.border import StaticBorder
from xentica_gb300.core.topology.neighborhood import VonNeumannNeighborhood
from xentica_gb300.tools.rules import LifeLike


def crc(a):
    return binascii.crc32(np.ascontiguousarray(a)) & 0xFFFFFFFF


def oracle_setup(job):
    """(topology, fld, col, model) for a fixture job, seeded by our API."""
    model = build_from_job(job)
    border = model.topology.border
    kind = "vonneumann" if isinstance(model.topology.neighborhood, VonNeumannNeighborhood) else "moore"
    topo = O.Topology(model.size, kind, border.value if isinstance(border, StaticBorder) else None)
    main = model.gpu.arrays.cells.get()[:model.cells_num]
    fld = topo.field(main, model.main.dtype)
    col = np.zeros(model.cells_num * 3, dtype=np.int32)
    return topo, fld, col, model


# colour of state 0 / state 1 of each fixture model's color(), written out
LUTS = {"GameOfLifeFade": (0, 10, 250, 200, 110, 0),
        "GameOfLifePlainColor": (0, 0, 7, 255, 3, 7)}


def shift_params(model):
    """(plane0, lut) of a ShiftingSands-style model for ``oracle.shift_run``:
    the plane its emit writes the state into, and the colour of every sum
    0..N of the neighbours' buffers, both from evaluating the traced
    programs."""
    from xentica_gb300.core import ir
    n = len(model.buffers)
    one = np.array([1], dtype=np.uint64)
    ev = ir.evaluate(model.programs["emit"], {("main", -1): one}, lanes=1)
    plane0 = [key[1] for key, v in ev.stores.items() if int(v[0]) & 1]
    assert len(plane0) == 1
    lanes = np.arange(n + 1, dtype=np.uint64)
    inputs = {("main", -1): np.zeros(n + 1, dtype=np.uint64)}
    for k in range(n):
        inputs[("nbuf", k)] = (lanes > np.uint64(k)).astype(np.uint64)
    ev = ir.evaluate(model.programs["absorb"], inputs, lanes=n + 1)
    rgb = ev.color[0]
    return plane0[0], [int(rgb[c][v]) for v in range(n + 1) for c in range(3)]


def life_params(model):
    tpl = model.gpu.template
    info = tpl.color.extra if tpl.color is not None else {"kind": "none"}
    color = O._color(info["kind"] == "moving_average", info.get("fade_in", 255),
                     info.get("fade_out", 255), info.get("smooth", 1))
    return tpl, color


REFERENCE_GOLDENS = [
    # (fixture case, steps, reference checksum, reference test file:line)
    ("gol_640x360", 1000, 2981695958),        # tests/core/test_base.py:41
    ("gol_static_640x360", 1000, 1098273940),  # tests/core/test_base.py:147
    ("lifelike_diamoeba", 1000, 4016906756),   # tests/core/test_base.py:225
    ("gol6d_64x36", 1000, 2742543959),         # tests/core/test_base.py:168
]


@pytest.mark.parametrize("case,steps,expected", REFERENCE_GOLDENS)
def test_oracle_reference_goldens(golden, case, steps, expected):
    job = golden[case]["job"]
    topo, fld, col, model = oracle_setup(job)
    assert crc(fld[:topo.cells]) == golden[case]["init"]
    tpl, color = life_params(model)
    schedule = None
    if case == "lifelike_diamoeba":
        rule = LifeLike.golly2int("B3/S23")
        schedule = {23: (rule & 511, (rule & 511) | (rule >> 9))}
    O.life_run(topo, fld, col, steps, born=tpl.rule0, sustain=tpl.rule1, color=color,
               rule_schedule=schedule)
    assert crc(fld[:topo.cells]) == expected


def test_oracle_shifting_sands_golden(golden):
    # reference tests/core/test_base.py:182-189: ShiftingSands after 1000 steps
    topo, fld, col, model = oracle_setup(golden["sands_640x360"]["job"])
    assert crc(fld[:topo.cells]) == golden["sands_640x360"]["init"]
    plane0, lut = shift_params(model)
    O.shift_run(topo, fld, col, 1000, plane0, lut, color=life_params(model)[1])
    assert crc(fld[:topo.cells]) == 1639048270


def test_oracle_render_golden(golden):
    # reference tests/core/test_base.py:55-70: crc32(img / 255) == 1955702083
    topo, fld, col, model = oracle_setup(golden["gol_640x360"]["job"])
    tpl, color = life_params(model)
    O.life_run(topo, fld, col, 1000, born=tpl.rule0, sustain=tpl.rule1, color=color)
    img = O.render(topo, col, 640, 360, zoom=1).astype(np.uint8)
    assert binascii.crc32(img / 255) == 1955702083


def _fixture_cases(golden_json):
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")) as fh:
        data = json.load(fh)
    return sorted(k for k, v in data.items()
                  if v["cells_num"] <= 200000 and "lifelike" not in k and "evolife" not in k)


@pytest.mark.parametrize("case", _fixture_cases(None))
def test_oracle_fixtures(golden, case):
    entry = golden[case]
    job = entry["job"]
    topo, fld, col, model = oracle_setup(job)
    assert crc(fld[:topo.cells]) == entry["init"]
    tpl, color = life_params(model) if type(model).__name__ != "MassTransfer" else (None, None)
    done = 0
    axes = model.renderer.projection_axes
    smooth = model.constants["SMOOTH_FACTOR"].value if model.is_constant("SMOOTH_FACTOR") else 0
    for cp in sorted(int(c) for c in entry["steps"]):
        if type(model).__name__ == "MassTransfer":
            O.mass_run(topo, fld, col, cp - done)
        elif type(model).__name__.startswith("ShiftingSands"):
            plane0, lut = shift_params(model)
            O.shift_run(topo, fld, col, cp - done, plane0, lut, color=color)
        else:
            O.life_run(topo, fld, col, cp - done, born=tpl.rule0, sustain=tpl.rule1, color=color,
                       bits=model.main.properties["state"].bit_width,
                       lut=LUTS.get(type(model).__name__, (0, 0, 0, 255, 255, 255)))
        done = cp
        exp = entry["steps"][str(cp)]
        assert crc(fld[:topo.cells]) == exp["cells"], "cells at step %d" % cp
        assert crc(col) == exp["colors"], "colours at step %d" % cp
        if "img" in exp:
            w, h = job["render"]["viewport"]
            pos = job.get("exp_overrides", {}).get("pos", [0, 0])
            zoom = job.get("exp_overrides", {}).get("zoom", model.zoom)
            img = O.render(topo, col, w, h, zoom=zoom, dx=pos[0], dy=pos[1], axes=axes,
                           smooth=smooth).astype(np.uint8)
            assert crc(img) == exp["img"], "image at step %d" % cp


def evolife_run(model, topo, fld, col, steps):
    tpl = model.gpu.template
    info = tpl.color.extra
    O.evolife_run(topo, fld, col, steps, death_speed=tpl.params["death_speed"],
                  max_genes=tpl.params["max_genes"], mutation_prob=tpl.params["mutation_prob"],
                  positional=not tpl.legacy, fade_in=info["fade_in"], fade_out=info["fade_out"],
                  smooth=info["smooth"])


@pytest.mark.parametrize("case", ["evolife_bigbang_160x120", "evolife_bigbang_mut_131x101"])
def test_oracle_evolife_fixtures(golden, case):
    entry = golden[case]
    topo, fld, col, model = oracle_setup(entry["job"])
    assert crc(fld[:topo.cells]) == entry["init"]
    done = 0
    for cp in sorted(int(c) for c in entry["steps"]):
        evolife_run(model, topo, fld, col, cp - done)
        done = cp
        assert crc(fld[:topo.cells]) == entry["steps"][str(cp)]["cells"], "cells at %d" % cp
        assert crc(col) == entry["steps"][str(cp)]["colors"], "colours at %d" % cp


def test_oracle_evolife_reference_golden(golden):
    # reference tests/core/test_base.py:208-216 (CrossbreedingExperiment2, 100 steps)
    topo, fld, col, model = oracle_setup(golden["evolife_cross2"]["job"])
    evolife_run(model, topo, fld, col, 100)
    assert crc(fld[:topo.cells]) == 3381214984
    assert crc(col) == 2253830262


def test_oracle_mass_conserved(golden):
    topo, fld, col, model = oracle_setup(golden["mass_64cube"]["job"])
    totals = []
    before = int(fld[:topo.cells].astype(np.uint64).sum())
    O.mass_run(topo, fld, col, 30, totals=totals)
    assert totals == [before] * 30
