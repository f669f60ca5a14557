"""GPU parity of the EvoLife kernel (bit-exact, including the random stream).

Fixture cases (reference checksums) run through ``test_gpu_life``'s fixture
replay; here: random 64-bit states far from any seed pattern, compared with
the oracle after every step, and a step-transition check after a long run.
"""
import numpy as np
import pytest

import oracle as O
from tests.models import (EvoLife, BigBangExperiment, CrossbreedingExperiment2,
                          PrimordialSoupExperiment, build_from_job)
from tests.test_oracle import crc

pytestmark = pytest.mark.gpu


def _model(size, legacy=True, **params):
    exp = type("E", (BigBangExperiment, ), dict({"size": size, "zoom": 1}, **params))
    for p in EvoLife.meta.__dict__.values():
        if hasattr(p, "default"):
            p.__set__(None, p.default)
    return EvoLife(exp, legacy_coloring=legacy)


def _oracle_step(model, fld, col, steps):
    tpl = model.gpu.template
    info = tpl.color.extra
    topo = O.Topology(model.size)
    O.evolife_run(topo, fld, col, steps, death_speed=tpl.params["death_speed"],
                  max_genes=tpl.params["max_genes"], mutation_prob=tpl.params["mutation_prob"],
                  positional=not tpl.legacy, fade_in=info["fade_in"], fade_out=info["fade_out"],
                  smooth=info["smooth"])


@pytest.mark.parametrize("legacy,mutation,live", [(True, 0.0, 0.6), (False, 0.2, 0.6),
                                                  (True, 0.0001, 0.6), (True, 0.0, 0.02),
                                                  (False, 0.2, 0.02), (True, 0.0001, 0.005)])
def test_random_states_vs_oracle(legacy, mutation, live):
    # live: share of cells with a rule; sparse lattices put whole warps of
    # cells with no parent on the composed-RNG path
    w, h = 131, 103          # at least the BigBang seed area (100 x 100)
    model = _model((w, h), legacy, mutation_prob=mutation, death_speed=9, max_genes=7,
                   fade_in=30, fade_out=7)
    rng = np.random.RandomState(int(mutation * 1e4) + legacy + int(live * 1000))
    n = w * h
    energy = rng.randint(0, 300, n).astype(np.uint64)
    rule = rng.randint(0, 2 ** 18, n).astype(np.uint64) * (rng.random_sample(n) < live)
    rnd = rng.randint(0, 2 ** 16, n).astype(np.uint64)     # 65535 included
    cells = energy + (rule << np.uint64(9)) + (rnd << np.uint64(27))
    colors = rng.randint(0, 256, 3 * n).astype(np.int32)
    model.gpu.load(cells, colors)
    topo = O.Topology((w, h))
    fld = topo.field(cells, np.uint64)
    col = colors.copy()
    for step in range(6):
        model.step()
        _oracle_step(model, fld, col, 1)
        assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n]), "step %d" % step
        assert np.array_equal(model.gpu.arrays.colors.get(), col), "colours step %d" % step


def test_long_run_step_transitions():
    # 1920x1080 CrossbreedingExperiment2: after 300 GPU generations, one and
    # three more generations agree with the oracle started from the GPU state
    model = build_from_job({"model": ":EvoLife", "experiment": ":CrossbreedingExperiment2"})
    model.gpu.step(300)
    n = model.cells_num
    cells = model.gpu.arrays.cells.get()[:n]
    colors = model.gpu.arrays.colors.get()
    topo = O.Topology(model.size)
    fld = topo.field(cells, np.uint64)
    col = colors.copy()
    model.gpu.step(1)
    _oracle_step(model, fld, col, 1)
    assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n])
    model.gpu.step(2)
    _oracle_step(model, fld, col, 2)
    assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n])
    assert np.array_equal(model.gpu.arrays.colors.get(), col)


def test_uniform_genomes_step_transitions_to_10000():
    """The benchmarked EvoLife configuration (1920x1080, every cell a uniform
    random genome, energy and random state): the GPU runs 10 000 generations;
    at generations drawn from a seeded stream the oracle, started from the GPU
    state, computes one more generation (cells with their random streams, and
    colours), compared with the GPU's next generation."""
    for p in EvoLife.meta.__dict__.values():
        if hasattr(p, "default"):
            p.__set__(None, p.default)
    model = EvoLife(PrimordialSoupExperiment)
    n = model.cells_num
    topo = O.Topology(model.size)
    draws = sorted(np.random.RandomState(2041).randint(1, 10000, 4).tolist()) + [9999]
    done = 0
    for g in draws:
        if g > done:
            model.gpu.step(g - done)
            done = g
        fld = topo.field(model.gpu.arrays.cells.get()[:n], np.uint64)
        col = model.gpu.arrays.colors.get()
        model.gpu.step(1)
        done += 1
        _oracle_step(model, fld, col, 1)
        assert np.array_equal(model.gpu.arrays.cells.get()[:n], fld[:n]), "generation %d" % g
        assert np.array_equal(model.gpu.arrays.colors.get(), col), "colours, generation %d" % g
