"""xk_batch_step_noalloc: the ensemble step for callers that cannot allocate.

Callers such as plugins inside a host framework's memory pool hand over a
device buffer they already own and cannot call cudaMalloc themselves.  This
checks, through the C-ABI, that stepping such a caller-owned buffer twice in
a row gives exactly what the allocating entry point (xk_batch_step) gives.
The device buffer is allocated by the test (as the caller would own it).
"""
import ctypes

import numpy as np
import pytest

from xentica_gb300 import _native as nat
from xentica_gb300.batch import Ensemble

pytestmark = pytest.mark.gpu

SIZES = [(64, 64), (37, 23), (1, 9), (1024, 96), (128, 1024), (95, 95), (512, 32)]


def test_noalloc_matches_batch_step_twice():
    torch = pytest.importorskip("torch")
    rng = np.random.RandomState(31)
    widths = np.array([w for w, _ in SIZES], dtype=np.int32)
    heights = np.array([h for _, h in SIZES], dtype=np.int32)
    rules = rng.randint(0, 2 ** 18, len(SIZES)).astype(np.uint32)
    ens = Ensemble(widths, heights, rules)
    cells = (rng.random_sample(ens.total_cells) < 0.45).astype(np.uint8)
    ens.upload(cells)
    generations = 13
    ens.step(generations)
    want1 = ens.download()
    ens.step(generations)
    want2 = ens.download()

    lib = nat.load()
    d_cells = torch.from_numpy(cells.copy()).to("cuda")   # the caller's own buffer
    for want in (want1, want2):
        rc = lib.xk_batch_step_noalloc(ctypes.c_void_p(d_cells.data_ptr()), len(SIZES),
                                       nat.ptr(widths), nat.ptr(heights), nat.ptr(rules),
                                       generations, None)
        nat.check(rc, "xk_batch_step_noalloc")
        got = d_cells.cpu().numpy()
        assert np.array_equal(got, want)


def test_noalloc_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    lib = nat.load()
    d_cells = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    too_many = np.ones(4097, dtype=np.int32)
    rules = np.zeros(4097, dtype=np.uint32)
    rc = lib.xk_batch_step_noalloc(ctypes.c_void_p(d_cells.data_ptr()), 4097, nat.ptr(too_many),
                                   nat.ptr(too_many), nat.ptr(rules), 1, None)
    assert rc != 0 and "limit" in nat.last_error()
    wide = np.array([2048], dtype=np.int32)
    one = np.array([2], dtype=np.int32)
    rc = lib.xk_batch_step_noalloc(ctypes.c_void_p(d_cells.data_ptr()), 1, nat.ptr(wide),
                                   nat.ptr(one), nat.ptr(rules[:1]), 1, None)
    assert rc != 0 and "one CTA" in nat.last_error()
