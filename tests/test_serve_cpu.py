"""Host-side logic of the serving loop (no GPU): the arena allocator through
its C-ABI, request validation and sizing, the seeded request mix and the
latency summary."""
import ctypes

import numpy as np
import pytest

from xentica_gb300 import _native as nat
from xentica_gb300 import serve
from xentica_gb300.core.exceptions import XenticaException


class Arena:
    def __init__(self, capacity):
        self.lib = nat.load()
        self.h = ctypes.c_void_p()
        nat.check(self.lib.xk_arena_create(capacity, ctypes.byref(self.h)), "xk_arena_create")

    def alloc(self, nbytes):
        off = ctypes.c_int64()
        rc = self.lib.xk_arena_alloc(self.h, nbytes, ctypes.byref(off))
        return off.value if rc == 0 else rc

    def free(self, off):
        return self.lib.xk_arena_free(self.h, off)

    def stats(self):
        used, largest, ranges = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
        nat.check(self.lib.xk_arena_stats(self.h, ctypes.byref(used), ctypes.byref(largest),
                                          ctypes.byref(ranges)), "xk_arena_stats")
        return used.value, largest.value, ranges.value

    def close(self):
        self.lib.xk_arena_destroy(self.h)


def test_arena_first_fit_and_merge():
    a = Arena(4096)
    offs = [a.alloc(100) for _ in range(16)]          # 16 granules of 256 B
    assert offs == [256 * i for i in range(16)]
    assert a.alloc(1) == nat.XK_ERR_OOM               # full
    assert a.stats() == (4096, 0, 0)
    for i in (1, 2, 5):
        assert a.free(offs[i]) == 0
    assert a.stats() == (4096 - 768, 512, 2)          # [256, 768) and [1280, 1536)
    assert a.alloc(300) == 256                        # first fit: the merged pair
    assert a.alloc(600) == nat.XK_ERR_OOM             # 768 free in total, 256 largest
    assert a.free(offs[1] + 8) == nat.XK_ERR_ARG      # not an allocation
    for i in range(16):
        if i not in (1, 2, 5):
            assert a.free(offs[i]) == 0
    assert a.free(256) == 0
    assert a.stats() == (0, 4096, 1)                  # everything merged back
    assert a.alloc(4096) == 0
    a.close()


def test_arena_random_against_model():
    rng = np.random.RandomState(5)
    cap = 1 << 20
    a = Arena(cap)
    live = {}
    for _ in range(2000):
        if live and rng.random_sample() < 0.45:
            off = list(live)[rng.randint(len(live))]
            assert a.free(off) == 0
            del live[off]
        else:
            size = int(rng.randint(1, 40000))
            off = a.alloc(size)
            if off < 0:
                assert off == nat.XK_ERR_OOM
                assert a.stats()[1] < (size + 255) // 256 * 256
                continue
            assert off % 256 == 0
            end = off + (size + 255) // 256 * 256
            assert end <= cap
            for o, e in live.items():
                assert end <= o or off >= e, "overlap"
            live[off] = end
        assert a.stats()[0] == sum(e - o for o, e in live.items())
    a.close()


def test_request_validation():
    assert serve.request_bytes("life2d", (10, 33), 6152) >= 330
    assert serve.request_bytes("mass", (4, 5, 6)) >= 2 * 4 * 120
    bad = [("life2d", (10, 33), 1 << 18, 1),           # rule bits above 17
           ("life3d", (3, 10, 33), 1 << 14, 1),        # rule bits above 13
           ("mass", (3, 10, 33), 5, 1),                # mass takes no rule
           ("life2d", (0, 33), 0, 1),                  # empty axis
           ("life2d", (10, 33), 0, -1),                # negative generations
           ("life2d", (2 ** 21, 2), 0, 1)]             # side above 2^20
    for kind, shape, rule, gens in bad:
        with pytest.raises(XenticaException):
            serve.request_bytes(kind, shape, rule, gens)
    with pytest.raises(XenticaException):
        serve.request_bytes("life4d", (3, 3), 0, 1)
    with pytest.raises(XenticaException):
        serve.request_bytes("life2d", (3, 3, 3), 0, 1)


def test_request_bytes_cover_both_2d_paths():
    # resident (bytes in place) and bit-packed (bytes + two word planes) both fit
    for h, w in ((32, 32), (100, 4000), (4096, 4096)):
        b = serve.request_bytes("life2d", (h, w), 6152, 10)
        assert b >= h * w + 2 * 4 * h * ((w + 31) // 32)


def test_serving_workload_is_seeded_and_in_range():
    a = serve.serving_workload(400, seed=7)
    b = serve.serving_workload(400, seed=7)
    assert a == b
    kinds = [s["kind"] for s in a]
    assert abs(kinds.count("life2d") / 400 - 0.5) < 0.1
    for s in a:
        assert 100 <= s["generations"] <= 10000
        if s["kind"] == "life2d":
            assert all(32 <= v <= 4096 for v in s["shape"]) and s["rule"] < 2 ** 18
        else:
            assert all(64 <= v <= 256 for v in s["shape"]) and len(s["shape"]) == 3
            assert s["rule"] < 2 ** 14
        assert 0.1 <= s["p"] <= 0.6
    sides = np.array([s["shape"][0] for s in a if s["kind"] == "life2d"])
    # log-uniform: the median side is near sqrt(32 * 4096) = 362
    assert 200 < np.median(sides) < 650
    cells = serve.make_cells(dict(a[0], shape=(9, 11) if a[0]["kind"] == "life2d" else (3, 9, 11)))
    assert cells.shape in ((9, 11), (3, 9, 11))


def test_poisson_arrivals_and_latency_summary():
    t = serve.poisson_arrivals(50.0, 20000, seed=3)
    assert np.all(np.diff(t) > 0)
    assert abs(t[-1] / 20000 - 1 / 50.0) < 0.001
    s = serve.latency_summary(np.arange(1, 101) / 100.0)
    assert abs(s["p50"] - 0.505) < 1e-9 and abs(s["p99"] - 0.9901) < 1e-9 and s["max"] == 1.0
    assert serve.latency_summary([])["p99"] is None


def test_server_needs_a_gpu_here():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(XenticaException):
        serve.Server(1 << 20)
