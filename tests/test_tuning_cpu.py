"""The autotuning cache (``xentica_gb300.tuning``) on the CPU, with a fake
library standing in for ``libxk.so``: where the file lives, what the keys
distinguish, that a stored choice is applied without timing and that a miss
times and stores."""
import json

import numpy as np
import pytest

from xentica_gb300 import tuning


class FakeLib:
    """Records the tuning calls a batch handle would get."""

    def __init__(self, device=b"GB300 sm_103 SMs=152 smem_optin=232448", best=16, sizes=()):
        self.device, self.best, self.sizes = device, best, [list(t) for t in sizes]
        self.tuned, self.set, self.set_sizes = [], [], []

    def xk_device_info(self, buf, n):
        buf.value = self.device[:n - 1]
        return 0

    def xk_batch_tune(self, handle, generations, chosen):
        self.tuned.append(generations)
        chosen._obj.value = self.best
        return 0

    def xk_batch_set_band(self, handle, rows):
        self.set.append(rows)
        return 0

    def xk_batch_size_bands(self, handle, buf, capacity):
        for k, t in enumerate(self.sizes[:capacity]):
            buf[3 * k:3 * k + 3] = t
        return len(self.sizes)

    def xk_batch_set_size_bands(self, handle, buf, count):
        self.set_sizes.append([list(buf[3 * k:3 * k + 3]) for k in range(count)])
        return 0


W = np.array([64, 128, 1024], np.int32)
H = np.array([64, 256, 512], np.int32)


def test_cache_path(monkeypatch, tmp_path):
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "t.json"))
    assert tuning.cache_path() == str(tmp_path / "t.json")
    for off in ("off", "0", "", "none"):
        monkeypatch.setenv("XK_TUNE_CACHE", off)
        assert tuning.cache_path() is None
    monkeypatch.delenv("XK_TUNE_CACHE")
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    assert tuning.cache_path() == str(tmp_path / "xentica_gb300" / "tune.json")


def test_keys_distinguish_workload_device_and_build():
    base = tuning.ensemble_key("dev", "lib", W, H, 256)
    assert base == tuning.ensemble_key("dev", "lib", W.copy(), H.copy(), 256)
    others = [tuning.ensemble_key("dev2", "lib", W, H, 256),
              tuning.ensemble_key("dev", "lib2", W, H, 256),
              tuning.ensemble_key("dev", "lib", W, H, 128),
              tuning.ensemble_key("dev", "lib", H, W, 256),
              tuning.ensemble_key("dev", "lib", W[:2], H[:2], 256)]
    assert len(set(others + [base])) == len(others) + 1


def test_file_round_trip_and_bad_files(tmp_path):
    path = tmp_path / "sub" / "t.json"
    cache = tuning.TuneCache(str(path))
    assert cache.get("a") is None                  # no file yet
    cache.put("a", 4)
    cache.put("b", 8)                              # merged, not overwritten
    assert cache.get("a") == 4 and cache.get("b") == 8
    assert json.loads(path.read_text()) == {"a": 4, "b": 8}
    path.write_text("{not json")
    assert cache.get("a") is None                  # a damaged file is a miss
    cache.put("c", 2)
    assert json.loads(path.read_text()) == {"c": 2}


def test_miss_times_and_stores_then_hit_applies(monkeypatch, tmp_path):
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "t.json"))
    lib = FakeLib(best=16)
    assert tuning.tuned_band(lib, None, W, H, 256, library="L1") == 16
    assert lib.tuned == [256] and lib.set == []
    lib.best = 2                                   # a new timing would now disagree
    assert tuning.tuned_band(lib, None, W, H, 256, library="L1") == 16
    assert lib.tuned == [256] and lib.set == [16]  # applied, not timed
    # another generation count, library build or device: timed again
    assert tuning.tuned_band(lib, None, W, H, 64, library="L1") == 2
    assert tuning.tuned_band(lib, None, W, H, 256, library="L2") == 2
    other = FakeLib(device=b"another device", best=32)
    assert tuning.tuned_band(other, None, W, H, 256, library="L1") == 32
    assert lib.tuned == [256, 64, 256] and other.tuned == [256]


def test_cache_off(monkeypatch, tmp_path):
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "t.json"))
    lib = FakeLib(best=8)
    assert tuning.tuned_band(lib, None, W, H, 256, cache=False, library="L") == 8
    assert tuning.tuned_band(lib, None, W, H, 256, cache=False, library="L") == 8
    assert lib.tuned == [256, 256] and not (tmp_path / "t.json").exists()
    monkeypatch.setenv("XK_TUNE_CACHE", "off")
    assert tuning.tuned_band(lib, None, W, H, 256, library="L") == 8
    assert lib.tuned == [256, 256, 256]


@pytest.mark.parametrize("bad", [0, 5000, "8", None, 2.5, True])
def test_invalid_entries_are_ignored(monkeypatch, tmp_path, bad):
    path = tmp_path / "t.json"
    monkeypatch.setenv("XK_TUNE_CACHE", str(path))
    key = tuning.ensemble_key(FakeLib().device.decode(), "L", W, H, 256)
    path.write_text(json.dumps({key: bad}))
    lib = FakeLib(best=4)
    assert tuning.tuned_band(lib, None, W, H, 256, library="L") == 4
    assert lib.tuned == [256] and lib.set == []
    assert json.loads(path.read_text())[key] == {"band": 4, "sizes": []}


@pytest.mark.parametrize("bad", [{"band": 0}, {"sizes": []}, {"band": 8, "sizes": [[64, 64]]},
                                 {"band": 8, "sizes": [[64, 64, 0]]},
                                 {"band": 8, "sizes": [[64, 64, True]]}, {"band": 8, "sizes": 3}])
def test_invalid_size_entries_are_ignored(monkeypatch, tmp_path, bad):
    path = tmp_path / "t.json"
    monkeypatch.setenv("XK_TUNE_CACHE", str(path))
    key = tuning.ensemble_key(FakeLib().device.decode(), "L", W, H, 256)
    path.write_text(json.dumps({key: bad}))
    lib = FakeLib(best=4)
    assert tuning.tuned_band(lib, None, W, H, 256, library="L") == 4
    assert lib.tuned == [256] and lib.set == [] and lib.set_sizes == []


def test_per_size_bands_are_stored_and_reapplied(monkeypatch, tmp_path):
    path = tmp_path / "t.json"
    monkeypatch.setenv("XK_TUNE_CACHE", str(path))
    lib = FakeLib(best=16, sizes=[[1024, 512, 32], [128, 256, 4]])
    assert tuning.tuned_band(lib, None, W, H, 256, library="L") == 16
    key = tuning.ensemble_key(lib.device.decode(), "L", W, H, 256)
    assert json.loads(path.read_text())[key] == {"band": 16,
                                                 "sizes": [[1024, 512, 32], [128, 256, 4]]}
    again = FakeLib(best=2)                        # would time differently: not asked
    assert tuning.tuned_band(again, None, W, H, 256, library="L") == 16
    assert again.tuned == [] and again.set == [16]
    assert again.set_sizes == [[[1024, 512, 32], [128, 256, 4]]]
    # the older form without per-size choices still applies
    path.write_text(json.dumps({key: 8}))
    old = FakeLib(best=2)
    assert tuning.tuned_band(old, None, W, H, 256, library="L") == 8
    assert old.tuned == [] and old.set == [8] and old.set_sizes == []


def test_library_id_tracks_the_file(tmp_path):
    f = tmp_path / "libxk.so"
    f.write_bytes(b"one")
    a = tuning.library_id(str(f))
    assert a == tuning.library_id(str(f))
    f.write_bytes(b"two!")
    assert tuning.library_id(str(f)) != a


def test_unidentifiable_library_tunes_without_cache(monkeypatch, tmp_path):
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "t.json"))
    monkeypatch.setattr(tuning, "library_id", lambda: (_ for _ in ()).throw(OSError("gone")))
    lib = FakeLib(best=8)
    assert tuning.tuned_band(lib, None, W, H, 256) == 8
    assert lib.tuned == [256] and not (tmp_path / "t.json").exists()


class FakePlanLib(FakeLib):
    """Records the plan calls a 2-D Life-like model handle would get."""

    def __init__(self, plan=(2, 16, 2, 0), form=0, **kw):
        super().__init__(**kw)
        self.plan, self.timed, self.applied, self.form = list(plan), 0, [], form

    def xk_model_rule_form(self, handle):
        return self.form

    def xk_model_plan(self, handle, out):
        self.timed += 1
        out[:] = self.plan
        return 0

    def xk_model_set_plan(self, handle, plan):
        self.applied.append(list(plan))
        return 0


@pytest.mark.parametrize("plan", [(0, 0, 0, 0), (1, 0, 0, 0), (2, 16, 2, 0), (3, 0, 0, 8)],
                         ids=["global", "resident", "cluster", "temporal"])
def test_lattice_plan_stored_then_applied(monkeypatch, tmp_path, plan):
    """Every kind of plan: a miss times (xk_model_plan) and stores it, a hit
    re-applies it (xk_model_set_plan) without timing, and the key separates
    sizes, borders, devices and library builds."""
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "t.json"))
    lib = FakePlanLib(plan=plan)
    assert tuning.lattice_plan(lib, None, 512, 512, "torus", library="L") == list(plan)
    assert lib.timed == 1 and lib.applied == []
    lib.plan = [0, 0, 0, 0]                        # a new timing would disagree
    assert tuning.lattice_plan(lib, None, 512, 512, "torus", library="L") == list(plan)
    assert lib.timed == 1 and lib.applied == [list(plan)]
    for args in [(512, 256, "torus", "L"), (512, 512, "static1", "L"), (512, 512, "torus", "L2")]:
        assert tuning.lattice_plan(lib, None, args[0], args[1], args[2], library=args[3]) == [0] * 4
    other = FakePlanLib(device=b"another device", plan=(3, 0, 0, 4))
    assert tuning.lattice_plan(other, None, 512, 512, "torus", library="L") == [3, 0, 0, 4]
    assert lib.timed == 4 and other.timed == 1


def test_lattice_plan_keys_on_the_rule_form(monkeypatch, tmp_path):
    """Conway's rule runs kernels with the rule compiled in: its plan is
    timed and kept apart from the plan of a rule read from a table."""
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "t.json"))
    table = FakePlanLib(plan=(2, 16, 2, 0), form=0)
    assert tuning.lattice_plan(table, None, 512, 512, "torus", library="L") == [2, 16, 2, 0]
    conway = FakePlanLib(plan=(2, 8, 4, 0), form=1)
    assert tuning.lattice_plan(conway, None, 512, 512, "torus", library="L") == [2, 8, 4, 0]
    assert table.timed == 1 and conway.timed == 1
    again = FakePlanLib(plan=(0, 0, 0, 0), form=1)
    assert tuning.lattice_plan(again, None, 512, 512, "torus", library="L") == [2, 8, 4, 0]
    assert again.timed == 0 and again.applied == [[2, 8, 4, 0]]
    assert tuning.lattice_key("d", "L", 512, 512, "torus", 0) != \
        tuning.lattice_key("d", "L", 512, 512, "torus", 1)


def test_lattice_plan_rejected_or_invalid_entries_retime(monkeypatch, tmp_path):
    path = tmp_path / "t.json"
    monkeypatch.setenv("XK_TUNE_CACHE", str(path))
    key = tuning.lattice_key(FakeLib().device.decode(), "L", 300, 200, "torus")
    for bad in ([9, 0, 0, 0], [1, 2], "x", [True, 0, 0, 0]):
        path.write_text(json.dumps({key: bad}))
        lib = FakePlanLib(plan=(3, 0, 0, 2))
        assert tuning.lattice_plan(lib, None, 300, 200, "torus", library="L") == [3, 0, 0, 2]
        assert lib.timed == 1 and lib.applied == []
    # a stored plan the library refuses (e.g. a size it no longer supports)
    path.write_text(json.dumps({key: [2, 16, 1, 0]}))
    lib = FakePlanLib(plan=(1, 0, 0, 0))
    lib.xk_model_set_plan = lambda handle, plan: -1
    assert tuning.lattice_plan(lib, None, 300, 200, "torus", library="L") == [1, 0, 0, 0]
    assert json.loads(path.read_text())[key] == [1, 0, 0, 0]


def test_models_without_plans(monkeypatch, tmp_path):
    monkeypatch.setenv("XK_TUNE_CACHE", str(tmp_path / "t.json"))
    lib = FakePlanLib(plan=(-1, 0, 0, 0))
    assert tuning.lattice_plan(lib, None, 50, 30, "torus", library="L") is None
    assert not (tmp_path / "t.json").exists()
