"""Persistent cache of autotuned launch choices.

Two choices are timed on the device and cached:

* the ensemble's band lengths (``xk_batch_tune`` times the resident kernel
  for several band lengths and keeps the fastest, then a band of its own for
  each lattice size with a large share of the cells where that is faster),
  re-applied with ``xk_batch_set_band`` and ``xk_batch_set_size_bands``;
* a single 2-D Life-like lattice's launch plan (``xk_model_plan``: the
  kernel family -- per-generation global kernel, one resident CTA, a
  thread-block cluster of a size and band length, or temporal blocking of a
  depth -- timed on the model's first step), re-applied with
  ``xk_model_set_plan``.

A choice depends on the device, on the kernels in ``libxk.so`` and on the
workload, so it is stored in a JSON file under a key made of

* the device (``xk_device_info``: name, compute capability, SM count, shared
  memory per block),
* the library build (SHA-1 of ``libxk.so``; any rebuild with changed kernels
  changes it),
* the workload: for an ensemble the SHA-1 of the lattice sizes and the
  generations per step; for a lattice its size, border (torus, or static
  with its state) and rule form.  Conway's B3/S23 runs kernels with the
  rule compiled in (fewer instructions per word, so a different best plan);
  every other rule is evaluated through the same multiplexer over a table
  loaded at run time, whose instruction stream and cost are the same for
  every rule, so the rule itself is not part of the key.

A later tune of the same workload on the same device and library applies the
stored choice instead of timing again.  The file is
``$XK_TUNE_CACHE``, else ``$XDG_CACHE_HOME/xentica_gb300/tune.json`` (default
``~/.cache``); ``XK_TUNE_CACHE=off`` disables the cache.  Writes replace the
file atomically; concurrent writers can lose each other's newest entry, never
corrupt the file.
"""
import ctypes
import hashlib
import json
import os
import threading

import numpy as np

from xentica_gb300 import _native as nat

_LOCK = threading.Lock()
_LIB_IDS = {}


def cache_path():
    """The cache file, or None when caching is off."""
    env = os.environ.get("XK_TUNE_CACHE")
    if env is not None:
        return None if env.strip().lower() in ("", "0", "off", "none") else env
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "xentica_gb300", "tune.json")


def library_id(path=nat.LIBPATH):
    """SHA-1 of the library file (memoised per path, size and mtime)."""
    st = os.stat(path)
    memo = (path, st.st_size, st.st_mtime_ns)
    with _LOCK:
        if memo not in _LIB_IDS:
            h = hashlib.sha1()
            with open(path, "rb") as fh:
                for chunk in iter(lambda: fh.read(1 << 20), b""):
                    h.update(chunk)
            _LIB_IDS[memo] = h.hexdigest()
        return _LIB_IDS[memo]


def device_id(lib):
    """``xk_device_info`` of the current device."""
    buf = ctypes.create_string_buffer(256)
    nat.check(lib.xk_device_info(buf, 256), "xk_device_info")
    return buf.value.decode()


def ensemble_key(device, library, widths, heights, generations):
    """Cache key of an ensemble tuning."""
    h = hashlib.sha1()
    h.update(np.ascontiguousarray(widths, dtype=np.int32).tobytes())
    h.update(b"|")
    h.update(np.ascontiguousarray(heights, dtype=np.int32).tobytes())
    h.update(b"|%d" % int(generations))
    return "ensemble_band|%s|%s|%s" % (device, library, h.hexdigest())


class TuneCache:
    """A JSON file of tuned choices (see the module docstring)."""

    def __init__(self, path):
        self.path = path

    def _read(self):
        try:
            with open(self.path) as fh:
                data = json.load(fh)
            return data if isinstance(data, dict) else {}
        except (OSError, ValueError):
            return {}

    def get(self, key):
        return self._read().get(key)

    def put(self, key, value):
        with _LOCK:
            data = self._read()
            data[key] = value
            folder = os.path.dirname(os.path.abspath(self.path))
            os.makedirs(folder, exist_ok=True)
            tmp = "%s.%d.%d.tmp" % (self.path, os.getpid(), threading.get_ident())
            with open(tmp, "w") as fh:
                json.dump(data, fh, indent=1, sort_keys=True)
            os.replace(tmp, self.path)


def _valid_bands(hit):
    """A cached ensemble entry: ``{"band": b, "sizes": [[W, H, b], ...]}`` (or
    a bare band length, the form without per-size choices)."""
    def band_ok(v):
        return isinstance(v, int) and not isinstance(v, bool) and 1 <= v <= 1024
    if band_ok(hit):
        return True
    if not (isinstance(hit, dict) and band_ok(hit.get("band"))):
        return False
    sizes = hit.get("sizes", [])
    return isinstance(sizes, list) and all(
        isinstance(t, list) and len(t) == 3 and all(band_ok(v) for v in t[2:]) and
        all(isinstance(v, int) and not isinstance(v, bool) and v >= 1 for v in t[:2])
        for t in sizes)


def size_bands(lib, handle):
    """The per-size band choices of a batch as ``[[W, H, band], ...]``."""
    n = lib.xk_batch_size_bands(handle, None, 0)
    if n <= 0:
        return []
    buf = (ctypes.c_int32 * (3 * n))()
    lib.xk_batch_size_bands(handle, buf, n)
    return [[int(buf[3 * k]), int(buf[3 * k + 1]), int(buf[3 * k + 2])] for k in range(n)]


def apply_bands(lib, handle, band, sizes=()):
    """Set the common band and the per-size choices of a batch."""
    nat.check(lib.xk_batch_set_band(handle, int(band)), "xk_batch_set_band")
    if sizes:
        flat = (ctypes.c_int32 * (3 * len(sizes)))(*[int(v) for t in sizes for v in t])
        nat.check(lib.xk_batch_set_size_bands(handle, flat, len(sizes)), "xk_batch_set_size_bands")


def tuned_band(lib, handle, widths, heights, generations, cache=True, library=None):
    """Band lengths for an ensemble: from the cache when present (applied with
    ``xk_batch_set_band`` and ``xk_batch_set_size_bands``), else timed by
    ``xk_batch_tune`` and stored.  Returns the common band length."""
    path = cache_path() if cache else None
    store = key = None
    if path is not None:
        try:
            lib_id = library if library is not None else library_id()
        except OSError:
            path = None   # no library file to identify: tune without the cache
    if path is not None:
        key = ensemble_key(device_id(lib), lib_id, widths, heights, generations)
        store = TuneCache(path)
        hit = store.get(key)
        if _valid_bands(hit):
            if isinstance(hit, dict):
                apply_bands(lib, handle, hit["band"], hit.get("sizes", []))
                return hit["band"]
            apply_bands(lib, handle, hit)
            return hit
    chosen = ctypes.c_int32()
    nat.check(lib.xk_batch_tune(handle, int(generations), ctypes.byref(chosen)), "xk_batch_tune")
    if store is not None:
        try:
            store.put(key, {"band": int(chosen.value), "sizes": size_bands(lib, handle)})
        except OSError:
            pass   # a read-only cache location only costs the next tuning run
    return int(chosen.value)


PLAN_KINDS = {0: "global", 1: "resident", 2: "cluster", 3: "temporal"}


def lattice_key(device, library, width, height, border, rule_form=0):
    """Cache key of a 2-D lattice's launch plan; ``border`` is "torus" or
    "static0" / "static1"; ``rule_form`` the kernels' rule form
    (``xk_model_rule_form``: 1 Conway compiled in, 0 a rule table)."""
    return "life2d_plan|%s|%s|%dx%d|%s|rule%d" % (device, library, int(width), int(height), border,
                                                 int(rule_form))


def _valid_plan(hit):
    return (isinstance(hit, list) and len(hit) == 4 and
            all(isinstance(v, int) and not isinstance(v, bool) for v in hit) and hit[0] in PLAN_KINDS)


def lattice_plan(lib, handle, width, height, border, cache=True, library=None):
    """The launch plan of a 2-D Life-like model: from the cache when present
    (applied with ``xk_model_set_plan``), else the one ``xk_model_plan``
    times, stored.  Returns the plan (4 ints) or None for models without
    plans."""
    path = cache_path() if cache else None
    store = key = None
    if path is not None:
        try:
            lib_id = library if library is not None else library_id()
        except OSError:
            path = None
    plan = (ctypes.c_int32 * 4)()
    if path is not None:
        form = lib.xk_model_rule_form(handle) if hasattr(lib, "xk_model_rule_form") else 0
        key = lattice_key(device_id(lib), lib_id, width, height, border, form)
        store = TuneCache(path)
        hit = store.get(key)
        if _valid_plan(hit):
            plan[:] = hit
            if lib.xk_model_set_plan(handle, plan) == 0:
                return list(hit)
    nat.check(lib.xk_model_plan(handle, plan), "xk_model_plan")
    chosen = [int(v) for v in plan]
    if chosen[0] < 0:
        return None
    if store is not None:
        try:
            store.put(key, chosen)
        except OSError:
            pass
    return chosen
