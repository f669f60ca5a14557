"""Persistent cache of autotuned launch choices.

The ensemble's autotuner (``xk_batch_tune``) times the resident kernel for
several band lengths and keeps the fastest.  Its choice depends on the device,
on the kernels in ``libxk.so`` and on the workload, so a choice is stored in a
JSON file under a key made of

* the device (``xk_device_info``: name, compute capability, SM count, shared
  memory per block),
* the library build (SHA-1 of ``libxk.so``; any rebuild with changed kernels
  changes it),
* the workload (SHA-1 of the lattice sizes and the generations per step),

and a later tune of the same workload on the same device and library applies
it with ``xk_batch_set_band`` instead of timing again.  The file is
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


def tuned_band(lib, handle, widths, heights, generations, cache=True, library=None):
    """Band length for an ensemble: from the cache when present (applied with
    ``xk_batch_set_band``), else timed by ``xk_batch_tune`` and stored."""
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
        if isinstance(hit, int) and not isinstance(hit, bool) and 1 <= hit <= 1024:
            nat.check(lib.xk_batch_set_band(handle, hit), "xk_batch_set_band")
            return hit
    chosen = ctypes.c_int32()
    nat.check(lib.xk_batch_tune(handle, int(generations), ctypes.byref(chosen)), "xk_batch_tune")
    if store is not None:
        try:
            store.put(key, int(chosen.value))
        except OSError:
            pass   # a read-only cache location only costs the next tuning run
    return int(chosen.value)
