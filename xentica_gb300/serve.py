"""Serving: simulation requests as they arrive, continuously batched on one GPU.

The reference has no request loop -- a caller builds one model per lattice
and steps it (``xentica/core/base.py:591-728``).  :class:`Server` wraps the
engine's ``xk_serve_*`` C-ABI: a worker thread inside ``libxk`` admits queued
requests by HBM budget, keeps their state resident on the device and advances
every active request in rounds (``quantum`` generations for large lattices;
about ``quantum`` x 2^18 cell-generations for 2-D lattices that fit one CTA,
which run together in one launch per shape class), so requests admitted while
others run overlap with them on the GPU; requests with less work run at a
greater stream priority.  Each request computes exactly what it computes
alone.

Request kinds (cells row-major, axis 0 = x fastest, i.e. NumPy shape
``(height, width)`` or ``(depth, height, width)``):

``life2d``  Life-like on a 2-D torus, Moore neighbourhood, golly-style rule
            int (B bits 0-8, S bits 9-17), the semantics of the reference's
            ``LifelikeCA`` (``examples/game_of_life.py:183-203``); uint8 0/1.
``life3d``  Life-like on a 3-D torus, von Neumann neighbourhood (6), B bits
            0-6, S bits 7-13; uint8 0/1.
``mass``    the mass-transfer model (3-D von Neumann, StaticBorder wall
            2**32-1); uint32 masses.  The total mass after the last generation
            is returned with the result.

:func:`serving_workload` draws the seeded request mix of the serving
benchmark: Poisson arrivals, 2-D sides log-uniform in [32, 4096], 3-D sides
log-uniform in [64, 256], generations uniform in [100, 10000].
"""
import ctypes

import numpy as np

from xentica_gb300 import _native as nat
from xentica_gb300.batch import hash64
from xentica_gb300.core.exceptions import XenticaException

__all__ = ['Server', 'Request', 'KINDS', 'request_bytes', 'serving_workload', 'make_cells',
           'poisson_arrivals', 'latency_summary']

KINDS = {"life2d": nat.XK_SERVE_LIFE2D, "life3d": nat.XK_SERVE_LIFE3D_VN,
         "mass": nat.XK_SERVE_MASS3D}
_DTYPES = {"life2d": np.uint8, "life3d": np.uint8, "mass": np.uint32}
_STATUS = {nat.XK_REQ_PENDING: "pending", nat.XK_REQ_ACTIVE: "active",
           nat.XK_REQ_DONE: "done", nat.XK_REQ_CANCELLED: "cancelled",
           nat.XK_REQ_FAILED: "failed"}


def _request(kind, shape, rule, generations):
    if kind not in KINDS:
        raise XenticaException("unknown request kind %r (one of %s)" % (kind, sorted(KINDS)))
    req = nat.XkRequest()
    req.kind = KINDS[kind]
    dims = tuple(int(s) for s in reversed(shape))      # axis 0 (x) first
    want = 2 if kind == "life2d" else 3
    if len(dims) != want:
        raise XenticaException("%s cells need %d dimensions, got shape %s" % (kind, want, shape))
    for i in range(3):
        req.size[i] = dims[i] if i < len(dims) else 1
    req.rule = int(rule)
    req.generations = int(generations)
    return req


def request_bytes(kind, shape, rule=0, generations=0):
    """Device bytes a request is admitted with (validates it)."""
    req = _request(kind, shape, rule, generations)
    out = ctypes.c_int64()
    nat.check(nat.load().xk_serve_request_bytes(ctypes.byref(req), ctypes.byref(out)),
              "xk_serve_request_bytes")
    return out.value


class Request:
    """Handle of a submitted request."""

    def __init__(self, server, rid, kind, shape):
        self.server = server
        self.id = rid
        self.kind = kind
        self.shape = tuple(shape)
        self._result = None
        self._info = None

    def info(self):
        """Status and timings (seconds since the server started)."""
        if self._info is not None:
            return self._info
        out = nat.XkRequestInfo()
        nat.check(self.server._lib.xk_serve_info(self.server._h, self.id, ctypes.byref(out)),
                  "xk_serve_info")
        return _info_dict(out)

    def status(self):
        return self.info()["status"]

    def wait(self, timeout=None):
        """Block until done, cancelled or failed; returns :meth:`info`."""
        if self._info is not None:
            return self._info
        out = nat.XkRequestInfo()
        rc = self.server._lib.xk_serve_wait(self.server._h, self.id,
                                            -1.0 if timeout is None else float(timeout),
                                            ctypes.byref(out))
        nat.check(rc, "xk_serve_wait")
        return _info_dict(out)

    def result(self, timeout=None):
        """The final cells (same shape as submitted); collects the request."""
        if self._result is not None:
            return self._result
        info = self.wait(timeout)
        if info["status"] != "done":
            raise XenticaException("request %d ended %s" % (self.id, info["status"]))
        out = np.empty(self.shape, dtype=_DTYPES[self.kind])
        nat.check(self.server._lib.xk_serve_result(self.server._h, self.id, nat.ptr(out), out.size),
                  "xk_serve_result")
        self._info = info
        self._result = out
        return out

    def cancel(self):
        nat.check(self.server._lib.xk_serve_cancel(self.server._h, self.id), "xk_serve_cancel")


def _info_dict(out):
    return {"status": _STATUS.get(out.status, str(out.status)),
            "generations_done": out.generations_done, "submit_s": out.submit_s,
            "admit_s": out.admit_s, "done_s": out.done_s, "mass_total": out.mass_total}


class Server:
    """A request loop on the current GPU.

    :param budget_bytes: device arena for request state (HBM budget).
    :param host_bytes: pinned host arena for results (0: min(budget, 8 GiB)).
    :param max_active: requests on the device at once.
    :param quantum: generations per round of a large lattice (small 2-D
        lattices run about quantum x 2^18 cell-generations per round).
    """

    def __init__(self, budget_bytes, host_bytes=0, max_active=1024, quantum=128):
        self._lib = nat.load()
        self._h = ctypes.c_void_p()
        nat.check(self._lib.xk_serve_create(int(budget_bytes), int(host_bytes), int(max_active),
                                            int(quantum), ctypes.byref(self._h)),
                  "xk_serve_create")

    def submit(self, kind, cells, rule=0, generations=1):
        """Queue a request; returns its :class:`Request`."""
        cells = np.ascontiguousarray(cells, dtype=_DTYPES.get(kind, np.uint8))
        req = _request(kind, cells.shape, rule, generations)
        rid = ctypes.c_int64()
        nat.check(self._lib.xk_serve_submit(self._h, ctypes.byref(req), nat.ptr(cells),
                                            ctypes.byref(rid)), "xk_serve_submit")
        return Request(self, rid.value, kind, cells.shape)

    def stats(self):
        st = nat.XkServeStats()
        nat.check(self._lib.xk_serve_stats_get(self._h, ctypes.byref(st)), "xk_serve_stats_get")
        return {name: getattr(st, name) for name, _ in nat.XkServeStats._fields_}

    def close(self):
        """Cancel what is left and free the device and host arenas."""
        if self._h:
            self._lib.xk_serve_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


# ---------------------------------------------------------------------------
# the serving benchmark's request mix

def _log_uniform_int(rng, lo, hi, size=None):
    return np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), size))).astype(np.int64)


def serving_workload(count, seed=2041, mix=(0.5, 0.25, 0.25), sides2d=(32, 4096),
                     sides3d=(64, 256), generations=(100, 10000)):
    """``count`` request specs: kind, shape, rule, density, generations and a
    per-request cell seed, all from ``numpy.random.default_rng(seed)``.

    ``mix`` is the share of (life2d, life3d, mass) requests; each side of a
    2-D lattice is log-uniform in ``sides2d``, of a 3-D lattice in ``sides3d``;
    Life rules are uniform over all rules of the kind, densities uniform in
    [0.1, 0.6]; masses are Poisson(4).
    """
    rng = np.random.default_rng(seed)
    kinds = rng.choice(["life2d", "life3d", "mass"], size=count, p=list(mix))
    specs = []
    for i, kind in enumerate(kinds):
        if kind == "life2d":
            w, h = _log_uniform_int(rng, *sides2d, size=2)
            shape, rule = (int(h), int(w)), int(rng.integers(0, 2 ** 18))
        else:
            w, h, d = _log_uniform_int(rng, *sides3d, size=3)
            shape = (int(d), int(h), int(w))
            rule = int(rng.integers(0, 2 ** 14)) if kind == "life3d" else 0
        specs.append({"kind": str(kind), "shape": shape, "rule": rule,
                      "p": float(rng.uniform(0.1, 0.6)),
                      "generations": int(rng.integers(generations[0], generations[1] + 1)),
                      "seed": hash64(seed, i + 1)})
    return specs


def make_cells(spec):
    """Initial cells of a request spec (seeded)."""
    rng = np.random.RandomState(spec["seed"] & 0xFFFFFFFF)
    n = int(np.prod(spec["shape"]))
    if spec["kind"] == "mass":
        return rng.poisson(4, n).astype(np.uint32).reshape(spec["shape"])
    return (rng.random_sample(n) < spec["p"]).astype(np.uint8).reshape(spec["shape"])


def poisson_arrivals(rate, count, seed=2041):
    """Arrival times (seconds from 0) of a Poisson process of ``rate`` per second."""
    gaps = np.random.default_rng(seed).exponential(1.0 / rate, count)
    return np.cumsum(gaps)


def latency_summary(values):
    """p50 / p90 / p99 / max / mean of a list of seconds."""
    v = np.asarray(values, dtype=np.float64)
    if v.size == 0:
        return {"p50": None, "p90": None, "p99": None, "max": None, "mean": None}
    return {"p50": float(np.percentile(v, 50)), "p90": float(np.percentile(v, 90)),
            "p99": float(np.percentile(v, 99)), "max": float(v.max()), "mean": float(v.mean())}
