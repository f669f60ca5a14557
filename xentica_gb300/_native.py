"""ctypes binding of ``libxk.so`` (the C-ABI declared in ``include/xk.h``).

The library is built in-tree by :mod:`xentica_gb300.build`.  Nothing here
falls back to another implementation: if the library or a CUDA device is
missing, every GPU entry point raises :class:`XenticaException`.
"""
import ctypes
import os
import threading

from xentica_gb300.core.exceptions import XenticaException

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libxk.so")

XK_ABI_VERSION = 1
XK_MAXDIM = 8
XK_MAXNBR = 32
XK_FAMILY_LIFE, XK_FAMILY_EVOLIFE, XK_FAMILY_MASS, XK_FAMILY_VM, XK_FAMILY_SHIFT = 1, 2, 3, 4, 5
XK_FAMILY_LIFECOLOR = 6
XK_FAMILY_NOISE = 7
XK_FAMILY_GRAVITY = 8
XK_COLOR_NONE, XK_COLOR_PLAIN, XK_COLOR_MOVING_AVERAGE = 0, 1, 2

_I32, _U32, _I64, _U64 = ctypes.c_int32, ctypes.c_uint32, ctypes.c_int64, ctypes.c_uint64
_P = ctypes.c_void_p


class XkDesc(ctypes.Structure):
    """Mirror of ``xk_desc``."""

    _fields_ = [
        ("abi_version", _I32), ("family", _I32), ("ndim", _I32), ("nbr", _I32),
        ("size", _I64 * XK_MAXDIM),
        ("delta", (ctypes.c_int8 * XK_MAXDIM) * XK_MAXNBR),
        ("torus", _I32), ("state_bytes", _I32),
        ("border_value", _U64),
        ("color_kind", _I32), ("fade_in", _I32), ("fade_out", _I32), ("smooth", _I32),
        ("proj_axis0", _I32), ("proj_axis1", _I32), ("render_smooth", _I32),
        ("rule0", _U32), ("rule1", _U32),
        ("color_lut", _I32 * 6),
        ("color_history_free", _I32),
        ("death_speed", _U32), ("max_genes", _U32),
        ("mutation_prob", ctypes.c_double),
        ("positional", _I32),
        ("palette", ctypes.c_double * 54),
        ("wall", _U32),
        ("reserved", _I32 * 8),
    ]


XK_SERVE_LIFE2D, XK_SERVE_LIFE3D_VN, XK_SERVE_MASS3D = 1, 2, 3
XK_REQ_PENDING, XK_REQ_ACTIVE, XK_REQ_DONE, XK_REQ_CANCELLED, XK_REQ_FAILED = 0, 1, 2, 3, 4
XK_ERR_ARG, XK_ERR_CUDA, XK_ERR_OOM, XK_ERR_UNSUPPORTED, XK_ERR_STATE, XK_ERR_TIMEOUT = -1, -2, -3, -4, -5, -6


class XkRequest(ctypes.Structure):
    """Mirror of ``xk_request``."""

    _fields_ = [("kind", _I32), ("reserved0", _I32), ("size", _I64 * 3), ("rule", _U32),
                ("reserved1", _I32), ("generations", _I64)]


class XkRequestInfo(ctypes.Structure):
    """Mirror of ``xk_request_info``."""

    _fields_ = [("status", _I32), ("reserved", _I32), ("generations_done", _I64),
                ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("done_s", ctypes.c_double), ("mass_total", _U64)]


class XkServeStats(ctypes.Structure):
    """Mirror of ``xk_serve_stats``."""

    _fields_ = [(name, _I64) for name in (
        "submitted", "admitted", "completed", "cancelled", "rejected", "failed", "pending",
        "active", "device_bytes_in_use", "device_bytes_peak", "budget_bytes", "cell_updates",
        "rounds", "launches")] + [("elapsed_s", ctypes.c_double)]


# name -> (restype, argtypes); every symbol declared in include/xk.h
SIGNATURES = {
    "xk_model_create": (_I32, [ctypes.POINTER(XkDesc), ctypes.POINTER(_P)]),
    "xk_model_destroy": (None, [_P]),
    "xk_upload": (_I32, [_P, _P, _I64]),
    "xk_download": (_I32, [_P, _P, _I64]),
    "xk_upload_colors": (_I32, [_P, _P, _I64]),
    "xk_colors_range": (_I32, [_P, _P]),
    "xk_download_colors": (_I32, [_P, _P, _I64]),
    "xk_life_set_rule": (_I32, [_P, _U32, _U32, _P]),
    "xk_set_color_mode": (_I32, [_P, _I32]),
    "xk_step": (_I32, [_P, _I64]),
    "xk_render": (_I32, [_P, _P, _I32, _I32, _I32, _I32, _I32]),
    "xk_step_frames": (_I32, [_P, _I64, _I32, _I32, _I32, _I32, _I32, _P, _I32]),
    "xk_model_plan": (_I32, [_P, _P]),
    "xk_model_set_plan": (_I32, [_P, _P]),
    "xk_mass_totals": (_I32, [_P, _P, _I64]),
    "xk_sync": (_I32, [_P]),
    "xk_last_step_ms": (ctypes.c_double, []),
    "xk_batch_create": (_I32, [_I32, _P, _P, _P, ctypes.POINTER(_P)]),
    "xk_batch_destroy": (None, [_P]),
    "xk_batch_upload": (_I32, [_P, _P, _I64]),
    "xk_batch_download": (_I32, [_P, _P, _I64]),
    "xk_batch_step": (_I32, [_P, _I32]),
    "xk_batch_step_plain": (_I32, [_P, _I32]),
    "xk_batch_seed_bernoulli": (_I32, [_P, _P, _P]),
    "xk_batch_run": (_I32, [_P, _P, _P, _I64, _I32]),
    "xk_batch_tune": (_I32, [_P, _I32, ctypes.POINTER(_I32)]),
    "xk_batch_set_band": (_I32, [_P, _I32]),
    "xk_batch_add": (_I32, [_P, _I32, _I32, _U32, _P]),
    "xk_batch_remove": (_I32, [_P, _I32]),
    "xk_batch_count": (_I32, [_P]),
    "xk_batch_band": (_I32, [_P]),
    "xk_model_rule_form": (_I32, [_P]),
    "xk_batch_set_size_bands": (_I32, [_P, _P, _I32]),
    "xk_batch_size_bands": (_I32, [_P, _P, _I32]),
    "xk_batch_total_cells": (_I64, [_P]),
    "xk_batch_launches": (_I64, [_P, _I32]),
    "xk_batch_step_noalloc": (_I32, [_P, _I32, _P, _P, _P, _I32, _P]),
    "xk_vm_load": (_I32, [_P, _I32, _P, _I32, _P, _I32, _I32]),
    "xk_vm_set_params": (_I32, [_P, _P, _I32]),
    "xk_serve_create": (_I32, [_I64, _I64, _I32, _I32, ctypes.POINTER(_P)]),
    "xk_serve_destroy": (_I32, [_P]),
    "xk_serve_request_bytes": (_I32, [ctypes.POINTER(XkRequest), ctypes.POINTER(_I64)]),
    "xk_serve_submit": (_I32, [_P, ctypes.POINTER(XkRequest), _P, ctypes.POINTER(_I64)]),
    "xk_serve_info": (_I32, [_P, _I64, ctypes.POINTER(XkRequestInfo)]),
    "xk_serve_wait": (_I32, [_P, _I64, ctypes.c_double, ctypes.POINTER(XkRequestInfo)]),
    "xk_serve_result": (_I32, [_P, _I64, _P, _I64]),
    "xk_serve_cancel": (_I32, [_P, _I64]),
    "xk_serve_stats_get": (_I32, [_P, ctypes.POINTER(XkServeStats)]),
    "xk_arena_create": (_I32, [_I64, ctypes.POINTER(_P)]),
    "xk_arena_alloc": (_I32, [_P, _I64, ctypes.POINTER(_I64)]),
    "xk_arena_free": (_I32, [_P, _I64]),
    "xk_arena_stats": (_I32, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                              ctypes.POINTER(_I32)]),
    "xk_arena_destroy": (_I32, [_P]),
    "xk_range_push": (_I32, [ctypes.c_char_p]),
    "xk_range_pop": (_I32, []),
    "xk_set_device": (_I32, [_I32]),
    "xk_host_register": (_I32, [_P, _I64]),
    "xk_host_unregister": (_I32, [_P]),
    "xk_last_error": (ctypes.c_char_p, []),
    "xk_device_info": (_I32, [ctypes.c_char_p, _I32]),
}

_LIB = None
_LOCK = threading.Lock()


def load(path=LIBPATH):
    """Load the library (no CUDA call is made); raises if it is missing."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        if not os.path.exists(path):
            raise XenticaException(
                "libxk.so is not built (%s); run `python -m xentica_gb300.build`" % path)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def last_error():
    msg = load().xk_last_error()
    return msg.decode(errors="replace") if msg else ""


def check(rc, what):
    """Raise :class:`XenticaException` for a non-zero status."""
    if rc != 0:
        raise XenticaException("%s failed (status %d): %s" % (what, rc, last_error()))


def device_info():
    buf = ctypes.create_string_buffer(256)
    check(load().xk_device_info(buf, 256), "xk_device_info")
    return buf.value.decode()


def set_device(device):
    """Make ``device`` current for libxk handles created on this thread."""
    check(load().xk_set_device(int(device)), "xk_set_device")


class PinnedBuffer:
    """A page-locked host array (NumPy) for fast host<->device copies."""

    def __init__(self, nbytes, dtype="uint8"):
        import numpy as np
        self.array = np.empty(nbytes, dtype=dtype)
        check(load().xk_host_register(ptr(self.array), self.array.nbytes), "xk_host_register")

    def release(self):
        if self.array is not None:
            load().xk_host_unregister(ptr(self.array))
            self.array = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def ptr(array):
    """Raw pointer of a contiguous NumPy array."""
    if not array.flags["C_CONTIGUOUS"]:
        raise XenticaException("array must be C-contiguous")
    return ctypes.c_void_p(array.ctypes.data)
