"""Python front-end of the CPU oracle (``oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the checker; the product path never
imports it.

Every function works on the reference's own memory layout
(``xentica/core/base.py:659-661``): a flat ``fld`` array of
``n * (N + 1) + 1`` packed cells (main plane first) and an ``int32`` colour
array of ``3 * n``.  Topology tables follow the reference exactly:

* Moore neighbours are ``itertools.product([-1, 0, 1], repeat=d)`` minus the
  2-D zero vector, truncated to ``3**d - 1`` entries, and ``rev_index_map`` is
  the reversed index list (``core/topology/neighborhood.py:151-167``);
* von Neumann neighbours are ``+e_i, -e_i`` per axis with pairwise-swapped
  ``rev_index_map`` (``neighborhood.py:170-190``).
"""
import ctypes
import itertools
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
MAXDIM = 16


def build():
    """Compile ``oracle.c`` (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return os.path.join(HERE, "_build", "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        src = os.path.join(HERE, "oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        _LIB = ctypes.CDLL(path)
    return _LIB


def neighborhood(kind, ndim):
    """(deltas [N x ndim] int8, rev_index_map [N] int32) as the reference builds them."""
    if kind == "moore":
        num = 3 ** ndim - 1
        deltas = [d for d in itertools.product([-1, 0, 1], repeat=ndim) if d != (0, 0)]
        deltas = deltas[:num]
        rev = list(range(num))[::-1]
    elif kind in ("vonneumann", "von_neumann", "vn"):
        deltas, rev = [], []
        for i in range(ndim):
            deltas.append(tuple(1 if i == j else 0 for j in range(ndim)))
            deltas.append(tuple(-1 if i == j else 0 for j in range(ndim)))
            rev += [i * 2 + 1, i * 2]
    else:
        raise ValueError(kind)
    return np.array(deltas, dtype=np.int8).reshape(-1, ndim), np.array(rev, dtype=np.int32)


class _Topo(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int), ("size", ctypes.c_int64 * MAXDIM),
                ("nbr", ctypes.c_int), ("delta", ctypes.c_void_p),
                ("rev", ctypes.c_void_p), ("torus", ctypes.c_int),
                ("border_value", ctypes.c_uint64)]


class _Color(ctypes.Structure):
    _fields_ = [("fade_in", ctypes.c_int32), ("fade_out", ctypes.c_int32),
                ("smooth", ctypes.c_int32), ("moving_average", ctypes.c_int)]


class _Evo(ctypes.Structure):
    _fields_ = [("death_speed", ctypes.c_uint32), ("max_genes", ctypes.c_uint32),
                ("mutation_prob", ctypes.c_double), ("positional", ctypes.c_int),
                ("pos_lut", ctypes.c_void_p)]


class Topology:
    """Lattice + neighbourhood + border in the form ``oracle.c`` takes."""

    def __init__(self, size, neighborhood_kind="moore", border=None):
        self.size = tuple(int(s) for s in size)
        self.ndim = len(self.size)
        self.deltas, self.rev = neighborhood(neighborhood_kind, self.ndim)
        self.nbr = len(self.rev)
        self.torus = border is None
        self.border_value = 0 if border is None else int(border)
        self.cells = int(np.prod(self.size))
        self._c = _Topo()
        self._c.ndim = self.ndim
        for d, s in enumerate(self.size):
            self._c.size[d] = s
        self._c.nbr = self.nbr
        self._c.delta = self.deltas.ctypes.data
        self._c.rev = self.rev.ctypes.data
        self._c.torus = int(self.torus)
        self._c.border_value = self.border_value

    def field(self, main, dtype):
        """Reference ``fld`` array with ``main`` in plane 0 (base.py:660-661)."""
        fld = np.zeros(self.cells * (self.nbr + 1) + 1, dtype=dtype)
        fld[:self.cells] = main
        return fld


def _color(moving_average=True, fade_in=255, fade_out=255, smooth=1):
    c = _Color()
    c.fade_in, c.fade_out, c.smooth = fade_in, fade_out, smooth
    c.moving_average = int(moving_average)
    return c


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def life_run(topo, fld, col, steps, born=8, sustain=12, bits=1, color=None,
             threads=None, rule_schedule=None, lut=(0, 0, 0, 255, 255, 255)):
    """Advance a Life-like model ``steps`` generations in place.

    next = ((born >> k) & 1) | ((sustain >> k) & 1 & state); ``lut`` is the
    rgb of state 0 then state 1 before the colour effect.  ``rule_schedule``
    optionally maps a timestep to a new ``(born, sustain)`` applied before
    that step (an interactive rule parameter).
    """
    threads = threads or os.cpu_count()
    cc = color or _color()
    lut6 = np.ascontiguousarray(lut, dtype=np.int32)
    fn = lib().xo_life_step
    fn.restype = None
    for t in range(steps):
        if rule_schedule and t in rule_schedule:
            born, sustain = rule_schedule[t]
        fn(ctypes.byref(topo._c), _ptr(fld), ctypes.c_int(fld.itemsize), ctypes.c_int(bits),
           ctypes.c_uint32(born), ctypes.c_uint32(sustain), _ptr(col),
           ctypes.byref(cc), _ptr(lut6), ctypes.c_int(threads))


def shift_run(topo, fld, col, steps, plane0, lut, color=None, threads=None):
    """Advance a ShiftingSands-style model ``steps`` generations in place:
    emit writes the state into plane ``plane0`` (1..N) and 0 into the others,
    absorb sums the neighbours' buffers; ``lut`` is the rgb for every sum
    0..N before the colour effect."""
    threads = threads or os.cpu_count()
    cc = color or _color()
    lut = np.ascontiguousarray(lut, dtype=np.int32)
    fn = lib().xo_shift_step
    fn.restype = None
    for _ in range(steps):
        fn(ctypes.byref(topo._c), _ptr(fld), ctypes.c_int(fld.itemsize), ctypes.c_int(plane0),
           _ptr(col), ctypes.byref(cc), _ptr(lut), ctypes.c_int(threads))


def gravity_run(topo, fld, col, steps, color=None, threads=None):
    """Advance a GraviCowboys model (uint64 ``fld``) ``steps`` generations in
    place (``oracle.c``: ``xo_gravity_step``)."""
    threads = threads or os.cpu_count()
    cc = color or _color()
    fn = lib().xo_gravity_step
    fn.restype = None
    for _ in range(steps):
        fn(ctypes.byref(topo._c), _ptr(fld), _ptr(col), ctypes.byref(cc), ctypes.c_int(threads))


def noise_run(topo, fld, col, steps, color=None, threads=None):
    """Advance a NoiseTV model (uint16 ``fld``) ``steps`` generations in place
    (``oracle.c``: ``xo_noise_step``)."""
    threads = threads or os.cpu_count()
    cc = color or _color()
    fn = lib().xo_noise_step
    fn.restype = None
    for _ in range(steps):
        fn(ctypes.byref(topo._c), _ptr(fld), _ptr(col), ctypes.byref(cc), ctypes.c_int(threads))


def lifecolor_run(topo, fld, col, steps, color=None, threads=None):
    """Advance a GameOfLifeColor model (uint32 ``fld``) ``steps`` generations
    in place (``oracle.c``: ``xo_lifecolor_step``)."""
    threads = threads or os.cpu_count()
    cc = color or _color()
    fn = lib().xo_lifecolor_step
    fn.restype = None
    for _ in range(steps):
        fn(ctypes.byref(topo._c), _ptr(fld), _ptr(col), ctypes.byref(cc), ctypes.c_int(threads))


def mass_run(topo, fld, col, steps, wall=2 ** 32 - 1, threads=None, totals=None):
    """Advance the mass-transfer model; optionally record the total mass per step."""
    threads = threads or os.cpu_count()
    fn = lib().xo_mass_step
    fn.restype = None
    for _ in range(steps):
        fn(ctypes.byref(topo._c), _ptr(fld), _ptr(col), ctypes.c_uint32(wall),
           ctypes.c_int(threads))
        if totals is not None:
            totals.append(int(fld[:topo.cells].astype(np.uint64).sum()))


def positional_lut(num_genes=18):
    """Per-gene double weights of GenomeColor.positional (tools/color.py:63-104),
    computed as the reference's non-deferred hsv2rgb branch does."""
    out = np.zeros((num_genes, 3), dtype=np.float64)
    for i in range(num_genes):
        hue, sat, val = i / num_genes, 1, 1 / num_genes
        hue_f = hue * 6
        hue_i = int(hue_f)
        hue_f -= hue_i
        grad_p = val * (1 - sat)
        grad_q = val * (1 - sat * hue_f)
        grad_t = val * (1 - sat * (1 - hue_f))
        red = ((hue_i == 0) | (hue_i >= 5)) * val
        red = red + (hue_i == 1) * grad_q
        red = red + ((hue_i == 2) | (hue_i == 3)) * grad_p
        red = red + (hue_i == 4) * grad_t
        green = ((hue_i == 0) | (hue_i >= 6)) * grad_t
        green = green + ((hue_i == 1) | (hue_i == 2)) * val
        green = green + (hue_i == 3) * grad_q
        green = green + ((hue_i == 4) | (hue_i == 5)) * grad_p
        blue = ((hue_i == 0) | (hue_i == 1) | (hue_i >= 6)) * grad_p
        blue = blue + (hue_i == 2) * grad_t
        blue = blue + ((hue_i == 3) | (hue_i == 4)) * val
        blue = blue + (hue_i == 5) * grad_q
        out[i] = (red, green, blue)
    return out


def evolife_run(topo, fld, col, steps, death_speed=15, max_genes=9,
                mutation_prob=0.0, positional=False, fade_in=18, fade_out=3,
                smooth=1, threads=None):
    """Advance EvoLife ``steps`` generations in place (uint64 ``fld``)."""
    threads = threads or os.cpu_count()
    lut = positional_lut()
    p = _Evo()
    p.death_speed, p.max_genes = death_speed, max_genes
    p.mutation_prob = float(mutation_prob)
    p.positional = int(positional)
    p.pos_lut = lut.ctypes.data
    cc = _color(True, fade_in, fade_out, smooth)
    fn = lib().xo_evolife_step
    fn.restype = None
    for _ in range(steps):
        fn(ctypes.byref(topo._c), _ptr(fld), _ptr(col), ctypes.byref(p),
           ctypes.byref(cc), ctypes.c_int(threads))


def render(topo, col, width, height, zoom=1, dx=0, dy=0, axes=(0, 1),
           smooth=1, threads=None):
    """RendererPlain image (int32, ``width * height * 3``); ``smooth=0`` when the
    model defines no SMOOTH_FACTOR (plain ColorEffect)."""
    threads = threads or os.cpu_count()
    img = np.zeros(width * height * 3, dtype=np.int32)
    fn = lib().xo_render
    fn.restype = None
    fn(ctypes.byref(topo._c), _ptr(col), _ptr(img), ctypes.c_int(width),
       ctypes.c_int(height), ctypes.c_int(zoom), ctypes.c_int(dx), ctypes.c_int(dy),
       ctypes.c_int(axes[0]), ctypes.c_int(axes[1]), ctypes.c_int(smooth),
       ctypes.c_int(threads))
    return img
