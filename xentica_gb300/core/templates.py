"""Template matcher: traced model -> hand-written GB300 kernel + parameters.

This replaces the reference's code generation (``xentica/core/base.py:440-541``,
PyCUDA ``SourceModule``).  A model's traced programs (``model.programs``) are
analysed and, when they implement a family one of the libxk kernels computes,
turned into an ``xk_desc``: the family and its rule parameters.  Anything else
raises :class:`XenticaException` -- there is no fallback.

Life-like family (``XK_FAMILY_LIFE``)
    one integer property whose values stay in {0, 1}; ``emit`` copies it to
    every buffer; ``absorb`` sets it from its own value and the *sum* of the
    neighbours' buffers; the colour is a function of the new state.  The rule
    is read off by executing the traced absorb (with C semantics) on every
    combination of a cell's state and its neighbours' buffers -- 2**(N+1)
    lanes at once -- and checking that the result depends on the neighbours
    only through their sum.  Interactive parameters are re-bound and the rule
    re-extracted whenever their values change (LifelikeCA,
    ``examples/game_of_life.py:183-203``).

Shifting family (``XK_FAMILY_SHIFT``)
    ShiftingSands: one 1-bit property sent into one buffer and absorbed as the
    sum of the neighbours' buffers, i.e. moved by one neighbour offset per
    generation (see :class:`ShiftTemplate`).

EvoLife (``XK_FAMILY_EVOLIFE``), mass transfer (``XK_FAMILY_MASS``), colour Life
(``XK_FAMILY_LIFECOLOR``) and noise (``XK_FAMILY_NOISE``)
    matched statement by statement against the canonical programs of
    ``core/canonical.py``.

Interpreter (``XK_FAMILY_VM``)
    any other model whose programs hold no opaque C text: compiled to
    register bytecode (``core/vm.py``) and run by the generic kernel.
"""
import os

import numpy as np

from xentica_gb300 import _native as nat
from xentica_gb300.core import ir
from xentica_gb300.core.exceptions import XenticaException
from xentica_gb300.core.properties import IntegerProperty
from xentica_gb300.core.topology.border import TorusBorder, StaticBorder
from xentica_gb300.core.topology.lattice import OrthogonalLattice
from xentica_gb300.core.topology.neighborhood import OrthogonalNeighborhood
from xentica_gb300.core.renderers import RendererPlain

__all__ = ['match', 'LifeTemplate', 'ShiftTemplate', 'LifeColorTemplate', 'NoiseTemplate', 'NoTemplate']

MAX_EXHAUSTIVE_NBR = 16


class NoTemplate(Exception):
    """Raised internally when a family does not match (with the reason)."""


def _topology(model):
    topo = model.topology
    if not isinstance(topo.lattice, OrthogonalLattice):
        raise NoTemplate("lattice %s" % type(topo.lattice).__name__)
    if not isinstance(topo.neighborhood, OrthogonalNeighborhood):
        raise NoTemplate("neighbourhood %s" % type(topo.neighborhood).__name__)
    deltas = topo.neighborhood.deltas
    if len(deltas) > nat.XK_MAXNBR - 1:
        raise NoTemplate("%d neighbours (max %d)" % (len(deltas), nat.XK_MAXNBR - 1))
    if topo.dimensions > nat.XK_MAXDIM:
        raise NoTemplate("%d dimensions (max %d)" % (topo.dimensions, nat.XK_MAXDIM))
    if isinstance(topo.border, TorusBorder):
        torus, border = True, 0
    elif isinstance(topo.border, StaticBorder):
        torus, border = False, int(topo.border.value)
    else:
        raise NoTemplate("border %s" % type(topo.border).__name__)
    return deltas, torus, border


def _base_desc(model, family):
    deltas, torus, border = _topology(model)
    d = nat.XkDesc()
    d.abi_version = nat.XK_ABI_VERSION
    d.family = family
    d.ndim = model.topology.dimensions
    d.nbr = len(deltas)
    for i, s in enumerate(model.size[:d.ndim]):
        d.size[i] = int(s)
    for k, delta in enumerate(deltas):
        for i, v in enumerate(delta):
            d.delta[k][i] = int(v)
    d.torus = int(torus)
    d.state_bytes = np.dtype(model.main.dtype).itemsize
    d.border_value = border & 0xFFFFFFFFFFFFFFFF
    renderer = model.renderer
    axes = tuple(getattr(renderer, "projection_axes", (0, 1)))
    d.proj_axis0, d.proj_axis1 = (int(axes[0]), int(axes[1])) if d.ndim > 1 else (0, 0)
    d.render_smooth = 0
    if model.is_constant("SMOOTH_FACTOR"):
        d.render_smooth = int(model.constants["SMOOTH_FACTOR"].value)
    return d


def _color_stmt(program):
    stmts = [st for st in program.stmts if st.op == "color"]
    if len(stmts) > 1:
        raise NoTemplate("colour written more than once")
    return stmts[0] if stmts else None


def _store_keys(program):
    return {st.extra for st in program.stmts if st.op == "store"}


class LifeTemplate:
    """Binary outer-totalistic rule; see the module docstring."""

    family = nat.XK_FAMILY_LIFE

    def __init__(self, model):
        props = list(model.main.properties.values())
        if len(props) != 1 or not isinstance(props[0], IntegerProperty):
            raise NoTemplate("needs exactly one IntegerProperty")
        self.model = model
        self.prop = props[0]
        self.mask = (1 << self.prop.bit_width) - 1
        deltas, torus, border = _topology(model)
        self.nbr = len(deltas)
        self.border_state = border & self.mask
        if not torus and self.border_state not in (0, 1):
            raise NoTemplate("static border state %d is not 0/1" % self.border_state)
        self._check_emit(model.programs["emit"])
        absorb = model.programs["absorb"]
        loads = absorb.loads()
        allowed = {("main", -1)} | {("nbuf", k) for k in range(self.nbr)}
        if not loads <= allowed:
            raise NoTemplate("absorb reads %s" % sorted(loads - allowed))
        if _store_keys(absorb) != {("main", 0)}:
            raise NoTemplate("absorb must write only the cell's own main state")
        self.absorb = absorb
        self.color = _color_stmt(absorb)
        if self.color is not None and self.color.extra["kind"] not in ("plain", "moving_average"):
            raise NoTemplate("custom colour effect")
        self.param_names = sorted(absorb.params())
        self._cache = {}
        self.rule0, self.rule1, self.lut = self.rule_for(self.current_params())

    # -- analysis ----------------------------------------------------------
    def _check_emit(self, emit):
        loads = emit.loads()
        if not loads <= {("main", -1)}:
            raise NoTemplate("emit reads %s" % sorted(loads))
        if emit.params():
            raise NoTemplate("emit depends on parameters")
        keys = _store_keys(emit)
        planes = {("buf", p) for p in range(1, self.nbr + 1)}
        if keys != planes:
            raise NoTemplate("emit must write every buffer")
        lanes = np.array([0, 1], dtype=np.uint64)
        ev = ir.evaluate(emit, {("main", -1): lanes}, lanes=2)
        for key in planes:
            out = ev.stores[key].astype(np.uint64) & np.uint64(self.mask)
            if not np.array_equal(out, lanes):
                raise NoTemplate("emit does not copy the state to every buffer")

    def current_params(self):
        return {name: self.model.meta.__dict__[name].value for name in self.param_names}

    def _inputs(self):
        n = self.nbr
        if n <= MAX_EXHAUSTIVE_NBR:
            combos = np.arange(2 ** (n + 1), dtype=np.uint64)
        else:
            rng = np.random.RandomState(12345)
            combos = rng.randint(0, 2 ** 62, size=1 << 17, dtype=np.int64).astype(np.uint64)
            # make sure every (state, count) pair is present
            extra = []
            for s in (0, 1):
                for k in range(n + 1):
                    extra.append((((1 << k) - 1) << 1) | s)
            combos = np.concatenate([combos & np.uint64((1 << (n + 1)) - 1),
                                     np.array(extra, dtype=np.uint64)])
        state = combos & np.uint64(1)
        inputs = {("main", -1): state}
        count = np.zeros(len(combos), dtype=np.int64)
        for k in range(n):
            bit = (combos >> np.uint64(k + 1)) & np.uint64(1)
            inputs[("nbuf", k)] = bit
            count += bit.astype(np.int64)
        return inputs, state.astype(np.int64), count

    def rule_for(self, params):
        """``(rule0, rule1, lut6)`` for the given interactive parameter values."""
        key = tuple(sorted(params.items()))
        if key in self._cache:
            return self._cache[key]
        inputs, state, count = self._inputs()
        ev = ir.evaluate(self.absorb, inputs, params=params, lanes=len(state))
        new = ev.stores[("main", 0)].astype(np.uint64) & np.uint64(self.mask)
        if np.any(new > 1):
            raise XenticaException("Life-like absorb produced a state other than 0/1")
        new = new.astype(np.int64)
        rules = [0, 0]
        for s in (0, 1):
            for k in range(self.nbr + 1):
                sel = (state == s) & (count == k)
                vals = np.unique(new[sel])
                if len(vals) > 1:
                    raise XenticaException(
                        "absorb depends on more than the number of live neighbours")
                if len(vals) and vals[0]:
                    rules[s] |= 1 << k
        lut = [0] * 6
        if ev.color is not None:
            rgb = ev.color[0]
            for s in (0, 1):
                sel = new == s
                for c in range(3):
                    vals = np.unique(rgb[c][sel])
                    if len(vals) > 1:
                        raise XenticaException("colour depends on more than the new state")
                    if len(vals):
                        lut[3 * s + c] = int(vals[0])
        result = (rules[0], rules[1], lut)
        self._cache[key] = result
        return result

    # -- colour bookkeeping ------------------------------------------------
    def color_kind(self):
        if self.color is None:
            return nat.XK_COLOR_NONE
        if self.color.extra["kind"] == "moving_average":
            return nat.XK_COLOR_MOVING_AVERAGE
        return nat.XK_COLOR_PLAIN

    def _fades(self):
        info = self.color.extra
        return info.get("fade_in", 0), info.get("fade_out", 0), info.get("smooth", 1)

    def history_free(self, lut, old_colors):
        """Whether one step makes every colour equal its state's table value,
        given the colours ``old_colors`` hold (min, max) before it."""
        kind = self.color_kind()
        if kind != nat.XK_COLOR_MOVING_AVERAGE:
            return True
        fade_in, fade_out, smooth = self._fades()
        vals = [v * smooth for v in lut]
        vmin, vmax = min(vals), max(vals)
        omin, omax = old_colors
        first = (omax - fade_out <= vmin) and (vmax <= omin + fade_in)
        steady = (vmax - vmin <= fade_in) and (vmax - vmin <= fade_out)
        return first and steady

    def descriptor(self):
        d = _base_desc(self.model, self.family)
        d.border_value = self.border_state
        d.rule0, d.rule1 = self.rule0, self.rule1
        for i, v in enumerate(self.lut):
            d.color_lut[i] = int(v)
        d.color_kind = self.color_kind()
        if self.color is not None:
            d.fade_in, d.fade_out, d.smooth = self._fades()
        else:
            d.smooth = 1
        d.color_history_free = int(self.history_free(self.lut, (0, 0)))
        return d


class ShiftTemplate(LifeTemplate):
    """ShiftingSands' family (``examples/shifting_sands.py:15-47``): one 1-bit
    property; emit copies it into exactly one buffer plane and writes 0 into
    every other; absorb sets it to the sum of the neighbours' buffers.  Which
    neighbour's plane faces a cell (the one whose state moves in) is read off
    the evaluated emit: the plane written with the state, p, is the plane a
    cell reads from neighbour p - 1.  Absorb is evaluated on every
    combination of the cell's state and its neighbours' buffers and must equal
    their sum masked to the field; the colour is a function of the new state,
    as for the Life-like family."""

    family = nat.XK_FAMILY_SHIFT

    def __init__(self, model):
        props = list(model.main.properties.values())
        if len(props) != 1 or not isinstance(props[0], IntegerProperty):
            raise NoTemplate("needs exactly one IntegerProperty")
        self.model = model
        self.prop = props[0]
        self.mask = (1 << self.prop.bit_width) - 1
        if self.mask != 1:
            raise NoTemplate("needs a 1-bit property")
        deltas, torus, border = _topology(model)
        self.nbr = len(deltas)
        self.border_state = border & self.mask
        emit = model.programs["emit"]
        if not emit.loads() <= {("main", -1)} or emit.params():
            raise NoTemplate("emit reads more than the cell's state")
        planes = {("buf", p) for p in range(1, self.nbr + 1)}
        if _store_keys(emit) != planes:
            raise NoTemplate("emit must write every buffer")
        lanes = np.array([0, 1], dtype=np.uint64)
        ev = ir.evaluate(emit, {("main", -1): lanes}, lanes=2)
        copies, zeros = [], []
        for key in sorted(planes):
            out = ev.stores[key].astype(np.uint64) & np.uint64(self.mask)
            if np.array_equal(out, lanes):
                copies.append(key[1])
            elif not out.any():
                zeros.append(key[1])
        if len(copies) != 1 or len(zeros) != self.nbr - 1:
            raise NoTemplate("emit does not send the state into exactly one buffer")
        self.i0 = copies[0] - 1
        if not torus and self.border_state:
            # edge cells would add the live border once per off-board
            # neighbour: sums above 1, whose colour no state table gives
            raise NoTemplate("static border of live cells")
        absorb = model.programs["absorb"]
        allowed = {("main", -1)} | {("nbuf", k) for k in range(self.nbr)}
        if not absorb.loads() <= allowed or absorb.params():
            raise NoTemplate("absorb reads %s" % sorted(absorb.loads() - allowed))
        if _store_keys(absorb) != {("main", 0)}:
            raise NoTemplate("absorb must write only the cell's own main state")
        self.absorb = absorb
        self.color = _color_stmt(absorb)
        if self.color is not None and self.color.extra["kind"] not in ("plain", "moving_average"):
            raise NoTemplate("custom colour effect")
        inputs, state, count = self._inputs()
        ev = ir.evaluate(absorb, inputs, lanes=len(state))
        new = ev.stores[("main", 0)].astype(np.uint64) & np.uint64(self.mask)
        if not np.array_equal(new.astype(np.int64), count & self.mask):
            raise NoTemplate("absorb is not the sum of the neighbours' buffers")
        # the colour on the inputs that occur: only neighbour i0's buffer can
        # hold a state, every other buffer a cell reads is 0
        reach = np.array([0, 1, 2, 3], dtype=np.uint64)
        rin = {("main", -1): reach & np.uint64(1)}
        for k in range(self.nbr):
            rin[("nbuf", k)] = (reach >> np.uint64(1)) if k == self.i0 else np.zeros(4, np.uint64)
        ev = ir.evaluate(absorb, rin, lanes=4)
        new = ev.stores[("main", 0)].astype(np.uint64) & np.uint64(self.mask)
        lut = [0] * 6
        if ev.color is not None:
            rgb = ev.color[0]
            for s in (0, 1):
                sel = new.astype(np.int64) == s
                for c in range(3):
                    vals = np.unique(rgb[c][sel])
                    if len(vals) > 1:
                        raise NoTemplate("colour depends on more than the new state")
                    if len(vals):
                        lut[3 * s + c] = int(vals[0])
        self.param_names = []
        self.rule0, self.rule1, self.lut = self.i0, 0, lut

    def rule_for(self, params):
        return self.rule0, self.rule1, self.lut


class EvoLifeTemplate:
    """EvoLife (``canonical.EvoLifeProgram``): matched by program fingerprint.

    Parameters come from the model's meta-parameters ``death_speed``,
    ``max_genes``, ``mutation_prob``, its ``_legacy_coloring`` flag and the
    MovingAverage settings; the model's traced programs must equal the
    reference program traced with those values.
    """

    family = nat.XK_FAMILY_EVOLIFE
    PARAMS = ("death_speed", "max_genes", "mutation_prob")

    def __init__(self, model):
        from xentica_gb300.core import canonical
        names = [type(p).__name__ for p in model.main.properties.values()]
        if names != ["IntegerProperty", "TotalisticRuleProperty", "RandomProperty"]:
            raise NoTemplate("not the EvoLife property layout")
        meta = model.meta.__dict__
        if not all(name in meta for name in self.PARAMS):
            raise NoTemplate("missing EvoLife meta-parameters")
        deltas, torus, border = _topology(model)
        if model.topology.dimensions != 2 or len(deltas) != 8 or not torus:
            raise NoTemplate("EvoLife kernel is 2-D Moore on a torus")
        self.model = model
        self.params = {name: meta[name].value for name in self.PARAMS}
        self.legacy = bool(getattr(model, "_legacy_coloring", True))
        attrs = {"_legacy_coloring": self.legacy}
        for name in ("fade_in", "fade_out", "smooth_factor"):
            if name in model.__dict__:
                attrs[name] = model.__dict__[name]
        programs = canonical.trace(canonical.EvoLifeProgram, model.size, self.params, attrs)
        for key in ("emit", "absorb"):
            if ir.fingerprint(programs[key]) != ir.fingerprint(model.programs[key]):
                raise NoTemplate("%s differs from the EvoLife program" % key)
        self.color = _color_stmt(model.programs["absorb"])

    def descriptor(self):
        from xentica_gb300.tools.color import hsv2rgb
        d = _base_desc(self.model, self.family)
        d.death_speed = int(self.params["death_speed"]) & 0xFFFFFFFF
        d.max_genes = int(self.params["max_genes"]) & 0xFFFFFFFF
        d.mutation_prob = float(self.params["mutation_prob"])
        d.positional = int(not self.legacy)
        for i in range(18):
            rgb = hsv2rgb(i / 18, 1, 1 / 18)
            for c in range(3):
                d.palette[3 * i + c] = float(rgb[c])
        info = self.color.extra
        d.color_kind = nat.XK_COLOR_MOVING_AVERAGE
        d.fade_in, d.fade_out, d.smooth = info["fade_in"], info["fade_out"], info["smooth"]
        return d


class MassTemplate:
    """Mass transfer (``canonical.MassTransferProgram``): 3-D von Neumann,
    StaticBorder(2**32 - 1), matched by program fingerprint."""

    family = nat.XK_FAMILY_MASS

    def __init__(self, model):
        from xentica_gb300.core import canonical
        names = [type(p).__name__ for p in model.main.properties.values()]
        if names != ["IntegerProperty"] or model.main.bit_width != 32:
            raise NoTemplate("not one 32-bit integer property")
        deltas, torus, border = _topology(model)
        if model.topology.dimensions != 3 or len(deltas) != 6 or torus \
                or border != canonical.MASS_WALL:
            raise NoTemplate("mass kernel is 3-D von Neumann with a 2**32-1 wall")
        programs = canonical.trace(canonical.MassTransferProgram, model.size, {}, {})
        for key in ("emit", "absorb"):
            if ir.fingerprint(programs[key]) != ir.fingerprint(model.programs[key]):
                raise NoTemplate("%s differs from the mass-transfer program" % key)
        self.model = model
        self.wall = canonical.MASS_WALL

    def descriptor(self):
        d = _base_desc(self.model, self.family)
        d.wall = self.wall
        d.color_kind = nat.XK_COLOR_PLAIN
        d.smooth = 1
        return d


class LifeColorTemplate:
    """Conway's Life whose cells carry three 8-bit colour channels inherited
    from their neighbours (``canonical.LifeColorProgram``: the reference's
    GameOfLifeColor, ``examples/game_of_life.py:112-159``), matched by
    program fingerprint; a 2-D Moore lattice, torus or static border (the
    border is not part of the traced programs), MovingAverage colours with
    the model's fades."""

    family = nat.XK_FAMILY_LIFECOLOR

    def __init__(self, model):
        from xentica_gb300.core import canonical
        props = list(model.main.properties.values())
        if [type(p).__name__ for p in props] != ["IntegerProperty"] * 4 or \
                [p.bit_width for p in props] != [1, 8, 8, 8]:
            raise NoTemplate("not one 1-bit and three 8-bit integer properties")
        deltas, torus, border = _topology(model)
        if model.topology.dimensions != 2 or len(deltas) != 8:
            raise NoTemplate("colour Life kernel is 2-D Moore")
        attrs = {name: model.__dict__[name] for name in ("fade_in", "fade_out", "smooth_factor")
                 if name in model.__dict__}
        programs = canonical.trace(canonical.LifeColorProgram, model.size, {}, attrs)
        for key in ("emit", "absorb"):
            if ir.fingerprint(programs[key]) != ir.fingerprint(model.programs[key]):
                raise NoTemplate("%s differs from the colour Life program" % key)
        self.model = model
        self.color = _color_stmt(model.programs["absorb"])

    def descriptor(self):
        d = _base_desc(self.model, self.family)
        info = self.color.extra
        d.color_kind = nat.XK_COLOR_MOVING_AVERAGE
        d.fade_in, d.fade_out, d.smooth = info["fade_in"], info["fade_out"], info["smooth"]
        return d


class NoiseTemplate:
    """Per-cell noise (``canonical.NoiseProgram``: the reference's NoiseTV,
    ``examples/noisetv.py:13-31``), matched by program fingerprint: one
    16-bit RandomProperty, nothing emitted, any lattice and border (no cell
    reads another), MovingAverage colours with the model's fades."""

    family = nat.XK_FAMILY_NOISE

    def __init__(self, model):
        from xentica_gb300.core import canonical
        props = list(model.main.properties.values())
        if [type(p).__name__ for p in props] != ["RandomProperty"]:
            raise NoTemplate("not one RandomProperty")
        _topology(model)
        attrs = {name: model.__dict__[name] for name in ("fade_in", "fade_out", "smooth_factor")
                 if name in model.__dict__}
        programs = canonical.trace(canonical.NoiseProgram, model.size, {}, attrs)
        for key in ("emit", "absorb"):
            if ir.fingerprint(programs[key]) != ir.fingerprint(model.programs[key]):
                raise NoTemplate("%s differs from the noise program" % key)
        self.model = model
        self.color = _color_stmt(model.programs["absorb"])

    def descriptor(self):
        d = _base_desc(self.model, self.family)
        info = self.color.extra
        d.color_kind = nat.XK_COLOR_MOVING_AVERAGE
        d.fade_in, d.fade_out, d.smooth = info["fade_in"], info["fade_out"], info["smooth"]
        return d


class GravityTemplate:
    """Energy flowing down a gravity field (``canonical.GravityProgram``: the
    reference's GraviCowboys, ``examples/gravicowboys.py:20-71``), matched by
    program fingerprint: two 12-bit integer properties and a float, a 2-D
    Moore lattice in the reference's neighbour order, torus or static border,
    MovingAverage colours with the model's fades."""

    family = nat.XK_FAMILY_GRAVITY
    MOORE = [(-1, -1), (-1, 0), (-1, 1), (0, -1), (0, 1), (1, -1), (1, 0), (1, 1)]

    def __init__(self, model):
        from xentica_gb300.core import canonical
        props = list(model.main.properties.values())
        if [type(p).__name__ for p in props] != ["IntegerProperty", "IntegerProperty", "FloatProperty"] or \
                [p.bit_width for p in props] != [12, 12, 32]:
            raise NoTemplate("not two 12-bit integer properties and a float")
        deltas, torus, border = _topology(model)
        if model.topology.dimensions != 2 or [tuple(d) for d in deltas] != self.MOORE:
            raise NoTemplate("GraviCowboys kernel is 2-D Moore")
        attrs = {name: model.__dict__[name] for name in ("fade_in", "fade_out", "smooth_factor")
                 if name in model.__dict__}
        programs = canonical.trace(canonical.GravityProgram, model.size, {}, attrs)
        for key in ("emit", "absorb"):
            if ir.fingerprint(programs[key]) != ir.fingerprint(model.programs[key]):
                raise NoTemplate("%s differs from the GraviCowboys program" % key)
        self.model = model
        self.color = _color_stmt(model.programs["absorb"])

    def descriptor(self):
        d = _base_desc(self.model, self.family)
        info = self.color.extra
        d.color_kind = nat.XK_COLOR_MOVING_AVERAGE
        d.fade_in, d.fade_out, d.smooth = info["fade_in"], info["fade_out"], info["smooth"]
        return d


class VMTemplate:
    """Any other traced model: its emit and absorb programs, compiled to
    register bytecode (``core/vm.py``), run on the generic interpreter kernel
    with the reference's two-pass execution model and memory layout.  Tried
    after every hand-written family; needs a plain or moving-average colour
    and programs without opaque C text."""

    family = nat.XK_FAMILY_VM

    def __init__(self, model):
        from xentica_gb300.core import vm
        _topology(model)
        self.model = model
        params = []
        try:
            self.programs = [vm.compile_program(model.programs[key], params)
                             for key in ("emit", "absorb")]
        except XenticaException as exc:
            raise NoTemplate(str(exc))
        self.param_names = list(params)
        color = _color_stmt(model.programs["absorb"])
        if _color_stmt(model.programs["emit"]) is not None:
            raise NoTemplate("emit writes a colour")
        self.color = color
        if color is not None and color.extra["kind"] not in ("plain", "moving_average"):
            raise NoTemplate("colour effect %s" % color.extra["kind"])
        self._bound = None

    def descriptor(self):
        d = _base_desc(self.model, self.family)
        if self.color is None:
            d.color_kind = nat.XK_COLOR_NONE
        elif self.color.extra["kind"] == "plain":
            d.color_kind = nat.XK_COLOR_PLAIN
        else:
            d.color_kind = nat.XK_COLOR_MOVING_AVERAGE
            d.fade_in = int(self.color.extra["fade_in"])
            d.fade_out = int(self.color.extra["fade_out"])
            d.smooth = int(self.color.extra["smooth"])
        return d

    def after_create(self, lib, handle):
        """Load both programs into the new device model."""
        import ctypes
        for which, prog in enumerate(self.programs):
            nat.check(lib.xk_vm_load(handle, which, prog.code.ctypes.data_as(ctypes.c_void_p),
                                     len(prog.code), prog.consts.ctypes.data_as(ctypes.c_void_p),
                                     len(prog.consts), prog.nregs), "xk_vm_load")
        self._bound = None

    def bind(self, lib, handle):
        """Send the interactive parameters' current values when they changed."""
        from xentica_gb300.core import vm
        if not self.param_names:
            return
        vals = []
        for name in self.param_names:
            param = self.model.meta.__dict__[name]
            ctype = ir.ctype_of(param.ctype) if hasattr(param, "ctype") else ir.I32
            vals.append(vm.pack_value(param.value, ctype))
        if vals == self._bound:
            return
        arr = np.array(vals, dtype=np.uint64)
        nat.check(lib.xk_vm_set_params(handle, nat.ptr(arr), len(arr)), "xk_vm_set_params")
        self._bound = vals


FAMILIES = (LifeTemplate, ShiftTemplate, EvoLifeTemplate, MassTemplate, LifeColorTemplate, NoiseTemplate,
            GravityTemplate, VMTemplate)


def match(model):
    """Template instance for ``model``; raises :class:`XenticaException`.

    The hand-written families are tried first, the interpreter last;
    ``XENTICA_GB300_TEMPLATE=vm`` in the environment runs every model on the
    interpreter (for comparing the two on the same model)."""
    reasons = []
    families = FAMILIES
    if os.environ.get("XENTICA_GB300_TEMPLATE", "") == "vm":
        families = (VMTemplate, )
    for family in families:
        try:
            return family(model)
        except NoTemplate as exc:
            reasons.append("%s: %s" % (family.__name__, exc))
    raise XenticaException("No GB300 kernel template implements model %s (%s)."
                           % (type(model).__name__, "; ".join(reasons)))
