"""Base class of all CA models (reference ``xentica/core/base.py``).

A model is a :class:`CellularAutomaton` subclass with a ``Topology`` class,
``Property`` attributes and ``emit()``, ``absorb()`` and ``color()`` methods,
following the buffered-state CA principle: at every step each cell first
*emits* values into its per-neighbour buffers, then *absorbs* its neighbours'
buffers into its new state and colour.

What changes from the reference is what happens to those methods.  They are
still executed once, on proxy objects, when a model is instantiated; the
proxies record a typed program (:mod:`xentica_gb300.core.ir`) instead of CUDA C
text, and :mod:`xentica_gb300.core.templates` maps that program onto one of the
hand-written GB300 kernels, filling in its rule parameters.  A model that no
template implements raises :class:`XenticaException`; there is no code
generation and no CPU fallback.

Usage is unchanged::

    ca = MyCA(MyExperiment)
    ca.set_viewport((320, 200))
    for _ in range(100):
        ca.step()
    frame = ca.render()
"""
import collections
import functools
import itertools
import operator
import threading
from copy import deepcopy

import numpy as np

from xentica_gb300.bridge import MoireBridge
from xentica_gb300.seeds.random import LocalRandom
from xentica_gb300.core import ir
from xentica_gb300.core.mixins import ACTIVE
from xentica_gb300.core.properties import Property, ContainerProperty
from xentica_gb300.core.renderers import RendererPlain
from xentica_gb300.core.exceptions import XenticaException
from xentica_gb300.utils import compat

__all__ = ['BSCA', 'CellularAutomaton', 'CachedNeighbor']


class CachedNeighbor:
    """Main and buffered state of one neighbour."""

    def __init__(self):
        self.main = ContainerProperty()
        self.buffer = ContainerProperty()


class BSCA(type):
    """Metaclass of :class:`CellularAutomaton`.

    Validates the ``Topology`` and builds the ``main``, ``buffers`` and
    ``neighbors`` containers (reference ``base.py:116-236``): buffer ``i`` is
    stored in plane ``rev_index_map[i] + 1``, neighbour ``i``'s buffer is read
    from plane ``i + 1``.
    """

    mandatory_fields = ('dimensions', 'lattice', 'neighborhood', 'border', )

    @classmethod
    def __prepare__(mcs, _name, _bases):
        return collections.OrderedDict()

    def __new__(mcs, name, bases, attrs):
        keys = [key for key in attrs.keys() if key not in ('__module__', '__qualname__')]
        attrs['__ordered__'] = keys
        new_class = super().__new__(mcs, name, bases, attrs)
        if not [b for b in bases if isinstance(b, BSCA)]:
            return new_class
        mcs._prepare_topology(new_class, attrs)
        new_class.main = None
        new_class.buffers = None
        new_class.neighbors = None
        mcs._prepare_properties(new_class, bases, attrs)
        new_class.constants = {}
        if not hasattr(new_class, 'renderer'):
            new_class.renderer = RendererPlain()
        new_class.size = tuple(1 for _ in range(new_class.topology.dimensions))
        return new_class

    def _prepare_topology(cls, attrs):
        if hasattr(cls, 'Topology'):
            attrs['Topology'] = cls.Topology
        cls.topology = attrs.get('Topology')
        if cls.topology is None:
            raise XenticaException("No Topology class declared.")
        for field in BSCA.mandatory_fields:
            if not hasattr(cls.topology, field):
                raise XenticaException("No %s declared in Topology class." % field)
        topo = cls.topology
        topo.lattice = deepcopy(topo.lattice)
        topo.neighborhood = deepcopy(topo.neighborhood)
        topo.border = deepcopy(topo.border)
        topo.lattice.dimensions = topo.dimensions
        topo.neighborhood.dimensions = topo.dimensions
        topo.border.dimensions = topo.dimensions
        topo.neighborhood.topology = topo
        topo.border.topology = topo

    def _prepare_properties(cls, bases, attrs):
        cls.main = ContainerProperty()
        cls.buffers = []
        cls.neighbors = []
        cls.meta = type('MetaParams', (object,), {})
        num_neighbors = len(cls.topology.neighborhood)
        for _ in range(num_neighbors):
            cls.buffers.append(ContainerProperty())
            cls.neighbors.append(CachedNeighbor())
        items = [base.__dict__.items() for base in bases]
        items.append(attrs.items())
        restricted = {"main", "buffer"}
        for obj_name, obj in itertools.chain.from_iterable(items):
            allowed = obj_name not in restricted
            if isinstance(obj, Property) and allowed:
                cls.main[obj_name] = deepcopy(obj)
                cls.main[obj_name].var_name = "_cell_%s" % obj_name
                for i in range(num_neighbors):
                    cls.buffers[i][obj_name] = deepcopy(obj)
                    cls.buffers[i][obj_name].var_name = "_bcell_%s%d" % (obj_name, i)
                    nbr = cls.neighbors[i]
                    nbr.main[obj_name] = deepcopy(obj)
                    nbr.main[obj_name].var_name = "_dcell_%s%d" % (obj_name, i)
                    nbr.buffer[obj_name] = deepcopy(obj)
                    nbr.buffer[obj_name].var_name = "_dbcell_%s%d" % (obj_name, i)
            elif obj.__class__.__name__ == "Parameter" and allowed:
                obj.name = obj_name
                setattr(cls.meta, obj_name, obj)
        cls.main.buf_num = 0
        cls.main.nbr_num = -1
        cls.main.var_name = "_cell"
        for i in range(num_neighbors):
            rev_i = cls.topology.neighborhood.rev_index_map[i]
            cls.buffers[i].buf_num = rev_i + 1
            cls.buffers[i].nbr_num = -1
            cls.buffers[i].var_name = "_bcell%i" % i
            cls.neighbors[i].main.buf_num = 0
            cls.neighbors[i].main.nbr_num = i
            cls.neighbors[i].main.var_name = "_dcell%d" % i
            cls.neighbors[i].buffer.buf_num = i + 1
            cls.neighbors[i].buffer.nbr_num = i
            cls.neighbors[i].buffer.var_name = "_dbcell%d" % i


class Translator:
    """Traces ``emit/absorb/color`` into typed programs (``self.programs``)."""

    def __init__(self):
        self.cuda_source = ""
        self.programs = {}
        self._program = ir.Program()
        self._deferred_writes = {}
        self._declarations = set()
        self._unpacks = set()
        self._params = {}
        self._emit_params = []
        self._absorb_params = []
        self._render_params = []
        self._coords_declared = False

    def _translate_code(self, *funcs):
        """Run ``funcs`` on proxies; return the recorded program."""
        self._program = ir.Program()
        self._deferred_writes = {}
        self._declarations = set()
        self._unpacks = set()
        self._params = {}
        self._coords_declared = False
        ACTIVE.append(self)
        try:
            for func in funcs:
                func()
            for prop in list(self._deferred_writes.values()):
                prop.deferred_write()
        finally:
            ACTIVE.pop()
        program = self._program
        self._program = ir.Program()
        return program

    # recording API used by the DSL objects
    def _record(self, stmt, code):
        self._program.add(stmt, code)

    def _record_many(self, stmts, code):
        self._program.stmts.extend(stmts)
        self._program.listing.append(code)

    def append_code(self, code):
        """Append raw text to the program listing (no semantics)."""
        self._program.add(None, code)

    def deferred_write(self, prop):
        """Schedule a container's packed write at the end of the kernel."""
        self._deferred_writes.setdefault(id(prop), prop)

    def declare(self, prop):
        """Mark a variable declared in the current kernel."""
        self._declarations.add(prop)

    def unpack(self, prop):
        """Mark a container unpacked in the current kernel."""
        self._unpacks.add(prop)

    def is_declared(self, prop):
        """Whether ``prop`` is declared in the current kernel."""
        return prop in self._declarations

    def is_unpacked(self, prop):
        """Whether ``prop`` is unpacked in the current kernel."""
        return prop in self._unpacks

    def declare_coords(self):
        """Mark the coordinate variables declared."""
        self._coords_declared = True

    def define_constant(self, constant):
        """Register a named constant."""
        self.constants[constant.name] = deepcopy(constant)

    def is_constant(self, constant_name):
        """Whether a constant with that name is registered."""
        return constant_name in self.constants

    def define_parameter(self, param):
        """Register an interactive parameter of the current kernel."""
        self._params[param.name] = param

    def is_parameter(self, param_name):
        """Whether the interactive parameter is registered."""
        return param_name in self._params

    @property
    def coords_declared(self):
        """Whether the coordinate variables are declared."""
        return self._coords_declared

    def build_source(self):
        """Trace the model; ``cuda_source`` gets the listing of the programs."""
        emit = self.build_emit()
        absorb = self.build_absorb()
        render = self.build_render()
        self.cuda_source = self.build_defines() + emit + absorb + render

    def build_defines(self):
        """Listing of the registered constants."""
        return "".join(const.get_define_code() for const in self.constants.values())

    @staticmethod
    def _listing(name, args, body):
        arg_string = ", ".join("%s %s" % (t, v) for t, v in args)
        return "\n// %s(%s, int n): traced body\n%s\n" % (name, arg_string, body)

    def build_emit(self):
        """Trace ``emit()``."""
        program = self._translate_code(self.emit)
        self.programs["emit"] = program
        self._emit_params = list(self._params.values())
        args = [(self.main.ctype, "*fld")]
        args += [(p.ctype, p.name) for p in self._emit_params]
        return self._listing("emit", args, program.text)

    def build_absorb(self):
        """Trace ``absorb()`` and ``color()`` into one program."""
        program = self._translate_code(self.absorb, self.color)
        self.programs["absorb"] = program
        self._absorb_params = list(self._params.values())
        args = [(self.main.ctype, "*fld"), ("int3", "*col")]
        args += [(p.ctype, p.name) for p in self._absorb_params]
        return self._listing("absorb", args, program.text)

    def build_render(self):
        """Describe the render kernel."""
        ACTIVE.append(self)
        try:
            return self._listing("render", self.renderer.args, self.renderer.render_code())
        finally:
            ACTIVE.pop()

    def index_to_coord(self, i):
        """Coordinates of cell index ``i`` (int or NumPy array)."""
        return self.topology.lattice.index_to_coord(i, self)

    def pack_state(self, state):
        """Pack ``{property: value}`` into the raw cell value (LSB first)."""
        val = 0
        shift = 0
        for name, prop in self.main.properties.items():
            if name in state:
                val += state[name] << shift
            shift += prop.bit_width
        return val


class CellularAutomaton(Translator, metaclass=BSCA):
    """Base class of all models.

    :param experiment_class: :class:`Experiment` subclass with the run's
        parameters (``word``, ``size``, ``zoom``, ``pos``, ``seed``, model
        meta-parameters and colour-effect settings).
    """

    def __init__(self, experiment_class):
        super().__init__()
        self.frame_buf = np.zeros((3, ), dtype=np.uint8)
        self.width, self.height = 0, 0
        self.random = LocalRandom(experiment_class.word)
        experiment_class.seed.random = self.random
        experiment_class.random = self.random
        for attr_name in dir(experiment_class):
            attr = getattr(experiment_class, attr_name)
            if not callable(attr) and not attr_name.startswith("__"):
                if attr_name == 'seed':
                    continue
                if hasattr(self.meta, attr_name):
                    self.meta.__dict__[attr_name].__set__(self, attr)
                    continue
                setattr(self, attr_name, attr)
        self.speed = 1
        self.paused = False
        self.timestep = 0
        self.cells_num = functools.reduce(operator.mul, self.size)
        if len(self.size) < self.topology.dimensions:
            msg = "Wrong field's dimensionality ({} instead of {})."
            raise XenticaException(msg.format(len(self.size), self.topology.dimensions))
        self.build_source()
        init_colors = np.zeros((self.cells_num * 3, ), dtype=np.int32)
        init_cells = np.zeros((self.cells_num, ), dtype=self.main.dtype)
        ACTIVE.append(self)
        try:
            experiment_class.seed.generate(init_cells, self)
        finally:
            ACTIVE.pop()
        from xentica_gb300.core.device import GPU
        self.gpu = GPU(self, init_cells, init_colors)
        self.bridge = MoireBridge
        self.renderer.setup_actions(self.bridge)
        self._lock = threading.Lock()

    def apply_speed(self, dval):
        """Change the simulation speed (minimum 1)."""
        self.speed = max(1, (self.speed + dval))

    def toggle_pause(self):
        """Toggle ``paused``; a paused model's ``step()`` does nothing."""
        self.paused = not self.paused

    def set_viewport(self, size):
        """Set the viewport size ``(width, height)`` in pixels."""
        self.width, self.height = size
        self.gpu.arrays.init_img(self.width * self.height * 3)

    def step(self):
        """Advance the model by one generation (``timestep`` counts them)."""
        if self.paused:
            return
        with self._lock:
            self.gpu.step(1)
            self.timestep += 1

    def render(self):
        """Render the current state.

        :returns: ``np.uint8`` array of ``width * height * 3`` RGB values.
        """
        if self.gpu.arrays.img is None:
            msg = "Viewport is not set, call set_viewport() before rendering."
            raise XenticaException(msg)
        with self._lock:
            img = self.gpu.render(self.width, self.height, int(self.zoom),
                                  int(self.pos[0]), int(self.pos[1]))
            return img.astype(np.uint8)

    def step_frames(self, nsteps, out=None):
        """Advance ``nsteps`` generations and render after each one: row ``g``
        of the result equals what ``step()`` followed by ``render()`` returns
        after generation ``g + 1`` -- the reference's viewer loop
        (``base.py:703-753``) in one call, with the frames copied to the host
        while the next generations run.  ``out`` (optional, uint8,
        ``nsteps x width * height * 3``) receives them; page-locked memory
        (``_native.PinnedBuffer``) makes the copies asynchronous.

        :returns: the frames, ``np.uint8`` of shape ``(nsteps, width * height * 3)``.
        """
        if self.gpu.arrays.img is None:
            msg = "Viewport is not set, call set_viewport() before rendering."
            raise XenticaException(msg)
        size = self.width * self.height * 3
        if out is None:
            out = np.empty((int(nsteps), size), dtype=np.uint8)
        if self.paused or nsteps <= 0:
            return out
        with self._lock:
            self.gpu.step_frames(int(nsteps), self.width, self.height, int(self.zoom),
                                 int(self.pos[0]), int(self.pos[1]), out.reshape(-1))
            self.timestep += int(nsteps)
        return out.reshape(int(nsteps), size)

    def save(self, filename):
        """Save the state (cells, colours, RNG) to ``filename``, in the
        reference's pickle layout (the reference can load it)."""
        with open(filename, "wb") as ca_file:
            ca_state = {
                "cells": self.gpu.arrays.cells.get(),
                "colors": self.gpu.arrays.colors.get(),
                "random": self.random,
            }
            compat.dump_state(ca_state, ca_file)

    def load(self, filename):
        """Load a state saved by :meth:`save` or by the reference."""
        with open(filename, "rb") as ca_file:
            ca_state = compat.load_state(ca_file)
            self.gpu.load(ca_state['cells'], ca_state['colors'])
            self.random.load(ca_state['random'])
