"""Cell-state properties (reference ``xentica/core/properties.py``).

Declared as model class attributes; the ``BSCA`` metaclass copies them into
``main``, ``buffers[i]`` and ``neighbors[i].{main,buffer}`` containers::

    class MyCA(core.CellularAutomaton):
        state = core.IntegerProperty(max_val=1)

``self.main.state`` reads and writes the cell's state, ``self.buffers[i].state``
its i-th emitted value, ``self.neighbors[i].buffer.state`` what neighbour i
emitted towards this cell.

Packing follows the reference exactly (``properties.py:82-98``, ``:496-541``):
properties are laid out LSB-first in declaration order, each with mask
``2**bit_width - 1``, in the smallest of uint8/16/32/64 that holds their sum.
Reads unpack the whole container once; writes are deferred and packed at the
end of the traced kernel body.
"""
import abc
import math
from collections import OrderedDict
from functools import cached_property

import numpy as np

from xentica_gb300.core import ir
from xentica_gb300.core.expressions import DeferredExpression
from xentica_gb300.core.exceptions import XenticaException
from xentica_gb300.core.mixins import BscaDetectorMixin
from xentica_gb300.tools import xmath

__all__ = ['Property', 'IntegerProperty', 'FloatProperty', 'ContainerProperty',
           'TotalisticRuleProperty', 'RandomProperty', ]


class Property(DeferredExpression, BscaDetectorMixin):
    """Base class of all properties."""

    def __init__(self):
        self._types = (
            # (bit width, NumPy dtype, C type)
            (8, np.uint8, 'char'),
            (16, np.uint16, 'short'),
            (32, np.uint32, 'int'),
            (64, np.uint64, 'long'),
        )
        self._buf_num, self._nbr_num = 1, 1
        super().__init__()

    @cached_property
    def best_type(self):
        """``(bit_width, numpy_dtype, c_type)`` of the smallest type that fits."""
        best = self._types[-1]
        for entry in self._types:
            if self.bit_width <= entry[0]:
                best = entry
                break
        return best

    @cached_property
    def dtype(self):
        """NumPy dtype that stores the property."""
        return self.best_type[1]

    @cached_property
    def ctype(self):
        """C type that stores the property."""
        return 'unsigned ' + self.best_type[2]

    @property
    def _num_neighbors(self):
        return len(self.bsca.buffers)

    @cached_property
    def bit_width(self):
        """Number of bits the property needs."""
        return self.calc_bit_width()

    @cached_property
    def width(self):
        """Number of storage words the property needs."""
        return int(math.ceil(self.bit_width / self.best_type[0]))

    @abc.abstractmethod
    def calc_bit_width(self):
        """Bit width of the property (override in subclasses)."""
        return 1

    @property
    def buf_num(self):
        """Buffer plane the property lives in."""
        return self._buf_num

    @buf_num.setter
    def buf_num(self, val):
        self._buf_num = val

    @property
    def nbr_num(self):
        """Neighbour index the property belongs to (-1: the cell itself)."""
        return self._nbr_num

    @nbr_num.setter
    def nbr_num(self, val):
        self._nbr_num = val

    def __getattribute__(self, attr):
        obj = object.__getattribute__(self, attr)
        if hasattr(obj, '__get__') and attr != "__class__":
            return obj.__get__(self, type(self))
        return obj

    def __setattr__(self, attr, val):
        try:
            obj = object.__getattribute__(self, attr)
        except AttributeError:
            object.__setattr__(self, attr, val)
        else:
            if hasattr(obj, '__set__'):
                obj.__set__(self, val)
            else:
                object.__setattr__(self, attr, val)

    def __get__(self, obj, objtype):
        self.declare_once()
        return self

    def __set__(self, obj, value):
        self.declare_once()
        code = "%s = %s;\n" % (self, value)
        self.bsca._record(ir.Stmt("assign", var=self.var_name, expr=ir.to_node(value)), code)

    @property
    def ir_ctype(self):
        """IR type of the property's variable."""
        return ir.ctype_of(self.ctype)

    def ir_node(self):
        try:
            ctype = self.ir_ctype
        except XenticaException:
            # outside a model (no neighbourhood to size the property): the
            # expression keeps its text but cannot be analysed
            return ir.Raw(self.var_name)
        return ir.VarRef(self.var_name, ctype)

    @cached_property
    def _mem_cell(self):
        """``(text, IR load)`` reading this cell's packed state from memory."""
        if self._nbr_num >= 0:
            neighborhood = self.bsca.topology.neighborhood
            text = neighborhood.neighbor_state(self._nbr_num, self._buf_num, "_nx")
            kind = "nmain" if self._buf_num == 0 else "nbuf"
            return text, (kind, self._nbr_num, self._buf_num)
        offset = ""
        if self._buf_num > 0:
            offset = " + n * %d" % self._buf_num
        kind = "main" if self._buf_num == 0 else "buf"
        return "fld[i%s]" % offset, (kind, self._buf_num - 1, self._buf_num)

    def _load_node(self):
        text, (kind, k, plane) = self._mem_cell
        return ir.Load(kind, k, plane, self.ir_ctype, text)

    def unpack_cast(self, expr):
        """Expression turning unpacked integer bits into the property's value."""
        return expr

    def unpack_cast_node(self, node):
        return node

    def pack_cast(self, expr):
        """Expression turning the property's value into integer bits."""
        return expr

    def pack_cast_node(self, node):
        return node

    @property
    def declared(self):
        """Whether the property's variable is declared in the current kernel."""
        return self.bsca.is_declared(self)

    @property
    def coords_declared(self):
        """Whether the coordinate variables are declared in the current kernel."""
        return self.bsca.coords_declared

    def declare_once(self):
        """Declare the variable holding the property, once per kernel."""
        if self.declared:
            return
        code = "%s %s;\n" % (self.ctype, self.var_name)
        self.bsca._record(ir.Stmt("decl", var=self.var_name, ctype=self.ir_ctype), code)
        self.bsca.declare(self)

    def __str__(self):
        return self.var_name


class IntegerProperty(Property):
    """A non-negative integer no larger than ``max_val``."""

    def __init__(self, max_val):
        self.max_val = max_val
        self._buf_num = 0
        super().__init__()

    def calc_bit_width(self):
        """Bits needed for ``max_val``."""
        return int(math.log2(self.max_val)) + 1


class FloatProperty(Property):
    """A 32-bit float stored by its bit pattern."""

    def __init__(self):
        self._buf_num = 0
        super().__init__()

    def calc_bit_width(self):
        """Always 32 bits."""
        return 32

    @cached_property
    def ctype(self):
        """Always ``float``."""
        return "float"

    def unpack_cast(self, expr):
        return f"(* reinterpret_cast<float*>(&({expr})))"

    def unpack_cast_node(self, node):
        return ir.BitCast(ir.F32, node, self.unpack_cast(node))

    def pack_cast(self, expr):
        return f"(* reinterpret_cast<int*>(&({expr})))"

    def pack_cast_node(self, node):
        return ir.BitCast(ir.I32, node, self.pack_cast(node))


class ContainerProperty(Property):
    """Holder of the model's properties: packs and unpacks them.

    Used by the framework for ``main``, ``buffers`` and ``neighbors``; not
    meant to be declared by models directly.
    """

    def __init__(self):
        super().__init__()
        self._properties = OrderedDict()
        self.init_val = None

    @property
    def properties(self):
        """Inner properties in declaration order."""
        return self._properties

    def values(self):
        """Iterate over inner properties."""
        for prop in self._properties.values():
            yield prop

    @property
    def unpacked(self):
        """Whether inner properties are unpacked in the current kernel."""
        return self.bsca.is_unpacked(self)

    def __getitem__(self, key):
        return self._properties[key]

    def __setitem__(self, key, val):
        self._properties[key] = val
        object.__setattr__(self, key, val)

    def calc_bit_width(self):
        """Sum of the inner properties' widths."""
        return sum(p.bit_width for p in self._properties.values())

    @Property.buf_num.setter
    def buf_num(self, val):
        self._buf_num = val
        for key in self._properties.keys():
            self[key].buf_num = val

    @Property.nbr_num.setter
    def nbr_num(self, val):
        self._nbr_num = val
        for key in self._properties.keys():
            self[key].nbr_num = val

    def __get__(self, obj, objtype):
        return self

    def __set__(self, obj, value):
        """Containers cannot be assigned as a whole."""

    def __getattribute__(self, attr):
        obj = object.__getattribute__(self, attr)
        if isinstance(obj, Property):
            self.init_val = self._mem_cell[0]
            self.declare_once()
            self._unpack_state()
            return obj.__get__(self, type(self))
        return obj

    def __setattr__(self, attr, val):
        try:
            obj = object.__getattribute__(self, attr)
        except AttributeError:
            object.__setattr__(self, attr, val)
        else:
            if isinstance(obj, Property):
                obj.declare_once()
                obj.__set__(self, val)
                self.declare_once()
                self.bsca.deferred_write(self)
                self.bsca.unpack(self)
            else:
                object.__setattr__(self, attr, val)

    def declare_once(self):
        """Declare the packed variable; for neighbours, locate the neighbour
        (torus wrap or static off-board value) first."""
        if self.declared:
            return
        bsca = self.bsca
        code = ""
        if self._nbr_num >= 0:
            topology = bsca.topology
            lattice, border = topology.lattice, topology.border
            if not self.coords_declared:
                code += lattice.index_to_coord_code("i", "_x")
                coord_vars = ["_nx%d" % i for i in range(topology.dimensions)]
                code += "int %s;\n" % ", ".join(coord_vars)
                bsca.declare_coords()
            code += topology.neighborhood.neighbor_coords(self._nbr_num, "_x", "_nx")
            off_board = lattice.is_off_board_code("_nx")
            if hasattr(border, "wrap_coords"):
                code += ("\n                    if (%s) {\n                        %s\n"
                         "                    }\n                " % (off_board, border.wrap_coords("_nx")))
            else:
                code += ("\n                    {type} {var};\n                    if ({off}) {{\n"
                         "                        {var} = {border};\n                    }} else {{\n"
                         "                        {var} = {nbr};\n                    }}\n                "
                         ).format(type=self.ctype, var=self.var_name, off=off_board,
                                  border=border.off_board_state("_nx"), nbr=self.init_val)
                bsca._record(ir.Stmt("decl", var=self.var_name, ctype=self.ir_ctype,
                                  expr=self._load_node()), code)
                bsca.declare(self)
                return
        if self.init_val is None:
            code += "%s %s;\n" % (self.ctype, self.var_name)
            stmt = ir.Stmt("decl", var=self.var_name, ctype=self.ir_ctype)
        else:
            code += "%s %s = %s;\n" % (self.ctype, self.var_name, self.init_val)
            stmt = ir.Stmt("decl", var=self.var_name, ctype=self.ir_ctype, expr=self._load_node())
        bsca._record(stmt, code)
        bsca.declare(self)

    def _unpack_state(self):
        """Unpack every inner property from the packed variable."""
        if self.unpacked:
            return
        bsca = self.bsca
        tmp_var = f"tmp_{self.var_name}"
        code = f"int {tmp_var};\n"
        stmts = [ir.Stmt("decl", var=tmp_var, ctype=ir.I32)]
        packed = ir.VarRef(self.var_name, self.ir_ctype)
        tmp = ir.VarRef(tmp_var, ir.I32)
        shift = 0
        for prop in self._properties.values():
            prop.declare_once()
            val = self.var_name
            src = packed
            if shift > 0:
                val += " >> %d" % shift
                src = ir.Bin(">>", packed, ir.Lit(shift))
            mask = 2 ** prop.bit_width - 1
            code += f"{tmp_var} = ({val}) & {mask};\n"
            stmts.append(ir.Stmt("assign", var=tmp_var, expr=ir.Bin("&", src, ir.Lit(mask))))
            val = prop.unpack_cast(tmp_var)
            code += "{var} = {val};\n".format(var=prop.var_name, val=val)
            stmts.append(ir.Stmt("assign", var=prop.var_name, expr=prop.unpack_cast_node(tmp)))
            shift += prop.bit_width
        bsca._record_many(stmts, code)
        bsca.unpack(self)

    def deferred_write(self):
        """Pack the inner properties and store the container (end of kernel)."""
        bsca = self.bsca
        shift = 0
        vals = []
        total = None
        cont_t = self.ir_ctype
        for prop in self._properties.values():
            prop.declare_once()
            mask = 2 ** prop.bit_width - 1
            val = "(({ctype}) {val} & {mask})".format(
                ctype=self.ctype, val=prop.pack_cast(prop.var_name), mask=mask)
            node = ir.Bin("&", ir.Cast(cont_t, prop.pack_cast_node(prop.ir_node())), ir.Lit(mask))
            if shift > 0:
                val = "({val} << {shift})".format(val=val, shift=shift)
                node = ir.Bin("<<", node, ir.Lit(shift))
            vals.append(val)
            total = node if total is None else ir.Bin("+", total, node)
            shift += prop.bit_width
        code = "{var} = {val};\n".format(var=self.var_name, val=" + ".join(vals))
        mem_text, (kind, k, plane) = self._mem_cell
        code += "%s = %s;\n" % (mem_text, self.var_name)
        key = (kind, plane) if kind in ("main", "buf") else (kind, k, plane)
        bsca._record_many([
            ir.Stmt("assign", var=self.var_name, expr=total),
            ir.Stmt("store", ctype=cont_t, expr=ir.VarRef(self.var_name, cont_t), extra=key),
        ], code)


class TotalisticRuleProperty(Property):
    """A per-cell outer-totalistic rule: born bits then sustain bits.

    With N neighbours it holds ``2 * (N + 1)`` bits; bit 0 of each half is
    masked off by the helpers (``properties.py:544-619``).
    """

    def __init__(self, outer=False):
        self._buf_num = 0
        self._outer = outer
        super().__init__()

    @property
    def _genome_mask(self):
        return 2 ** (self._num_neighbors + 1) - 2

    def calc_bit_width(self):
        """``2 * (N + 1)`` bits for N neighbours."""
        return (self._num_neighbors + 1) * 2

    def is_sustained(self, num_neighbors):
        """Sustain bit for ``num_neighbors`` living neighbours."""
        if not self._outer:
            raise XenticaException("Can not get a sustained flag from the pure totalistic rule.")
        mask = (self._genome_mask << (self._num_neighbors + 1))
        return ((self & mask) >> (num_neighbors + self._num_neighbors + 1)) & 1

    def is_born(self, num_neighbors):
        """Birth bit for ``num_neighbors`` living neighbours."""
        if not self._outer:
            raise XenticaException("Can not get a born flag from the pure totalistic rule.")
        return ((self & self._genome_mask) >> num_neighbors) & 1

    def __get__(self, obj, objtype):
        self.declare_once()
        return self

    def next_val(self, cur_val, num_neighbors):
        """Next state for current value ``cur_val``."""
        if not self._outer:
            return (self >> (num_neighbors + cur_val)) & 1
        alive_shift = cur_val * (self._num_neighbors + 1)
        return (self >> (num_neighbors + alive_shift)) & 1


class RandomProperty(Property):
    """A 16-bit per-cell random stream.

    Every read through a container advances it with
    ``x = (x * 58321 + 11113) % 65535`` (``properties.py:622-660``) and
    schedules the container's write-back.
    """

    def __init__(self):
        self._buf_num = 0
        super().__init__()

    def __get__(self, obj, objtype):
        self.declare_once()
        self._get_next(obj)
        return self

    def calc_bit_width(self):
        """Always 16 bits."""
        return 16

    def _get_next(self, container):
        var = DeferredExpression(self.var_name, self.ir_node())
        val = ((xmath.int(var) * 58321 + 11113)) % 65535
        self.__set__(self, val)
        if isinstance(container, ContainerProperty):
            self.bsca.deferred_write(container)

    @property
    def uniform(self):
        """The current value scaled to ``[0, 1)`` as a float."""
        var = DeferredExpression(self.var_name, self.ir_node())
        return xmath.float(var) / 65535
