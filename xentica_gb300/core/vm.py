"""Register bytecode for the generic interpreter kernel (``csrc/vm.cu``).

Models that no hand-written GB300 template implements still run on the GPU:
their traced ``emit`` and ``absorb`` programs (``core/ir.py``) are compiled
here into a flat list of typed register instructions that one kernel
interprets, one thread per cell, with the reference's execution model
(``xentica/core/base.py:461-487``): an emit pass writing every cell's buffer
planes, then an absorb pass reading the neighbours' buffers and writing the
main plane and the colour, on the reference's own memory layout.

Every C conversion the reference's generated code performs implicitly
(integer promotions, usual arithmetic conversions, assignment to a narrower
type) is made an explicit ``CVT`` instruction here, by the rules
``ir.Evaluator`` implements, so the kernel's arithmetic instructions always
see operands of their own type.  Programs hold no branches (conditionals are
selects), so every thread runs the same instruction stream.
"""
import numpy as np

from xentica_gb300.core import ir
from xentica_gb300.core.exceptions import XenticaException

__all__ = ['compile_program', 'optimize', 'VmProgram', 'TYPE_CODES', 'type_code', 'pack_value']

# type codes shared with csrc/vm.cu
TYPE_CODES = {"bool": 0, "unsigned char": 1, "unsigned short": 2, "int": 3, "unsigned int": 4,
              "long": 5, "unsigned long": 6, "float": 7, "double": 8}

# opcodes shared with csrc/vm.cu
OP = {"const": 1, "param": 2, "load": 3, "mov": 4, "cvt": 5,
      "+": 10, "-": 11, "*": 12, "/": 13, "%": 14, "&": 15, "|": 16, "^": 17, "<<": 18, ">>": 19,
      "<": 20, "<=": 21, ">": 22, ">=": 23, "==": 24, "!=": 25,
      "neg": 30, "~": 31, "abs": 32,
      "sel": 40, "f2i": 41, "i2f": 42, "popc": 50, "exp": 51,
      "store": 60, "color": 61}
LOAD_KINDS = {"main": 0, "buf": 1, "nmain": 2, "nbuf": 3}

#: largest register file the kernel provides (64-bit registers per thread)
MAX_REGS = 256

INS_DTYPE = np.dtype([("op", np.uint8), ("ty", np.uint8), ("dst", np.uint16), ("a", np.uint16),
                      ("b", np.uint16), ("c", np.uint16), ("reserved", np.uint16)])


def type_code(ctype):
    return TYPE_CODES[ctype.name]


def pack_value(value, ctype):
    """64-bit register image of ``value`` as a ``ctype``: integers sign- or
    zero-extended from their width, floats as their IEEE bits."""
    if ctype is ir.F32:
        return int(np.array([value], dtype=np.float32).view(np.uint32)[0])
    if ctype is ir.F64:
        return int(np.array([value], dtype=np.float64).view(np.uint64)[0])
    if ctype is ir.BOOL:
        return 1 if value else 0
    v = int(value) & ((1 << ctype.bits) - 1)
    if ctype.kind == "i" and v >> (ctype.bits - 1):
        v -= 1 << ctype.bits
    return v & ((1 << 64) - 1)


class VmProgram:
    """Compiled program: instructions, constant pool, registers used, the
    interactive parameters it reads (in slot order) and whether it colours."""

    def __init__(self, code, consts, nregs, params, colors):
        self.code = code
        self.consts = consts
        self.nregs = nregs
        self.params = params
        self.colors = colors


class _Compiler:
    def __init__(self):
        self.code = []
        self.consts = []
        self.const_slot = {}
        self.vars = {}        # name -> (reg, ctype)
        self.free = []
        self.nregs = 0
        self.params = []
        self.colors = False

    # -- registers ---------------------------------------------------------
    def alloc(self):
        if self.free:
            return self.free.pop()
        self.nregs += 1
        if self.nregs > MAX_REGS:
            raise XenticaException("model needs more than %d interpreter registers" % MAX_REGS)
        return self.nregs - 1

    def release(self, reg, temp):
        if temp:
            self.free.append(reg)

    def emit(self, op, ty, dst=0, a=0, b=0, c=0):
        self.code.append((OP[op], ty, dst, a, b, c, 0))

    # -- expressions: each returns (register, ctype, is_temporary) ----------
    def const(self, value, ctype):
        key = (pack_value(value, ctype), ctype.name)
        slot = self.const_slot.get(key)
        if slot is None:
            slot = len(self.consts)
            self.consts.append(key[0])
            self.const_slot[key] = slot
        r = self.alloc()
        self.emit("const", type_code(ctype), r, slot)
        return r, ctype, True

    def cvt(self, val, to):
        r, t, temp = val
        if t is to:
            return val
        out = self.alloc()
        self.emit("cvt", type_code(to), out, r, type_code(t))
        self.release(r, temp)
        return out, to, True

    def expr(self, n):
        if isinstance(n, ir.Lit):
            return self.const(n.value, n.ctype)
        if isinstance(n, ir.VarRef):
            if n.name not in self.vars:
                raise XenticaException("interpreter: variable %s read before it is declared" % n.name)
            reg, t = self.vars[n.name]
            return reg, t, False
        if isinstance(n, ir.ParamRef):
            if n.name not in self.params:
                self.params.append(n.name)
            r = self.alloc()
            self.emit("param", type_code(n.ctype), r, self.params.index(n.name))
            return r, n.ctype, True
        if isinstance(n, ir.Load):
            if n.kind not in LOAD_KINDS:
                raise XenticaException("interpreter: unknown load %s" % n.kind)
            r = self.alloc()
            k = n.k if n.kind in ("nmain", "nbuf") else 0
            self.emit("load", type_code(n.ctype), r, LOAD_KINDS[n.kind], k, n.plane)
            return r, n.ctype, True
        if isinstance(n, ir.Cast):
            return self.cvt(self.expr(n.a), n.ctype)
        if isinstance(n, ir.BitCast):
            src = self.cvt(self.expr(n.a), ir.I32 if n.ctype is ir.F32 else ir.F32)
            out = self.alloc()
            self.emit("i2f" if n.ctype is ir.F32 else "f2i", type_code(n.ctype), out, src[0])
            self.release(src[0], src[2])
            return out, n.ctype, True
        if isinstance(n, ir.Cond):
            c = self.truth(self.expr(n.c))
            a = self.cvt(self.expr(n.a), n.ctype)
            b = self.cvt(self.expr(n.b), n.ctype)
            out = self.alloc()
            self.emit("sel", type_code(n.ctype), out, c[0], a[0], b[0])
            for v in (c, a, b):
                self.release(v[0], v[2])
            return out, n.ctype, True
        if isinstance(n, ir.Un):
            a = self.expr(n.a)
            rt = a[1] if a[1].kind == "f" else ir.promote(a[1])
            a = self.cvt(a, rt)
            if n.op == "+":
                return a
            if n.op not in ("-", "~", "abs"):
                raise XenticaException("interpreter: unary %s" % n.op)
            if n.op == "~" and rt.kind == "f":
                raise XenticaException("interpreter: ~ on a float")
            out = self.alloc()
            self.emit("neg" if n.op == "-" else n.op, type_code(rt), out, a[0])
            self.release(a[0], a[2])
            return out, rt, True
        if isinstance(n, ir.Bin):
            return self.binary(n.op, self.expr(n.a), self.expr(n.b))
        if isinstance(n, ir.Call):
            if n.fn == "__popc":
                a = self.cvt(self.expr(n.args[0]), ir.U32)
                out = self.alloc()
                self.emit("popc", type_code(ir.I32), out, a[0])
                self.release(a[0], a[2])
                return out, ir.I32, True
            if n.fn == "exp":
                a = self.cvt(self.expr(n.args[0]), ir.F64)
                out = self.alloc()
                self.emit("exp", type_code(ir.F64), out, a[0])
                self.release(a[0], a[2])
                return out, ir.F64, True
            raise XenticaException("interpreter: call to %s" % n.fn)
        raise XenticaException("interpreter: %s node (opaque C text) cannot run"
                               % type(n).__name__)

    def truth(self, val):
        """A condition as an int register (floats compared with 0.0)."""
        if val[1].kind != "f":
            return val
        return self.binary("!=", val, self.const(0.0, val[1]))

    def binary(self, op, a, b):
        if op in ("<<", ">>"):
            rt = ir.promote(a[1])
            if rt.kind == "f" or ir.promote(b[1]).kind == "f":
                raise XenticaException("interpreter: shift of a float")
            a = self.cvt(a, rt)
            b = self.cvt(b, ir.I32)
            out = self.alloc()
            self.emit(op, type_code(rt), out, a[0], b[0])
            self.release(a[0], a[2])
            self.release(b[0], b[2])
            return out, rt, True
        ct = ir.common(a[1], b[1])
        if ct.kind == "f" and op in ("%", "&", "|", "^"):
            raise XenticaException("interpreter: %s on floats" % op)
        a = self.cvt(a, ct)
        b = self.cvt(b, ct)
        out = self.alloc()
        if op not in OP:
            raise XenticaException("interpreter: binary %s" % op)
        self.emit(op, type_code(ct), out, a[0], b[0])
        self.release(a[0], a[2])
        self.release(b[0], b[2])
        return out, ir.I32 if op in ir.Bin.CMP else ct, True

    # -- statements --------------------------------------------------------
    def assign_to(self, name, val):
        reg, t = self.vars[name]
        val = self.cvt(val, t)
        if val[0] != reg:
            self.emit("mov", type_code(t), reg, val[0])
        self.release(val[0], val[2])

    def stmt(self, st):
        if st.op == "decl":
            if st.var not in self.vars:
                self.vars[st.var] = (self.alloc(), st.ctype)
            elif self.vars[st.var][1] is not st.ctype:
                raise XenticaException("interpreter: %s declared twice with two types" % st.var)
            if st.expr is None:
                self.assign_to(st.var, self.const(0, st.ctype))
            else:
                self.assign_to(st.var, self.expr(st.expr))
        elif st.op == "assign":
            if st.var not in self.vars:
                raise XenticaException("interpreter: assignment to undeclared %s" % st.var)
            self.assign_to(st.var, self.expr(st.expr))
        elif st.op == "aug":
            if st.var not in self.vars:
                raise XenticaException("interpreter: assignment to undeclared %s" % st.var)
            reg, t = self.vars[st.var]
            self.assign_to(st.var, self.binary(st.aug, (reg, t, False), self.expr(st.expr)))
        elif st.op == "store":
            kind, plane = st.extra
            val = self.cvt(self.expr(st.expr), st.ctype)
            self.emit("store", type_code(st.ctype), 0, val[0], int(plane))
            self.release(val[0], val[2])
        elif st.op == "color":
            regs = [self.cvt(self.expr(node), ir.I32) for node in st.extra["rgb"]]
            self.emit("color", type_code(ir.I32), 0, regs[0][0], regs[1][0], regs[2][0])
            for v in regs:
                self.release(v[0], v[2])
            self.colors = True
        else:
            raise XenticaException("interpreter: statement %s" % st.op)


# -- optimisation -----------------------------------------------------------
# The compiler above emits one instruction per C operation and conversion, a
# move per assignment and a constant load per literal; the traced programs
# unpack and repack every field of every buffer.  The programs are straight
# lines (no branches), so every register value can be numbered: each
# instruction result becomes a value, a move only renames one, equal pure
# operations on equal values (constant loads included) share one value, an
# integer conversion or integer arithmetic of constants becomes a constant
# (with the kernel's semantics: wrap-around, truncating division, division
# by zero giving 0, shift counts modulo the width), integer identities (x + 0,
# x * 1, x | 0, x * 0, ...) fold, values nothing stored or coloured depends on
# are dropped, and registers are allocated again over the live ranges that
# remain.  Loads are shared only up to the next store.

_BINARY = set(range(OP["+"], OP["!="] + 1))
_SIDE = {OP["store"], OP["color"]}
_CODE_TYPES = {v: k for k, v in TYPE_CODES.items()}
_INT_CODES = {TYPE_CODES[n] for n in ("bool", "unsigned char", "unsigned short", "int", "unsigned int",
                                      "long", "unsigned long")}


def _reg_fields(op):
    """The instruction fields that name registers (the others are immediates)."""
    if op in _BINARY:
        return ("a", "b")
    if op in (OP["sel"], OP["color"]):
        return ("a", "b", "c")
    if op in (OP["const"], OP["param"], OP["load"]):
        return ()
    return ("a", )    # mov, cvt, neg, ~, abs, f2i, i2f, popc, exp, store


def _image_value(image, code):
    """The integer a register image of integer type ``code`` holds."""
    image = int(image)
    if code in (TYPE_CODES["int"], TYPE_CODES["long"]) and image >> 63:
        return image - (1 << 64)
    return image


# the integer types binary instructions compute in, with their widths
_ARITH_BITS = {TYPE_CODES["int"]: 32, TYPE_CODES["unsigned int"]: 32, TYPE_CODES["long"]: 64,
               TYPE_CODES["unsigned long"]: 64}


def _fold_binary(op, code, x, y):
    """The register image ``csrc/vm.cu`` computes for integer operation ``op``
    of type ``code`` on the values ``x`` and ``y``, or None."""
    bits = _ARITH_BITS[code]
    if op == OP["+"]:
        v = x + y
    elif op == OP["-"]:
        v = x - y
    elif op == OP["*"]:
        v = x * y
    elif op in (OP["/"], OP["%"]):
        if y == 0:
            v = 0
        else:
            q = abs(x) // abs(y)
            q = -q if (x < 0) != (y < 0) else q
            v = q if op == OP["/"] else x - q * y
    elif op == OP["&"]:
        v = x & y
    elif op == OP["|"]:
        v = x | y
    elif op == OP["^"]:
        v = x ^ y
    elif op == OP["<<"]:
        v = x << (y & (bits - 1))
    elif op == OP[">>"]:
        v = x >> (y & (bits - 1))
    elif OP["<"] <= op <= OP["!="]:
        return int({OP["<"]: x < y, OP["<="]: x <= y, OP[">"]: x > y, OP[">="]: x >= y,
                    OP["=="]: x == y, OP["!="]: x != y}[op])
    else:
        return None
    return pack_value(v, ir.ctype_of(_CODE_TYPES[code]))


def optimize(code, consts):
    """Straight-line value numbering, constant conversion folding, dead-value
    removal and register re-allocation of compiled instructions; returns
    ``(code, consts, nregs)`` computing the same stores and colours."""
    consts = [int(c) for c in consts]
    const_slot = {}
    for slot, c in enumerate(consts):
        const_slot.setdefault(c, slot)
    nodes = []            # (op, ty, arg values, immediates)
    cur = {}              # register -> value it holds
    table = {}            # (op, ty, args, immediates) -> value
    load_keys = []
    for ins in code:
        op, ty = int(ins["op"]), int(ins["ty"])
        fields = _reg_fields(op)
        args = tuple(cur[int(ins[f])] for f in fields)
        imm = tuple(int(ins[f]) if f not in fields else -1 for f in ("a", "b", "c"))
        if op == OP["mov"]:
            cur[int(ins["dst"])] = args[0]
            continue
        if op in _SIDE:
            nodes.append((op, ty, args, imm))
            if op == OP["store"]:
                for k in load_keys:
                    table.pop(k, None)
                load_keys = []
            continue
        if op == OP["cvt"]:
            src = nodes[args[0]]
            frm = imm[1]
            if frm == ty:
                cur[int(ins["dst"])] = args[0]
                continue
            if src[0] == OP["const"] and frm in _INT_CODES and ty in _INT_CODES:
                value = _image_value(consts[src[3][0]], frm)
                image = pack_value(value, ir.ctype_of(_CODE_TYPES[ty]))
                if image not in const_slot:
                    const_slot[image] = len(consts)
                    consts.append(image)
                op, args, imm = OP["const"], (), (const_slot[image], -1, -1)
        if op in _BINARY and ty in _ARITH_BITS:
            na, nb = nodes[args[0]], nodes[args[1]]
            ca = _image_value(consts[na[3][0]], ty) if na[0] == OP["const"] else None
            cb = _image_value(consts[nb[3][0]], ty) if nb[0] == OP["const"] else None
            folded = None
            if ca is not None and cb is not None:
                folded = _fold_binary(op, ty, ca, cb)
            elif cb == 0 and op in (OP["+"], OP["-"], OP["|"], OP["^"], OP["<<"], OP[">>"]) or \
                    cb == 1 and op in (OP["*"], OP["/"]) or ca == 0 and op in (OP["+"], OP["|"], OP["^"]) or \
                    ca == 1 and op == OP["*"]:
                cur[int(ins["dst"])] = args[0] if cb is not None else args[1]
                continue
            elif (ca == 0 or cb == 0) and op in (OP["*"], OP["&"]):
                folded = 0
            if folded is not None:
                if folded not in const_slot:
                    const_slot[folded] = len(consts)
                    consts.append(folded)
                op, args, imm = OP["const"], (), (const_slot[folded], -1, -1)
        if op == OP["const"]:
            imm = (const_slot.get(consts[imm[0]], imm[0]), -1, -1)
        key = (op, ty, args, imm)
        vid = table.get(key)
        if vid is None:
            vid = len(nodes)
            nodes.append(key)
            table[key] = vid
            if op == OP["load"]:
                load_keys.append(key)
        cur[int(ins["dst"])] = vid
    # values the stores and colours depend on
    live = [False] * len(nodes)
    stack = [i for i, n in enumerate(nodes) if n[0] in _SIDE]
    while stack:
        i = stack.pop()
        if live[i]:
            continue
        live[i] = True
        stack.extend(nodes[i][2])
    last = {}
    for i, n in enumerate(nodes):
        if live[i]:
            for a in n[2]:
                last[a] = i
    reg_of, free, nregs, out = {}, [], 0, []
    for i, (op, ty, args, imm) in enumerate(nodes):
        if not live[i]:
            continue
        regs = [reg_of[a] for a in args]
        for a in set(args):
            if last[a] == i:
                free.append(reg_of[a])
        dst = 0
        if op not in _SIDE:
            if free:
                dst = free.pop()
            else:
                dst, nregs = nregs, nregs + 1
            reg_of[i] = dst
        fields = _reg_fields(op)
        vals = {"a": 0, "b": 0, "c": 0}
        it = iter(regs)
        for k, f in enumerate(("a", "b", "c")):
            vals[f] = next(it) if f in fields else max(imm[k], 0)
        out.append((op, ty, dst, vals["a"], vals["b"], vals["c"], 0))
    if nregs > MAX_REGS:
        raise XenticaException("model needs more than %d interpreter registers" % MAX_REGS)
    code = np.array(out, dtype=INS_DTYPE) if out else np.zeros(0, dtype=INS_DTYPE)
    return code, np.array(consts or [0], dtype=np.uint64), max(nregs, 1)


def compile_program(program, params=None):
    """Compile a traced :class:`ir.Program` into a :class:`VmProgram`.

    ``params`` (a list, shared by the programs of one model) gives the
    interactive parameters their slots; names read first are appended."""
    comp = _Compiler()
    if params is not None:
        comp.params = params
    for st in program.stmts:
        comp.stmt(st)
    code = np.array(comp.code, dtype=INS_DTYPE) if comp.code else np.zeros(0, dtype=INS_DTYPE)
    consts = np.array(comp.consts, dtype=np.uint64) if comp.consts else np.zeros(1, dtype=np.uint64)
    code, consts, nregs = optimize(code, consts)
    return VmProgram(code, consts, nregs, comp.params, comp.colors)
