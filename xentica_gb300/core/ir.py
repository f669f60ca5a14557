"""Typed expression IR for traced ``emit`` / ``absorb`` / ``color`` bodies.

The reference translator turns the model's Python methods into C text
(``xentica/core/base.py:285-306``).  Here the same tracing builds a small typed
program instead: expression trees whose nodes carry their C type, and a list of
statements (declare, assign, compound-assign, store, colour).  Two consumers:

* the template matcher (``templates.py``), which decides which hand-written
  GB300 kernel runs the model and with which parameters;
* :class:`Evaluator`, a NumPy interpreter with exact C semantics (integer
  promotions, usual arithmetic conversions, unsigned wrap-around, truncating
  division, IEEE float/double), used to extract rule tables by evaluating the
  traced program over every relevant input combination at once.

Every node also renders the same C-like text the reference would have produced
(``str(node)``), so traced expressions keep the reference's textual form.
"""
import numpy as np

from xentica_gb300.core.exceptions import XenticaException


class CType:
    """A C scalar type: ``kind`` is 'u' (unsigned), 'i' (signed) or 'f'."""

    __slots__ = ("name", "kind", "bits", "rank", "np")

    def __init__(self, name, kind, bits, rank, np_dtype):
        self.name, self.kind, self.bits, self.rank, self.np = name, kind, bits, rank, np_dtype

    def __repr__(self):
        return self.name

    @property
    def is_float(self):
        return self.kind == "f"


BOOL = CType("bool", "u", 8, 0, np.uint8)
U8 = CType("unsigned char", "u", 8, 1, np.uint8)
U16 = CType("unsigned short", "u", 16, 2, np.uint16)
I32 = CType("int", "i", 32, 3, np.int32)
U32 = CType("unsigned int", "u", 32, 3, np.uint32)
I64 = CType("long", "i", 64, 4, np.int64)
U64 = CType("unsigned long", "u", 64, 4, np.uint64)
F32 = CType("float", "f", 32, 10, np.float32)
F64 = CType("double", "f", 64, 11, np.float64)

CTYPES = {t.name: t for t in (BOOL, U8, U16, I32, U32, I64, U64, F32, F64)}
CTYPES["int32"] = I32


def ctype_of(name):
    try:
        return CTYPES[name]
    except KeyError:
        raise XenticaException("Unsupported C type '%s'." % name)


def promote(t):
    """Integer promotion: everything narrower than int becomes int."""
    if t.kind != "f" and t.rank < I32.rank:
        return I32
    return t


def common(a, b):
    """Usual arithmetic conversions (C11 6.3.1.8) for the LP64 data model."""
    if a.kind == "f" or b.kind == "f":
        if a is F64 or b is F64:
            return F64
        return F32
    a, b = promote(a), promote(b)
    if a is b:
        return a
    if a.kind == b.kind:
        return a if a.rank >= b.rank else b
    uns, sig = (a, b) if a.kind == "u" else (b, a)
    if uns.rank >= sig.rank:
        return uns
    if sig.bits > uns.bits:
        return sig
    return U64 if sig is I64 else U32


def literal_type(value):
    """Type of the C literal the reference emits for a Python value."""
    if isinstance(value, float):
        return F64
    if -2 ** 31 <= value < 2 ** 31:
        return I32
    if -2 ** 63 <= value < 2 ** 63:
        return I64
    return U64


# --------------------------------------------------------------------------
# nodes

class Node:
    ctype = I32

    def text(self):
        raise NotImplementedError

    def __str__(self):
        return self.text()


class Lit(Node):
    def __init__(self, value, ctype=None, text=None):
        if isinstance(value, bool):
            value = int(value)
        self.value = value
        self.ctype = ctype or literal_type(value)
        self._text = text

    def text(self):
        return self._text if self._text is not None else str(self.value)


class Raw(Node):
    """Opaque C text (a user string or an undeclared name): not evaluable."""

    def __init__(self, text_):
        self._text = text_
        self.ctype = I32

    def text(self):
        return self._text


class VarRef(Node):
    def __init__(self, name, ctype):
        self.name, self.ctype = name, ctype

    def text(self):
        return self.name


class ParamRef(Node):
    """An interactive model parameter (a kernel argument in the reference)."""

    def __init__(self, name, ctype):
        self.name, self.ctype = name, ctype

    def text(self):
        return self.name


class Load(Node):
    """Packed container read: ``kind`` is 'main', 'buf' (own buffer plane),
    'nmain' (neighbour's main) or 'nbuf' (neighbour's buffer); ``k`` is the
    buffer / neighbour index; ``plane`` the reference plane number."""

    def __init__(self, kind, k, plane, ctype, text_):
        self.kind, self.k, self.plane, self.ctype, self._text = kind, k, plane, ctype, text_

    def text(self):
        return self._text


class Bin(Node):
    CMP = ("<", "<=", ">", ">=", "==", "!=")

    def __init__(self, op, a, b, text_=None):
        self.op, self.a, self.b = op, a, b
        if op in self.CMP:
            self.ctype = I32
        elif op in ("<<", ">>"):
            self.ctype = promote(a.ctype)
        else:
            self.ctype = common(a.ctype, b.ctype)
        self._text = text_

    def text(self):
        if self._text is not None:
            return self._text
        return "(%s %s %s)" % (self.a, self.op, self.b)


class Un(Node):
    def __init__(self, op, a, text_=None):
        self.op, self.a = op, a
        self.ctype = a.ctype if a.ctype.kind == "f" else promote(a.ctype)
        self._text = text_

    def text(self):
        if self._text is not None:
            return self._text
        return "(%s(%s))" % (self.op, self.a)


class Cast(Node):
    def __init__(self, ctype, a, text_=None):
        self.ctype, self.a = ctype, a
        self._text = text_

    def text(self):
        if self._text is not None:
            return self._text
        return "((%s) (%s))" % (self.ctype.name, self.a)


class BitCast(Node):
    """``reinterpret_cast`` between a 32-bit integer and float."""

    def __init__(self, ctype, a, text_):
        self.ctype, self.a, self._text = ctype, a, text_

    def text(self):
        return self._text


class Cond(Node):
    def __init__(self, c, a, b, text_):
        self.c, self.a, self.b = c, a, b
        self.ctype = common(a.ctype, b.ctype)
        self._text = text_

    def text(self):
        return self._text


class Call(Node):
    def __init__(self, fn, args, ctype, text_):
        self.fn, self.args, self.ctype, self._text = fn, args, ctype, text_

    def text(self):
        return self._text


def to_node(value):
    """IR node of any operand the DSL may combine."""
    node = getattr(value, "ir_node", None)
    if node is not None:
        return node() if callable(node) else node
    if isinstance(value, Node):
        return value
    if isinstance(value, (bool, int, np.integer)):
        return Lit(int(value))
    if isinstance(value, (float, np.floating)):
        return Lit(float(value))
    return Raw(str(value))


def parse_literal(text_):
    """Node for an initial-value string such as ``"0"`` or ``"0.0f"``."""
    s = text_.strip()
    try:
        return Lit(int(s), text=s)
    except ValueError:
        pass
    try:
        if s.endswith("f"):
            return Lit(float(s[:-1]), F32, text=s)
        return Lit(float(s), text=s)
    except ValueError:
        return Raw(s)


# --------------------------------------------------------------------------
# statements

class Stmt:
    __slots__ = ("op", "var", "ctype", "expr", "aug", "extra")

    def __init__(self, op, var=None, ctype=None, expr=None, aug=None, extra=None):
        self.op, self.var, self.ctype, self.expr, self.aug, self.extra = op, var, ctype, expr, aug, extra


class Program:
    """Statements of one traced kernel body plus its C-syntax listing."""

    def __init__(self):
        self.stmts = []
        self.listing = []

    def add(self, stmt, text_):
        if stmt is not None:
            self.stmts.append(stmt)
        self.listing.append(text_)

    @property
    def text(self):
        return "".join(self.listing)

    def loads(self):
        out = set()

        def walk(n):
            if isinstance(n, Load):
                out.add((n.kind, n.k))
            for attr in ("a", "b", "c"):
                sub = getattr(n, attr, None)
                if isinstance(sub, Node):
                    walk(sub)
            for sub in getattr(n, "args", ()) or ():
                if isinstance(sub, Node):
                    walk(sub)
        for st in self.stmts:
            if isinstance(st.expr, Node):
                walk(st.expr)
            if st.op == "color":
                for n in st.extra["rgb"]:
                    walk(n)
        return out

    def params(self):
        out = set()

        def walk(n):
            if isinstance(n, ParamRef):
                out.add(n.name)
            for attr in ("a", "b", "c"):
                sub = getattr(n, attr, None)
                if isinstance(sub, Node):
                    walk(sub)
            for sub in getattr(n, "args", ()) or ():
                if isinstance(sub, Node):
                    walk(sub)
        for st in self.stmts:
            if isinstance(st.expr, Node):
                walk(st.expr)
            if st.op == "color":
                for n in st.extra["rgb"]:
                    walk(n)
        return out


# --------------------------------------------------------------------------
# evaluator

class _Unsupported(Exception):
    pass


def _convert(arr, src, dst):
    """C conversion of ``arr`` (typed ``src``) to ``dst``."""
    if src is dst:
        return arr
    if dst.kind == "f":
        return arr.astype(dst.np)
    if src.kind == "f":
        # truncation toward zero; out-of-range values are undefined in C and
        # never occur in supported models -- NaN maps to 0 as on the GPU
        a = np.where(np.isnan(arr), 0, np.trunc(arr))
        if dst.kind == "u":
            a = np.where(a < 0, 0, a)
        return a.astype(np.float64).astype(np.int64 if dst.bits <= 32 or dst.kind == "i" else np.uint64).astype(dst.np)
    if dst is BOOL:
        return (arr != 0).astype(np.uint8)
    # integer -> integer: modular reinterpretation (what every target does)
    return arr.astype(dst.np, copy=False)


class Evaluator:
    """Vectorised C-semantics interpreter for a :class:`Program`.

    ``inputs`` maps ``(kind, k)`` load keys to packed container arrays;
    ``params`` maps interactive parameter names to values.  Every statement is
    executed for all lanes at once; the result holds the final variable values
    and the stored containers.
    """

    def __init__(self, program, inputs, params=None, lanes=None):
        self.p = program
        self.inputs = inputs
        self.params = params or {}
        self.lanes = lanes if lanes is not None else len(next(iter(inputs.values())))
        self.env = {}
        self.stores = {}
        self.color = None

    # -- expressions -------------------------------------------------------
    def ev(self, n):
        if isinstance(n, Lit):
            return np.full(self.lanes, n.value, dtype=n.ctype.np), n.ctype
        if isinstance(n, VarRef):
            if n.name not in self.env:
                raise _Unsupported("undeclared variable %s" % n.name)
            return self.env[n.name]
        if isinstance(n, ParamRef):
            if n.name not in self.params:
                raise _Unsupported("unbound parameter %s" % n.name)
            return np.full(self.lanes, self.params[n.name], dtype=n.ctype.np), n.ctype
        if isinstance(n, Load):
            key = (n.kind, n.k)
            if key not in self.inputs:
                raise _Unsupported("no input for %s" % (key,))
            return self.inputs[key].astype(n.ctype.np), n.ctype
        if isinstance(n, Cast):
            a, t = self.ev(n.a)
            return _convert(a, t, n.ctype), n.ctype
        if isinstance(n, BitCast):
            a, t = self.ev(n.a)
            a = _convert(a, t, I32 if n.ctype is F32 else t)
            if n.ctype is F32:
                return a.astype(np.int32).view(np.float32), F32
            return np.asarray(a, dtype=np.float32).view(np.int32), I32
        if isinstance(n, Cond):
            c, tc = self.ev(n.c)
            a, ta = self.ev(n.a)
            b, tb = self.ev(n.b)
            t = n.ctype
            return np.where(c != 0, _convert(a, ta, t), _convert(b, tb, t)), t
        if isinstance(n, Un):
            a, t = self.ev(n.a)
            rt = n.ctype
            a = _convert(a, t, rt)
            with np.errstate(over="ignore"):
                if n.op == "-":
                    return (-a).astype(rt.np), rt
                if n.op == "+":
                    return a, rt
                if n.op == "~":
                    if rt.kind == "f":
                        raise _Unsupported("~ on float")
                    return (~a).astype(rt.np), rt
                if n.op == "abs":
                    return np.abs(a).astype(rt.np), rt
            raise _Unsupported("unary %s" % n.op)
        if isinstance(n, Bin):
            return self._bin(n)
        if isinstance(n, Call):
            if n.fn == "__popc":
                a, t = self.ev(n.args[0])
                a = _convert(a, t, U32).astype(np.uint64)
                cnt = np.zeros(self.lanes, dtype=np.int32)
                for bit in range(32):
                    cnt += ((a >> np.uint64(bit)) & np.uint64(1)).astype(np.int32)
                return cnt, I32
            raise _Unsupported("call %s" % n.fn)
        raise _Unsupported(type(n).__name__)

    def _bin(self, n):
        op = n.op
        a, ta = self.ev(n.a)
        b, tb = self.ev(n.b)
        if op in ("<<", ">>"):
            rt = promote(ta)
            if rt.kind == "f" or promote(tb).kind == "f":
                raise _Unsupported("float shift")
            a = _convert(a, ta, rt)
            cnt = b.astype(np.int64)
            if np.any((cnt < 0) | (cnt >= rt.bits)):
                raise _Unsupported("shift count out of range")
            ua = a.astype(np.uint64) if rt.kind == "u" else a.astype(np.int64)
            if op == "<<":
                res = (a.astype(np.uint64) << cnt.astype(np.uint64)).astype(rt.np)
            else:
                res = (ua >> (cnt.astype(np.uint64) if rt.kind == "u" else cnt)).astype(rt.np)
            return res, rt
        ct = common(ta, tb)
        a = _convert(a, ta, ct)
        b = _convert(b, tb, ct)
        with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
            if op in Bin.CMP:
                fn = {"<": np.less, "<=": np.less_equal, ">": np.greater,
                      ">=": np.greater_equal, "==": np.equal, "!=": np.not_equal}[op]
                return fn(a, b).astype(np.int32), I32
            if op == "+":
                return (a + b).astype(ct.np), ct
            if op == "-":
                return (a - b).astype(ct.np), ct
            if op == "*":
                return (a * b).astype(ct.np), ct
            if op in ("/", "%"):
                if ct.kind == "f":
                    if op == "%":
                        raise _Unsupported("float %")
                    return (a / b).astype(ct.np), ct
                if np.any(b == 0):
                    raise _Unsupported("integer division by zero")
                if ct.kind == "u":
                    return ((a // b) if op == "/" else (a % b)).astype(ct.np), ct
                q = np.trunc(a.astype(np.float64) / b.astype(np.float64))
                if ct.bits > 32:
                    raise _Unsupported("64-bit signed division")
                q = q.astype(np.int64)
                if op == "/":
                    return q.astype(ct.np), ct
                return (a.astype(np.int64) - q * b.astype(np.int64)).astype(ct.np), ct
            if op in ("&", "|", "^"):
                if ct.kind == "f":
                    raise _Unsupported("bitwise op on float")
                fn = {"&": np.bitwise_and, "|": np.bitwise_or, "^": np.bitwise_xor}[op]
                return fn(a, b).astype(ct.np), ct
        raise _Unsupported("binary %s" % op)

    # -- statements --------------------------------------------------------
    def run(self):
        for st in self.p.stmts:
            if st.op == "decl":
                if st.expr is None:
                    self.env[st.var] = (np.zeros(self.lanes, dtype=st.ctype.np), st.ctype)
                else:
                    v, t = self.ev(st.expr)
                    self.env[st.var] = (_convert(v, t, st.ctype), st.ctype)
            elif st.op == "assign":
                cur = self.env.get(st.var)
                if cur is None:
                    raise _Unsupported("assign to undeclared %s" % st.var)
                v, t = self.ev(st.expr)
                self.env[st.var] = (_convert(v, t, cur[1]), cur[1])
            elif st.op == "aug":
                cur = self.env.get(st.var)
                if cur is None:
                    raise _Unsupported("compound assign to undeclared %s" % st.var)
                node = Bin(st.aug, VarRef(st.var, cur[1]), st.expr)
                v, t = self._bin(node)
                self.env[st.var] = (_convert(v, t, cur[1]), cur[1])
            elif st.op == "store":
                v, t = self.ev(st.expr)
                self.stores[st.extra] = _convert(v, t, st.ctype)
            elif st.op == "color":
                rgb = []
                for node in st.extra["rgb"]:
                    v, t = self.ev(node)
                    rgb.append(_convert(v, t, I32))
                self.color = (rgb, st.extra)
        return self


def evaluate(program, inputs, params=None, lanes=None):
    """Run ``program``; returns the :class:`Evaluator` or raises
    :class:`XenticaException` when the program is outside what it can decide."""
    try:
        return Evaluator(program, inputs, params, lanes).run()
    except _Unsupported as exc:
        raise XenticaException("Model cannot be analysed: %s." % exc)


def _reads(n, out):
    """Add the variable names ``n`` reads to ``out``; False if ``n`` holds
    opaque text (which may read anything)."""
    if n is None:
        return True
    if isinstance(n, Raw):
        return False
    if isinstance(n, VarRef):
        out.add(n.name)
        return True
    if isinstance(n, Call):
        return all(_reads(a, out) for a in n.args)
    return all(_reads(getattr(n, attr, None), out) for attr in ("a", "b", "c"))


def dead_initializers(program):
    """Indices of ``decl`` statements whose initial value is overwritten by a
    plain assignment before anything reads the variable.

    The translator declares a packed container with a load of its memory cell
    once any earlier kernel of the same model class has read that container,
    so a second model of a class declares the buffer cells it only writes
    with a load that the first model omits; the loaded value is dead.
    """
    stmts = program.stmts
    dead = set()
    for i, st in enumerate(stmts):
        if st.op != "decl" or st.expr is None:
            continue
        for later in stmts[i + 1:]:
            reads = set()
            nodes = [later.expr]
            if later.op == "color":
                nodes = list(later.extra["rgb"])
            if not all(_reads(x, reads) for x in nodes) or st.var in reads:
                break
            if later.op == "aug" and later.var == st.var:
                break
            if later.op == "assign" and later.var == st.var:
                dead.add(i)
                break
    return dead


def fingerprint(program):
    """Structure of a program with variables renamed by first appearance.

    Two programs with equal fingerprints execute the same statements on the
    same types and constants, whatever their variables are called; dead
    initial values of declarations (``dead_initializers``) are left out.
    """
    names = {}
    dead = dead_initializers(program)

    def nm(name):
        return names.setdefault(name, "v%d" % len(names))

    def fp(n):
        if n is None:
            return None
        if isinstance(n, Lit):
            return ("L", n.ctype.name, repr(n.value))
        if isinstance(n, VarRef):
            return ("V", nm(n.name), n.ctype.name)
        if isinstance(n, ParamRef):
            return ("P", n.name, n.ctype.name)
        if isinstance(n, Load):
            return ("M", n.kind, n.k, n.plane, n.ctype.name)
        if isinstance(n, Bin):
            return ("B", n.op, fp(n.a), fp(n.b))
        if isinstance(n, Un):
            return ("U", n.op, fp(n.a))
        if isinstance(n, Cast):
            return ("C", n.ctype.name, fp(n.a))
        if isinstance(n, BitCast):
            return ("X", n.ctype.name, fp(n.a))
        if isinstance(n, Cond):
            return ("Q", fp(n.c), fp(n.a), fp(n.b))
        if isinstance(n, Call):
            return ("F", n.fn, tuple(fp(a) for a in n.args))
        return ("R", n.text())

    out = []
    for i, st in enumerate(program.stmts):
        if st.op == "color":
            out.append(("color", st.extra["kind"], tuple(fp(x) for x in st.extra["rgb"])))
        else:
            out.append((st.op, nm(st.var) if st.var else None,
                        st.ctype.name if st.ctype is not None else None,
                        None if i in dead else fp(st.expr), st.aug, st.extra))
    return tuple(out)
