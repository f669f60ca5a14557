"""NumPy executor of the interpreter bytecode (test infrastructure).

Runs a model's compiled emit/absorb programs (``xentica_gb300.core.vm``) over
all cells at once with the semantics ``csrc/vm.cu`` implements, on the
reference's layout, so the compiler can be checked against the reference's
fixtures without a GPU; the GPU kernel is then checked against the same
fixtures.
"""
import numpy as np

from xentica_gb300.core import vm

T = {0: np.uint8, 1: np.uint8, 2: np.uint16, 3: np.int32, 4: np.uint32, 5: np.int64,
     6: np.uint64, 7: np.float32, 8: np.float64}
U32MASK = np.uint64(0xFFFFFFFF)


def view(v, ty):
    """Typed values of 64-bit register images."""
    if ty == 3:
        return (v & U32MASK).astype(np.uint32).view(np.int32)
    if ty == 4:
        return (v & U32MASK).astype(np.uint32)
    if ty == 5:
        return v.view(np.int64)
    if ty == 6:
        return v
    if ty == 7:
        return (v & U32MASK).astype(np.uint32).view(np.float32)
    if ty == 8:
        return v.view(np.float64)
    return v.astype(T[ty])


def image(x, ty):
    """64-bit register images of typed values."""
    if ty in (3, 5):
        return x.astype(np.int64).view(np.uint64)
    if ty == 7:
        return x.astype(np.float32).view(np.uint32).astype(np.uint64)
    if ty == 8:
        return x.astype(np.float64).view(np.uint64)
    if ty == 0:
        return (x != 0).astype(np.uint64)
    return x.astype(T[ty]).astype(np.uint64)


def norm(v, ty):
    if ty == 0:
        return (v != 0).astype(np.uint64)
    if ty == 1:
        return v & np.uint64(0xFF)
    if ty == 2:
        return v & np.uint64(0xFFFF)
    if ty == 3:
        return (v & U32MASK).astype(np.uint32).view(np.int32).astype(np.int64).view(np.uint64)
    if ty in (4, 7):
        return v & U32MASK
    return v


def cvt(v, frm, to):
    if frm == to:
        return v
    if to in (7, 8):
        if frm in (7, 8):
            return image(view(v, frm), to)
        src = v if frm == 6 else v.view(np.int64)
        return image(src.astype(np.float32 if to == 7 else np.float64), to)
    if frm in (7, 8):
        d = view(v, frm).astype(np.float64)
        d = np.where(np.isnan(d), 0.0, np.trunc(d))
        if to == 0:
            return (d != 0).astype(np.uint64)
        if to not in (3, 5):
            d = np.where(d < 0, 0.0, d)
        w = d.astype(np.uint64) if to == 6 else d.astype(np.int64).view(np.uint64)
        return norm(w, to)
    if to == 0:
        return (v != 0).astype(np.uint64)
    return norm(v, to)


def _int_div(x, y, mod, signed):
    zero = y == 0
    ys = np.where(zero, 1, y).astype(y.dtype)
    if signed:
        # floor quotient turned toward zero (an absolute value of the most
        # negative integer would overflow)
        q = np.floor_divide(x, ys)
        r = x - q * ys
        q = np.where((r != 0) & ((x < 0) ^ (ys < 0)), q + 1, q).astype(x.dtype)
    else:
        q = x // ys
    r = (x - q * ys).astype(x.dtype)
    return np.where(zero, 0, r if mod else q).astype(x.dtype)


def binary(op, ty, a, b):
    with np.errstate(all="ignore"):
        if ty in (7, 8):
            x, y = view(a, ty), view(b, ty)
            if op == 10: return image(x + y, ty)
            if op == 11: return image(x - y, ty)
            if op == 12: return image(x * y, ty)
            if op == 13: return image(x / y, ty)
        else:
            x, y = view(a, ty), view(b, ty)
            signed = ty in (3, 5)
            bits = 32 if ty in (3, 4) else 64
            ux = x.view(np.uint32 if bits == 32 else np.uint64)
            if op == 10: return image(x + y, ty)
            if op == 11: return image(x - y, ty)
            if op == 12: return image(x * y, ty)
            if op == 13: return image(_int_div(x, y, False, signed), ty)
            if op == 14: return image(_int_div(x, y, True, signed), ty)
            if op == 15: return image(x & y, ty)
            if op == 16: return image(x | y, ty)
            if op == 17: return image(x ^ y, ty)
            cnt = (b & np.uint64(bits - 1)).astype(ux.dtype)
            if op == 18: return image((ux << cnt).view(x.dtype), ty)
            if op == 19: return image(x >> cnt.astype(x.dtype), ty)
        fn = {20: np.less, 21: np.less_equal, 22: np.greater, 23: np.greater_equal,
              24: np.equal, 25: np.not_equal}[op]
        return fn(x, y).astype(np.uint64)


def unary(op, ty, a):
    with np.errstate(all="ignore"):
        x = view(a, ty)
        if op == 30:
            return image(-x, ty)
        if op == 31:
            return image(~x, ty)
        return image(np.abs(x), ty)


class Lattice:
    """Coordinates, neighbour indices and the static border of a model."""

    def __init__(self, model=None, size=None, deltas=None, torus=True, border=0):
        if model is not None:
            size = tuple(model.size)
            deltas = model.topology.neighborhood.deltas
            torus = not hasattr(model.topology.border, "value")
            border = 0 if torus else int(model.topology.border.value)
        self.size = tuple(int(s) for s in size)
        self.n = int(np.prod(self.size))
        self.torus = bool(torus)
        self.border = int(border)
        idx = np.arange(self.n, dtype=np.int64)
        coords, rest = [], idx
        for s in self.size:
            coords.append(rest % s)
            rest = rest // s
        self.nbr, self.off = [], []
        for delta in deltas:
            j = np.zeros(self.n, dtype=np.int64)
            off = np.zeros(self.n, dtype=bool)
            stride = 1
            for d, s in enumerate(self.size):
                c = coords[d] + int(delta[d])
                out = (c < 0) | (c >= s)
                if self.torus:
                    c = (c + s) % s
                else:
                    off |= out
                    c = np.clip(c, 0, s - 1)
                j += c * stride
                stride *= s
            self.nbr.append(j)
            self.off.append(off)


def run(prog, fld, col, lat, esz, params, color):
    """One pass of a compiled program over every cell (``fld``, ``col`` in place)."""
    n = lat.n
    R = {}
    ctype = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[esz]
    for ins in prog.code:
        op, ty, dst, a, b, c = (int(ins[k]) for k in ("op", "ty", "dst", "a", "b", "c"))
        if op == 1:
            R[dst] = np.full(n, prog.consts[a], dtype=np.uint64)
        elif op == 2:
            R[dst] = np.full(n, params[a], dtype=np.uint64)
        elif op == 3:
            if a < 2:
                R[dst] = fld[c * n:(c + 1) * n].astype(np.uint64)
            else:
                v = fld[c * n + lat.nbr[b]].astype(np.uint64)
                R[dst] = np.where(lat.off[b], np.uint64(lat.border), v)
        elif op == 4:
            R[dst] = R[a].copy()
        elif op == 5:
            R[dst] = cvt(R[a], b, ty)
        elif 10 <= op <= 25:
            R[dst] = binary(op, ty, R[a], R[b])
        elif op in (30, 31, 32):
            R[dst] = unary(op, ty, R[a])
        elif op == 40:
            R[dst] = np.where(R[a] != 0, R[b], R[c])
        elif op == 41:
            R[dst] = norm(R[a] & U32MASK, 3)
        elif op == 42:
            R[dst] = R[a] & U32MASK
        elif op == 50:
            v = R[a] & U32MASK
            cnt = np.zeros(n, dtype=np.uint64)
            for bit in range(32):
                cnt += (v >> np.uint64(bit)) & np.uint64(1)
            R[dst] = cnt
        elif op == 51:
            R[dst] = image(np.exp(view(R[a], 8)), 8)
        elif op == 60:
            fld[b * n:(b + 1) * n] = R[a].astype(ctype)
        elif op == 61:
            rgb = [view(R[r], 3).astype(np.int64) for r in (a, b, c)]
            if color and color["kind"] == "moving_average":
                old = col.reshape(n, 3).astype(np.int64)
                for k in range(3):
                    v = rgb[k] * color["smooth"]
                    rgb[k] = np.maximum(np.minimum(v, old[:, k] + color["fade_in"]),
                                        old[:, k] - color["fade_out"])
            col.reshape(n, 3)[:] = np.stack(rgb, axis=1).astype(np.int32)
        else:
            raise ValueError("opcode %d" % op)


def step(model, fld, col, steps=1, params=None):
    """Advance ``fld``/``col`` (reference layout) by ``steps`` generations."""
    names = []
    progs = [vm.compile_program(model.programs[k], names) for k in ("emit", "absorb")]
    vals = [vm.pack_value(model.meta.__dict__[nm].value, vm.ir.ctype_of(model.meta.__dict__[nm].ctype))
            for nm in names]
    lat = Lattice(model)
    colst = [st for st in model.programs["absorb"].stmts if st.op == "color"]
    color = colst[0].extra if colst else None
    esz = fld.dtype.itemsize
    for _ in range(steps):
        for p in progs:
            run(p, fld, col, lat, esz, vals, color)


def replay(desc, programs, params, fld, col, steps):
    """Run stored programs (``[(code, consts, nregs), ...]``) for a model
    described by an ``XkDesc`` (as the GPU interpreter would)."""
    size = [desc.size[i] for i in range(desc.ndim)]
    deltas = [[desc.delta[k][i] for i in range(desc.ndim)] for k in range(desc.nbr)]
    lat = Lattice(size=size, deltas=deltas, torus=desc.torus, border=desc.border_value)
    color = None
    if desc.color_kind == 2:
        color = {"kind": "moving_average", "fade_in": desc.fade_in, "fade_out": desc.fade_out,
                 "smooth": desc.smooth}
    progs = [vm.VmProgram(code, consts, nregs, [], False) for code, consts, nregs in programs]
    for _ in range(steps):
        for p in progs:
            run(p, fld, col, lat, fld.dtype.itemsize, list(params), color)
