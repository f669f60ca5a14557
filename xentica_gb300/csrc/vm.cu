// Generic interpreter for traced models no hand-written template implements.
//
// xentica_gb300/core/vm.py compiles a model's emit and absorb programs into
// typed register instructions; this kernel runs them with the reference's
// execution model (xentica/core/base.py:461-487): one thread per cell, an
// emit pass that writes the cell's buffer planes, then an absorb pass that
// reads the neighbours' buffers (plane rev_index_map[k] + 1 of neighbour k,
// base.py:475-487) and writes the main plane and the colour.  Memory is the
// reference's own layout: N + 1 planes of packed containers (1/2/4/8 bytes)
// plus int32 x 3 colours.  Off-board neighbours of a static border read the
// border's whole container value (properties.py:444-483).
//
// Registers are 64-bit images of C values: integers sign- or zero-extended
// from their width, floats as their IEEE bits.  Every instruction has a type
// and operands already converted to it (the compiler made every C implicit
// conversion explicit), so the semantics are C's: wrap-around integer
// arithmetic, truncating division, IEEE float and double with no
// contraction (-fmad=false), shift counts taken modulo the width.  Integer
// division by zero yields 0 instead of trapping.  No instruction branches, so
// every thread runs the same stream and the dispatch stays warp-uniform.
#include <math.h>

#include "xk_internal.cuh"

enum { VT_BOOL = 0, VT_U8, VT_U16, VT_I32, VT_U32, VT_I64, VT_U64, VT_F32, VT_F64 };
enum {
    OP_CONST = 1, OP_PARAM = 2, OP_LOAD = 3, OP_MOV = 4, OP_CVT = 5,
    OP_ADD = 10, OP_SUB, OP_MUL, OP_DIV, OP_MOD, OP_AND, OP_OR, OP_XOR, OP_SHL, OP_SHR,
    OP_LT = 20, OP_LE, OP_GT, OP_GE, OP_EQ, OP_NE,
    OP_NEG = 30, OP_BNOT, OP_ABS,
    OP_SEL = 40, OP_F2I, OP_I2F, OP_POPC = 50, OP_EXP = 51,
    OP_STORE = 60, OP_COLOR = 61
};

#define XK_VM_MAXREG 256

__device__ __forceinline__ uint64_t vm_norm(uint64_t v, int ty)
{
    switch (ty) {
    case VT_BOOL: return v != 0;
    case VT_U8: return v & 0xFFull;
    case VT_U16: return v & 0xFFFFull;
    case VT_I32: return (uint64_t)(int64_t)(int32_t)(uint32_t)v;
    case VT_U32: return v & 0xFFFFFFFFull;
    case VT_F32: return v & 0xFFFFFFFFull;
    default: return v;
    }
}

__device__ __forceinline__ bool vm_signed(int ty) { return ty == VT_I32 || ty == VT_I64; }
__device__ __forceinline__ float vm_f(uint64_t v) { return __int_as_float((int)(uint32_t)v); }
__device__ __forceinline__ double vm_d(uint64_t v) { return __longlong_as_double((long long)v); }
__device__ __forceinline__ uint64_t vm_of(float x) { return (uint64_t)(uint32_t)__float_as_int(x); }
__device__ __forceinline__ uint64_t vm_of(double x) { return (uint64_t)__double_as_longlong(x); }

// C conversion of register image v from type `from` to type `to`
__device__ uint64_t vm_cvt(uint64_t v, int from, int to)
{
    if (from == to) return v;
    if (to == VT_F32 || to == VT_F64) {
        double dv;
        float fv;
        if (from == VT_F32) {
            if (to == VT_F64) return vm_of((double)vm_f(v));
            return v;
        }
        if (from == VT_F64) return vm_of(__double2float_rn(vm_d(v)));
        // integer source: its 64-bit image is the value (signed types sign-extended)
        if (from == VT_U64) {
            if (to == VT_F32) { fv = __ull2float_rn(v); return vm_of(fv); }
            dv = __ull2double_rn(v);
            return vm_of(dv);
        }
        if (to == VT_F32) { fv = __ll2float_rn((long long)v); return vm_of(fv); }
        dv = __ll2double_rn((long long)v);
        return vm_of(dv);
    }
    if (from == VT_F32 || from == VT_F64) {
        // truncation toward zero; NaN -> 0; negative -> 0 for unsigned targets
        double d = from == VT_F32 ? (double)vm_f(v) : vm_d(v);
        if (d != d) d = 0.0;
        d = trunc(d);
        if (to == VT_BOOL) return d != 0.0;
        const bool uns = !(to == VT_I32 || to == VT_I64);
        if (uns && d < 0.0) d = 0.0;
        const uint64_t w = (to == VT_U64) ? (uint64_t)__double2ull_rz(d)
                                          : (uint64_t)__double2ll_rz(d);
        return vm_norm(w, to);
    }
    if (to == VT_BOOL) return v != 0;
    return vm_norm(v, to);   // integer -> integer: modular
}

template <class T>
__device__ __forceinline__ T vm_int_div(T x, T y, bool mod)
{
    if (y == 0) return 0;
    if (mod) return x % y;
    return x / y;
}

// arithmetic / comparison on integers of type T (register images in a, b)
template <class T>
__device__ __forceinline__ uint64_t vm_int_op(int op, uint64_t ra, uint64_t rb, int ty)
{
    const T x = (T)ra, y = (T)rb;
    const int bits = (int)sizeof(T) * 8;
    switch (op) {
    case OP_ADD: return vm_norm((uint64_t)(T)(x + y), ty);
    case OP_SUB: return vm_norm((uint64_t)(T)(x - y), ty);
    case OP_MUL: return vm_norm((uint64_t)(T)(x * y), ty);
    case OP_DIV: return vm_norm((uint64_t)vm_int_div<T>(x, y, false), ty);
    case OP_MOD: return vm_norm((uint64_t)vm_int_div<T>(x, y, true), ty);
    case OP_AND: return vm_norm((uint64_t)(T)(x & y), ty);
    case OP_OR: return vm_norm((uint64_t)(T)(x | y), ty);
    case OP_XOR: return vm_norm((uint64_t)(T)(x ^ y), ty);
    case OP_SHL: return vm_norm((uint64_t)(T)(x << ((int)rb & (bits - 1))), ty);
    case OP_SHR: return vm_norm((uint64_t)(T)(x >> ((int)rb & (bits - 1))), ty);
    case OP_LT: return x < y;
    case OP_LE: return x <= y;
    case OP_GT: return x > y;
    case OP_GE: return x >= y;
    case OP_EQ: return x == y;
    case OP_NE: return x != y;
    }
    return 0;
}

template <class F>
__device__ __forceinline__ uint64_t vm_float_op(int op, F x, F y)
{
    switch (op) {
    case OP_ADD: return vm_of((F)(x + y));
    case OP_SUB: return vm_of((F)(x - y));
    case OP_MUL: return vm_of((F)(x * y));
    case OP_DIV: return vm_of((F)(x / y));
    case OP_LT: return x < y;
    case OP_LE: return x <= y;
    case OP_GT: return x > y;
    case OP_GE: return x >= y;
    case OP_EQ: return x == y;
    case OP_NE: return x != y;
    }
    return 0;
}

__device__ uint64_t vm_binary(int op, int ty, uint64_t a, uint64_t b)
{
    switch (ty) {
    case VT_I32: return vm_int_op<int32_t>(op, a, b, ty);
    case VT_U32: return vm_int_op<uint32_t>(op, a, b, ty);
    case VT_I64: return vm_int_op<int64_t>(op, a, b, ty);
    case VT_U64: return vm_int_op<uint64_t>(op, a, b, ty);
    case VT_F32: return vm_float_op<float>(op, vm_f(a), vm_f(b));
    case VT_F64: return vm_float_op<double>(op, vm_d(a), vm_d(b));
    }
    return 0;
}

__device__ uint64_t vm_unary(int op, int ty, uint64_t a)
{
    if (ty == VT_F32) {
        const float x = vm_f(a);
        return vm_of(op == OP_NEG ? -x : fabsf(x));
    }
    if (ty == VT_F64) {
        const double x = vm_d(a);
        return vm_of(op == OP_NEG ? -x : fabs(x));
    }
    if (op == OP_NEG) return vm_norm((uint64_t)0 - a, ty);
    if (op == OP_BNOT) return vm_norm(~a, ty);
    // abs of a signed value (unsigned: itself)
    if (vm_signed(ty) && (int64_t)a < 0) return vm_norm((uint64_t)0 - a, ty);
    return a;
}

__device__ __forceinline__ uint64_t vm_ld(const uint8_t *fld, int esz, int64_t idx)
{
    switch (esz) {
    case 1: return fld[idx];
    case 2: return ((const uint16_t *)fld)[idx];
    case 4: return ((const uint32_t *)fld)[idx];
    default: return ((const uint64_t *)fld)[idx];
    }
}

__device__ __forceinline__ void vm_st(uint8_t *fld, int esz, int64_t idx, uint64_t v)
{
    switch (esz) {
    case 1: fld[idx] = (uint8_t)v; break;
    case 2: ((uint16_t *)fld)[idx] = (uint16_t)v; break;
    case 4: ((uint32_t *)fld)[idx] = (uint32_t)v; break;
    default: ((uint64_t *)fld)[idx] = v; break;
    }
}

__global__ void __launch_bounds__(128)
xk_k_vm(const xk_vm_ins *__restrict__ code, int ncode, const uint64_t *__restrict__ consts,
        const uint64_t *__restrict__ params, uint8_t *__restrict__ fld, int32_t *__restrict__ col,
        VmGeo g)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    uint64_t R[XK_VM_MAXREG];
    int64_t coord[XK_MAXDIM];
    {
        int64_t rest = i;
        for (int d = 0; d < g.ndim; ++d) {
            coord[d] = rest % g.size[d];
            rest /= g.size[d];
        }
    }
    for (int pc = 0; pc < ncode; ++pc) {
        const xk_vm_ins in = code[pc];
        const int op = in.op, ty = in.ty;
        uint64_t v = 0;
        switch (op) {
        case OP_CONST: v = consts[in.a]; break;
        case OP_PARAM: v = params[in.a]; break;
        case OP_LOAD: {
            const int kind = in.a;
            const int plane = in.c;
            if (kind == 0 || kind == 1) {
                v = vm_ld(fld, g.esz, i + g.n * plane);
            } else {
                // neighbour in.b: its coordinates, wrapped or off the board
                int64_t j = 0, stride = 1;
                bool off = false;
                for (int d = 0; d < g.ndim; ++d) {
                    int64_t c = coord[d] + g.delta[in.b][d];
                    if (c < 0 || c >= g.size[d]) {
                        if (g.torus) c = (c + g.size[d]) % g.size[d];
                        else off = true;
                    }
                    j += c * stride;
                    stride *= g.size[d];
                }
                v = off ? g.border : vm_ld(fld, g.esz, j + g.n * plane);
            }
            break;
        }
        case OP_MOV: v = R[in.a]; break;
        case OP_CVT: v = vm_cvt(R[in.a], in.b, ty); break;
        case OP_NEG: case OP_BNOT: case OP_ABS: v = vm_unary(op, ty, R[in.a]); break;
        case OP_SEL: v = R[in.a] != 0 ? R[in.b] : R[in.c]; break;
        case OP_F2I: v = vm_norm((uint64_t)(int64_t)(int32_t)(uint32_t)R[in.a], VT_I32); break;
        case OP_I2F: v = R[in.a] & 0xFFFFFFFFull; break;
        case OP_POPC: v = (uint64_t)__popc((unsigned)R[in.a]); break;
        case OP_EXP: v = vm_of(exp(vm_d(R[in.a]))); break;
        case OP_STORE: vm_st(fld, g.esz, i + g.n * in.b, R[in.a]); continue;
        case OP_COLOR: {
            int r = (int)(int32_t)R[in.a], gg = (int)(int32_t)R[in.b], b = (int)(int32_t)R[in.c];
            if (g.color_kind == XK_COLOR_MOVING_AVERAGE) {
                const int s = g.smooth;
                r *= s;
                gg *= s;
                b *= s;
                const int orr = col[3 * i], og = col[3 * i + 1], ob = col[3 * i + 2];
                r = max(min(r, orr + g.fade_in), orr - g.fade_out);
                gg = max(min(gg, og + g.fade_in), og - g.fade_out);
                b = max(min(b, ob + g.fade_in), ob - g.fade_out);
            }
            col[3 * i] = r;
            col[3 * i + 1] = gg;
            col[3 * i + 2] = b;
            continue;
        }
        default:
            if (op >= OP_ADD && op <= OP_NE) v = vm_binary(op, ty, R[in.a], R[in.b]);
            break;
        }
        R[in.dst] = v;
    }
}

cudaError_t xk_vm_run(const xk_vm_ins *code, int ncode, const uint64_t *consts,
                      const uint64_t *params, uint8_t *fld, int32_t *col, const VmGeo &g,
                      cudaStream_t s)
{
    if (ncode <= 0) return cudaSuccess;
    const int threads = 128;
    const int64_t blocks = (g.n + threads - 1) / threads;
    xk_k_vm<<<(unsigned)blocks, threads, 0, s>>>(code, ncode, consts, params, fld, col, g);
    return cudaGetLastError();
}
