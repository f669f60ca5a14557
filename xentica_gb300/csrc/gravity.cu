// Energy flowing down a gravity field (the reference's GraviCowboys,
// examples/gravicowboys.py:20-71) for sm_103a.
//
// A cell is a uint64 packed LSB first in declaration order
// (properties.py:496-541): energy (12 bits) | new_energy << 12 | gravity
// (float bits) << 24.  One generation, per cell, in the reference's
// arithmetic (its emit and absorb as traced):
//   emit    lowest = 0 + min over the neighbours' gravities (a < b ? a : b, in
//           neighbour order); for buffer k in order, one unit goes to
//           neighbour k when its gravity equals lowest and energy - sent > 0
//           (unsigned); every buffer carries gravity + energy (float);
//           new_energy = energy - sent
//   absorb  energy = (uint16)(new_energy + the units sent towards the cell),
//           gravity = (float)((double)(the float sum of the buffers'
//           gravities in neighbour order) / 8.008)
// and the colour (MovingAverage, color_effects.py:106-130) energy * 255,
// (unsigned)(gravity * 108) twice.  An off-board neighbour of a static border
// reads as the whole border container (border.py:144-151).
//
// One launch per generation: a block loads the gravities and energies of its
// 32 x 32 cells with a halo of two into shared memory, runs emit on the tile
// and a halo of one (what a neighbour sends is a bit of an 8-bit mask, its
// new energy and the one float every buffer carries), then absorb on the
// tile, four rows a thread.  A cell's state is read and written once per
// generation; the reference's nine containers per cell never exist.  The
// division by 8.008 runs in float arithmetic with an exactness test (the
// double-precision pipe is narrow on this part).  What a cell emits is one
// 64-bit shared entry, so absorb reads each neighbour's with one load.
#include "xk_internal.cuh"

struct GravParams {
    int32_t W, H;
    uint64_t border;            // off-board container (static border)
    int32_t color_kind;         // XK_COLOR_*
    int32_t fade_in, fade_out, smooth;
    uint8_t *frame;             // null, or the W x H RendererPlain frame (zoom 1, no offset)
    int32_t frame_smooth;       // its SMOOTH_FACTOR (0: none)
};

#define XK_GC_TX 32
#define XK_GC_TY 32             // rows of a tile; each of the 8 warps runs four of them
#define XK_GC_THREADS 256

// the Moore deltas in the reference's order (x, y): (-1,-1) (-1,0) (-1,1)
// (0,-1) (0,1) (1,-1) (1,0) (1,1); neighbour 7 - k points back along k
__device__ __forceinline__ int xk_gc_dx(int k) { return k < 3 ? -1 : k < 5 ? 0 : 1; }
__device__ __forceinline__ int xk_gc_dy(int k) { return (k == 0 || k == 3 || k == 5) ? -1 : (k == 1 || k == 6) ? 0 : 1; }

__device__ __forceinline__ float xk_gc_grav(uint64_t c) { return __uint_as_float((uint32_t)(c >> 24)); }

// (float)((double)f / 8.008) by the division itself: zeros keep their sign
__device__ __noinline__ float xk_gc_mean_f64(float f)
{
    if (f == 0.0f) return f;
    return __double2float_rn(__ddiv_rn((double)f, 8.008));
}

// (float)((double)f / 8.008) in float arithmetic: the quotient as the
// unevaluated sum q1 + t (8.008 split as CH + CL, R = RN(1/8.008); the
// remainder f - q1 * 8.008 by two fmas), relative error below 2^-45; s =
// RN(q1 + t) and err = q1 + t - s exactly (Fast2Sum).  When q1 + t lies more
// than 2^-43 |s| from the midpoint between s and its neighbour on err's side,
// the exact quotient, and its double rounding, round to s; otherwise (and for
// |f| outside [2^-60, 2^120], zeros and non-finite values) the division
// itself.  Checked equal to the double division for every finite float.
__device__ __forceinline__ float xk_gc_mean(float f)
{
    constexpr float CH = 0x1.00418ap+3f, CL = -0x1.916872p-22f, R = 0x1.ff7d1p-4f;
    const float af = fabsf(f);
    if (!(af >= 0x1p-60f && af <= 0x1p+120f)) return xk_gc_mean_f64(f);
    const float q1 = __fmul_rn(f, R);
    const float e = __fmaf_rn(-q1, CH, f);
    const float e2 = __fmaf_rn(-q1, CL, e);
    const float t = __fmul_rn(e2, R);
    const float s = __fadd_rn(q1, t);
    const float err = __fsub_rn(t, __fsub_rn(s, q1));
    const uint32_t sb = __float_as_uint(s), es = sb & 0x7F800000u;
    float h = __fmul_rn(__uint_as_float(es - (23u << 23)), 0.5f);     // ulp(s) / 2
    if ((sb & 0x007FFFFFu) == 0 && ((__float_as_uint(err) ^ sb) >> 31)) h = __fmul_rn(h, 0.5f);
    const float bound = __fmul_rn(__uint_as_float(es), 0x1p-43f);
    if (fabsf(__fsub_rn(fabsf(err), h)) <= bound) return xk_gc_mean_f64(f);
    return s;
}

struct GravTile {
    float g[XK_GC_TY + 4][XK_GC_TX + 4];        // gravities, halo of two
    uint32_t e[XK_GC_TY + 4][XK_GC_TX + 4];     // energies
    // emitted: .x units sent (bit k: to neighbour k) | new_energy << 8, .y the
    // bits of the gravity every buffer carries (one 64-bit load in absorb)
    uint2 x[XK_GC_TY + 2][XK_GC_TX + 2];
};

// emit of the cell at tile position (y, x): the units go to the neighbours of
// the lowest gravity in neighbour order, one each while energy lasts, i.e. to
// the first min(energy, ties) of them
__device__ __forceinline__ void xk_gc_emit(GravTile &T, int y, int x, int ey, int ex)
{
    const uint32_t energy = T.e[y][x];
    float gk[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) gk[k] = T.g[y + xk_gc_dy(k)][x + xk_gc_dx(k)];
    float m = gk[0];
#pragma unroll
    for (int k = 1; k < 8; ++k) m = m < gk[k] ? m : gk[k];
    const float lowest = __fadd_rn(0.0f, m);
    uint32_t ties = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) ties |= (uint32_t)(lowest == gk[k]) << k;
    uint32_t mask = ties;
    if (energy < (uint32_t)__popc(ties)) {       // energy < 8: only its first set bits
        uint32_t rest = ties;
        mask = 0;
        for (uint32_t j = 0; j < energy; ++j) {
            const uint32_t low = rest & (0u - rest);
            mask |= low;
            rest ^= low;
        }
    }
    T.x[ey][ex] = make_uint2(mask | (energy - (uint32_t)__popc(mask)) << 8,
                             __float_as_uint(__fadd_rn(T.g[y][x], (float)energy)));
}

template <bool TORUS>
__global__ void __launch_bounds__(XK_GC_THREADS)
xk_k_gravity(const uint64_t *__restrict__ src, uint64_t *__restrict__ dst, int32_t *__restrict__ col,
             GravParams p)
{
    __shared__ GravTile T;
    const int tid = threadIdx.y * XK_GC_TX + threadIdx.x;
    const int x0 = blockIdx.x * XK_GC_TX, y0 = blockIdx.y * XK_GC_TY;
    xk_grid_dep_wait();                 // launched as a dependent of the previous generation
    for (int e = tid; e < (XK_GC_TY + 4) * (XK_GC_TX + 4); e += XK_GC_THREADS) {
        const int sy = e / (XK_GC_TX + 4), sx = e % (XK_GC_TX + 4);
        int gx = x0 + sx - 2, gy = y0 + sy - 2;
        uint64_t v;
        if (TORUS) {
            if ((unsigned)gx >= (unsigned)p.W) { gx %= p.W; if (gx < 0) gx += p.W; }
            if ((unsigned)gy >= (unsigned)p.H) { gy %= p.H; if (gy < 0) gy += p.H; }
            v = __ldg(src + (int64_t)gy * p.W + gx);
        } else {
            v = (gx >= 0 && gx < p.W && gy >= 0 && gy < p.H) ? __ldg(src + (int64_t)gy * p.W + gx) : p.border;
        }
        T.g[sy][sx] = xk_gc_grav(v);
        T.e[sy][sx] = (uint32_t)v & 4095u;
    }
    __syncthreads();
    for (int e = tid; e < (XK_GC_TY + 2) * (XK_GC_TX + 2); e += XK_GC_THREADS) {
        const int ey = e / (XK_GC_TX + 2), ex = e % (XK_GC_TX + 2);
        xk_gc_emit(T, ey + 1, ex + 1, ey, ex);   // off-board positions are never read
    }
    __syncthreads();
    const int gx = x0 + threadIdx.x;
    if (gx >= p.W) return;
#pragma unroll
    for (int r = 0; r < XK_GC_TY / 8; ++r) {
        const int ly = threadIdx.y + 8 * r, gy = y0 + ly;
        if (gy >= p.H) return;
        const int ty = ly + 1, tx = threadIdx.x + 1;
        uint32_t got = 0, received = 0;
        float gk[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int dx = xk_gc_dx(k), dy = xk_gc_dy(k);
            const bool on = TORUS || ((unsigned)(gx + dx) < (unsigned)p.W && (unsigned)(gy + dy) < (unsigned)p.H);
            if (on) {
                const uint2 w = T.x[ty + dy][tx + dx];
                got |= w.x & (1u << (7 - k));   // the unit neighbour k sent back along k
                gk[k] = __uint_as_float(w.y);
            } else {
                received += (uint32_t)p.border & 4095u;
                gk[k] = xk_gc_grav(p.border);
            }
        }
        received += (uint32_t)__popc(got);
        float field = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) field = __fadd_rn(field, gk[k]);
        const uint32_t newe = T.x[ty][tx].x >> 8;
        const uint32_t energy = (newe + received) & 0xFFFFu;
        const float g = xk_gc_mean(field);
        const int64_t i = (int64_t)gy * p.W + gx;
        dst[i] = (uint64_t)(energy & 4095u) | (uint64_t)newe << 12 | (uint64_t)__float_as_uint(g) << 24;
        if (p.color_kind == XK_COLOR_NONE) continue;
        const int gg = (int)__float2uint_rz(__fmul_rn(g, 108.0f));
        int rgb[3] = {(int)energy * 255 * p.smooth, gg * p.smooth, gg * p.smooth};
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            const int old = col[3 * i + ch];
            const int m = rgb[ch] < old + p.fade_in ? rgb[ch] : old + p.fade_in;
            rgb[ch] = m > old - p.fade_out ? m : old - p.fade_out;
        }
        col[3 * i] = rgb[0];
        col[3 * i + 1] = rgb[1];
        col[3 * i + 2] = rgb[2];
        if (p.frame) {
            // RendererPlain at zoom 1: the colour as a float, / SMOOTH_FACTOR,
            // truncated, its low byte; exact without the division below 2^24
            const bool small = (((uint32_t)rgb[0] + (1u << 24)) | ((uint32_t)rgb[1] + (1u << 24)) |
                                ((uint32_t)rgb[2] + (1u << 24))) < (1u << 25);
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                uint8_t px;
                if (p.frame_smooth <= 1 && small) {
                    px = (uint8_t)rgb[ch];
                } else {
                    float v = (float)rgb[ch];
                    if (p.frame_smooth > 0) v = __fdiv_rn(v, (float)p.frame_smooth);
                    px = (uint8_t)(int)v;
                }
                p.frame[3 * i + ch] = px;
            }
        }
    }
}

cudaError_t xk_gravity_step(const uint64_t *src, uint64_t *dst, int32_t *col, const xk_desc &d,
                            cudaStream_t s, uint8_t *frame, int frame_smooth)
{
    GravParams p;
    p.W = (int32_t)d.size[0];
    p.H = (int32_t)d.size[1];
    p.border = d.border_value;
    p.color_kind = d.color_kind;
    p.fade_in = d.fade_in;
    p.fade_out = d.fade_out;
    p.smooth = d.smooth;
    p.frame = frame;
    p.frame_smooth = frame_smooth;
    dim3 block(XK_GC_TX, XK_GC_THREADS / XK_GC_TX);
    dim3 grid((p.W + XK_GC_TX - 1) / XK_GC_TX, (p.H + XK_GC_TY - 1) / XK_GC_TY);
    return d.torus ? xk_launch_pdl(xk_k_gravity<true>, grid, block, 0, s, src, dst, col, p)
                   : xk_launch_pdl(xk_k_gravity<false>, grid, block, 0, s, src, dst, col, p);
}
