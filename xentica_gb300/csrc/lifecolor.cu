// Life with inherited colour channels (the reference's GameOfLifeColor,
// examples/game_of_life.py:112-159) for sm_103a.
//
// A cell is a uint32 packed LSB first in declaration order
// (properties.py:496-541): state (1 bit) | red << 1 | green << 9 | blue << 17.
// Emit copies every field into every buffer, so a neighbour's buffer is its
// main state: emit is fused away and the kernel reads the neighbours' cells
// directly (ping-pong state buffers).  Per cell, in the reference's integer
// arithmetic (its absorb as traced):
//   alive  = sum_k state_k
//   state' = ((8 >> alive) & 1) | ((12 >> alive) & 1 & state)
//   c'     = (unsigned char)((sum_k (c_k + 1)) * state')      for c = r, g, b
// and the colour (MovingAverage, color_effects.py:106-130)
//   new = state' * c' * SMOOTH, clamped to [old - FADE_OUT, old + FADE_IN].
// An off-board neighbour of a static border reads as the whole border
// container (border.py:144-151).  The unsigned sums commute, so the
// neighbour order does not matter; red and blue are summed together as the
// two 16-bit halves of (w >> 1) & 0x00FF00FF (a sum is at most 8 * 255).
// (Measured and not kept: column sums shared between lanes by shuffles, whose
// warp- and lattice-edge columns cost more than the loads they saved.)
#include "xk_internal.cuh"

struct LColorParams {
    int32_t W, H;
    int32_t torus;
    uint32_t border;            // off-board container (static border)
    int32_t color_kind;         // XK_COLOR_*
    int32_t fade_in, fade_out, smooth;
    uint8_t *frame;             // null, or the W x H RendererPlain frame (zoom 1, no offset)
    int32_t frame_smooth;       // its SMOOTH_FACTOR (0: none)
};

#define XK_LC_BX 32
#define XK_LC_BY 8

// TORUS: every neighbour on the lattice (wrapped), else off-board ones read
// the border container
template <bool TORUS>
__global__ void __launch_bounds__(XK_LC_BX * XK_LC_BY)
xk_k_lifecolor(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, int32_t *__restrict__ col,
               LColorParams p)
{
    const int x = blockIdx.x * XK_LC_BX + threadIdx.x;
    const int y = blockIdx.y * XK_LC_BY + threadIdx.y;
    if (x >= p.W || y >= p.H) return;   // no block-wide synchronisation below
    xk_grid_dep_wait();                 // launched as a dependent of the previous generation
    const int xl = x > 0 ? x - 1 : p.W - 1, xr = x + 1 < p.W ? x + 1 : 0;
    const int yu = y > 0 ? y - 1 : p.H - 1, yd = y + 1 < p.H ? y + 1 : 0;
    const int nxs[3] = {xl, x, xr}, nys[3] = {yu, y, yd};
    const bool xon[3] = {x > 0, true, x + 1 < p.W}, yon[3] = {y > 0, true, y + 1 < p.H};
    uint32_t alive = 0, rb = 0, gs = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            if (a == 1 && b == 1) continue;
            const bool on = TORUS || (yon[a] && xon[b]);
            const uint32_t w = on ? __ldg(src + (int64_t)nys[a] * p.W + nxs[b]) : p.border;
            alive += w & 1u;
            rb += (w >> 1) & 0x00FF00FFu;
            gs += (w >> 9) & 0xFFu;
        }
    const int64_t i = (int64_t)y * p.W + x;
    const uint32_t s = __ldg(src + i) & 1u;
    const uint32_t ns = ((8u >> alive) & 1u) | ((12u >> alive) & 1u & s);
    const uint32_t r = (((rb & 0xFFFFu) + 8u) * ns) & 255u;
    const uint32_t g = ((gs + 8u) * ns) & 255u;
    const uint32_t b = (((rb >> 16) + 8u) * ns) & 255u;
    dst[i] = ns | (r << 1) | (g << 9) | (b << 17);
    if (p.color_kind == XK_COLOR_NONE) return;
    int rgb[3] = {(int)(ns * r) * p.smooth, (int)(ns * g) * p.smooth, (int)(ns * b) * p.smooth};
    if (p.color_kind == XK_COLOR_MOVING_AVERAGE) {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            const int old = col[3 * i + ch];
            const int m = rgb[ch] < old + p.fade_in ? rgb[ch] : old + p.fade_in;
            rgb[ch] = m > old - p.fade_out ? m : old - p.fade_out;
        }
    }
    col[3 * i] = rgb[0];
    col[3 * i + 1] = rgb[1];
    col[3 * i + 2] = rgb[2];
    if (p.frame) {
        // the pixel of this cell as RendererPlain computes it at zoom 1: the
        // colour as a float, / SMOOTH_FACTOR, truncated, its low byte; int ->
        // float -> int and a division by 1 are exact below 2^24 in magnitude
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

cudaError_t xk_lifecolor_step(const uint32_t *src, uint32_t *dst, int32_t *col, const xk_desc &d,
                              cudaStream_t s, uint8_t *frame, int frame_smooth)
{
    LColorParams p;
    p.W = (int32_t)d.size[0];
    p.H = (int32_t)d.size[1];
    p.torus = d.torus;
    p.border = (uint32_t)d.border_value;
    p.color_kind = d.color_kind;
    p.fade_in = d.fade_in;
    p.fade_out = d.fade_out;
    p.smooth = d.smooth;
    p.frame = frame;
    p.frame_smooth = frame_smooth;
    dim3 block(XK_LC_BX, XK_LC_BY);
    dim3 grid((p.W + XK_LC_BX - 1) / XK_LC_BX, (p.H + XK_LC_BY - 1) / XK_LC_BY);
    return p.torus ? xk_launch_pdl(xk_k_lifecolor<true>, grid, block, 0, s, src, dst, col, p)
                   : xk_launch_pdl(xk_k_lifecolor<false>, grid, block, 0, s, src, dst, col, p);
}
