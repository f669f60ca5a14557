// Per-cell noise (the reference's NoiseTV, examples/noisetv.py:13-31) for
// sm_103a.
//
// A cell is one RandomProperty (uint16).  Emit writes nothing; absorb reads
// the property once and the colour reads its uniform draw, each read one
// advance of x = (x * 58321 + 11113) % 65535 (properties.py:638-660); the
// colour is (unsigned)((float)x / 65535 * 255) on every channel, through
// MovingAverage (color_effects.py:106-130), and the cell stores x.  No cell
// reads another, so one launch may run many generations of a cell in
// registers: its state and colour are read once and written once.  The two
// advances of a generation are one composed map x -> (a x + c) % 65535 (a, c
// below 65535, so a x + c stays below 2^32 for every 16-bit x).  (Measured
// and not kept: the grey level of every x from a 65 535-byte table, which put
// a load in each generation's dependent chain: 930 against 1 246 G.)
#include "xk_internal.cuh"

struct NoiseParams {
    int64_t n;
    int32_t color_kind;          // XK_COLOR_*
    int32_t fade_in, fade_out, smooth;
    int32_t generations;         // generations per launch (1 when a frame is written)
    uint8_t *frame;              // null, or the zoom-1 RendererPlain frame of a 2-D lattice
    int32_t frame_smooth;        // its SMOOTH_FACTOR (0: none)
};

// the two advances of a generation composed: 58321^2 and 58321 * 11113 + 11113, mod 65535
#define XK_NOISE_A2 ((58321ull * 58321ull) % 65535ull)
#define XK_NOISE_C2 ((58321ull * 11113ull + 11113ull) % 65535ull)

__global__ void __launch_bounds__(256)
xk_k_noise(uint16_t *__restrict__ cells, int32_t *__restrict__ col, NoiseParams p)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    xk_grid_dep_wait();                 // launched as a dependent of the previous generation
    uint32_t x = cells[i];
    const bool ma = p.color_kind == XK_COLOR_MOVING_AVERAGE;
    int c0 = 0, c1 = 0, c2 = 0;
    if (ma) {
        c0 = col[3 * i];
        c1 = col[3 * i + 1];
        c2 = col[3 * i + 2];
    }
    for (int g = 0; g < p.generations; ++g) {
        x = ((uint32_t)XK_NOISE_A2 * x + (uint32_t)XK_NOISE_C2) % 65535u;
        int v = (int)__float2uint_rz(__fmul_rn(__fdiv_rn((float)x, 65535.0f), 255.0f));
        if (ma) {
            v *= p.smooth;
            auto clamp = [&](int old) {
                const int m = v < old + p.fade_in ? v : old + p.fade_in;
                return m > old - p.fade_out ? m : old - p.fade_out;
            };
            c0 = clamp(c0);
            c1 = clamp(c1);
            c2 = clamp(c2);
        } else {
            c0 = c1 = c2 = v;
        }
    }
    cells[i] = (uint16_t)x;
    if (p.color_kind == XK_COLOR_NONE) return;
    col[3 * i] = c0;
    col[3 * i + 1] = c1;
    col[3 * i + 2] = c2;
    if (p.frame) {
        // RendererPlain at zoom 1: the colour as a float, / SMOOTH_FACTOR,
        // truncated, its low byte; exact without the division below 2^24
        const int c[3] = {c0, c1, c2};
        const bool small = (((uint32_t)c0 + (1u << 24)) | ((uint32_t)c1 + (1u << 24)) |
                            ((uint32_t)c2 + (1u << 24))) < (1u << 25);
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            uint8_t px;
            if (p.frame_smooth <= 1 && small) {
                px = (uint8_t)c[ch];
            } else {
                float f = (float)c[ch];
                if (p.frame_smooth > 0) f = __fdiv_rn(f, (float)p.frame_smooth);
                px = (uint8_t)(int)f;
            }
            p.frame[3 * i + ch] = px;
        }
    }
}

cudaError_t xk_noise_step(uint16_t *cells, int32_t *col, const xk_desc &d, int64_t n, int generations,
                          cudaStream_t s, uint8_t *frame, int frame_smooth)
{
    if (generations < 1 || (frame && generations != 1)) return cudaErrorInvalidValue;
    NoiseParams p;
    p.n = n;
    p.color_kind = d.color_kind;
    p.fade_in = d.fade_in;
    p.fade_out = d.fade_out;
    p.smooth = d.smooth;
    p.generations = generations;
    p.frame = frame;
    p.frame_smooth = frame_smooth;
    const int threads = 256;
    return xk_launch_pdl(xk_k_noise, dim3((unsigned)((n + threads - 1) / threads)), dim3(threads), 0, s,
                         cells, col, p);
}
