// Mass-transfer generation kernel (3-D von Neumann, wall border) for sm_103a.
//
// The model (a sand-transfer CA written in the reference's DSL): every cell
// sends mass / 7 to each neighbour whose mass is not the wall value and
// absorbs what its neighbours send; off-board neighbours read as the wall
// (StaticBorder, border.py:144-151, properties.py:444-483).  Per cell, in the
// reference's unsigned 32-bit arithmetic:
//   sent_k     = (m / 7) * (m_k != WALL)                    (emit, buffer k)
//   incoming_k = off-board ? 0 : nb_k * (nb_k != WALL),
//                nb_k = (m_k / 7) * (m != WALL)             (neighbour's buffer)
//   m'         = m - sum_k sent_k + sum_k incoming_k
// Colour (plain ColorEffect): min(m' * 32, 255) on every channel.
//
// One thread per (x, y) column walks z with a three-deep register queue; the
// x/y neighbours of plane z come from a shared tile with a one-cell halo.  The
// same pass writes the column's colour sum (RendererPlain's projection over
// z, exact in float because it is a sum of integers below 2^24) and adds the
// column's mass to the generation's total (the conserved quantity).
#include "xk_internal.cuh"

#define XK_MASS_BX 32
#define XK_MASS_BY 8

struct MassParams {
    int32_t W, H, D;
    uint32_t wall;
};

__device__ __forceinline__ uint32_t xk_mass_color(uint32_t m)
{
    const uint32_t v = m * 32u;
    return v < 255u ? v : 255u;
}

__global__ void __launch_bounds__(XK_MASS_BX * XK_MASS_BY)
xk_k_mass(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, uint32_t *__restrict__ proj,
          unsigned long long *__restrict__ total, MassParams p)
{
    __shared__ uint32_t tile[XK_MASS_BY + 2][XK_MASS_BX + 2];
    __shared__ unsigned long long warp_sums[XK_MASS_BX * XK_MASS_BY / 32];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = blockIdx.x * XK_MASS_BX + tx, y = blockIdx.y * XK_MASS_BY + ty;
    const bool in = x < p.W && y < p.H;
    const int64_t plane = (int64_t)p.W * p.H;
    const int64_t col = (int64_t)y * p.W + x;
    // in-board flags of the x/y neighbours (z neighbours are checked per plane)
    const bool has_xp = x + 1 < p.W, has_xm = x > 0, has_yp = y + 1 < p.H, has_ym = y > 0;
    uint32_t m_prev = p.wall;
    uint32_t m_cur = in ? src[col] : p.wall;
    uint32_t proj_sum = 0;
    unsigned long long mass_sum = 0;
    for (int z = 0; z < p.D; ++z) {
        const uint32_t m_next = (in && z + 1 < p.D) ? src[(int64_t)(z + 1) * plane + col] : p.wall;
        tile[ty + 1][tx + 1] = m_cur;
        const int64_t zb = (int64_t)z * plane;
        if (tx == 0)
            tile[ty + 1][0] = (y < p.H && x > 0 && x - 1 < p.W) ? src[zb + col - 1] : p.wall;
        if (tx == XK_MASS_BX - 1)
            tile[ty + 1][XK_MASS_BX + 1] = (y < p.H && x + 1 < p.W) ? src[zb + col + 1] : p.wall;
        if (ty == 0)
            tile[0][tx + 1] = (x < p.W && y > 0 && y - 1 < p.H) ? src[zb + col - p.W] : p.wall;
        if (ty == XK_MASS_BY - 1)
            tile[XK_MASS_BY + 1][tx + 1] = (x < p.W && y + 1 < p.H) ? src[zb + col + p.W] : p.wall;
        __syncthreads();
        if (in) {
            const uint32_t m = m_cur;
            // von Neumann order: +x, -x, +y, -y, +z, -z
            const uint32_t mk[6] = {tile[ty + 1][tx + 2], tile[ty + 1][tx], tile[ty + 2][tx + 1],
                                    tile[ty][tx + 1], m_next, m_prev};
            const bool on[6] = {has_xp, has_xm, has_yp, has_ym, z + 1 < p.D, z > 0};
            const uint32_t share = m / 7u;
            const uint32_t keep = (uint32_t)(m != p.wall);
            uint32_t v = m;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const uint32_t mkk = on[k] ? mk[k] : p.wall;
                v -= share * (uint32_t)(mkk != p.wall);
                const uint32_t nb = (mkk / 7u) * keep;
                v += on[k] ? nb * (uint32_t)(nb != p.wall) : 0u;
            }
            dst[zb + col] = v;
            proj_sum += xk_mass_color(v);
            mass_sum += v;
        }
        __syncthreads();
        m_prev = m_cur;
        m_cur = m_next;
    }
    if (in && proj) proj[col] = proj_sum;
    // block total -> one atomic per CTA
    for (int off = 16; off > 0; off >>= 1) mass_sum += __shfl_down_sync(0xFFFFFFFFu, mass_sum, off);
    const int tid = ty * XK_MASS_BX + tx;
    if ((tid & 31) == 0) warp_sums[tid >> 5] = mass_sum;
    __syncthreads();
    if (tid == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < XK_MASS_BX * XK_MASS_BY / 32; ++w) s += warp_sums[w];
        atomicAdd(total, s);
    }
}

// column colour sums of a state (after an upload, before any step)
__global__ void xk_k_mass_project(const uint32_t *__restrict__ src, uint32_t *__restrict__ proj,
                                  MassParams p)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t plane = (int64_t)p.W * p.H;
    if (c >= plane) return;
    uint32_t s = 0;
    for (int z = 0; z < p.D; ++z) s += xk_mass_color(src[(int64_t)z * plane + c]);
    proj[c] = s;
}

__global__ void xk_k_mass_colors(const uint32_t *__restrict__ src, int32_t *__restrict__ col, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int v = (int)xk_mass_color(src[i]);
    col[3 * i] = v;
    col[3 * i + 1] = v;
    col[3 * i + 2] = v;
}

// RendererPlain over axes (0, 1) from the column sums: the float sum of a
// column's colours equals its integer sum, divided by the depth
__global__ void xk_k_mass_render(const uint32_t *__restrict__ proj, int32_t *__restrict__ img,
                                 MassParams p, int width, int height, int zoom, int dx, int dy)
{
    const int64_t ip = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= (int64_t)width * height) return;
    const unsigned i = (unsigned)ip;
    int xa = (int)(__fdiv_rn((float)(i % (unsigned)width), (float)zoom)) + dx;
    int xb = (int)(__fdiv_rn((float)(i / (unsigned)width), (float)zoom)) + dy;
    if (xa < 0) xa = p.W - (-xa % p.W);
    if (xa >= p.W) xa = xa % p.W;
    if (xb < 0) xb = p.H - (-xb % p.H);
    if (xb >= p.H) xb = xb % p.H;
    const float s = (float)proj[(int64_t)xb * p.W + xa];
    const int v = (int)__fdiv_rn(s, (float)p.D);
    img[3 * ip] = v;
    img[3 * ip + 1] = v;
    img[3 * ip + 2] = v;
}

static MassParams mass_params(const xk_desc &d)
{
    MassParams p;
    p.W = (int32_t)d.size[0];
    p.H = (int32_t)d.size[1];
    p.D = (int32_t)d.size[2];
    p.wall = d.wall;
    return p;
}

cudaError_t xk_mass_step(const uint32_t *src, uint32_t *dst, uint32_t *proj,
                         unsigned long long *total, const xk_desc &d, cudaStream_t s)
{
    const MassParams p = mass_params(d);
    dim3 block(XK_MASS_BX, XK_MASS_BY);
    dim3 grid((p.W + XK_MASS_BX - 1) / XK_MASS_BX, (p.H + XK_MASS_BY - 1) / XK_MASS_BY);
    xk_k_mass<<<grid, block, 0, s>>>(src, dst, proj, total, p);
    return cudaGetLastError();
}

cudaError_t xk_mass_project(const uint32_t *src, uint32_t *proj, const xk_desc &d, cudaStream_t s)
{
    const MassParams p = mass_params(d);
    const int64_t plane = (int64_t)p.W * p.H;
    xk_k_mass_project<<<(unsigned)((plane + 255) / 256), 256, 0, s>>>(src, proj, p);
    return cudaGetLastError();
}

cudaError_t xk_mass_colors(const uint32_t *src, int32_t *col, int64_t n, cudaStream_t s)
{
    xk_k_mass_colors<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, col, n);
    return cudaGetLastError();
}

cudaError_t xk_mass_render(const uint32_t *proj, int32_t *img, const xk_desc &d, int width,
                           int height, int zoom, int dx, int dy, cudaStream_t s)
{
    const MassParams p = mass_params(d);
    const int64_t n = (int64_t)width * height;
    xk_k_mass_render<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(proj, img, p, width, height, zoom,
                                                                 dx, dy);
    return cudaGetLastError();
}
