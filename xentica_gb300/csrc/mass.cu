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
// Two kernels: xk_k_mass_rows for widths that are a multiple of 4 (below)
// and the generic xk_k_mass for any width.  Work split of the generic one: a
// CTA owns a 32-wide, 8-row tile of a run of zc planes; a thread owns one
// cell of a row and walks its z run with a three-plane register queue.
// x neighbours come from the neighbouring lanes (shuffles; lanes 0 and 31
// load the one cell beyond the warp), y neighbours are 128-bit loads of the
// rows above and below (the neighbouring warps' own rows, so mostly L1
// hits), z neighbours are the queue.  No shared-memory tile and no barrier
// inside the loop.  Each cell carries (m, m / 7); an off-board cell reads as
// (WALL, 0), which makes the sent and incoming sums need no bounds test:
//   m' = m - (m / 7) * #{k : m_k != WALL} + (m != WALL) * sum_k q_k
// (q_k = m_k / 7 < WALL, so the reference's "incoming != WALL" test always
// holds).  Each CTA adds its cells' new mass to the generation's total with
// one 64-bit atomic.  Colours and the RendererPlain projection are derived
// from the state when they are read, not every generation.
#include <cstdlib>

#include "xk_internal.cuh"

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

template <int V>
struct MassRow {
    uint32_t m[V];
    uint32_t q[V];
};

// V cells from element index idx of src when ok, else V off-board cells
template <int V>
__device__ __forceinline__ void xk_mass_load(const uint32_t *__restrict__ src, int64_t idx, bool ok,
                                             uint32_t wall, MassRow<V> &r)
{
    if (V == 4) {
        uint4 u = make_uint4(wall, wall, wall, wall);
        if (ok) u = __ldg(reinterpret_cast<const uint4 *>(src + idx));
        r.m[0] = u.x;
        r.m[1] = u.y;
        r.m[2] = u.z;
        r.m[3] = u.w;
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) r.m[i] = ok ? __ldg(src + idx + i) : wall;
    }
#pragma unroll
    for (int i = 0; i < V; ++i) r.q[i] = ok ? r.m[i] / 7u : 0u;
}

template <int V>
__global__ void __launch_bounds__(32 * XK_MASS_BY)
xk_k_mass(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst,
          unsigned long long *__restrict__ total, MassParams p, int zc)
{
    __shared__ unsigned long long warp_sums[XK_MASS_BY];
    const int lane = threadIdx.x;
    const int x0 = (blockIdx.x * 32 + lane) * V;
    const int y = blockIdx.y * XK_MASS_BY + threadIdx.y;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, p.D);
    const bool in = x0 < p.W && y < p.H;
    const int64_t plane = (int64_t)p.W * p.H;
    const int64_t col = in ? (int64_t)y * p.W + x0 : 0;
    const bool has_ym = in && y > 0, has_yp = in && y + 1 < p.H;
    const bool has_xl = in && x0 > 0, has_xr = in && x0 + V < p.W;
    const uint32_t wall = p.wall;
    MassRow<V> prv, cur, nxt, ym, yp;
    xk_mass_load<V>(src, (int64_t)(z0 - 1) * plane + col, in && z0 > 0, wall, prv);
    xk_mass_load<V>(src, (int64_t)z0 * plane + col, in && z0 < p.D, wall, cur);
    unsigned long long mass_sum = 0;
    for (int z = z0; z < z1; ++z) {
        const int64_t zb = (int64_t)z * plane;
        xk_mass_load<V>(src, zb + plane + col, in && z + 1 < p.D, wall, nxt);
        xk_mass_load<V>(src, zb + col - p.W, has_ym, wall, ym);
        xk_mass_load<V>(src, zb + col + p.W, has_yp, wall, yp);
        uint32_t lm = __shfl_up_sync(0xFFFFFFFFu, cur.m[V - 1], 1);
        uint32_t lq = __shfl_up_sync(0xFFFFFFFFu, cur.q[V - 1], 1);
        uint32_t rm = __shfl_down_sync(0xFFFFFFFFu, cur.m[0], 1);
        uint32_t rq = __shfl_down_sync(0xFFFFFFFFu, cur.q[0], 1);
        if (lane == 0) {
            lm = has_xl ? __ldg(src + zb + col - 1) : wall;
            lq = has_xl ? lm / 7u : 0u;
        }
        if (lane == 31) {
            rm = has_xr ? __ldg(src + zb + col + V) : wall;
            rq = has_xr ? rm / 7u : 0u;
        }
        uint32_t out[V];
#pragma unroll
        for (int i = 0; i < V; ++i) {
            const uint32_t m = cur.m[i];
            // von Neumann: +x, -x, +y, -y, +z, -z (order does not change the sums)
            const uint32_t mx_p = i + 1 < V ? cur.m[i + 1 < V ? i + 1 : 0] : rm;
            const uint32_t qx_p = i + 1 < V ? cur.q[i + 1 < V ? i + 1 : 0] : rq;
            const uint32_t mx_m = i > 0 ? cur.m[i > 0 ? i - 1 : 0] : lm;
            const uint32_t qx_m = i > 0 ? cur.q[i > 0 ? i - 1 : 0] : lq;
            const uint32_t cnt = (uint32_t)(mx_p != wall) + (uint32_t)(mx_m != wall) +
                                 (uint32_t)(yp.m[i] != wall) + (uint32_t)(ym.m[i] != wall) +
                                 (uint32_t)(nxt.m[i] != wall) + (uint32_t)(prv.m[i] != wall);
            const uint32_t sq = qx_p + qx_m + yp.q[i] + ym.q[i] + nxt.q[i] + prv.q[i];
            out[i] = m - cur.q[i] * cnt + (m != wall ? sq : 0u);
            mass_sum += out[i];
        }
        if (in) {
            if (V == 4)
                *reinterpret_cast<uint4 *>(dst + zb + col) = make_uint4(out[0], out[V > 1 ? 1 : 0],
                                                                        out[V > 2 ? 2 : 0],
                                                                        out[V > 3 ? 3 : 0]);
            else
#pragma unroll
                for (int i = 0; i < V; ++i) dst[zb + col + i] = out[i];
        }
        prv = cur;
        cur = nxt;
    }
    if (!in) mass_sum = 0;
    for (int off = 16; off > 0; off >>= 1) mass_sum += __shfl_down_sync(0xFFFFFFFFu, mass_sum, off);
    if (lane == 0) warp_sums[threadIdx.y] = mass_sum;
    __syncthreads();
    if (threadIdx.y == 0 && lane == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < XK_MASS_BY; ++w) s += warp_sums[w];
        atomicAdd(total, s);
    }
}

// Helpers of the W % 4 == 0 kernel.  Division by the invariant 7 as a
// multiply-high (Granlund and Montgomery, "Division by invariant integers
// using multiplication", 1994): c = 0x24924925 = (2^32 + 3) / 7, so
// umulhi(m, c) = floor(m / 7 + 3m / (7 * 2^32)), which is floor(m / 7) while
// the error term stays below 1/7 (the smallest gap to the next integer), i.e.
// for all m < 2^32 / 3 = 1 431 655 765.  Cells below 2^30 use it; larger
// cells take the compiler's exact division.
#define XK_MASS_SMALL 0x40000000u

__device__ __forceinline__ uint4 xk_mass_ld4(const uint32_t *__restrict__ src, uint32_t off, bool ok,
                                              uint32_t wall)
{
    uint4 u = make_uint4(wall, wall, wall, wall);
    if (ok) u = __ldg(reinterpret_cast<const uint4 *>(src + off));
    return u;
}

__device__ __forceinline__ uint32_t xk_div7(uint32_t m, bool small)
{
    return small ? __umulhi(m, 0x24924925u) : m / 7u;
}

// q of four loaded cells (0 when off-board), exact; `big` marks a loaded
// cell at or above 2^30
__device__ __forceinline__ uint4 xk_mass_q4(const uint4 m, bool ok, bool &big)
{
    const bool b = ok && ((m.x | m.y | m.z | m.w) >= XK_MASS_SMALL);
    big |= b;
    uint4 q;
    if (b)
        q = make_uint4(m.x / 7u, m.y / 7u, m.z / 7u, m.w / 7u);
    else
        q = make_uint4(__umulhi(m.x, 0x24924925u), __umulhi(m.y, 0x24924925u),
                       __umulhi(m.z, 0x24924925u), __umulhi(m.w, 0x24924925u));
    return ok ? q : make_uint4(0u, 0u, 0u, 0u);
}

__device__ __forceinline__ uint32_t xk_get(const uint4 &u, int i)
{
    return i == 0 ? u.x : i == 1 ? u.y : i == 2 ? u.z : u.w;
}

// Form for W % 4 == 0 (the usual case): a thread owns four consecutive
// cells of one row (128-bit loads and stores) and walks its run of zc planes
// with a register queue of planes z - 1 .. z + 2; the rows above and below and
// the x halo cell of lanes 0 and 31 are loaded one plane ahead.  Each
// loaded cell gets its q = m / 7 by the one-instruction division when it is
// below 2^30.  No shared tile and no barrier: x neighbours are lane shuffles,
// y neighbours the thread's own loads of the rows above and below (mostly L1
// hits: they are the neighbouring warps' rows).  A warp takes the fast path
// when none of the cells its lanes read is at or above 2^30 (__any_sync), so
// no cell is the wall value and every on-board neighbour counts in the sent
// sum:  m' = m - q * (#on-board neighbours) + sum_k q_k;  otherwise the exact
// per-neighbour form of the generic kernel.
__device__ __forceinline__ uint4 xk_mass_ld4z(const uint32_t *__restrict__ src, uint32_t off, bool ok)
{
    uint4 u = make_uint4(0u, 0u, 0u, 0u);
    if (ok) u = __ldg(reinterpret_cast<const uint4 *>(src + off));
    return u;
}

__device__ __forceinline__ uint32_t xk_or4(const uint4 &u) { return u.x | u.y | u.z | u.w; }

__device__ __forceinline__ uint32_t xk_q_small(uint32_t m) { return __umulhi(m, 0x24924925u); }

template <int MINB>
__global__ void __launch_bounds__(32 * XK_MASS_BY, MINB)
xk_k_mass_rows(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst,
               unsigned long long *__restrict__ total, MassParams p, int zc)
{
    __shared__ unsigned long long warp_sums[XK_MASS_BY];
    const int lane = threadIdx.x, ty = threadIdx.y;
    const int x0 = (blockIdx.x * 32 + lane) * 4;
    const int y = blockIdx.y * XK_MASS_BY + ty;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, p.D);
    const bool in = x0 < p.W && y < p.H;
    const uint32_t plane = (uint32_t)p.W * (uint32_t)p.H;
    const uint32_t wall = p.wall;
    uint32_t off = in ? (uint32_t)z0 * plane + (uint32_t)y * p.W + x0 : 0u;
    const bool hx_ok = in && ((lane == 0 && x0 > 0) || (lane == 31 && x0 + 4 < p.W));
    const int hx_d = lane == 0 ? -1 : 4;
    const bool has_ym = in && y > 0, has_yp = in && y + 1 < p.H;
    const bool has_xl = x0 > 0, has_xr = x0 + 4 < p.W;   // outside the thread's four cells
    // on-board x/y neighbours of cells 0 and 3 (cells 1 and 2 have both x neighbours)
    const int cy = (y > 0) + (y + 1 < p.H);
    const int c0 = cy + 1 + (int)has_xl, c3 = cy + 1 + (int)has_xr;

    // Off-board cells load as 0 (their q is 0, nothing comes in from them);
    // the exact path counts on-board neighbours from the flags above.
    uint4 prv_m = xk_mass_ld4z(src, off - plane, in && z0 > 0);
    uint4 cur_m = xk_mass_ld4z(src, off, in);
    uint4 nxt_m = xk_mass_ld4z(src, off + plane, in && z0 + 1 < p.D);
    uint4 ym_pf = xk_mass_ld4z(src, off - p.W, has_ym);
    uint4 yp_pf = xk_mass_ld4z(src, off + p.W, has_yp);
    uint32_t hx_pf = hx_ok ? __ldg(src + (off + hx_d)) : 0u;
    unsigned long long mass_sum = 0;
    for (int z = z0; z < z1; ++z) {
        const uint4 nn_m = xk_mass_ld4z(src, off + 2 * plane, in && z + 2 < p.D);
        const uint4 ym_m = ym_pf, yp_m = yp_pf;
        const uint32_t hx_m = hx_pf;
        const bool more = z + 1 < z1;
        ym_pf = xk_mass_ld4z(src, off + plane - p.W, has_ym && more);
        yp_pf = xk_mass_ld4z(src, off + plane + p.W, has_yp && more);
        hx_pf = hx_ok && more ? __ldg(src + (off + plane + hx_d)) : 0u;
        const uint32_t ors = xk_or4(prv_m) | xk_or4(cur_m) | xk_or4(nxt_m) | xk_or4(ym_m) |
                             xk_or4(yp_m) | hx_m;
        uint32_t out[4];
        if (!__any_sync(0xFFFFFFFFu, ors >= XK_MASS_SMALL)) {
            // every cell the warp reads is below 2^30: no wall value, exact
            // one-instruction q, every on-board neighbour counts
            const uint32_t q0 = xk_q_small(cur_m.x), q1 = xk_q_small(cur_m.y);
            const uint32_t q2 = xk_q_small(cur_m.z), q3 = xk_q_small(cur_m.w);
            uint32_t xl = xk_q_small(__shfl_up_sync(0xFFFFFFFFu, cur_m.w, 1));
            uint32_t xr = xk_q_small(__shfl_down_sync(0xFFFFFFFFu, cur_m.x, 1));
            const uint32_t hq = xk_q_small(hx_m);
            if (lane == 0) xl = hq;
            if (lane == 31) xr = hq;
            if (!has_xl && lane == 0) xl = 0u;
            if (!has_xr && lane == 31) xr = 0u;
            const int cz = (z > 0) + (z + 1 < p.D);
            const uint32_t vz0 = xk_q_small(prv_m.x) + xk_q_small(nxt_m.x) + xk_q_small(ym_m.x) + xk_q_small(yp_m.x);
            const uint32_t vz1 = xk_q_small(prv_m.y) + xk_q_small(nxt_m.y) + xk_q_small(ym_m.y) + xk_q_small(yp_m.y);
            const uint32_t vz2 = xk_q_small(prv_m.z) + xk_q_small(nxt_m.z) + xk_q_small(ym_m.z) + xk_q_small(yp_m.z);
            const uint32_t vz3 = xk_q_small(prv_m.w) + xk_q_small(nxt_m.w) + xk_q_small(ym_m.w) + xk_q_small(yp_m.w);
            out[0] = cur_m.x - q0 * (uint32_t)(c0 + cz) + xl + q1 + vz0;
            out[1] = cur_m.y - q1 * (uint32_t)(cy + 2 + cz) + q0 + q2 + vz1;
            out[2] = cur_m.z - q2 * (uint32_t)(cy + 2 + cz) + q1 + q3 + vz2;
            out[3] = cur_m.w - q3 * (uint32_t)(c3 + cz) + q2 + xr + vz3;
            if (in)   // each value < 2^31 here, so pairs sum without overflow
                mass_sum += (unsigned long long)(out[0] + out[1]) + (unsigned long long)(out[2] + out[3]);
        } else {
            // the reference's arithmetic per neighbour: sent to each on-board
            // neighbour whose mass is not the wall, its share taken in while
            // the cell itself is not the wall
            const uint32_t xl_m = __shfl_up_sync(0xFFFFFFFFu, cur_m.w, 1);
            const uint32_t xr_m = __shfl_down_sync(0xFFFFFFFFu, cur_m.x, 1);
            const uint32_t left = lane == 0 ? hx_m : xl_m, right = lane == 31 ? hx_m : xr_m;
            const bool zm = z > 0, zp = z + 1 < p.D, ym_on = y > 0, yp_on = y + 1 < p.H;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t m = xk_get(cur_m, i);
                const uint32_t ml = i == 0 ? left : xk_get(cur_m, i > 0 ? i - 1 : 0);
                const uint32_t mr = i == 3 ? right : xk_get(cur_m, i < 3 ? i + 1 : 3);
                const bool lo = i > 0 || has_xl, ro = i < 3 || has_xr;
                const uint32_t nb[6] = {ml, mr, xk_get(ym_m, i), xk_get(yp_m, i), xk_get(prv_m, i),
                                        xk_get(nxt_m, i)};
                const bool on[6] = {lo, ro, ym_on, yp_on, zm, zp};
                uint32_t cnt = 0, sq = 0;
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    cnt += (uint32_t)(on[k] && nb[k] != wall);
                    sq += on[k] ? nb[k] / 7u : 0u;
                }
                out[i] = m - (m / 7u) * cnt + (m != wall ? sq : 0u);
            }
            if (in)
                mass_sum += (unsigned long long)out[0] + out[1] + (unsigned long long)out[2] + out[3];
        }
        if (in) *reinterpret_cast<uint4 *>(dst + off) = make_uint4(out[0], out[1], out[2], out[3]);
        prv_m = cur_m;
        cur_m = nxt_m;
        nxt_m = nn_m;
        off += plane;
    }
    for (int o = 16; o > 0; o >>= 1) mass_sum += __shfl_down_sync(0xFFFFFFFFu, mass_sum, o);
    if (lane == 0) warp_sums[ty] = mass_sum;
    __syncthreads();
    if (ty == 0 && lane == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < XK_MASS_BY; ++w) s += warp_sums[w];
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

// planes per CTA: enough CTAs for about 2048 per generation
static int mass_zchunk(const MassParams &p, int gx, int gy)
{
    if (const char *e = getenv("XK_MASS_ZC")) {
        const int v = atoi(e);
        if (v > 0) return v;
    }
    const int64_t tiles = (int64_t)gx * gy;
    int64_t chunks = (2048 + tiles - 1) / tiles;
    if (chunks > p.D) chunks = p.D;
    if (chunks < 1) chunks = 1;
    return (int)((p.D + chunks - 1) / chunks);
}

cudaError_t xk_mass_step(const uint32_t *src, uint32_t *dst, unsigned long long *total,
                         const xk_desc &d, cudaStream_t s)
{
    const MassParams p = mass_params(d);
    const bool vec = p.W % 4 == 0;
    const int cells_x = 32 * (vec ? 4 : 1);
    const int gx = (p.W + cells_x - 1) / cells_x, gy = (p.H + XK_MASS_BY - 1) / XK_MASS_BY;
    const int zc = mass_zchunk(p, gx, gy);
    dim3 block(32, XK_MASS_BY);
    dim3 grid(gx, gy, (p.D + zc - 1) / zc);
    // four CTAs per SM (64 registers) measured faster than three; XK_MASS_MINB=1 lifts the cap
    static const int minb = getenv("XK_MASS_MINB") ? atoi(getenv("XK_MASS_MINB")) : 4;
    if (vec && minb >= 4)
        xk_k_mass_rows<4><<<grid, block, 0, s>>>(src, dst, total, p, zc);
    else if (vec)
        xk_k_mass_rows<1><<<grid, block, 0, s>>>(src, dst, total, p, zc);
    else
        xk_k_mass<1><<<grid, block, 0, s>>>(src, dst, total, p, zc);
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
