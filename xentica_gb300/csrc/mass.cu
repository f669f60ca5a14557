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
// Three kernels: xk_k_mass_tma (tensor copies into a shared-memory ring,
// widths that are a multiple of 4: the default), xk_k_mass_rows (the same
// widths, register queue and plain loads; XK_MASS_KERNEL=rows) and the
// generic xk_k_mass for any width.  Work split of the generic one: a
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
#include <cuda.h>          // CUtensorMap and its enums (types only; no driver link)
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "xk_internal.cuh"

#define XK_MASS_BY 8

struct MassParams {
    int32_t W, H, D;
    int32_t P;          // row pitch in cells: W rounded up to a multiple of 4
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
    const int64_t plane = (int64_t)p.P * p.H;
    const int64_t col = in ? (int64_t)y * p.P + x0 : 0;
    const bool has_ym = in && y > 0, has_yp = in && y + 1 < p.H;
    const bool has_xl = in && x0 > 0, has_xr = in && x0 + V < p.W;
    const uint32_t wall = p.wall;
    MassRow<V> prv, cur, nxt, ym, yp;
    xk_grid_dep_wait();       // launched as a dependent of the previous generation
    xk_mass_load<V>(src, (int64_t)(z0 - 1) * plane + col, in && z0 > 0, wall, prv);
    xk_mass_load<V>(src, (int64_t)z0 * plane + col, in && z0 < p.D, wall, cur);
    unsigned long long mass_sum = 0;
    for (int z = z0; z < z1; ++z) {
        const int64_t zb = (int64_t)z * plane;
        xk_mass_load<V>(src, zb + plane + col, in && z + 1 < p.D, wall, nxt);
        xk_mass_load<V>(src, zb + col - p.P, has_ym, wall, ym);
        xk_mass_load<V>(src, zb + col + p.P, has_yp, wall, yp);
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

// The generic form's fast-only counterpart (any width): used when the
// lattice's total mass is below 2^30, so no cell reaches 2^30 and no wall
// value is inside (see the TMA kernel).  One cell per thread marching its z
// run; q = m / 7 by the one-instruction division; off-board neighbours read
// as 0 and the cell's on-board neighbours are counted once:
//   m' = m - q * (#on-board neighbours) + sum_k q_k.
__global__ void __launch_bounds__(32 * XK_MASS_BY)
xk_k_mass_small(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst,
                unsigned long long *__restrict__ total, MassParams p, int zc)
{
    __shared__ unsigned long long warp_sums[XK_MASS_BY];
    const int lane = threadIdx.x;
    const int x = blockIdx.x * 32 + lane;
    const int y = blockIdx.y * XK_MASS_BY + threadIdx.y;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, p.D);
    const bool in = x < p.W && y < p.H;
    const uint32_t plane = (uint32_t)p.P * (uint32_t)p.H;
    uint32_t off = in ? (uint32_t)z0 * plane + (uint32_t)y * p.P + x : 0u;
    const bool has_xl = in && x > 0, has_xr = in && x + 1 < p.W;
    const bool has_ym = in && y > 0, has_yp = in && y + 1 < p.H;
    const uint32_t cxy = (uint32_t)has_xl + has_xr + has_ym + has_yp;
    auto ld = [&](uint32_t o, bool ok) { return ok ? __ldg(src + o) : 0u; };
    xk_grid_dep_wait();       // launched as a dependent of the previous generation
    uint32_t q_prv = xk_q_small(ld(off - plane, in && z0 > 0));
    uint32_t m_cur = ld(off, in);
    uint32_t q_cur = xk_q_small(m_cur);
    uint32_t m_nxt = ld(off + plane, in && z0 + 1 < p.D);
    uint32_t q_nxt = xk_q_small(m_nxt);
    // the rows above and below and the cell beyond the warp (lanes 0 and 31)
    // are loaded one plane ahead
    const bool edge_l = lane == 0 && has_xl, edge_r = lane == 31 && has_xr;
    uint32_t ym_pf = ld(off - p.P, has_ym), yp_pf = ld(off + p.P, has_yp);
    uint32_t hl_pf = ld(off - 1, edge_l), hr_pf = ld(off + 1, edge_r);
    uint32_t sum = 0;         // below 2^30: the whole lattice's total is
    for (int z = z0; z < z1; ++z) {
        const uint32_t m_nn = ld(off + 2 * plane, in && z + 2 < p.D);
        const uint32_t ym_m = ym_pf, yp_m = yp_pf, hl_m = hl_pf, hr_m = hr_pf;
        const bool more = z + 1 < z1;
        ym_pf = ld(off + plane - p.P, has_ym && more);
        yp_pf = ld(off + plane + p.P, has_yp && more);
        hl_pf = ld(off + plane - 1, edge_l && more);
        hr_pf = ld(off + plane + 1, edge_r && more);
        const uint32_t qy = xk_q_small(ym_m) + xk_q_small(yp_m);
        // x neighbours from the neighbouring lanes (same row); lanes 0 and 31
        // take the cell beyond the warp
        const uint32_t sl = __shfl_up_sync(0xFFFFFFFFu, q_cur, 1);
        const uint32_t sr = __shfl_down_sync(0xFFFFFFFFu, q_cur, 1);
        const uint32_t hl = lane == 0 ? xk_q_small(hl_m) : sl;
        const uint32_t hr = lane == 31 ? xk_q_small(hr_m) : sr;
        const uint32_t ql = has_xl ? hl : 0u, qr = has_xr ? hr : 0u;
        const uint32_t cz = (uint32_t)((z > 0) + (z + 1 < p.D));
        const uint32_t out = m_cur - q_cur * (cxy + cz) + ql + qr + qy + q_prv + q_nxt;
        if (in) {
            dst[off] = out;
            sum += out;
        }
        q_prv = q_cur;
        m_cur = m_nxt;
        q_cur = q_nxt;
        m_nxt = m_nn;
        q_nxt = xk_q_small(m_nn);
        off += plane;
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
    if (lane == 0) warp_sums[threadIdx.y] = sum;
    __syncthreads();
    if (threadIdx.y == 0 && lane == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < XK_MASS_BY; ++w) t += warp_sums[w];
        atomicAdd(total, t);
    }
}


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
    const uint32_t plane = (uint32_t)p.P * (uint32_t)p.H;
    const uint32_t wall = p.wall;
    uint32_t off = in ? (uint32_t)z0 * plane + (uint32_t)y * p.P + x0 : 0u;
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
    uint4 ym_pf = xk_mass_ld4z(src, off - p.P, has_ym);
    uint4 yp_pf = xk_mass_ld4z(src, off + p.P, has_yp);
    uint32_t hx_pf = hx_ok ? __ldg(src + (off + hx_d)) : 0u;
    unsigned long long mass_sum = 0;
    for (int z = z0; z < z1; ++z) {
        const uint4 nn_m = xk_mass_ld4z(src, off + 2 * plane, in && z + 2 < p.D);
        const uint4 ym_m = ym_pf, yp_m = yp_pf;
        const uint32_t hx_m = hx_pf;
        const bool more = z + 1 < z1;
        ym_pf = xk_mass_ld4z(src, off + plane - p.P, has_ym && more);
        yp_pf = xk_mass_ld4z(src, off + plane + p.P, has_yp && more);
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

// ---------------------------------------------------------------------------
// TMA form (W % 4 == 0, the default): a CTA owns a 128-cell by XK_MT_BY-row
// tile of a run of zc planes.  Each plane of the tile, with one halo row
// above and below and four halo columns either side, arrives in shared
// memory by one tensor copy (cp.async.bulk.tensor, issued by one thread into
// a ring of XK_MT_STAGES stages, completion on an mbarrier); coordinates off
// the lattice read as 0, which is exactly what an off-board neighbour
// contributes in the fast path.  Each cell's q = m / 7 is computed once,
// when its plane arrives, and written to a q tile (three of them in turn, so
// one barrier per plane separates writers and readers); a thread owns four
// consecutive cells of a row and keeps q of planes z - 1, z, z + 1 of its own
// column in registers, reads the q of the rows above and below from the q
// tile, the x neighbours from its lanes (shuffles) and, at the tile's edge,
// from the tile's halo columns.  The barrier also ORs a flag: some cell of
// the plane's tile or halo is at or above 2^30 (so the one-instruction q may
// be inexact, or a wall value is inside).  A plane whose tile saw such a
// cell in planes z - 1 .. z + 1 takes the exact per-neighbour form for the
// whole CTA, reading the neighbours from global memory.  When the uploaded
// lattice's total mass is below 2^30, no cell can ever reach 2^30 (mass is
// conserved and never negative) and the fast-only instantiation runs: plain
// barriers, no flag and no exact path, so fewer registers.
#define XK_MT_BY 8
#define XK_MT_STAGES 4
#define XK_MT_COLS 136                                  // 4 + 128 + 4
#define XK_MT_ROWS (XK_MT_BY + 2)
#define XK_MT_TILE_WORDS (XK_MT_COLS * XK_MT_ROWS)
#define XK_MT_STAGE_BYTES (XK_MT_TILE_WORDS * 4)
#define XK_MT_STAGE_STRIDE (((XK_MT_STAGE_BYTES + 127) / 128) * 128)
#define XK_MT_SMEM \
    (128 + XK_MT_STAGES * XK_MT_STAGE_STRIDE + 3 * XK_MT_STAGE_BYTES + 8 * XK_MT_STAGES + 8 * XK_MT_BY + 16)
#define XK_MT_SPIN (1u << 20)                           // try_wait rounds before giving up

// set when a CTA gave up waiting for a tensor copy (never expected)
__device__ unsigned int xk_mass_wait_failed;

__device__ __forceinline__ uint32_t xk_smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool xk_mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return done != 0;
}

// bounded wait for the copy of one stage; false after XK_MT_SPIN rounds
__device__ __forceinline__ bool xk_mbar_wait(uint32_t bar, uint32_t parity)
{
    for (uint32_t i = 0; i < XK_MT_SPIN; ++i)
        if (xk_mbar_try_wait(bar, parity)) return true;
    return false;
}

// one thread: plane z of the tile (x from x_lo, y from y_lo) into a stage
__device__ __forceinline__ void xk_mt_issue(const CUtensorMap *tm, uint32_t stage, uint32_t bar, int x_lo,
                                            int y_lo, int z)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :
                 : "r"(bar), "r"((uint32_t)XK_MT_STAGE_BYTES)
                 : "memory");
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
                 "[%0], [%1, {%2, %3, %4}], [%5];"
                 :
                 : "r"(stage), "l"(reinterpret_cast<uint64_t>(tm)), "r"(x_lo), "r"(y_lo), "r"(z),
                   "r"(bar)
                 : "memory");
}

// the barrier of a plane; the general kernel also ORs the flags of its threads
template <bool GENERAL>
__device__ __forceinline__ bool xk_mt_barrier(bool flag)
{
    if (GENERAL) return __syncthreads_or(flag);
    __syncthreads();
    return false;
}

// q of four cells, and whether one of them is at or above 2^30
__device__ __forceinline__ uint4 xk_mt_q4(const uint4 m, bool &big)
{
    big |= (m.x | m.y | m.z | m.w) >= XK_MASS_SMALL;
    return make_uint4(xk_q_small(m.x), xk_q_small(m.y), xk_q_small(m.z), xk_q_small(m.w));
}

// PROJ: also add the colours of the cells it writes, per column, into
// proj[y * W + x] (the z-projection RendererPlain renders; proj zeroed
// before the launch): a thread sums its four columns over its run of planes
// (two columns per register, 16 bits each: a colour is at most 255 and a run
// at most 256 planes, which the host checks) and adds each sum with one
// atomic, so the projection needs no second pass over the state.  Integer
// sums: the order of the additions does not matter.
//
// With PROJ, the launch can also finish the previous generation's frame:
// proj_prev holds that generation's column sums (its launch has completed
// when this one passes its dependency wait), and the CTAs of the first run
// of planes turn each of their columns into the frame_prev pixel, as
// RendererPlain renders it at zoom 1, and zero the column for the generation
// after this one (the sums alternate between two buffers).  So a frame every
// generation adds no launch between two generations.
template <int MINB, bool GENERAL, bool PROJ>
__global__ void __launch_bounds__(32 * XK_MT_BY, MINB)
xk_k_mass_tma(const __grid_constant__ CUtensorMap tm, const uint32_t *__restrict__ src,
              uint32_t *__restrict__ dst, unsigned long long *__restrict__ total, MassParams p, int zc,
              uint32_t *__restrict__ proj, uint32_t *__restrict__ proj_prev, uint8_t *__restrict__ frame_prev)
{
    extern __shared__ __align__(128) uint8_t xk_mt_raw[];
    // tensor copies land on 128-byte boundaries: round the window's start up
    uint8_t *base = xk_mt_raw + ((128u - (xk_smem_addr(xk_mt_raw) & 127u)) & 127u);
    uint8_t *stages = base;
    uint32_t *qt = reinterpret_cast<uint32_t *>(base + XK_MT_STAGES * XK_MT_STAGE_STRIDE);
    uint64_t *bars = reinterpret_cast<uint64_t *>(qt + 3 * XK_MT_TILE_WORDS);
    unsigned long long *warp_sums = reinterpret_cast<unsigned long long *>(bars + XK_MT_STAGES);
    volatile int *fail = reinterpret_cast<volatile int *>(warp_sums + XK_MT_BY);

    const int lane = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + lane;
    const int x_lo = blockIdx.x * 128 - 4, y_lo = blockIdx.y * XK_MT_BY - 1;
    const int x0 = blockIdx.x * 128 + lane * 4, y = blockIdx.y * XK_MT_BY + ty;
    const int z0 = blockIdx.z * zc, z1 = min(z0 + zc, p.D);
    const int nplanes = z1 - z0 + 2;                  // planes z0 - 1 .. z1
    // a thread's four cells start at x0; when W is not a multiple of 4 the
    // last quad of a row is partly in the row's padding (pitch P)
    const bool in = x0 < p.W && y < p.H;
    const uint32_t plane = (uint32_t)p.P * (uint32_t)p.H;
    const uint32_t bar0 = xk_smem_addr(bars), stage0 = xk_smem_addr(stages);

    if (tid == 0) {
        *fail = 0;
        for (int s = 0; s < XK_MT_STAGES; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8 * s) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // launched as a programmatic dependent of the previous generation: all of
    // the above overlaps its last CTAs; every thread waits here for that
    // grid to complete (and its writes to be visible) before any global
    // access -- the previous generation still reads the buffer this one
    // writes.  Without a programmatic launch this returns at once.
    xk_grid_dep_wait();
    if (tid == 0)
        for (int k = 0; k < XK_MT_STAGES && k < nplanes; ++k)
            xk_mt_issue(&tm, stage0 + k * XK_MT_STAGE_STRIDE, bar0 + 8 * k, x_lo, y_lo, z0 - 1 + k);
    if (PROJ && frame_prev && blockIdx.z == 0 && in) {
        // the previous generation's frame from its column sums (this
        // thread's four columns), and those sums zeroed for the next one
        const int64_t c0 = (int64_t)y * p.W + x0;
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (x0 + i < p.W) {
                const uint8_t v = (uint8_t)(int)__fdiv_rn((float)proj_prev[c0 + i], (float)p.D);
                uint8_t *px = frame_prev + 3 * (c0 + i);
                px[0] = v;
                px[1] = v;
                px[2] = v;
                proj_prev[c0 + i] = 0u;
            }
    }
    __syncthreads();

    // own cells of a stage (row ty + 1, columns 4 + 4 lane ..); the halo
    // column this lane converts when it is lane 0 or 31 (every lane reads one,
    // in bounds, so the code has no lane-dependent branch)
    const int own = (ty + 1) * XK_MT_COLS + 4 + 4 * lane;
    const int hcol = (ty + 1) * XK_MT_COLS + (lane == 0 ? 3 : 4 + 128);
    const bool hlane = lane == 0 || lane == 31;
    const bool hrow = ty == 0 || ty == XK_MT_BY - 1;
    const int hrow_at = (ty == 0 ? 0 : XK_MT_BY + 1) * XK_MT_COLS + 4 + 4 * lane;
    uint32_t *const qt0 = qt, *const qt1 = qt + XK_MT_TILE_WORDS, *const qt2 = qt + 2 * XK_MT_TILE_WORDS;
    int st_idx = 0;                                   // ring stage of the next plane taken
    uint32_t par = 0;                                 // its mbarrier phase parity
    // next plane of the ring: wait for it, return this thread's cells; the q
    // of its cells and of the halo cells it converts go to q tile qdst (null:
    // own cells only).  A wait that gives up marks `fail`, which every thread
    // reads after the next barrier.
    auto take = [&](uint32_t *qdst, uint4 &m, uint4 &q, bool &big) {
        if (!xk_mbar_wait(bar0 + 8 * st_idx, par)) *fail = 1;
        const uint32_t *st = reinterpret_cast<const uint32_t *>(stages + st_idx * XK_MT_STAGE_STRIDE);
        m = *reinterpret_cast<const uint4 *>(st + own);
        q = xk_mt_q4(m, big);
        if (qdst) {
            *reinterpret_cast<uint4 *>(qdst + own) = q;
            const uint32_t hm = st[hcol];
            if (hlane) {
                big |= hm >= XK_MASS_SMALL;
                qdst[hcol] = xk_q_small(hm);
            }
            if (hrow) {
                const uint4 rm = *reinterpret_cast<const uint4 *>(st + hrow_at);
                *reinterpret_cast<uint4 *>(qdst + hrow_at) = xk_mt_q4(rm, big);
            }
        }
    };
    // after the barrier that follows the last read of the plane just taken
    // (ring index k): its stage receives plane k + XK_MT_STAGES
    int k_taken = -1;
    auto advance = [&]() {
        ++k_taken;
        // warp 0 alone (a warp-uniform branch: the other warps skip the
        // issue code instead of running it predicated off), lane 0 issues
        if (ty == 0 && k_taken + XK_MT_STAGES < nplanes) {
            if (lane == 0)
                xk_mt_issue(&tm, stage0 + st_idx * XK_MT_STAGE_STRIDE, bar0 + 8 * st_idx, x_lo, y_lo,
                            z0 - 1 + k_taken + XK_MT_STAGES);
        }
        if (++st_idx == XK_MT_STAGES) {
            st_idx = 0;
            par ^= 1u;
        }
    };

    // three register sets (m, q) take the roles previous / current / next
    // plane in turn, and three q tiles the roles current / next: plane
    // z0 + j uses tile j % 3 and set (j + 1) % 3
    uint4 m0, q0, m1, q1, m2, q2;
    bool b_prev = false, b_cur = false;
    take(nullptr, m0, q0, b_prev);                    // plane z0 - 1: q of the own column
    b_prev = xk_mt_barrier<GENERAL>(b_prev);
    if (*fail) {
        if (tid == 0) atomicOr(&xk_mass_wait_failed, 1u);
        return;
    }
    advance();
    take(qt0, m1, q1, b_cur);                         // plane z0
    b_cur = xk_mt_barrier<GENERAL>(b_cur);
    if (*fail) {
        if (tid == 0) atomicOr(&xk_mass_wait_failed, 1u);
        return;
    }
    advance();

    // on-board neighbours in x and y of the four cells
    const int cy = (y > 0) + (y + 1 < p.H);
    // per cell: x neighbours on the lattice (0 for cells in the padding)
    const uint32_t c0 = cy + (x0 > 0) + (x0 + 1 < p.W), c1 = cy + 1 + (x0 + 2 < p.W);
    const uint32_t c2 = cy + 1 + (x0 + 3 < p.W), c3 = cy + 1 + (x0 + 4 < p.W);
    // cells at or beyond W (padding) are written as 0
    const bool v1 = x0 + 1 < p.W, v2 = x0 + 2 < p.W, v3 = x0 + 3 < p.W;
    // the fast-only form runs when the lattice's whole total is below 2^30,
    // so every partial sum of its cells fits 32 bits
    typename std::conditional<GENERAL, unsigned long long, uint32_t>::type mass_sum = 0;
    uint32_t cs01 = 0u, cs23 = 0u;                   // PROJ: colour sums, two columns per word
    uint32_t off = in ? (uint32_t)z0 * plane + (uint32_t)y * p.P + x0 : 0u;
    int z = z0;
    // one plane: take plane z + 1 into (mn, qn) and tile qnext, then compute
    // plane z from tile qcur, qp (z - 1), (mc, qc) (z) and qn (z + 1)
    auto step = [&](const uint4 &qp, const uint4 &mc, const uint4 &qc, uint4 &mn, uint4 &qn,
                    const uint32_t *qcur, uint32_t *qnext) -> bool {
        bool b_t = false;
        take(qnext, mn, qn, b_t);
        const bool b_next = xk_mt_barrier<GENERAL>(b_t);
        if (*fail) return false;
        advance();
        const uint32_t cz = (uint32_t)((z > 0) + (z + 1 < p.D));
        uint32_t out[4];
        if (!GENERAL || !(b_prev | b_cur | b_next)) {
            const uint4 up = *reinterpret_cast<const uint4 *>(qcur + own - XK_MT_COLS);
            const uint4 dn = *reinterpret_cast<const uint4 *>(qcur + own + XK_MT_COLS);
            const uint32_t hl = qcur[own - 1], hr = qcur[own + 4];
            const uint32_t sl = __shfl_up_sync(0xFFFFFFFFu, qc.w, 1);
            const uint32_t sr = __shfl_down_sync(0xFFFFFFFFu, qc.x, 1);
            const uint32_t xl = lane == 0 ? hl : sl, xr = lane == 31 ? hr : sr;
            out[0] = mc.x - qc.x * (c0 + cz) + xl + qc.y + up.x + dn.x + qp.x + qn.x;
            out[1] = mc.y - qc.y * (c1 + cz) + qc.x + qc.z + up.y + dn.y + qp.y + qn.y;
            out[2] = mc.z - qc.z * (c2 + cz) + qc.y + qc.w + up.z + dn.z + qp.z + qn.z;
            out[3] = mc.w - qc.w * (c3 + cz) + qc.z + xr + up.w + dn.w + qp.w + qn.w;
        } else if (GENERAL && in) {
            // the reference's arithmetic per neighbour, neighbours from global memory
            const uint32_t wall = p.wall;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t m = xk_get(mc, i);
                const uint32_t o = off + i;
                const bool on[6] = {x0 + i > 0, x0 + i + 1 < p.W, y > 0, y + 1 < p.H, z > 0, z + 1 < p.D};
                const uint32_t at[6] = {o - 1, o + 1, o - p.P, o + p.P, o - plane, o + plane};
                uint32_t cnt = 0, sq = 0;
#pragma unroll
                for (int n = 0; n < 6; ++n) {
                    const uint32_t nb = on[n] ? __ldg(src + at[n]) : 0u;
                    cnt += (uint32_t)(on[n] && nb != wall);
                    sq += on[n] ? nb / 7u : 0u;
                }
                out[i] = m - (m / 7u) * cnt + (m != wall ? sq : 0u);
            }
        }
        out[1] = v1 ? out[1] : 0u;
        out[2] = v2 ? out[2] : 0u;
        out[3] = v3 ? out[3] : 0u;
        if (in) {
            *reinterpret_cast<uint4 *>(dst + off) = make_uint4(out[0], out[1], out[2], out[3]);
            if (GENERAL)
                mass_sum += (unsigned long long)out[0] + out[1] + (unsigned long long)out[2] + out[3];
            else
                mass_sum += out[0] + out[1] + out[2] + out[3];
            if (PROJ) {
                cs01 += xk_mass_color(out[0]) + (xk_mass_color(out[1]) << 16);
                cs23 += xk_mass_color(out[2]) + (xk_mass_color(out[3]) << 16);
            }
        }
        b_prev = b_cur;
        b_cur = b_next;
        off += plane;
        return ++z < z1;
    };
    bool go = true;
    while (go) {
        go = step(q0, m1, q1, m2, q2, qt0, qt1) && step(q1, m2, q2, m0, q0, qt1, qt2) &&
             step(q2, m0, q0, m1, q1, qt2, qt0);
    }
    if (*fail) {
        if (tid == 0) atomicOr(&xk_mass_wait_failed, 1u);
        return;
    }
    if (PROJ && in) {
        uint32_t *pc = proj + (int64_t)y * p.W + x0;
        const uint32_t csum[4] = {cs01 & 0xFFFFu, cs01 >> 16, cs23 & 0xFFFFu, cs23 >> 16};
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (x0 + i < p.W) atomicAdd(pc + i, csum[i]);
    }
    for (int o = 16; o > 0; o >>= 1) mass_sum += __shfl_down_sync(0xFFFFFFFFu, mass_sum, o);
    if (lane == 0) warp_sums[ty] = mass_sum;
    __syncthreads();
    if (tid == 0) {
        unsigned long long s = 0;
        for (int w = 0; w < XK_MT_BY; ++w) s += warp_sums[w];
        atomicAdd(total, s);
    }
}

// column colour sums of a state (pitched rows; the sums are W * H, unpadded).
// A CTA owns 32 columns of one row y: its 8 warps take every 8th plane each
// (a warp reads 32 consecutive cells of a plane row, 128 bytes), four loads
// in flight per thread, and the 8 partial sums of a column meet in shared
// memory.  Integer sums, so the order of the additions does not matter.
// grid: x over row chunks of 32, y striding over the rows
#define XK_PROJ_ZS 8
// frame: null, or the W x H frame of RendererPlain over axes (0, 1) at zoom 1
// with no offset, written from the column sums as xk_k_mass_render does
__global__ void __launch_bounds__(32 * XK_PROJ_ZS)
xk_k_mass_project(const uint32_t *__restrict__ src, uint32_t *__restrict__ proj, MassParams p,
                  uint8_t *__restrict__ frame)
{
    __shared__ uint32_t part[XK_PROJ_ZS][33];
    const int x = blockIdx.x * 32 + threadIdx.x;
    const int64_t plane = (int64_t)p.P * p.H;
    for (int64_t y = blockIdx.y; y < p.H; y += gridDim.y) {
        uint32_t s = 0;
        if (x < p.W) {
            const uint32_t *col = src + y * p.P + x;
            int z = threadIdx.y;
            for (; z + 3 * XK_PROJ_ZS < p.D; z += 4 * XK_PROJ_ZS) {
                const uint32_t a = __ldg(col + (int64_t)z * plane);
                const uint32_t b = __ldg(col + (int64_t)(z + XK_PROJ_ZS) * plane);
                const uint32_t c = __ldg(col + (int64_t)(z + 2 * XK_PROJ_ZS) * plane);
                const uint32_t d = __ldg(col + (int64_t)(z + 3 * XK_PROJ_ZS) * plane);
                s += xk_mass_color(a) + xk_mass_color(b) + xk_mass_color(c) + xk_mass_color(d);
            }
            for (; z < p.D; z += XK_PROJ_ZS) s += xk_mass_color(__ldg(col + (int64_t)z * plane));
        }
        part[threadIdx.y][threadIdx.x] = s;
        __syncthreads();
        if (threadIdx.y == 0 && x < p.W) {
            uint32_t t = 0;
#pragma unroll
            for (int k = 0; k < XK_PROJ_ZS; ++k) t += part[k][threadIdx.x];
            proj[y * p.W + x] = t;
            if (frame) {
                const uint8_t v = (uint8_t)(int)__fdiv_rn((float)t, (float)p.D);
                uint8_t *px = frame + 3 * (y * p.W + x);
                px[0] = v;
                px[1] = v;
                px[2] = v;
            }
        }
        __syncthreads();
    }
}

// colours of every cell in the reference's order (3 ints per cell, no
// padding); grid: x over a row's cells, y striding over the H * D rows
__global__ void xk_k_mass_colors(const uint32_t *__restrict__ src, int32_t *__restrict__ col, MassParams p)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= p.W) return;
    const int64_t rows = (int64_t)p.H * p.D;
    for (int64_t row = blockIdx.y; row < rows; row += gridDim.y) {
        const int v = (int)xk_mass_color(src[row * p.P + x]);
        const int64_t i = row * p.W + x;
        col[3 * i] = v;
        col[3 * i + 1] = v;
        col[3 * i + 2] = v;
    }
}

// RendererPlain over axes (0, 1) from the column sums: the float sum of a
// column's colours equals its integer sum, divided by the depth
template <typename T>
__global__ void xk_k_mass_render(const uint32_t *__restrict__ proj, T *__restrict__ img,
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
    const T v = (T)(int)__fdiv_rn(s, (float)p.D);
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
    p.P = (int32_t)xk_mass_pitch(p.W);
    p.wall = d.wall;
    return p;
}

// planes per CTA: enough CTAs for about `target` per generation (2048 for
// the register-queue forms; 1024 for the TMA form, whose CTAs load two halo
// planes per run and fill a four-stage ring before their first plane)
static int mass_zchunk(const MassParams &p, int gx, int gy, int target = 2048)
{
    if (const char *e = getenv("XK_MASS_ZC")) {
        const int v = atoi(e);
        if (v > 0) return v;
    }
    const int64_t tiles = (int64_t)gx * gy;
    int64_t chunks = (target + tiles - 1) / tiles;
    if (chunks > p.D) chunks = p.D;
    if (chunks < 1) chunks = 1;
    return (int)((p.D + chunks - 1) / chunks);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
static PFN_cuTensorMapEncodeTiled_v12000 xk_tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
        else
            cudaGetLastError();
    });
    return fn;
}

// XK_MASS_KERNEL=rows in the environment selects the register-queue form
// for widths that are a multiple of 4 instead of the TMA form
static bool mass_tma_enabled()
{
    const char *v = getenv("XK_MASS_KERNEL");
    return !(v && !strcmp(v, "rows"));
}

// the TMA form's grid and planes per CTA for a lattice
// runs of at least 4 planes (a run loads 2 halo planes and sets up its ring
// once): with a frame every generation 64^3 46 -> 62 G, 96^3 154 -> 180 G,
// 128^3 237 -> 301 G cell-updates/s against the 1024-CTA target alone
static void mass_tma_shape(const MassParams &p, int *gx, int *gy, int *zc)
{
    *gx = (p.W + 127) / 128;
    *gy = (p.H + XK_MT_BY - 1) / XK_MT_BY;
    *zc = mass_zchunk(p, *gx, *gy, 1024);
    if (!getenv("XK_MASS_ZC")) *zc = std::max(*zc, std::min(4, p.D));
}

bool xk_mass_fuses_projection(const xk_desc &d)
{
    if (!mass_tma_enabled()) return false;
    int gx, gy, zc;
    mass_tma_shape(mass_params(d), &gx, &gy, &zc);
    return zc <= 256;   // the 16-bit column sums of a run of planes
}

// the zoom-1 frame of the whole lattice from column sums (RendererPlain over
// axes (0, 1), no smoothing): the float sum of a column's colours equals its
// integer sum, divided by the depth
__global__ void xk_k_mass_frame(const uint32_t *__restrict__ proj, uint8_t *__restrict__ frame, MassParams p)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)p.W * p.H) return;
    const uint8_t v = (uint8_t)(int)__fdiv_rn((float)proj[i], (float)p.D);
    frame[3 * i] = v;
    frame[3 * i + 1] = v;
    frame[3 * i + 2] = v;
}

cudaError_t xk_mass_frame(const uint32_t *proj, uint8_t *frame, const xk_desc &d, cudaStream_t s)
{
    const MassParams p = mass_params(d);
    const int64_t n = (int64_t)p.W * p.H;
    xk_k_mass_frame<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(proj, frame, p);
    return cudaGetLastError();
}

cudaError_t xk_mass_step(const uint32_t *src, uint32_t *dst, unsigned long long *total,
                         const xk_desc &d, bool small, cudaStream_t s, uint32_t *proj, uint32_t *proj_prev,
                         uint8_t *frame_prev)
{
    const MassParams p = mass_params(d);
    const bool vec = p.W % 4 == 0;
    if (mass_tma_enabled()) {
        PFN_cuTensorMapEncodeTiled_v12000 enc = xk_tensor_map_encoder();
        if (!enc) return cudaErrorNotSupported;
        CUtensorMap tm;
        const cuuint64_t dims[3] = {(cuuint64_t)p.W, (cuuint64_t)p.H, (cuuint64_t)p.D};
        // logical width W with the pitched row stride: columns at or beyond W
        // read as 0 like every other off-lattice coordinate
        const cuuint64_t strides[2] = {(cuuint64_t)p.P * 4, (cuuint64_t)p.P * p.H * 4};
        const cuuint32_t box[3] = {XK_MT_COLS, XK_MT_ROWS, 1};
        const cuuint32_t estr[3] = {1, 1, 1};
        if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<uint32_t *>(src), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
        int gx, gy, zc;
        mass_tma_shape(p, &gx, &gy, &zc);
        dim3 block(32, XK_MT_BY);
        dim3 grid(gx, gy, (p.D + zc - 1) / zc);
        // a lattice whose total mass is below 2^30 keeps every cell below 2^30
        // (mass is conserved and never negative), so no cell can need the exact
        // form and no wall value can be inside: the fast-only instantiation.
        // XK_MASS_GENERAL=1 in the environment takes the general one anyway.
        const char *g = getenv("XK_MASS_GENERAL");
        const bool fast = small && !(g && g[0] == '1');
        // programmatic dependent launch: this generation's CTAs may start
        // their set-up while the previous generation's last CTAs run
        if (proj) {
            if (zc > 256) return cudaErrorNotSupported;   // the 16-bit column sums would overflow
            if (fast)
                return xk_launch_pdl(xk_k_mass_tma<4, false, true>, grid, block, XK_MT_SMEM, s, tm, src, dst, total,
                                     p, zc, proj, proj_prev, frame_prev);
            return xk_launch_pdl(xk_k_mass_tma<3, true, true>, grid, block, XK_MT_SMEM, s, tm, src, dst, total, p,
                                 zc, proj, proj_prev, frame_prev);
        }
        uint32_t *const none = nullptr;
        uint8_t *const no_frame = nullptr;
        if (fast)
            return xk_launch_pdl(xk_k_mass_tma<4, false, false>, grid, block, XK_MT_SMEM, s, tm, src, dst, total, p,
                                 zc, none, none, no_frame);
        return xk_launch_pdl(xk_k_mass_tma<4, true, false>, grid, block, XK_MT_SMEM, s, tm, src, dst, total, p, zc,
                             none, none, no_frame);
    }
    if (proj) return cudaErrorNotSupported;   // the other forms write no projection
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
    else if (small && !(getenv("XK_MASS_GENERAL") && getenv("XK_MASS_GENERAL")[0] == '1'))
        return xk_launch_pdl(xk_k_mass_small, grid, block, 0, s, src, dst, total, p, zc);
    else
        return xk_launch_pdl(xk_k_mass<1>, grid, block, 0, s, src, dst, total, p, zc);
    return cudaGetLastError();
}

__global__ void xk_k_mass_sum(const uint32_t *__restrict__ src, int64_t n, unsigned long long *__restrict__ out)
{
    unsigned long long s = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += src[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

cudaError_t xk_mass_sum(const uint32_t *src, int64_t n, unsigned long long *out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    xk_k_mass_sum<<<(unsigned)blocks, 256, 0, s>>>(src, n, out);
    return cudaGetLastError();
}

// copy of the TMA kernel's give-up flag, cleared; true when a CTA gave up
// waiting for a tensor copy since the last call
bool xk_mass_take_wait_failure()
{
    unsigned int v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, xk_mass_wait_failed, sizeof(v)) != cudaSuccess) return false;
    if (v) cudaMemcpyToSymbol(xk_mass_wait_failed, &z, sizeof(z));
    return v != 0;
}

cudaError_t xk_mass_project(const uint32_t *src, uint32_t *proj, const xk_desc &d, cudaStream_t s,
                            uint8_t *frame)
{
    const MassParams p = mass_params(d);
    const unsigned gy = (unsigned)(p.H < 65535 ? p.H : 65535);
    xk_k_mass_project<<<dim3((unsigned)((p.W + 31) / 32), gy), dim3(32, XK_PROJ_ZS), 0, s>>>(src, proj,
                                                                                            p, frame);
    return cudaGetLastError();
}

cudaError_t xk_mass_colors(const uint32_t *src, int32_t *col, const xk_desc &d, cudaStream_t s)
{
    const MassParams p = mass_params(d);
    const int64_t rows = (int64_t)p.H * p.D;
    const unsigned gy = (unsigned)(rows < 65535 ? rows : 65535);
    xk_k_mass_colors<<<dim3((unsigned)((p.W + 255) / 256), gy), 256, 0, s>>>(src, col, p);
    return cudaGetLastError();
}

cudaError_t xk_mass_render(const uint32_t *proj, int32_t *img, const xk_desc &d, int width,
                           int height, int zoom, int dx, int dy, cudaStream_t s)
{
    const MassParams p = mass_params(d);
    const int64_t n = (int64_t)width * height;
    xk_k_mass_render<int32_t><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(proj, img, p, width, height,
                                                                          zoom, dx, dy);
    return cudaGetLastError();
}

cudaError_t xk_mass_render_u8(const uint32_t *proj, uint8_t *img, const xk_desc &d, int width,
                              int height, int zoom, int dx, int dy, cudaStream_t s)
{
    const MassParams p = mass_params(d);
    const int64_t n = (int64_t)width * height;
    xk_k_mass_render<uint8_t><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(proj, img, p, width, height,
                                                                          zoom, dx, dy);
    return cudaGetLastError();
}
