// Temporally blocked Life-like generations for 2-D lattices too large for one
// CTA: T generations per launch (T <= XK_TB_MAXT), each CTA on a tile of its
// own in shared memory.
//
// Tile: 32 words (1024 cells) by XK_TB_ROWS rows, read from the lattice with
// a halo -- one word left and right, T rows above and below -- so the
// interior (words 1..30, rows T..T + TH - 1 with TH = XK_TB_ROWS - 2T) is
// exact after T generations: a cell's value after k generations depends only
// on cells within k of it, and the halo is T >= k cells deep in rows and 32
// cells deep in columns.  Tile cell b of word w is the lattice cell
// x0 - 32 + 32 w + b of row y0 - T + r; on a torus that coordinate is taken
// modulo W and H (the tile is a window onto the periodic lattice, so a word
// may straddle the wrap), with a static border cells outside the lattice
// hold the border state and are reset to it after every generation.
//
// Each of the 8 warps owns a band of 8 tile rows, lane w holding word w; a
// band is updated walking down its rows with the column sums (s, c) =
// FA(L, C, R) of the rows above, at and below carried in registers (each
// row's sums computed once per generation), the left and right neighbour
// bits from the adjacent lanes by shuffles.  Generations alternate between
// two shared buffers, one barrier each.  Lanes 0 and 31 and the rows outside
// the interior compute on incomplete neighbourhoods; their values are never
// stored.
//
// Requires W >= 64 (a 32-cell window wraps at most once).
#include <string.h>

#include "life_word.cuh"

#define XK_TB_ROWS 64
#define XK_TB_MAXT 8
#define XK_TB_WARPS 8
#define XK_TB_BAND (XK_TB_ROWS / XK_TB_WARPS)

struct TbParams {
    LifeGeo g;
    int32_t T, TH;             // generations, interior rows
};

// 32 cells of row `row` starting at cell X (0 <= X < W), wrapping past W to
// the row's start (torus); bits past the row's end are 0 when `wrap` is 0
__device__ __forceinline__ uint32_t xk_tb_cells32(const uint32_t *__restrict__ row, int X, const LifeGeo &g,
                                                  bool wrap)
{
    const int jw = X >> 5, sh = X & 31;
    const uint32_t a = __ldg(row + jw);
    const uint32_t b = jw + 1 < g.wpr ? __ldg(row + jw + 1) : 0u;   // padding bits are 0
    uint32_t v = sh ? __funnelshift_r(a, b, sh) : a;
    const int avail = g.W - X;
    if (avail < 32) {
        const uint32_t keep = (1u << avail) - 1u;
        v &= keep;
        if (wrap) v |= __ldg(row) << avail;   // W >= 64: word 0 holds 32 cells
    }
    return v;
}

template <int RF>
__global__ void __launch_bounds__(32 * XK_TB_WARPS)
xk_k_life_tb(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, TbParams p, LifeTable9 t9)
{
    const auto &t = RuleForm<RF>::make(t9);
    __shared__ uint32_t tile[2][XK_TB_ROWS][32];
    const LifeGeo &g = p.g;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 30 * 32;                   // first interior cell
    const int y0 = blockIdx.y * p.TH;                      // first interior row
    const int X = x0 - 32 + 32 * lane;                     // this lane's first cell
    // bits of this lane's word outside the lattice (static border only)
    uint32_t outside = 0;
    if (!g.torus) {
        if (X < 0 || X >= g.W) outside = 0xFFFFFFFFu;
        else if (g.W - X < 32) outside = ~((1u << (g.W - X)) - 1u);
    }
    xk_grid_dep_wait();       // launched as a dependent of the previous launch
    const int r0 = warp * XK_TB_BAND;
#pragma unroll
    for (int i = 0; i < XK_TB_BAND; ++i) {
        const int r = r0 + i;
        int vy = y0 - p.T + r;
        uint32_t w;
        if (g.torus) {
            vy %= g.H;
            if (vy < 0) vy += g.H;
            int xm = X % g.W;
            if (xm < 0) xm += g.W;
            w = xk_tb_cells32(src + (int64_t)vy * g.wpr, xm, g, true);
        } else if (vy < 0 || vy >= g.H || outside == 0xFFFFFFFFu) {
            w = g.bfill;
        } else {
            w = xk_tb_cells32(src + (int64_t)vy * g.wpr, X, g, false);
            w = (w & ~outside) | (g.bfill & outside);
        }
        tile[0][r][lane] = w;
    }
    __syncthreads();
    for (int gen = 0; gen < p.T; ++gen) {
        const int cur = gen & 1;
        // column sums of the row above the band and of its first row
        uint32_t su, cu, sm, cm, Cm;
        {
            const uint32_t c = r0 > 0 ? tile[cur][r0 - 1][lane] : 0u;
            const uint32_t l = __shfl_up_sync(0xFFFFFFFFu, c, 1), rr = __shfl_down_sync(0xFFFFFFFFu, c, 1);
            const uint32_t L = (c << 1) | (lane > 0 ? l >> 31 : 0u);
            const uint32_t R = (c >> 1) | (lane < 31 ? rr << 31 : 0u);
            su = xk_lop3_xor3(L, c, R);
            cu = xk_maj(L, c, R);
        }
        {
            const uint32_t c = tile[cur][r0][lane];
            const uint32_t l = __shfl_up_sync(0xFFFFFFFFu, c, 1), rr = __shfl_down_sync(0xFFFFFFFFu, c, 1);
            const uint32_t L = (c << 1) | (lane > 0 ? l >> 31 : 0u);
            const uint32_t R = (c >> 1) | (lane < 31 ? rr << 31 : 0u);
            sm = xk_lop3_xor3(L, c, R);
            cm = xk_maj(L, c, R);
            Cm = c;
        }
#pragma unroll
        for (int i = 0; i < XK_TB_BAND; ++i) {
            const int r = r0 + i;
            const uint32_t c = r + 1 < XK_TB_ROWS ? tile[cur][r + 1][lane] : 0u;
            const uint32_t l = __shfl_up_sync(0xFFFFFFFFu, c, 1), rr = __shfl_down_sync(0xFFFFFFFFu, c, 1);
            const uint32_t L = (c << 1) | (lane > 0 ? l >> 31 : 0u);
            const uint32_t R = (c >> 1) | (lane < 31 ? rr << 31 : 0u);
            const uint32_t sd = xk_lop3_xor3(L, c, R), cd = xk_maj(L, c, R);
            uint32_t out = xk_life_word9(su, cu, sm, cm, sd, cd, Cm, t);
            if (!g.torus) {
                const int vy = y0 - p.T + r;
                out = (vy < 0 || vy >= g.H) ? g.bfill : (out & ~outside) | (g.bfill & outside);
            }
            tile[cur ^ 1][r][lane] = out;
            su = sm;
            cu = cm;
            sm = sd;
            cm = cd;
            Cm = c;
        }
        __syncthreads();
    }
    // the interior: lanes 1..30, rows T .. T + TH - 1, where they are cells
    if (lane >= 1 && lane <= 30) {
        const int j = (x0 >> 5) + lane - 1;
        if (j < g.wpr) {
#pragma unroll
            for (int i = 0; i < XK_TB_BAND; ++i) {
                const int r = r0 + i;
                const int y = y0 - p.T + r;
                if (r >= p.T && r < p.T + p.TH && y < g.H) {
                    uint32_t w = tile[p.T & 1][r][lane];
                    if (j == g.wpr - 1) w &= g.lastmask;
                    dst[(int64_t)y * g.wpr + j] = w;
                }
            }
        }
    }
}

int xk_life_tb_supported(const LifeGeo &g) { return g.W >= 64; }

cudaError_t xk_life_step_tb(const uint32_t *src, uint32_t *dst, const LifeGeo &g, const LifeTable9 &t,
                            int T, cudaStream_t s)
{
    if (T < 1 || T > XK_TB_MAXT || g.W < 64) return cudaErrorInvalidValue;
    TbParams p;
    p.g = g;
    p.T = T;
    p.TH = XK_TB_ROWS - 2 * T;
    const dim3 grid((unsigned)((g.W + 30 * 32 - 1) / (30 * 32)), (unsigned)((g.H + p.TH - 1) / p.TH));
    if (grid.y > 65535u) return cudaErrorInvalidValue;
    // B3/S23 runs the instantiation with the rule compiled in
    const LifeTable9 conway = xk_life_table9(8u, 12u);
    if (memcmp(&t, &conway, sizeof(t)) == 0)
        return xk_launch_pdl(xk_k_life_tb<XK_RULE_CONWAY>, grid, dim3(32 * XK_TB_WARPS), 0, s, src, dst, p, t);
    return xk_launch_pdl(xk_k_life_tb<XK_RULE_TABLE>, grid, dim3(32 * XK_TB_WARPS), 0, s, src, dst, p, t);
}
