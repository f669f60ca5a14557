// One Life-like lattice on a thread-block cluster (single-model path).
//
// The resident kernel runs a lattice on one CTA, i.e. one SM.  Here the rows
// of a bit-packed lattice (W <= 1024) are cut into C bands, one per CTA of a
// cluster of C (up to 16) CTAs; each CTA keeps its band in shared memory,
// double-buffered by generation parity, for every generation of the launch.
// The row above a band and the row below it belong to the neighbouring CTAs
// and are read straight from their shared memory (distributed shared memory,
// cluster.map_shared_rank).  One cluster barrier per generation orders it all:
// after barrier g every CTA has finished generation g - 1, so buffer g & 1
// holds generation g everywhere and nobody still reads buffer (g + 1) & 1,
// which generation g overwrites.  The barrier is the hardware cluster barrier
// (every thread of every CTA arrives once per generation; no CTA leaves the
// loop early), so there is no software spin to bound.
//
// Inside a band, P = next_pow2(wpr) lanes cover one row (lane j owns column
// word j) and each group of P lanes walks down a run of consecutive rows
// keeping three rows' neighbour vectors in registers, as in the resident
// kernel; the neighbour count and rule are xk_life_word's.
#include <cooperative_groups.h>

#include <string.h>

#include "life_word.cuh"
#include "xk_internal.cuh"

namespace cg = cooperative_groups;

template <bool TORUS>
__global__ void __launch_bounds__(1024)
xk_k_life_cluster(uint32_t *__restrict__ bits, LifeGeo g, LifeTable t, int generations, int R)
{
    extern __shared__ uint32_t band[];   // [2][R][wpr]
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int)cluster.num_blocks();
    const int c = (int)cluster.block_rank();
    const int wpr = g.wpr, H = g.H;
    const int r0 = c * R;
    const int Rc = min(H, r0 + R) - r0;                       // rows of this CTA (>= 1)
    const int cu = c > 0 ? c - 1 : C - 1, cd = c + 1 < C ? c + 1 : 0;
    const int Ru = min(H, cu * R + R) - cu * R;               // rows of the CTA above
    const bool top_off = !TORUS && c == 0, bot_off = !TORUS && c == C - 1;
    const uint32_t *up_band = cluster.map_shared_rank(band, cu);
    const uint32_t *dn_band = cluster.map_shared_rank(band, cd);
    const int buf = R * wpr;

    for (int w = threadIdx.x; w < Rc * wpr; w += blockDim.x) band[w] = bits[(int64_t)r0 * wpr + w];

    int P = 1;
    while (P < wpr) P <<= 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gpw = 32 / P;
    const int groups = (int)(blockDim.x / 32) * gpw;
    const int q = lane / P, j = lane - q * P;
    const int grp = warp * gpw + q;
    const int L = (Rc + groups - 1) / groups;                 // rows per group
    const int gy0 = grp * L, gy1 = min(Rc, gy0 + L);
    const bool jok = j < wpr;
    const int jc = jok ? j : wpr - 1;
    const int last = wpr - 1;
    const int gbase = q * P;
    const int src_l = gbase + (jc > 0 ? jc - 1 : last);
    const int src_r = gbase + (jc < last ? jc + 1 : 0);
    const int lshift = jc > 0 ? 31 : g.rlast - 1;
    const int lpre = 31 - lshift;
    const int top = jc == last ? g.rlast - 1 : 31;
    const uint32_t topbit = 1u << top;
    const uint32_t outmask = jc == last ? g.lastmask : 0xFFFFFFFFu;
    const uint32_t edge = g.bfill & 1u;
    const int use_le = (!TORUS) && jc == 0, use_re = (!TORUS) && jc == last;

    cluster.sync();   // every band loaded before anyone reads a neighbour's
    for (int gen = 0; gen < generations; ++gen) {
        const int pb = (gen & 1) * buf;
        const uint32_t *cur = band + pb;
        uint32_t *nxt = band + (buf - pb);
        // word of local row y (-1 .. Rc) at this lane's column; rows outside
        // the band come from the neighbouring CTAs (or the static border)
        auto fetch = [&](int y, bool &off) -> uint32_t {
            off = false;
            if (y < 0) {
                if (top_off) { off = true; return g.bfill; }
                return up_band[pb + (Ru - 1) * wpr + jc];
            }
            if (y >= Rc) {
                if (bot_off) { off = true; return g.bfill; }
                return dn_band[pb + jc];
            }
            return cur[y * wpr + jc];
        };
        auto vec = [&](uint32_t w, bool off) -> RowVec {
            const uint32_t l = __shfl_sync(0xFFFFFFFFu, w, src_l);
            const uint32_t r = __shfl_sync(0xFFFFFFFFu, w, src_r);
            RowVec v;
            if (TORUS) {
                v = xk_torus_vec(w, l, r, lpre, top, topbit);
            } else {
                v = xk_row_vec(w, l, r, lshift, top, edge, edge, use_le, use_re);
                if (off) v.L = v.C = v.R = g.bfill;
            }
            return v;
        };
        // every lane runs L iterations so the shuffles always see the whole
        // warp; groups past the band's end compute and discard
        const int ys = min(gy0, Rc);
        bool off;
        uint32_t w = fetch(ys - 1, off);
        RowVec vu = vec(w, off);
        w = fetch(ys, off);
        RowVec vm = vec(w, off);
        for (int i = 0; i < L; ++i) {
            const int y = ys + i;
            w = fetch(min(y + 1, Rc), off);
            const RowVec vd = vec(w, off);
            const uint32_t out = xk_life_word(vu.L, vu.C, vu.R, vm.L, vm.C, vm.R, vd.L, vd.C,
                                                 vd.R, t) & outmask;
            if (jok && y < gy1) nxt[y * wpr + j] = out;
            vu = vm;
            vm = vd;
        }
        cluster.sync();
    }
    const uint32_t *fin = band + (generations & 1) * buf;
    for (int w = threadIdx.x; w < Rc * wpr; w += blockDim.x) bits[(int64_t)r0 * wpr + w] = fin[w];
}

template <bool TORUS>
static cudaError_t cluster_attrs(size_t smem)
{
    cudaError_t e = cudaFuncSetAttribute(xk_k_life_cluster<TORUS>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(xk_k_life_cluster<TORUS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
}

static void cluster_cfg(cudaLaunchConfig_t &cfg, cudaLaunchAttribute &attr, int C, int threads,
                        size_t smem, cudaStream_t s)
{
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(C, 1, 1);
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = C;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
}

// rows per CTA and threads for a cluster of (up to) C CTAs; 0 if the lattice
// does not fit or no such cluster can be resident on this device
int xk_life_cluster_config(const LifeGeo &g, int C, int *C_out, int *R, int *threads)
{
    if (g.wpr > 32 || C < 2 || C > 16 || g.H < C) return 0;
    const int rows = (g.H + C - 1) / C;
    const int Cr = (g.H + rows - 1) / rows;                    // no empty CTA
    if (Cr < 2) return 0;
    const size_t smem = 2ull * rows * g.wpr * 4;
    if ((int64_t)smem > xk_max_smem_optin()) return 0;
    int P = 1;
    while (P < g.wpr) P <<= 1;
    int th = ((P * rows + 31) / 32) * 32;
    th = th < 32 ? 32 : (th > 1024 ? 1024 : th);
    const bool torus = g.torus != 0;
    if ((torus ? cluster_attrs<true>(smem) : cluster_attrs<false>(smem)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr;
    cluster_cfg(cfg, attr, Cr, th, smem, 0);
    int active = 0;
    cudaError_t e = torus ? cudaOccupancyMaxActiveClusters(&active, xk_k_life_cluster<true>, &cfg)
                          : cudaOccupancyMaxActiveClusters(&active, xk_k_life_cluster<false>, &cfg);
    if (e != cudaSuccess || active < 1) {
        cudaGetLastError();
        return 0;
    }
    *C_out = Cr;
    *R = rows;
    *threads = th;
    return 1;
}

cudaError_t xk_life_step_cluster(uint32_t *bits, const LifeGeo &g, const LifeTable &t,
                                 int generations, int C, int R, int threads, cudaStream_t s)
{
    const size_t smem = 2ull * R * g.wpr * 4;
    const bool torus = g.torus != 0;
    cudaError_t e = torus ? cluster_attrs<true>(smem) : cluster_attrs<false>(smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr;
    cluster_cfg(cfg, attr, C, threads, smem, s);
    if (torus) return cudaLaunchKernelEx(&cfg, xk_k_life_cluster<true>, bits, g, t, generations, R);
    return cudaLaunchKernelEx(&cfg, xk_k_life_cluster<false>, bits, g, t, generations, R);
}
