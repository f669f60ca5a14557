// One Life-like lattice on a thread-block cluster (single-model path).
//
// The resident kernel runs a lattice on one CTA, i.e. one SM.  Here the rows
// of a bit-packed lattice (W <= 1024) are cut into C slabs of R rows, one per
// CTA of a cluster of C (up to 16) CTAs, and each CTA keeps its slab in shared
// memory for every generation of the launch, in the resident kernel's band
// layout (a group of P = next_pow2(wpr) lanes per row, each group walking down
// a band of L rows with the column sums of three rows in registers, the rule
// indexed by the 3 x 3 block count: xk_life_word9).  Updates are in place.
//
// Each band's first and last row are also kept in a halo area, which the
// bands next to it read; the slab's first row also goes to the CTA above's
// "row below" slot and its last row to the CTA below's "row above" slot
// (remote stores to distributed shared memory).  Halos and slots are
// double-buffered by generation parity: generation g reads the parity-g
// buffers (all local loads) and, as it computes a band's first and last row,
// stores them straight from registers into the parity-(g + 1) buffers, last
// read by generation g - 1.  Two ways to order that:
//
// * barrier form: one cluster barrier starts every generation; it orders the
//   stores of generation g - 1 before the loads of generation g and the loads
//   of generation g - 1 before the stores of generation g (release / acquire
//   at cluster scope; every thread of every CTA arrives once per generation
//   and no CTA leaves the loop early).  It is the hardware cluster barrier,
//   so there is no software spin to bound.
// * neighbour form (P2P): only the two CTAs a slab exchanges rows with are
//   waited for.  Each CTA has one mbarrier per slot parity, expecting 2 wpr
//   arrivals a phase: every lane that stores a row word into a neighbour's
//   slot then arrives on that neighbour's mbarrier with release semantics at
//   cluster scope, and the lanes of a slab's first and last band wait
//   (acquire, cluster scope) on their own mbarrier before reading the slots.
//   Bands inside the CTA are ordered by one __syncthreads per generation.
//   The write-after-read order needs nothing more: a lane writes parity
//   (g + 1) slots of a neighbour only after it has received that
//   neighbour's generation g - 1 row, which the neighbour sent after reading
//   the parity (g - 1) = (g + 1) slot; and a phase's arrivals all come
//   before the next phase's can start.  The last generation sends nothing.
//   Waits are bounded (1 s): a CTA that gives up sets xk_cluster_wait_failed and
//   leaves the generation loop (every thread at once, through
//   __syncthreads_or), its neighbours then give up in turn, and the step
//   reports XK_ERR_TIMEOUT.
//
// * async form: the neighbour form's protocol, with each row word sent by an
//   asynchronous remote store (st.async) that completes 4 bytes of a
//   transaction count on the neighbour's mbarrier of that parity; the
//   receiving CTA's thread 0 arms its own mbarrier once per phase (one
//   arrival expecting the 8 wpr bytes of the two rows), so no release fence
//   per sending lane.  A store may land before the arming: the phase still
//   needs the arrival.  Bands of 2, 4 or 8 rows (the same length in every
//   CTA) compute their first and last row before the inner ones, so the rows
//   leave early.
//
// * split form (bands of exactly 4 or 8 rows in every CTA): the barrier form with
//   the cluster barrier's arrive and wait apart.  A band computes its first
//   and last row first (from the halos and its own rows, whose old values it
//   keeps in registers) and publishes them, then arrives; its two inner rows,
//   which no other band reads, are computed while the barrier completes, and
//   the wait comes at the top of the next generation.  The ordering argument
//   is the barrier form's: every halo read of generation g precedes the
//   arrival of generation g, every halo write of generation g + 1 follows its
//   wait.
//
// A last cluster barrier after the loop keeps every CTA's shared memory alive
// until the remote stores of the final generation have landed (the mbarrier
// forms send nothing in the final generation, and every earlier row is
// waited for by its receiver).  A lane only
// ever touches its own column word of its own band.
#include <cooperative_groups.h>

#include <string.h>

#include "life_word.cuh"
#include "xk_internal.cuh"

namespace cg = cooperative_groups;

// shared words: slab of the widest CTA (R rows), halos [2][G][2][wpr], slots
// [2][2][wpr], then (rounded to 8 bytes) the neighbour form's two mbarriers;
// the offsets are the same in every CTA of the cluster, which the remote
// stores and arrivals rely on
static inline int64_t cluster_data_words(int wpr, int R, int threads)
{
    const ResidentPlan p = xk_resident_plan(wpr, R, threads);
    return xk_res_lat_words(p) + 4LL * p.G * wpr + 4LL * wpr;
}

static inline int64_t cluster_words(int wpr, int R, int threads)
{
    return ((cluster_data_words(wpr, R, threads) + 1) & ~1LL) + 4;
}

#define XK_CL_WAIT_NS 1000000000ull   // a CTA gives up after 1 s of waiting (never expected)

// set when a CTA of the neighbour form gave up waiting (never expected)
__device__ unsigned int xk_cluster_wait_failed;

__device__ __forceinline__ bool xk_cl_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return done != 0;
}

__device__ __forceinline__ uint64_t xk_globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for the phase of `parity` to complete; false after XK_CL_WAIT_NS
__device__ __forceinline__ bool xk_cl_wait(uint32_t bar, uint32_t parity)
{
    if (xk_cl_try_wait(bar, parity)) return true;
    const uint64_t t0 = xk_globaltimer();
    while (!xk_cl_try_wait(bar, parity))
        if (xk_globaltimer() - t0 > XK_CL_WAIT_NS) return false;
    return true;
}

// arrive on the mbarrier at shared::cluster address `bar` (another CTA's),
// ordering this thread's earlier stores before it
__device__ __forceinline__ void xk_cl_arrive_remote(uint32_t bar)
{
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" : : "r"(bar) : "memory");
}

// store v at shared::cluster address `addr` (another CTA's) asynchronously;
// its completion counts 4 bytes on the mbarrier at shared::cluster address
// `bar` of the same CTA
__device__ __forceinline__ void xk_cl_st_async(uint32_t addr, uint32_t v, uint32_t bar)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.u32 [%0], %1, [%2];"
                 : : "r"(addr), "r"(v), "r"(bar) : "memory");
}

// this CTA's arrival on its own mbarrier, expecting `bytes` of transactions
__device__ __forceinline__ void xk_cl_arm(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" : : "r"(bar), "r"(bytes) : "memory");
}

// the hardware cluster barrier's two halves (every thread of every CTA
// alternates them)
__device__ __forceinline__ void xk_cl_barrier_arrive()
{
    asm volatile("barrier.cluster.arrive.release.aligned;" : : : "memory");
}

__device__ __forceinline__ void xk_cl_barrier_wait()
{
    asm volatile("barrier.cluster.wait.acquire.aligned;" : : : "memory");
}

__device__ __forceinline__ uint32_t xk_cl_mapa(uint32_t addr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

// TORUS: wrap, else static border; FULLW: torus rows of whole words (each
// neighbour vector one funnel shift); LB: every band of the widest CTA has
// exactly LB rows (1, 2, 4 or 8; the row loop is unrolled), 0 for any length;
// RF: the rule form (XK_RULE_TABLE: `t`; XK_RULE_CONWAY: B3/S23 compiled in);
// SYNC: the synchronisation form (XK_SYNC_*)
template <bool TORUS, bool FULLW, int LB, int RF, int SYNC>
__global__ void __launch_bounds__(1024)
xk_k_life_cluster(uint32_t *__restrict__ bits, LifeGeo g, LifeTable9 t9, int generations, int R)
{
    constexpr bool ASYNC = SYNC == XK_SYNC_ASYNC, SPLIT = SYNC == XK_SYNC_SPLIT;
    constexpr bool P2P = SYNC == XK_SYNC_NEIGHBOUR || ASYNC;     // mbarrier waits
    constexpr bool EDGE_FIRST = SPLIT || (ASYNC && LB >= 2);      // edge rows, then the inner ones
    static_assert(!SPLIT || LB == 4 || LB == 8, "the split form runs bands of 4 or 8 rows");
    static_assert(!ASYNC || LB > 0, "the async form runs bands of a fixed length");
    const auto &t = RuleForm<RF>::make(t9);
    extern __shared__ uint32_t sm[];
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int)cluster.num_blocks();
    const int c = (int)cluster.block_rank();
    const int wpr = g.wpr, H = g.H;
    const int r0 = c * R;
    const int Rc = min(H, r0 + R) - r0;                       // rows of this CTA (>= 1)
    const int cu = c > 0 ? c - 1 : C - 1, cd = c + 1 < C ? c + 1 : 0;
    const ResidentPlan pw = xk_resident_plan(wpr, R, blockDim.x);
    const ResidentPlan p = xk_resident_plan(wpr, Rc, blockDim.x);
    uint32_t *lat = sm;
    uint32_t *halo = sm + xk_res_lat_words(pw);               // [parity][band][first, last][wpr]
    uint32_t *slot = halo + 4 * pw.G * wpr;                   // [parity][above, below][wpr]
    uint32_t *slot_up = cluster.map_shared_rank(slot, cu);
    uint32_t *slot_dn = cluster.map_shared_rank(slot, cd);
    const int hwords = 2 * pw.G * wpr;
    // neighbour form: mbarrier [parity] (8-byte aligned, after the data)
    const int64_t dwords = xk_res_lat_words(pw) + 4LL * pw.G * wpr + 4LL * wpr;
    uint64_t *mbar = (uint64_t *)(sm + ((dwords + 1) & ~1LL));
    const uint32_t mbar0 = (uint32_t)__cvta_generic_to_shared(mbar);
    if (P2P && threadIdx.x == 0) {
        // neighbour form: the 2 wpr sending lanes arrive; async form: this
        // CTA's arming is the one arrival, the stores count bytes
        for (int q = 0; q < 2; ++q)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" : : "r"(mbar0 + 8u * q), "r"(ASYNC ? 1 : 2 * wpr)
                         : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" : : : "memory");
    }
    // the neighbours' mbarriers [parity] at shared::cluster addresses
    const uint32_t mb_up = P2P ? xk_cl_mapa(mbar0, (uint32_t)cu) : 0u;
    const uint32_t mb_dn = P2P ? xk_cl_mapa(mbar0, (uint32_t)cd) : 0u;
    // async form: the neighbours' slots at shared::cluster addresses
    const uint32_t slot0 = (uint32_t)__cvta_generic_to_shared(slot);
    const uint32_t sa_up = ASYNC ? xk_cl_mapa(slot0, (uint32_t)cu) : 0u;
    const uint32_t sa_dn = ASYNC ? xk_cl_mapa(slot0, (uint32_t)cd) : 0u;

    for (int w = threadIdx.x; w < Rc * wpr; w += blockDim.x) {
        const int y = w / wpr, jj = w - y * wpr;
        const int b = y / p.L, i = y - b * p.L;
        lat[xk_res_at(p, b, i, jj)] = bits[(int64_t)r0 * wpr + w];
    }

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int q = lane / p.P, j = lane - q * p.P;
    const int band = warp * p.gpw + q;
    const bool active = band < p.nb && j < wpr;
    // clamped indices: idle lanes compute on valid (ignored) words, so the
    // shuffles always see the whole warp
    const int bc = band < p.nb ? band : p.nb - 1;
    const int jc = j < wpr ? j : wpr - 1;
    const int y0 = bc * p.L;
    const int y1 = min(Rc, y0 + p.L);
    const int last = wpr - 1;
    const int gbase = q * p.P;
    const int src_l = gbase + (jc > 0 ? jc - 1 : last);
    const int src_r = gbase + (jc < last ? jc + 1 : 0);
    const int lshift = jc > 0 ? 31 : g.rlast - 1;
    const int lpre = 31 - lshift;
    const int top = jc == last ? g.rlast - 1 : 31;
    const uint32_t topbit = 1u << top;
    const uint32_t outmask = jc == last ? g.lastmask : 0xFFFFFFFFu;
    const uint32_t edge = g.bfill & 1u;
    const int use_le = (!TORUS) && jc == 0, use_re = (!TORUS) && jc == last;
    const bool first_band = bc == 0, last_band = bc == p.nb - 1;
    const bool top_off = !TORUS && c == 0 && first_band;      // row above is off the lattice
    const bool bot_off = !TORUS && c == C - 1 && last_band;   // row below is off the lattice
    uint32_t *wp = lat + xk_res_at(p, bc, 0, jc);             // this lane's word of band row i: wp[32 i]

    // column sums (s, c) = FA(L, C, R) of the row whose word at this lane's
    // column is w
    auto colsum = [&](uint32_t w, uint32_t &s, uint32_t &cy) {
        const uint32_t l = __shfl_sync(0xFFFFFFFFu, w, src_l);
        const uint32_t r = __shfl_sync(0xFFFFFFFFu, w, src_r);
        if (FULLW) {
            const uint32_t L = __funnelshift_l(l, w, 1), Rr = __funnelshift_r(w, r, 1);
            s = xk_lop3_xor3(L, w, Rr);
            cy = xk_maj(L, w, Rr);
            return;
        }
        const RowVec v = TORUS ? xk_torus_vec(w, l, r, lpre, top, topbit)
                               : xk_row_vec(w, l, r, lshift, top, edge, edge, use_le, use_re);
        s = xk_lop3_xor3(v.L, v.C, v.R);
        cy = xk_maj(v.L, v.C, v.R);
    };

    // a band's first row goes to its halo and, for the slab's first band, to
    // the CTA above ("row below" slot); its last row likewise downwards
    const bool send_up = active && band == 0, send_dn = active && band == p.nb - 1;
    // `remote`: also store into the neighbours' slots (and, in the neighbour
    // form, arrive on their parity-npar mbarrier)
    // (active lanes) a band's first row, and its last row
    auto publish_first = [&](int npar, uint32_t w, bool remote) {
        halo[npar * hwords + (band * 2 + 0) * wpr + j] = w;
        if (send_up && remote) {
            if (ASYNC) {
                xk_cl_st_async(sa_up + 4u * (uint32_t)((npar * 2 + 1) * wpr + j), w, mb_up + 8u * (uint32_t)npar);
            } else {
                slot_up[(npar * 2 + 1) * wpr + j] = w;
                if (P2P) xk_cl_arrive_remote(mb_up + 8u * (uint32_t)npar);
            }
        }
    };
    auto publish_last = [&](int npar, uint32_t w, bool remote) {
        halo[npar * hwords + (band * 2 + 1) * wpr + j] = w;
        if (send_dn && remote) {
            if (ASYNC) {
                xk_cl_st_async(sa_dn + 4u * (uint32_t)((npar * 2 + 0) * wpr + j), w, mb_dn + 8u * (uint32_t)npar);
            } else {
                slot_dn[(npar * 2 + 0) * wpr + j] = w;
                if (P2P) xk_cl_arrive_remote(mb_dn + 8u * (uint32_t)npar);
            }
        }
    };
    auto publish = [&](int npar, int i, uint32_t w, bool remote) {
        if (!active) return;
        if (i == 0) publish_first(npar, w, remote);
        if (i == y1 - 1 - y0) publish_last(npar, w, remote);
    };

    cluster.sync();   // every CTA running (before any remote store), slabs loaded, mbarriers set
    // each edge row sent once (a one-row band's row is its first and last);
    // nothing when no generation will read them
    if (generations > 0) {
        publish(0, 0, wp[0], true);
        if (y1 - 1 - y0 != 0) publish(0, y1 - 1 - y0, wp[32 * (y1 - 1 - y0)], true);
    }
    bool failed = false;
    if (SPLIT) xk_cl_barrier_arrive();
    for (int gen = 0; gen < generations; ++gen) {
        const int par = gen & 1;
        const uint32_t *hp = halo + par * hwords;
        if (P2P) {
            // async form: one arrival per phase, expecting the two rows
            if (ASYNC && threadIdx.x == 0) xk_cl_arm(mbar0 + 8u * (uint32_t)par, 8u * (uint32_t)wpr);
            // bands of this CTA; every thread leaves together after a failure
            if (__syncthreads_or(failed)) break;
            if ((first_band || last_band) &&
                !xk_cl_wait(mbar0 + 8u * (uint32_t)par, (uint32_t)(gen >> 1) & 1u)) {
                failed = true;
                atomicOr(&xk_cluster_wait_failed, 1u);
            }
        } else if (SPLIT) {
            xk_cl_barrier_wait();
        } else {
            cluster.sync();
        }
        const bool remote = gen + 1 < generations || !P2P;
        const uint32_t wu = first_band ? slot[(par * 2 + 0) * wpr + jc] : hp[((bc - 1) * 2 + 1) * wpr + jc];
        const uint32_t wl = last_band ? slot[(par * 2 + 1) * wpr + jc] : hp[((bc + 1) * 2 + 0) * wpr + jc];
        if constexpr (EDGE_FIRST) {
            // every band has LB rows: the first and last row, then the inner
            // ones after the arrival (split form) or the sends (async form),
            // the old rows' column sums in registers
            uint32_t w[LB], s[LB], cy[LB];
            uint32_t s_u, c_u, s_d, c_d;
#pragma unroll
            for (int i = 0; i < LB; ++i) w[i] = wp[32 * i];
            colsum(wu, s_u, c_u);
            if (top_off) s_u = c_u = g.bfill;
#pragma unroll
            for (int i = 0; i < LB; ++i) colsum(w[i], s[i], cy[i]);
            colsum(wl, s_d, c_d);
            if (bot_off) s_d = c_d = g.bfill;
            uint32_t o0 = xk_life_word9(s_u, c_u, s[0], cy[0], s[1], cy[1], w[0], t);
            uint32_t oL = xk_life_word9(s[LB - 2], cy[LB - 2], s[LB - 1], cy[LB - 1], s_d, c_d, w[LB - 1], t);
            if (!FULLW) {
                o0 &= outmask;
                oL &= outmask;
            }
            if (active) {
                wp[0] = o0;
                wp[32 * (LB - 1)] = oL;
                publish_first(par ^ 1, o0, remote);
                publish_last(par ^ 1, oL, remote);
            }
            if (SPLIT) xk_cl_barrier_arrive();
#pragma unroll
            for (int i = 1; i < LB - 1; ++i) {
                uint32_t o = xk_life_word9(s[i - 1], cy[i - 1], s[i], cy[i], s[i + 1], cy[i + 1], w[i], t);
                if (!FULLW) o &= outmask;
                if (active) wp[32 * i] = o;
            }
            continue;
        }
        uint32_t su, cu_, sm_, cm_, Cm = wp[0];
        colsum(wu, su, cu_);
        if (top_off) su = cu_ = g.bfill;
        colsum(Cm, sm_, cm_);
        auto row = [&](int i) {
            const int y = y0 + i;
            const bool below = y + 1 >= y1;                       // next row is the band's neighbour
            const uint32_t wd = below ? wl : wp[32 * (i + 1)];
            uint32_t sd, cd_;
            colsum(wd, sd, cd_);
            if (below && bot_off) sd = cd_ = g.bfill;
            uint32_t out = xk_life_word9(su, cu_, sm_, cm_, sd, cd_, Cm, t);
            if (!FULLW) out &= outmask;
            if (active && y < y1) {
                wp[32 * i] = out;
                publish(par ^ 1, i, out, remote);
            }
            su = sm_;
            cu_ = cm_;
            sm_ = sd;
            cm_ = cd_;
            Cm = wd;
        };
        if (LB > 0) {
#pragma unroll
            for (int i = 0; i < LB; ++i) row(i);
        } else {
#pragma unroll 2
            for (int i = 0; i < p.L; ++i) row(i);
        }
    }
    if (SPLIT) xk_cl_barrier_wait();   // the phase of the last arrival
    cluster.sync();
    for (int w = threadIdx.x; w < Rc * wpr; w += blockDim.x) {
        const int y = w / wpr, jj = w - y * wpr;
        const int b = y / p.L, i = y - b * p.L;
        bits[(int64_t)r0 * wpr + w] = lat[xk_res_at(p, b, i, jj)];
    }
}

typedef void (*ClusterKernel)(uint32_t *, LifeGeo, LifeTable9, int, int);

// the neighbour form has instantiations for bands of 1, 2 and 4 rows, the
// split form for bands of 4 and 8, the async form for 1, 2, 4 and 8
template <bool TORUS, bool FULLW, int RF>
static ClusterKernel cluster_kernel_l(int L, int sync)
{
    if (sync == XK_SYNC_NEIGHBOUR) {
        switch (L) {
        case 1: return xk_k_life_cluster<TORUS, FULLW, 1, RF, XK_SYNC_NEIGHBOUR>;
        case 2: return xk_k_life_cluster<TORUS, FULLW, 2, RF, XK_SYNC_NEIGHBOUR>;
        case 4: return xk_k_life_cluster<TORUS, FULLW, 4, RF, XK_SYNC_NEIGHBOUR>;
        default: return nullptr;
        }
    }
    if (sync == XK_SYNC_SPLIT) {
        if (L == 4) return xk_k_life_cluster<TORUS, FULLW, 4, RF, XK_SYNC_SPLIT>;
        if (L == 8) return xk_k_life_cluster<TORUS, FULLW, 8, RF, XK_SYNC_SPLIT>;
        return nullptr;
    }
    if (sync == XK_SYNC_ASYNC) {
        switch (L) {
        case 1: return xk_k_life_cluster<TORUS, FULLW, 1, RF, XK_SYNC_ASYNC>;
        case 2: return xk_k_life_cluster<TORUS, FULLW, 2, RF, XK_SYNC_ASYNC>;
        case 4: return xk_k_life_cluster<TORUS, FULLW, 4, RF, XK_SYNC_ASYNC>;
        case 8: return xk_k_life_cluster<TORUS, FULLW, 8, RF, XK_SYNC_ASYNC>;
        default: return nullptr;
        }
    }
    switch (L) {
    case 1: return xk_k_life_cluster<TORUS, FULLW, 1, RF, XK_SYNC_BARRIER>;
    case 2: return xk_k_life_cluster<TORUS, FULLW, 2, RF, XK_SYNC_BARRIER>;
    case 4: return xk_k_life_cluster<TORUS, FULLW, 4, RF, XK_SYNC_BARRIER>;
    case 8: return xk_k_life_cluster<TORUS, FULLW, 8, RF, XK_SYNC_BARRIER>;
    default: return xk_k_life_cluster<TORUS, FULLW, 0, RF, XK_SYNC_BARRIER>;
    }
}

template <int RF>
static ClusterKernel cluster_kernel_rf(const LifeGeo &g, int L, int sync)
{
    if (!g.torus) return cluster_kernel_l<false, false, RF>(L, sync);
    if (g.rlast == 32) return cluster_kernel_l<true, true, RF>(L, sync);
    return cluster_kernel_l<true, false, RF>(L, sync);
}

// the instantiation for a lattice, launch shape (L: band length of the
// widest CTA), rule form and synchronisation form (null: none)
static ClusterKernel cluster_kernel(const LifeGeo &g, int R, int threads, int rf = XK_RULE_TABLE,
                                    int sync = XK_SYNC_BARRIER)
{
    const int L = xk_resident_plan(g.wpr, R, threads).L;
    return rf == XK_RULE_CONWAY ? cluster_kernel_rf<XK_RULE_CONWAY>(g, L, sync)
                                : cluster_kernel_rf<XK_RULE_TABLE>(g, L, sync);
}

static cudaError_t cluster_attrs(ClusterKernel k, size_t smem)
{
    cudaError_t e = cudaFuncSetAttribute((const void *)k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    return xk_smem_attr_at_least((const void *)k, (int)smem);
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

int xk_rule_form(uint32_t rule0, uint32_t rule1)
{
    return rule0 == 8u && rule1 == 12u ? XK_RULE_CONWAY : XK_RULE_TABLE;
}

LifeTable9 xk_life_table9(uint32_t rule0, uint32_t rule1)
{
    // dead D[n] = rule0 bit n, live L[n] = rule1 bit n - 1 (n: 3 x 3 count)
    auto D = [&](int n) { return 0u - ((rule0 >> n) & 1u); };
    auto L = [&](int n) { return 0u - ((rule1 >> (n > 0 ? n - 1 : 0)) & 1u); };
    LifeTable9 t;
    for (int q = 0; q < 8; ++q) {
        const uint32_t A = q < 4 ? D(2 * q) : L(2 * (q - 4));
        const uint32_t B = q < 4 ? D(2 * q + 1) : L(2 * (q - 4) + 1);
        t.a[q] = A;
        t.k[q] = xk_mux_coef(A, B);
    }
    t.d8 = D(8);
    t.a9 = L(8);
    t.k9 = xk_mux_coef(L(8), L(9));
    return t;
}

// rows per CTA and threads for a cluster of (up to) C CTAs whose lane groups
// walk bands of about `band` rows; 0 if the lattice does not fit or no such
// cluster can be resident on this device
int xk_life_cluster_config(const LifeGeo &g, int C, int band, int *C_out, int *R, int *threads)
{
    if (g.wpr > 32 || C < 2 || C > 16 || g.H < C || band < 1) return 0;
    const int rows = (g.H + C - 1) / C;
    const int Cr = (g.H + rows - 1) / rows;                    // no empty CTA
    if (Cr < 2) return 0;
    int P = 1;
    while (P < g.wpr) P <<= 1;
    const int groups = (rows + band - 1) / band;
    int th = ((P * groups + 31) / 32) * 32;
    th = th < 32 ? 32 : (th > 1024 ? 1024 : th);
    const size_t smem = 4ull * cluster_words(g.wpr, rows, th);
    if ((int64_t)smem > xk_max_smem_optin()) return 0;
    const ClusterKernel k = cluster_kernel(g, rows, th);
    bool attrs_ok = true;
    for (int rf = XK_RULE_TABLE; rf <= XK_RULE_CONWAY && attrs_ok; ++rf)
        for (int sync = XK_SYNC_BARRIER; sync <= XK_SYNC_ASYNC && attrs_ok; ++sync) {
            const ClusterKernel kk = cluster_kernel(g, rows, th, rf, sync);
            attrs_ok = !kk || cluster_attrs(kk, smem) == cudaSuccess;
        }
    if (!attrs_ok) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr;
    cluster_cfg(cfg, attr, Cr, th, smem, 0);
    int active = 0;
    cudaError_t e = cudaOccupancyMaxActiveClusters(&active, (const void *)k, &cfg);
    if (e != cudaSuccess || active < 1) {
        cudaGetLastError();
        return 0;
    }
    *C_out = Cr;
    *R = rows;
    *threads = th;
    return 1;
}

int xk_life_cluster_has_sync(const LifeGeo &g, int C, int R, int threads, int sync)
{
    if (sync == XK_SYNC_BARRIER) return 1;
    const ResidentPlan p = xk_resident_plan(g.wpr, R, threads);
    if (sync == XK_SYNC_SPLIT) {
        // every CTA has R rows, cut into bands of exactly 4 or 8
        if ((int64_t)C * R != g.H || (p.L != 4 && p.L != 8) || p.nb * p.L != R) return 0;
    }
    if (sync == XK_SYNC_ASYNC && p.L >= 2) {
        // the edge rows computed first: every CTA has R rows, cut into bands
        // of exactly 2, 4 or 8
        if ((int64_t)C * R != g.H || (p.L != 2 && p.L != 4 && p.L != 8) || p.nb * p.L != R) return 0;
    }
    return cluster_kernel(g, R, threads, XK_RULE_TABLE, sync) != nullptr;
}

bool xk_cluster_take_wait_failure()
{
    unsigned int v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, xk_cluster_wait_failed, sizeof(v)) != cudaSuccess) return false;
    if (v) cudaMemcpyToSymbol(xk_cluster_wait_failed, &z, sizeof(z));
    return v != 0;
}

cudaError_t xk_life_step_cluster(uint32_t *bits, const LifeGeo &g, uint32_t rule0, uint32_t rule1,
                                 int generations, int C, int R, int threads, cudaStream_t s, int sync)
{
    const size_t smem = 4ull * cluster_words(g.wpr, R, threads);
    if (!xk_life_cluster_has_sync(g, C, R, threads, sync)) return cudaErrorInvalidValue;
    const ClusterKernel k = cluster_kernel(g, R, threads, xk_rule_form(rule0, rule1), sync);
    if (!k) return cudaErrorInvalidValue;
    cudaError_t e = cluster_attrs(k, smem);
    if (e != cudaSuccess) return e;
    const LifeTable9 t = xk_life_table9(rule0, rule1);
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr;
    cluster_cfg(cfg, attr, C, threads, smem, s);
    return cudaLaunchKernelEx(&cfg, k, bits, g, t, generations, R);
}
