// Life-like (outer-totalistic, binary state) generation kernels for sm_103a.
//
// Reference semantics: GameOfLife / LifelikeCA emit copies the state to every
// buffer and absorb applies  next = ((B >> k) & 1) | ((S >> k) & 1 & state)
// with k = sum of the neighbours' buffers (examples/game_of_life.py:42-70,
// :183-203; buffers and planes per xentica/core/base.py:226-236).  Emit and
// absorb are fused: a cell's buffer towards each neighbour equals its state,
// so absorb can read the neighbours' states directly and the N buffer planes
// never exist.  The rule arrives as a truth table (rule0 for dead cells,
// rule1 for live ones) extracted from the traced model.
//
// Layout: 32 cells per 32-bit word, LSB = lowest x; a generation is pure
// bitwise logic -- a carry-save adder network counts the 8 neighbours of 32
// cells at once and a LOP3 multiplexer tree applies the runtime rule.
#include <string.h>

#include <type_traits>

#include "xk_internal.cuh"

LifeTable xk_life_table(uint32_t rule0, uint32_t rule1)
{
    LifeTable t;
    auto mask = [](uint32_t r, int n) { return 0u - ((r >> n) & 1u); };
    for (int q = 0; q < 8; ++q) {
        const uint32_t r = q < 4 ? rule0 : rule1;
        const int n = 2 * (q & 3);
        t.a[q] = mask(r, n);
        t.k[q] = xk_mux_coef(mask(r, n), mask(r, n + 1));
    }
    t.a8 = mask(rule0, 8);
    t.k8 = xk_mux_coef(mask(rule0, 8), mask(rule1, 8));
    return t;
}

LifeGeo xk_life_geo(int64_t W, int64_t H, int torus, int border_state)
{
    LifeGeo g;
    g.W = (int32_t)W;
    g.H = (int32_t)H;
    g.wpr = (int32_t)((W + 31) / 32);
    g.rlast = (int32_t)(W - 32 * (int64_t)(g.wpr - 1));
    g.lastmask = g.rlast == 32 ? 0xFFFFFFFFu : ((1u << g.rlast) - 1u);
    g.torus = torus;
    g.bfill = border_state ? 0xFFFFFFFFu : 0u;
    g.div_wpr = xk_div_magic((uint64_t)g.wpr, (uint64_t)g.H * (uint64_t)g.wpr);
    return g;
}

#include "life_word.cuh"

// ---------------------------------------------------------------------------
// one generation straight from global memory (lattices too large for a CTA)

__global__ void __launch_bounds__(256)
xk_k_life_global(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, LifeGeo g,
                 LifeTable t)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (uint32_t)g.H * (uint32_t)g.wpr) return;
    xk_grid_dep_wait();       // launched as a dependent of the previous generation
    const int y = (int)xk_divu(idx, (uint32_t)g.wpr, g.div_wpr);
    const int j = (int)(idx - (uint32_t)y * g.wpr);
    const int last = g.wpr - 1;
    const int jl = j > 0 ? j - 1 : last, jr = j < last ? j + 1 : 0;
    const int lshift = j > 0 ? 31 : g.rlast - 1;
    const int top = j == last ? g.rlast - 1 : 31;
    const int use_le = (!g.torus) && j == 0, use_re = (!g.torus) && j == last;
    const uint32_t edge = g.bfill & 1u;
    RowVec v[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        int yy = y + r - 1;
        bool off = yy < 0 || yy >= g.H;
        if (off && !g.torus) {
            v[r].L = v[r].C = v[r].R = g.bfill;
            continue;
        }
        if (yy < 0) yy += g.H;
        if (yy >= g.H) yy -= g.H;
        const uint32_t *row = src + (int64_t)yy * g.wpr;
        v[r] = xk_row_vec(__ldg(row + j), __ldg(row + jl), __ldg(row + jr), lshift, top, edge,
                          edge, use_le, use_re);
    }
    uint32_t out = xk_life_word(v[0].L, v[0].C, v[0].R, v[1].L, v[1].C, v[1].R, v[2].L, v[2].C,
                                v[2].R, t);
    if (j == last) out &= g.lastmask;
    dst[idx] = out;
}

cudaError_t xk_life_step_global(const uint32_t *src, uint32_t *dst, const LifeGeo &g,
                                const LifeTable &t, cudaStream_t s)
{
    const int64_t total = (int64_t)g.H * g.wpr;
    if (total > 0xFFFFFFFFll) return cudaErrorInvalidValue;   // 32-bit word indices
    const int threads = 256;
    const int64_t blocks = (total + threads - 1) / threads;
    return xk_launch_pdl(xk_k_life_global, dim3((unsigned)blocks), dim3(threads), 0, s, src, dst, g, t);
}

// ---------------------------------------------------------------------------
// 3-D von Neumann Life-like on a torus (the serving loop's 3-D requests),
// bit-packed along x: row (y, z) is row z * H + y of the 2-D packing, so the
// pack/unpack kernels above serve unchanged with H * D rows.  One thread per
// word: the x neighbours come from the row's own words (torus wrap as in 2-D),
// y and z neighbours are the same word of four other rows.  Six one-bit
// inputs reduce to a 3-bit count with two full adders and a third on the
// carries; the count and the cell's state select the rule bit through the
// same multiplexer tree as in 2-D (counts 0..6).

__global__ void __launch_bounds__(256)
xk_k_life3d_vn(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, Life3Geo g,
               LifeTable t)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (uint32_t)g.H * (uint32_t)g.D * (uint32_t)g.wpr) return;
    xk_grid_dep_wait();       // launched as a dependent of the previous generation
    const uint32_t r = xk_divu(idx, (uint32_t)g.wpr, g.div_wpr);
    const int j = (int)(idx - r * (uint32_t)g.wpr);
    const int z = (int)xk_divu(r, (uint32_t)g.H, g.div_h), y = (int)(r - (uint32_t)z * g.H);
    const int last = g.wpr - 1;
    const int jl = j > 0 ? j - 1 : last, jr = j < last ? j + 1 : 0;
    const int lshift = j > 0 ? 31 : g.rlast - 1;
    const int top = j == last ? g.rlast - 1 : 31;
    const uint32_t *row = src + r * g.wpr;
    const RowVec v = xk_row_vec(__ldg(row + j), __ldg(row + jl), __ldg(row + jr), lshift, top, 0u,
                                0u, 0, 0);
    const int yu = y > 0 ? y - 1 : g.H - 1, yd = y + 1 < g.H ? y + 1 : 0;
    const int zf = z > 0 ? z - 1 : g.D - 1, zb = z + 1 < g.D ? z + 1 : 0;
    const uint32_t U = __ldg(src + ((int64_t)z * g.H + yu) * g.wpr + j);
    const uint32_t Dn = __ldg(src + ((int64_t)z * g.H + yd) * g.wpr + j);
    const uint32_t F = __ldg(src + ((int64_t)zf * g.H + y) * g.wpr + j);
    const uint32_t B = __ldg(src + ((int64_t)zb * g.H + y) * g.wpr + j);
    const uint32_t s1 = xk_lop3_xor3(v.L, v.R, U), c1 = xk_maj(v.L, v.R, U);
    const uint32_t s2 = xk_lop3_xor3(Dn, F, B), c2 = xk_maj(Dn, F, B);
    const uint32_t b0 = s1 ^ s2, c3 = s1 & s2;
    const uint32_t b1 = xk_lop3_xor3(c1, c2, c3), b2 = xk_maj(c1, c2, c3);
    uint32_t m[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) m[q] = xk_imux(b0, t.a[q], t.k[q]);
    uint32_t n[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) n[q] = xk_mux(b1, m[2 * q], m[2 * q + 1]);
    const uint32_t dead = xk_mux(b2, n[0], n[1]);
    const uint32_t live = xk_mux(b2, n[2], n[3]);
    uint32_t out = xk_mux(v.C, dead, live);
    if (j == last) out &= g.lastmask;
    dst[idx] = out;
}

cudaError_t xk_life_step3d_vn(const uint32_t *src, uint32_t *dst, const Life3Geo &g,
                              const LifeTable &t, cudaStream_t s)
{
    const int64_t total = (int64_t)g.H * g.D * g.wpr;
    if (total > 0xFFFFFFFFll) return cudaErrorInvalidValue;   // 32-bit word indices
    const int threads = 256;
    const int64_t blocks = (total + threads - 1) / threads;
    return xk_launch_pdl(xk_k_life3d_vn, dim3((unsigned)blocks), dim3(threads), 0, s, src, dst, g, t);
}

// ---------------------------------------------------------------------------
// resident lattices: a whole lattice (W <= 1024) lives in shared memory for
// all generations of a launch; one CTA per lattice.
//
// Lanes are grouped: a group of P = next_pow2(wpr) lanes covers one row, lane
// j of the group owning column word j.  The lattice's rows are cut into one
// band of consecutive rows per group; a group walks down its band keeping the
// column sums (s, c) = FA(L, C, R) of three rows and the cells of the middle
// row in registers (each row's sums are computed once, when it is the row
// below), so every generation costs one shared load, two shuffles and one
// shared store per 32 cells.  The rule is indexed by the count of the 3 x 3
// block including the cell (LifeTable9, xk_life_word9).  Updates are
// in place: a lane only ever touches its own column word of its own band, and
// the first and last row of every band are copied to a halo area, so
// neighbouring bands read the previous generation.  The halos are
// double-buffered by generation parity: generation g reads the parity-g
// halos and, once its band is done, copies its new first and last row into
// the parity-(g + 1) halos, last read by generation g - 1; one barrier per
// generation (at its end) then orders everything.
//
// Shared layout is warp-major: the bands of warp w hold their local row i at
// words (w * L + i) * 32 + lane, lane = group * P + column word, so a warp's
// accesses to one row hit 32 consecutive words and a lane's next row is
// always 32 words further on (a constant stride: the unrolled band loop
// addresses its rows with immediate offsets).  The rule table sits after the
// halo and is read into registers once.

#define XK_TAB_WORDS 32

int64_t xk_life_resident_words(int W, int H, int threads)
{
    const int wpr = (W + 31) / 32;
    if (wpr > 32) return -1;
    ResidentPlan p = xk_resident_plan(wpr, H, threads);
    return xk_res_lat_words(p) + 4LL * p.G * wpr + XK_TAB_WORDS;
}

template <bool BYTES, bool TORUS, int RF>
__global__ void __launch_bounds__(1024)
xk_k_life_resident(const LifeInst *__restrict__ insts, const void *in, void *out, void *mirror,
                   int generations, const int32_t *__restrict__ gens, uint32_t bfill,
                   unsigned int *__restrict__ bad)
{
    extern __shared__ uint32_t sm[];
    const LifeInst I = insts[blockIdx.x];
    if (gens) generations = gens[blockIdx.x];         // per-lattice generation counts
    const int wpr = I.wpr, H = I.H, W = I.W;
    const ResidentPlan p = xk_resident_plan(wpr, H, blockDim.x);
    uint32_t *lat = sm;
    uint32_t *halo = sm + xk_res_lat_words(p);       // [parity][band][first, last][wpr]
    uint32_t *tabs = halo + 4 * p.G * wpr;            // rule table
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    // load: global row-major -> band-interleaved shared layout
    if (BYTES) {
        // one thread per word: 32 bytes in two 16-byte loads when the row
        // segment is whole and aligned, byte by byte otherwise
        const uint8_t *src = (const uint8_t *)in + I.off;
        unsigned int flag = 0;
#pragma unroll 4
        for (int w = threadIdx.x; w < H * wpr; w += blockDim.x) {
            const int y = w / wpr, jj = w - y * wpr;
            const int b = y / p.L, i = y - b * p.L;
            const int x0 = jj * 32;
            const uint8_t *seg = src + (int64_t)y * W + x0;
            uint32_t word = 0;
            if (x0 + 32 <= W && ((uintptr_t)seg & 15u) == 0) {
                const uint4 lo = *(const uint4 *)seg, hi = *(const uint4 *)(seg + 16);
                const uint64_t q[4] = {((uint64_t)lo.y << 32) | lo.x, ((uint64_t)lo.w << 32) | lo.z,
                                       ((uint64_t)hi.y << 32) | hi.x, ((uint64_t)hi.w << 32) | hi.z};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    flag |= (q[k] & 0xFEFEFEFEFEFEFEFEull) != 0;
                    word |= (uint32_t)((q[k] * 0x0102040810204080ull) >> 56) << (8 * k);
                }
            } else {
                const int nb = min(32, W - x0);
                for (int k = 0; k < nb; ++k) {
                    const uint32_t v = seg[k];
                    flag |= v > 1u;
                    word |= (v != 0u) << k;
                }
            }
            lat[xk_res_at(p, b, i, jj)] = word;
        }
        if (flag) atomicOr(bad, 1u);
    } else {
        const uint32_t *src = (const uint32_t *)in + I.off;
        for (int w = threadIdx.x; w < H * wpr; w += blockDim.x) {
            const int y = w / wpr, jj = w - y * wpr;
            const int b = y / p.L, i = y - b * p.L;
            lat[xk_res_at(p, b, i, jj)] = src[w];
        }
    }
    if (threadIdx.x < 10) {
        // first-level multiplexer coefficients (LifeTable9) of this rule:
        // masks of dead D[n] = rule0 bit n, live L[n] = rule1 bit n - 1
        auto D = [&](int n) { return 0u - ((I.rule0 >> n) & 1u); };
        auto L = [&](int n) { return 0u - ((I.rule1 >> (n > 0 ? n - 1 : 0)) & 1u); };
        const int q = threadIdx.x;
        if (q < 8) {
            const uint32_t A = q < 4 ? D(2 * q) : L(2 * (q - 4));
            const uint32_t B = q < 4 ? D(2 * q + 1) : L(2 * (q - 4) + 1);
            tabs[2 * q] = A;
            tabs[2 * q + 1] = xk_mux_coef(A, B);
        } else if (q == 8) {
            tabs[16] = D(8);
        } else {
            tabs[17] = L(8);
            tabs[18] = xk_mux_coef(L(8), L(9));
        }
    }

    const int q = lane / p.P, j = lane - q * p.P;
    const int band = warp * p.gpw + q;
    const bool active = band < p.nb && j < wpr;
    // clamped indices: idle lanes read valid (ignored) words, so no load
    // needs a predicate
    const int bc = band < p.nb ? band : p.nb - 1;
    const int jc = j < wpr ? j : wpr - 1;
    const int y0 = bc * p.L;
    const int y1 = min(H, y0 + p.L);
    const int last = wpr - 1;
    const int gbase = q * p.P;
    const int src_l = gbase + (jc > 0 ? jc - 1 : last);
    const int src_r = gbase + (jc < last ? jc + 1 : 0);
    const int lshift = jc > 0 ? 31 : I.rlast - 1;
    const int lpre = 31 - lshift;
    const int top = jc == last ? I.rlast - 1 : 31;
    const uint32_t topbit = 1u << top;
    const uint32_t outmask = jc == last ? I.lastmask : 0xFFFFFFFFu;
    const uint32_t edge = bfill & 1u;
    const int use_le = (!TORUS) && jc == 0, use_re = (!TORUS) && jc == last;
    const int hup = bc > 0 ? bc - 1 : p.nb - 1;        // band holding the row above
    const int hdn = bc + 1 < p.nb ? bc + 1 : 0;         // band holding the row below
    const bool full = (H % p.L) == 0;                   // every band has L rows
    __syncthreads();
    LifeTable9 t9;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        t9.a[q] = tabs[2 * q];
        t9.k[q] = tabs[2 * q + 1];
    }
    t9.d8 = tabs[16];
    t9.a9 = tabs[17];
    t9.k9 = tabs[18];
    const auto &t = RuleForm<RF>::make(t9);   // RF != XK_RULE_TABLE: the table is not read

    const int hw = 2 * p.G * wpr;                      // halo words per parity
    // a band's first and last row into the halos of parity `par`
    const uint32_t *first_row = lat + xk_res_at(p, bc, 0, jc);
    const int last_off = 32 * (y1 - 1 - y0);            // warp-major: rows 32 words apart
    uint32_t *hslot = halo + (bc * 2) * wpr + jc;
    auto publish = [&](int par) {
        if (active) {
            hslot[par * hw] = first_row[0];
            hslot[par * hw + wpr] = first_row[last_off];
        }
    };
    publish(0);
    __syncthreads();
    for (int gen = 0; gen < generations; ++gen) {
        const uint32_t *hc = halo + (gen & 1) * hw;
        RowVec vu, vm, vd;
        const uint32_t wu = (!TORUS && bc == 0) ? bfill : hc[(hup * 2 + 1) * wpr + jc];
        const uint32_t wm = lat[xk_res_at(p, bc, 0, jc)];
        if (TORUS) {
            uint32_t l = __shfl_sync(0xFFFFFFFFu, wu, src_l), r = __shfl_sync(0xFFFFFFFFu, wu, src_r);
            vu = xk_torus_vec(wu, l, r, lpre, top, topbit);
            l = __shfl_sync(0xFFFFFFFFu, wm, src_l);
            r = __shfl_sync(0xFFFFFFFFu, wm, src_r);
            vm = xk_torus_vec(wm, l, r, lpre, top, topbit);
        } else {
            uint32_t l = __shfl_sync(0xFFFFFFFFu, wu, src_l), r = __shfl_sync(0xFFFFFFFFu, wu, src_r);
            vu = xk_row_vec(wu, l, r, lshift, top, edge, edge, use_le, use_re);
            if (bc == 0) vu.L = vu.C = vu.R = bfill;
            l = __shfl_sync(0xFFFFFFFFu, wm, src_l);
            r = __shfl_sync(0xFFFFFFFFu, wm, src_r);
            vm = xk_row_vec(wm, l, r, lshift, top, edge, edge, use_le, use_re);
        }
        if (TORUS && full) {
            // fast path: every band has exactly L rows; the word of the row
            // below comes from the band itself except for the band's last
            // row (halo).  Rows whose width is a multiple of 32 need no
            // partial-word handling: both neighbour vectors are one funnel
            // shift and no output mask applies.  The width test is uniform
            // per CTA and taken outside the row loop.
            uint32_t su = xk_lop3_xor3(vu.L, vu.C, vu.R), cu = xk_maj(vu.L, vu.C, vu.R);
            uint32_t sm_ = xk_lop3_xor3(vm.L, vm.C, vm.R), cm_ = xk_maj(vm.L, vm.C, vm.R);
            uint32_t Cm = vm.C;
            constexpr int stride = 32;                          // words between band rows
            uint32_t *wp = lat + xk_res_at(p, bc, 0, jc);       // this lane's word of row i
            const uint32_t whalo = hc[(hdn * 2 + 0) * wpr + jc];
            auto band_rows = [&](auto fullw_tag) {
                constexpr bool FULLW = decltype(fullw_tag)::value;
                auto row = [&](uint32_t wd, uint32_t *dst) {
                    const uint32_t l = __shfl_sync(0xFFFFFFFFu, wd, src_l);
                    const uint32_t r = __shfl_sync(0xFFFFFFFFu, wd, src_r);
                    uint32_t Ld, Rd;
                    if (FULLW) {
                        Ld = __funnelshift_l(l, wd, 1);
                        Rd = __funnelshift_r(wd, r, 1);
                    } else {
                        const RowVec d = xk_torus_vec(wd, l, r, lpre, top, topbit);
                        Ld = d.L;
                        Rd = d.R;
                    }
                    const uint32_t sd = xk_lop3_xor3(Ld, wd, Rd), cd = xk_maj(Ld, wd, Rd);
                    uint32_t out = xk_life_word9(su, cu, sm_, cm_, sd, cd, Cm, t);
                    if (!FULLW) out &= outmask;
                    if (active) *dst = out;
                    su = sm_;
                    cu = cm_;
                    sm_ = sd;
                    cm_ = cd;
                    Cm = wd;
                };
                if (p.L == 1) {
                    row(whalo, wp);
                    return;
                }
                uint32_t wd = wp[stride];
                uint32_t *dst = wp;
                const uint32_t *src = wp + 2 * stride;
                const uint32_t *src_end = wp + p.L * stride;
#pragma unroll 6
                for (; src < src_end; src += stride, dst += stride) {
                    const uint32_t wnext = *src;
                    row(wd, dst);
                    wd = wnext;
                }
                row(wd, dst);              // row L-2: row below is the band's last row
                row(whalo, dst + stride);  // row L-1: row below is the next band's first
            };
            if (I.rlast == 32) band_rows(std::true_type());
            else band_rows(std::false_type());
        } else {
            // general path: bands may be shorter than L; every lane still
            // runs L iterations so the shuffles always see the full warp
            for (int i = 0; i < p.L; ++i) {
                const int y = y0 + i;
                const bool row_ok = active && y < y1;
                uint32_t wd;
                bool off_d = false;
                if (y + 1 < y1) wd = lat[xk_res_at(p, bc, i + 1, jc)];
                else if (y + 1 < H) wd = hc[((bc + 1) * 2 + 0) * wpr + jc];
                else if (TORUS) wd = hc[(0 * 2 + 0) * wpr + jc];
                else { wd = bfill; off_d = true; }
                const uint32_t l = __shfl_sync(0xFFFFFFFFu, wd, src_l);
                const uint32_t r = __shfl_sync(0xFFFFFFFFu, wd, src_r);
                if (TORUS) {
                    vd = xk_torus_vec(wd, l, r, lpre, top, topbit);
                } else {
                    vd = xk_row_vec(wd, l, r, lshift, top, edge, edge, use_le, use_re);
                    if (off_d) vd.L = vd.C = vd.R = bfill;
                }
                const uint32_t out = xk_life_word9(
                    xk_lop3_xor3(vu.L, vu.C, vu.R), xk_maj(vu.L, vu.C, vu.R), xk_lop3_xor3(vm.L, vm.C, vm.R),
                    xk_maj(vm.L, vm.C, vm.R), xk_lop3_xor3(vd.L, vd.C, vd.R), xk_maj(vd.L, vd.C, vd.R), vm.C, t);
                if (row_ok) lat[xk_res_at(p, bc, i, jc)] = out & outmask;
                vu = vm;
                vm = vd;
            }
        }
        publish((gen & 1) ^ 1);
        __syncthreads();
    }
    if (BYTES) {
        uint8_t *dst = (uint8_t *)out + I.off;
        uint8_t *dst2 = mirror ? (uint8_t *)mirror + I.off : nullptr;
        for (int w = threadIdx.x; w < H * wpr; w += blockDim.x) {
            const int y = w / wpr, jj = w - y * wpr;
            const int b = y / p.L, i = y - b * p.L;
            const uint32_t word = lat[xk_res_at(p, b, i, jj)];
            const int x0 = jj * 32;
            const int64_t at = (int64_t)y * W + x0;
            uint8_t *seg = dst + at;
            if (x0 + 32 <= W && ((uintptr_t)seg & 15u) == 0 &&
                (!dst2 || ((uintptr_t)(dst2 + at) & 15u) == 0)) {
                uint64_t qq[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    uint64_t u = ((uint64_t)((word >> (8 * k)) & 0xFFu) * 0x0101010101010101ull) &
                                 0x8040201008040201ull;
                    qq[k] = ((u + 0x7F7F7F7F7F7F7F7Full) >> 7) & 0x0101010101010101ull;
                }
                const uint4 lo = make_uint4((uint32_t)qq[0], (uint32_t)(qq[0] >> 32), (uint32_t)qq[1],
                                            (uint32_t)(qq[1] >> 32));
                const uint4 hi = make_uint4((uint32_t)qq[2], (uint32_t)(qq[2] >> 32), (uint32_t)qq[3],
                                            (uint32_t)(qq[3] >> 32));
                *(uint4 *)seg = lo;
                *(uint4 *)(seg + 16) = hi;
                if (dst2) {
                    *(uint4 *)(dst2 + at) = lo;
                    *(uint4 *)(dst2 + at + 16) = hi;
                }
            } else {
                const int nb = min(32, W - x0);
                for (int k = 0; k < nb; ++k) seg[k] = (uint8_t)((word >> k) & 1u);
                if (dst2)
                    for (int k = 0; k < nb; ++k) dst2[at + k] = (uint8_t)((word >> k) & 1u);
            }
        }
    } else {
        uint32_t *dst = (uint32_t *)out + I.off;
        for (int w = threadIdx.x; w < H * wpr; w += blockDim.x) {
            const int y = w / wpr, jj = w - y * wpr;
            const int b = y / p.L, i = y - b * p.L;
            dst[w] = lat[xk_res_at(p, b, i, jj)];
        }
    }
}

template <bool BYTES, bool TORUS, int RF = XK_RULE_TABLE>
static cudaError_t xk_launch_resident(const LifeInst *inst, int ninst, const void *in, void *out,
                                      void *mirror, int generations, uint32_t bfill, unsigned int *bad,
                                      int threads, int smem_bytes, cudaStream_t s,
                                      const int32_t *gens = nullptr, int priority = XK_NO_PRIORITY)
{
    cudaError_t e = xk_smem_attr_at_least((const void *)xk_k_life_resident<BYTES, TORUS, RF>, smem_bytes);
    if (e != cudaSuccess || ninst <= 0) return e;
    if (priority == XK_NO_PRIORITY) {
        xk_k_life_resident<BYTES, TORUS, RF><<<ninst, threads, smem_bytes, s>>>(inst, in, out, mirror,
                                                                                generations, gens, bfill, bad);
        return cudaGetLastError();
    }
    // a launch priority (kept by a graph instantiated with node priorities)
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cudaLaunchAttribute attr;
    cfg.gridDim = dim3(ninst);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem_bytes;
    cfg.stream = s;
    attr.id = cudaLaunchAttributePriority;
    attr.val.priority = priority;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, xk_k_life_resident<BYTES, TORUS, RF>, inst, in, out, mirror, generations,
                              gens, bfill, bad);
}

// ninst == 0 only sets the kernel's shared-memory attribute (done before a
// graph capture, where attribute changes are not recorded)
cudaError_t xk_life_step_resident(const LifeInst *inst, int ninst, void *state, int bytes_io,
                                  int generations, int torus, uint32_t bfill, unsigned int *bad,
                                  int threads, int smem_bytes, cudaStream_t s, int rule_form, int priority)
{
    if (bytes_io && torus && priority != XK_NO_PRIORITY)
        return xk_launch_resident<true, true>(inst, ninst, state, state, nullptr, generations, bfill, bad,
                                              threads, smem_bytes, s, nullptr, priority);
    if (!bytes_io && rule_form == XK_RULE_CONWAY)
        return torus ? xk_launch_resident<false, true, XK_RULE_CONWAY>(inst, ninst, state, state, nullptr,
                                                                       generations, bfill, bad, threads,
                                                                       smem_bytes, s)
                     : xk_launch_resident<false, false, XK_RULE_CONWAY>(inst, ninst, state, state, nullptr,
                                                                        generations, bfill, bad, threads,
                                                                        smem_bytes, s);
    if (bytes_io)
        return torus ? xk_launch_resident<true, true>(inst, ninst, state, state, nullptr, generations,
                                                      bfill, bad, threads, smem_bytes, s)
                     : xk_launch_resident<true, false>(inst, ninst, state, state, nullptr, generations,
                                                       bfill, bad, threads, smem_bytes, s);
    return torus ? xk_launch_resident<false, true>(inst, ninst, state, state, nullptr, generations,
                                                   bfill, bad, threads, smem_bytes, s)
                 : xk_launch_resident<false, false>(inst, ninst, state, state, nullptr, generations,
                                                    bfill, bad, threads, smem_bytes, s);
}

cudaError_t xk_life_step_resident_each(const LifeInst *inst, const int32_t *gens, int ninst, void *state,
                                       unsigned int *bad, int threads, int smem_bytes, cudaStream_t s)
{
    return xk_launch_resident<true, true>(inst, ninst, state, state, nullptr, 0, 0u, bad, threads,
                                          smem_bytes, s, gens);
}

// CTAs of the one-byte torus resident kernel one SM holds at once
int xk_life_resident_ctas_per_sm(int threads, int smem_bytes)
{
    int n = 0;
    if (xk_smem_attr_at_least((const void *)xk_k_life_resident<true, true, XK_RULE_TABLE>, smem_bytes) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, xk_k_life_resident<true, true, XK_RULE_TABLE>, threads,
                                                      smem_bytes) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n;
}

cudaError_t xk_life_step_resident_io(const LifeInst *inst, int ninst, const uint8_t *in, uint8_t *out,
                                     uint8_t *mirror, int generations, unsigned int *bad, int threads,
                                     int smem_bytes, cudaStream_t s)
{
    return xk_launch_resident<true, true>(inst, ninst, in, out, mirror, generations, 0u, bad, threads,
                                          smem_bytes, s);
}

// ---------------------------------------------------------------------------
// layout conversion: reference main plane (esz bytes per cell, values 0/1)
// <-> bit-packed rows.  One warp builds one word with a ballot.

__device__ __forceinline__ uint64_t xk_load_cell(const void *src, int esz, int64_t i)
{
    switch (esz) {
    case 1: return ((const uint8_t *)src)[i];
    case 2: return ((const uint16_t *)src)[i];
    case 4: return ((const uint32_t *)src)[i];
    default: return ((const uint64_t *)src)[i];
    }
}

__device__ __forceinline__ void xk_store_cell(void *dst, int esz, int64_t i, uint64_t v)
{
    switch (esz) {
    case 1: ((uint8_t *)dst)[i] = (uint8_t)v; break;
    case 2: ((uint16_t *)dst)[i] = (uint16_t)v; break;
    case 4: ((uint32_t *)dst)[i] = (uint32_t)v; break;
    default: ((uint64_t *)dst)[i] = v; break;
    }
}

__global__ void xk_k_life_pack(const void *__restrict__ src, int esz, uint32_t *__restrict__ dst,
                               LifeGeo g, unsigned int *__restrict__ bad)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t word = t >> 5;
    if (word >= (int64_t)g.H * g.wpr) return;   // whole warps exit together
    const int lane = threadIdx.x & 31;
    const int y = (int)(word / g.wpr);
    const int j = (int)(word - (int64_t)y * g.wpr);
    const int x = j * 32 + lane;
    uint64_t v = 0;
    if (x < g.W) v = xk_load_cell(src, esz, (int64_t)y * g.W + x);
    if (v > 1u) atomicOr(bad, 1u);
    const uint32_t bits = __ballot_sync(0xFFFFFFFFu, v != 0);
    if (lane == 0) dst[word] = bits;
}

cudaError_t xk_life_pack(const void *src, int esz, uint32_t *dst, const LifeGeo &g, cudaStream_t s)
{
    // `bad` lives right after the packed words (the caller sizes the buffer)
    unsigned int *bad = (unsigned int *)(dst + (int64_t)g.H * g.wpr);
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    const int64_t threads_total = (int64_t)g.H * g.wpr * 32;
    const int threads = 256;
    xk_k_life_pack<<<(unsigned)((threads_total + threads - 1) / threads), threads, 0, s>>>(
        src, esz, dst, g, bad);
    return cudaGetLastError();
}

__global__ void xk_k_life_unpack(const uint32_t *__restrict__ src, void *__restrict__ dst, int esz,
                                 LifeGeo g)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)g.W * g.H) return;
    const int y = (int)(i / g.W), x = (int)(i - (int64_t)y * g.W);
    const uint32_t w = src[(int64_t)y * g.wpr + (x >> 5)];
    xk_store_cell(dst, esz, i, (w >> (x & 31)) & 1u);
}

cudaError_t xk_life_unpack(const uint32_t *src, void *dst, int esz, const LifeGeo &g, cudaStream_t s)
{
    const int64_t n = (int64_t)g.W * g.H;
    const int threads = 256;
    xk_k_life_unpack<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(src, dst, esz, g);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// colours of Life-like models: the traced colour is a function of the new
// state; lut6 = rgb of state 0 then of state 1 (before the effect).

__device__ __forceinline__ int xk_clamp_ma(int v, int old, int fade_in, int fade_out)
{
    // max(min(v, old + FADE_IN), old - FADE_OUT)  (color_effects.py:118-129)
    int m = v < old + fade_in ? v : old + fade_in;
    return m > old - fade_out ? m : old - fade_out;
}

struct Lut6 {
    int32_t v[6];
};

__global__ void xk_k_life_colors(const uint32_t *__restrict__ bits, int32_t *__restrict__ col,
                                 LifeGeo g, Lut6 lut, int smooth)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)g.W * g.H) return;
    const int y = (int)(i / g.W), x = (int)(i - (int64_t)y * g.W);
    const int s = (bits[(int64_t)y * g.wpr + (x >> 5)] >> (x & 31)) & 1;
    for (int c = 0; c < 3; ++c) col[3 * i + c] = lut.v[3 * s + c] * smooth;
}

cudaError_t xk_life_colors(const uint32_t *bits, int32_t *col, const LifeGeo &g,
                           const int32_t *lut6, int smooth, cudaStream_t s)
{
    Lut6 l;
    for (int c = 0; c < 6; ++c) l.v[c] = lut6[c];
    const int64_t n = (int64_t)g.W * g.H;
    xk_k_life_colors<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(bits, col, g, l, smooth);
    return cudaGetLastError();
}

__global__ void xk_k_life_color_step(const uint32_t *__restrict__ bits, int32_t *__restrict__ col,
                                     LifeGeo g, Lut6 lut, int fade_in, int fade_out, int smooth,
                                     int plain)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)g.W * g.H) return;
    const int y = (int)(i / g.W), x = (int)(i - (int64_t)y * g.W);
    const int s = (bits[(int64_t)y * g.wpr + (x >> 5)] >> (x & 31)) & 1;
    for (int c = 0; c < 3; ++c) {
        const int v = lut.v[3 * s + c];
        col[3 * i + c] = plain ? v : xk_clamp_ma(v * smooth, col[3 * i + c], fade_in, fade_out);
    }
}

cudaError_t xk_life_color_step(const uint32_t *bits, int32_t *col, const LifeGeo &g,
                               const int32_t *lut6, int fade_in, int fade_out, int smooth,
                               int plain, cudaStream_t s)
{
    Lut6 l;
    for (int c = 0; c < 6; ++c) l.v[c] = lut6[c];
    const int64_t n = (int64_t)g.W * g.H;
    xk_k_life_color_step<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(bits, col, g, l, fade_in,
                                                                        fade_out, smooth, plain);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// byte-per-cell lattices: any dimensionality and neighbourhood

__global__ void xk_k_nd_pack(const void *__restrict__ src, int esz, uint8_t *__restrict__ dst,
                             int64_t n, unsigned int *__restrict__ bad)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t v = xk_load_cell(src, esz, i);
    if (v > 1u) atomicOr(bad, 1u);
    dst[i] = (uint8_t)(v != 0);
}

cudaError_t xk_nd_pack(const void *src, int esz, uint8_t *dst, int64_t n, cudaStream_t s)
{
    unsigned int *bad = (unsigned int *)(dst + ((n + 15) / 16) * 16);
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    xk_k_nd_pack<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, esz, dst, n, bad);
    return cudaGetLastError();
}

__global__ void xk_k_nd_unpack(const uint8_t *__restrict__ src, void *__restrict__ dst, int esz,
                               int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xk_store_cell(dst, esz, i, src[i]);
}

cudaError_t xk_nd_unpack(const uint8_t *src, void *dst, int esz, int64_t n, cudaStream_t s)
{
    xk_k_nd_unpack<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, esz, n);
    return cudaGetLastError();
}

// index -> coords with axis 0 fastest (lattice.py:146-170); neighbour k at
// coords + delta_k, wrapped (border.py:104-117) or off-board (static value).
__global__ void xk_k_life_nd(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst, NdGeo g,
                             uint32_t rule0, uint32_t rule1, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t x[XK_MAXDIM];
    int64_t rem = i;
    for (int d = 0; d < g.ndim; ++d) {
        if (d < g.ndim - 1) { x[d] = rem % g.size[d]; rem /= g.size[d]; }
        else x[d] = rem;
    }
    uint32_t alive = 0;
    for (int k = 0; k < g.nbr; ++k) {
        int64_t idx = 0, stride = 1;
        bool off = false;
        for (int d = 0; d < g.ndim; ++d) {
            int64_t c = x[d] + g.delta[k][d];
            if (c < 0 || c >= g.size[d]) {
                off = true;
                c = (c + g.size[d]) % g.size[d];
            }
            idx += c * stride;
            stride *= g.size[d];
        }
        alive += (off && !g.torus) ? g.border_state : src[idx];
    }
    const uint32_t rule = src[i] ? rule1 : rule0;
    dst[i] = (uint8_t)((rule >> alive) & 1u);
}

cudaError_t xk_life_step_nd(const uint8_t *src, uint8_t *dst, const NdGeo &g, uint32_t rule0,
                            uint32_t rule1, cudaStream_t s)
{
    int64_t n = 1;
    for (int d = 0; d < g.ndim; ++d) n *= g.size[d];
    xk_k_life_nd<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, g, rule0, rule1, n);
    return cudaGetLastError();
}

// plain 2-D Moore torus on bytes: the reference's one-byte-per-cell layout,
// one launch per lattice per generation (the "plain form" of the ensemble)
__global__ void xk_k_life_bytes2d(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst, int W,
                                  int H, uint32_t rule0, uint32_t rule1)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)W * H) return;
    const int y = (int)(i / W), x = (int)(i - (int64_t)y * W);
    const int xl = x > 0 ? x - 1 : W - 1, xr = x < W - 1 ? x + 1 : 0;
    const int yu = y > 0 ? y - 1 : H - 1, yd = y < H - 1 ? y + 1 : 0;
    const uint8_t *ru = src + (int64_t)yu * W, *rm = src + (int64_t)y * W, *rd = src + (int64_t)yd * W;
    const uint32_t k = ru[xl] + ru[x] + ru[xr] + rm[xl] + rm[xr] + rd[xl] + rd[x] + rd[xr];
    const uint32_t rule = rm[x] ? rule1 : rule0;
    dst[i] = (uint8_t)((rule >> k) & 1u);
}

cudaError_t xk_life_step_bytes2d(const uint8_t *src, uint8_t *dst, int W, int H, uint32_t rule0,
                                 uint32_t rule1, cudaStream_t s)
{
    const int64_t n = (int64_t)W * H;
    xk_k_life_bytes2d<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, W, H, rule0, rule1);
    return cudaGetLastError();
}

__global__ void xk_k_nd_colors(const uint8_t *__restrict__ st, int32_t *__restrict__ col, int64_t n,
                               Lut6 lut, int smooth)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = st[i];
    for (int c = 0; c < 3; ++c) col[3 * i + c] = lut.v[3 * s + c] * smooth;
}

cudaError_t xk_nd_colors(const uint8_t *st, int32_t *col, int64_t n, const int32_t *lut6,
                         int smooth, cudaStream_t s)
{
    Lut6 l;
    for (int c = 0; c < 6; ++c) l.v[c] = lut6[c];
    xk_k_nd_colors<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(st, col, n, l, smooth);
    return cudaGetLastError();
}

__global__ void xk_k_nd_color_step(const uint8_t *__restrict__ st, int32_t *__restrict__ col,
                                   int64_t n, Lut6 lut, int fade_in, int fade_out, int smooth,
                                   int plain)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = st[i];
    for (int c = 0; c < 3; ++c) {
        const int v = lut.v[3 * s + c];
        col[3 * i + c] = plain ? v : xk_clamp_ma(v * smooth, col[3 * i + c], fade_in, fade_out);
    }
}

cudaError_t xk_nd_color_step(const uint8_t *st, int32_t *col, int64_t n, const int32_t *lut6,
                             int fade_in, int fade_out, int smooth, int plain, cudaStream_t s)
{
    Lut6 l;
    for (int c = 0; c < 6; ++c) l.v[c] = lut6[c];
    xk_k_nd_color_step<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(st, col, n, l, fade_in,
                                                                     fade_out, smooth, plain);
    return cudaGetLastError();
}
