// Word-level Life-like logic shared by the bit-sliced kernels (life.cu,
// cluster.cu): 32 cells per 32-bit word, neighbour counts from carry-save
// adders and the rule from a multiplexer tree over warp-uniform masks (its
// first level as integer multiply-adds, LifeTable).
#pragma once

#include <stdint.h>

#include "xk_internal.cuh"

// Three-input boolean functions as single lop3 instructions (PTX lop3.b32:
// the immediate is the function evaluated on a = 0xF0, b = 0xCC, c = 0xAA).
__device__ __forceinline__ uint32_t xk_lop3_mux(uint32_t sel, uint32_t a, uint32_t b)
{
    uint32_t d;   // sel ? b : a, bitwise
    asm("lop3.b32 %0, %1, %2, %3, 0xAC;" : "=r"(d) : "r"(sel), "r"(a), "r"(b));
    return d;
}

__device__ __forceinline__ uint32_t xk_lop3_maj(uint32_t a, uint32_t b, uint32_t c)
{
    uint32_t d;   // majority: carry of a full adder
    asm("lop3.b32 %0, %1, %2, %3, 0xE8;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

__device__ __forceinline__ uint32_t xk_lop3_xor3(uint32_t a, uint32_t b, uint32_t c)
{
    uint32_t d;   // sum of a full adder
    asm("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

__device__ __forceinline__ uint32_t xk_mux(uint32_t sel, uint32_t a, uint32_t b)
{
    return xk_lop3_mux(sel, a, b);
}

__device__ __forceinline__ uint32_t xk_maj(uint32_t a, uint32_t b, uint32_t c)
{
    return xk_lop3_maj(a, b, c);
}

// sel ? B : A for warp-uniform masks A, B (0 or ~0) given as A and
// k = xk_mux_coef(A, B): one integer multiply-add
__device__ __forceinline__ uint32_t xk_imux(uint32_t sel, uint32_t a, uint32_t k)
{
    return sel * k + a;
}

// Next state of 32 cells.  (Lu, Cu, Ru) are the row above shifted so that bit
// b holds the up-left, up and up-right neighbour of cell b; (Lm, Rm) the left
// and right neighbours; (Ld, Cd, Rd) the row below; Cm the cells themselves.
template <class Tab>
__device__ __forceinline__ uint32_t xk_life_word(uint32_t Lu, uint32_t Cu, uint32_t Ru,
                                                 uint32_t Lm, uint32_t Cm, uint32_t Rm,
                                                 uint32_t Ld, uint32_t Cd, uint32_t Rd,
                                                 const Tab &t)
{
    // neighbour count k = b0 + 2 b1 + 4 b2 + 8 b3 (k <= 8, so b3 implies k == 8)
    const uint32_t su = xk_lop3_xor3(Lu, Cu, Ru), cu = xk_maj(Lu, Cu, Ru);
    const uint32_t sd = xk_lop3_xor3(Ld, Cd, Rd), cd = xk_maj(Ld, Cd, Rd);
    const uint32_t sm = Lm ^ Rm, cm = Lm & Rm;
    const uint32_t b0 = xk_lop3_xor3(su, sd, sm), k1 = xk_maj(su, sd, sm);
    const uint32_t tw = xk_lop3_xor3(cu, cd, cm), k2 = xk_maj(cu, cd, cm);
    const uint32_t b1 = tw ^ k1, k3 = tw & k1;
    const uint32_t b2 = k2 ^ k3, b3 = k2 & k3;
    // rule lookup: multiplexer tree over (state, b2, b1, b0), then b3
    uint32_t m[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) m[q] = xk_imux(b0, t.a[q], t.k[q]);
    uint32_t n[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) n[q] = xk_mux(b1, m[2 * q], m[2 * q + 1]);
    const uint32_t dead = xk_mux(b2, n[0], n[1]);
    const uint32_t live = xk_mux(b2, n[2], n[3]);
    const uint32_t low = xk_mux(Cm, dead, live);
    const uint32_t eight = xk_imux(Cm, t.a8, t.k8);
    return xk_mux(b3, low, eight);
}

// Same as xk_life_word, with the rows above and below already reduced to
// their column sums: (su, cu) = FA(Lu, Cu, Ru) and (sd, cd) = FA(Ld, Cd, Rd).
// A row's sums are computed once and reused while it is the row below and,
// two rows later, the row above.
template <class Tab>
__device__ __forceinline__ uint32_t xk_life_word_fa(uint32_t su, uint32_t cu, uint32_t Lm,
                                                    uint32_t Cm, uint32_t Rm, uint32_t sd,
                                                    uint32_t cd, const Tab &t)
{
    const uint32_t sm = Lm ^ Rm, cm = Lm & Rm;
    const uint32_t b0 = xk_lop3_xor3(su, sd, sm), k1 = xk_maj(su, sd, sm);
    const uint32_t tw = xk_lop3_xor3(cu, cd, cm), k2 = xk_maj(cu, cd, cm);
    const uint32_t b1 = tw ^ k1, k3 = tw & k1;
    const uint32_t b2 = k2 ^ k3, b3 = k2 & k3;
    uint32_t m[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) m[q] = xk_imux(b0, t.a[q], t.k[q]);
    uint32_t n[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) n[q] = xk_mux(b1, m[2 * q], m[2 * q + 1]);
    const uint32_t dead = xk_mux(b2, n[0], n[1]);
    const uint32_t live = xk_mux(b2, n[2], n[3]);
    const uint32_t low = xk_mux(Cm, dead, live);
    const uint32_t eight = xk_imux(Cm, t.a8, t.k8);
    return xk_mux(b3, low, eight);
}

// The rule stage: next state of 32 cells from the bits of the 3 x 3 block
// count n9 = b0 + 2 b1 + 4 b2 + 8 b3 (the cell included; b3: n9 is 8 or 9,
// so b1 = b2 = 0) and the cells themselves (C).  A rule loaded at run time
// (LifeTable9): a multiplexer tree over warp-uniform masks, its first level
// as integer multiply-adds.
__device__ __forceinline__ uint32_t xk_rule9(const LifeTable9 &t, uint32_t b0, uint32_t b1, uint32_t b2,
                                             uint32_t b3, uint32_t C)
{
    uint32_t m[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) m[q] = xk_imux(b0, t.a[q], t.k[q]);
    uint32_t n[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) n[q] = xk_mux(b1, m[2 * q], m[2 * q + 1]);
    const uint32_t dead = xk_mux(b2, n[0], n[1]);
    const uint32_t live = xk_mux(b2, n[2], n[3]);
    const uint32_t low = xk_mux(C, dead, live);
    const uint32_t high = xk_mux(C, t.d8, xk_imux(b0, t.a9, t.k9));
    return xk_mux(b3, low, high);
}

// A rule fixed at compile time: a dead cell is born with k neighbours iff
// bit k of B is set, a live cell survives with k iff bit k of S is set (the
// golly int B | S << 9 of LifelikeCA).  The same multiplexer tree written in
// plain C over compile-time masks: the compiler folds every constant leaf,
// so Conway's B3/S23 takes about four logic instructions instead of the
// eighteen of a rule loaded at run time.
template <uint32_t B, uint32_t S>
struct FixedRule9 {
    static constexpr uint32_t born = B, sustain = S;
};

__device__ __forceinline__ uint32_t xk_cmux(uint32_t sel, uint32_t a, uint32_t b)
{
    return (a & ~sel) | (b & sel);
}

template <uint32_t B, uint32_t S>
__device__ __forceinline__ uint32_t xk_rule9(const FixedRule9<B, S> &, uint32_t b0, uint32_t b1, uint32_t b2,
                                             uint32_t b3, uint32_t C)
{
    // dead cell: D(n9) = born bit n9; live cell: L(n9) = sustain bit n9 - 1
    auto D = [](int n) -> uint32_t { return n <= 8 && ((B >> n) & 1u) ? 0xFFFFFFFFu : 0u; };
    auto L = [](int n) -> uint32_t { return n >= 1 && ((S >> (n - 1)) & 1u) ? 0xFFFFFFFFu : 0u; };
    uint32_t m[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
        m[q] = q < 4 ? xk_cmux(b0, D(2 * q), D(2 * q + 1)) : xk_cmux(b0, L(2 * (q - 4)), L(2 * (q - 4) + 1));
    uint32_t n[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) n[q] = xk_cmux(b1, m[2 * q], m[2 * q + 1]);
    const uint32_t dead = xk_cmux(b2, n[0], n[1]);
    const uint32_t live = xk_cmux(b2, n[2], n[3]);
    const uint32_t low = xk_cmux(C, dead, live);
    const uint32_t high = xk_cmux(C, D(8), xk_cmux(b0, L(8), L(9)));
    return xk_cmux(b3, low, high);
}

// Next state of 32 cells from the column sums (s, c) = FA(L, C, R) of the
// rows above (u), at (m) and below (d) -- the 3 x 3 block including the cell
// -- and the cells themselves (C).  A row's sums are computed once, when it
// is the row below, and reused twice; the count n9 = (su + sm + sd) +
// 2 (cu + cm + cd) <= 9 needs one fewer logic instruction than the
// neighbour count of xk_life_word_fa, and the rule is indexed by it (a
// LifeTable9 or a FixedRule9).
template <class Rule>
__device__ __forceinline__ uint32_t xk_life_word9(uint32_t su, uint32_t cu, uint32_t sm, uint32_t cm,
                                                  uint32_t sd, uint32_t cd, uint32_t C, const Rule &t)
{
    const uint32_t b0 = xk_lop3_xor3(su, sm, sd), k1 = xk_maj(su, sm, sd);
    const uint32_t tw = xk_lop3_xor3(cu, cm, cd), k2 = xk_maj(cu, cm, cd);
    const uint32_t b1 = tw ^ k1, k3 = tw & k1;
    const uint32_t b2 = k2 ^ k3, b3 = k2 & k3;
    return xk_rule9(t, b0, b1, b2, b3, C);
}

// the rule form's rule object (XK_RULE_* in xk_internal.cuh)
template <int RF>
struct RuleForm {
    typedef LifeTable9 type;
    __device__ static const LifeTable9 &make(const LifeTable9 &t) { return t; }
};

template <>
struct RuleForm<XK_RULE_CONWAY> {
    typedef FixedRule9<8u, 12u> type;
    __device__ static FixedRule9<8u, 12u> make(const LifeTable9 &) { return FixedRule9<8u, 12u>(); }
};

// Neighbour vectors of word j of a row, given the row's word and the words
// left and right of it (already wrapped).  lshift: bit of `left` that is
// the cell left of bit 0; top: bit of R that receives the cell right of the
// word's last cell.
struct RowVec {
    uint32_t L, C, R;
};

__device__ __forceinline__ RowVec xk_row_vec(uint32_t c, uint32_t left, uint32_t right,
                                             int lshift, int top, uint32_t ledge, uint32_t redge,
                                             int use_ledge, int use_redge)
{
    RowVec v;
    uint32_t lb = use_ledge ? ledge : ((left >> lshift) & 1u);
    uint32_t rb = use_redge ? redge : (right & 1u);
    v.C = c;
    v.L = (c << 1) | lb;
    v.R = (c >> 1) | (rb << top);
    return v;
}

// neighbour vectors of a torus row: left bit taken from `left` (already the
// wrapped neighbour word), right bit from `right`; lpre moves the left
// neighbour's bit to position 31, top / topbit place the right neighbour
// after the row's last cell
__device__ __forceinline__ RowVec xk_torus_vec(uint32_t c, uint32_t left, uint32_t right, int lpre,
                                               int top, uint32_t topbit)
{
    RowVec v;
    v.C = c;
    v.L = __funnelshift_l(left << lpre, c, 1);
    v.R = (c >> 1) | ((right << top) & topbit);
    return v;
}

// Band layout of a lattice held in shared memory (life.cu's resident kernel,
// cluster.cu): a group of P = next_pow2(wpr) lanes covers one row, the rows
// are cut into bands of L consecutive rows, one per group, and local row i
// of band b, column word jj, sits at ((b / gpw) * L + i) * 32 + (b % gpw) * P
// + jj (warp-major: a lane's next row is always 32 words further on).
struct ResidentPlan {
    int P, gpw, G, L, nb;  // lanes per group, groups per warp, groups, band length, live bands
};

// shared word of local row i, column word jj of band b (warp-major layout)
__host__ __device__ __forceinline__ int xk_res_at(const ResidentPlan &p, int b, int i, int jj)
{
    return ((b / p.gpw) * p.L + i) * 32 + (b % p.gpw) * p.P + jj;
}

// shared words of the lattice area: L rows of 32 words per warp holding bands
__host__ __device__ __forceinline__ int64_t xk_res_lat_words(const ResidentPlan &p)
{
    return (int64_t)p.L * ((p.G + p.gpw - 1) / p.gpw) * 32;
}

__host__ __device__ inline ResidentPlan xk_resident_plan(int wpr, int H, int threads)
{
    ResidentPlan p;
    int P = 1;
    while (P < wpr) P <<= 1;
    p.P = P;
    p.gpw = 32 / P;
    int groups = (threads / 32) * p.gpw;
    if (groups > H) groups = H;
    p.G = groups;
    p.L = (H + groups - 1) / groups;
    p.nb = (H + p.L - 1) / p.L;
    return p;
}
