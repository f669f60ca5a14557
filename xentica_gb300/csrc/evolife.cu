// EvoLife generation kernel for sm_103a.
//
// Restates, per cell and in the same operation order, the absorb + colour
// program the reference generates for EvoLife (examples/evolife.py:20-128,
// tools/genetics.py:7-56, tools/color.py:8-125):
//   cell = energy (9 bits) | rule (18 bits) << 9 | rng (16 bits) << 27, uint64
//   (properties.py:496-541); 2-D Moore torus, neighbour k at the reference's
//   delta order (-1,-1) (-1,0) (-1,1) (0,-1) (0,1) (1,-1) (1,0) (1,1).
// Emit copies energy and rule to every buffer, so a neighbour's buffer is its
// main state: emit is fused away and the kernel reads neighbours directly
// (ping-pong state buffers).  Every read of the cell's RandomProperty advances
// x = (x * 58321 + 11113) % 65535 (properties.py:638-660): once for the start
// gene, then once per gene (twice with mutation).  Floats follow IEEE
// round-to-nearest with no contraction (__fdiv_rn, __fmul_rn, __fadd_rn).
//
// The crossover's draws depend only on the cell's 16-bit random state x0 at
// the start of the crossover and on the number n of parents: the start gene,
// and for every gene which parent wins it (and, with mutation, whether it
// mutates).  So for every (x0, n) the winners are precomputed once per
// process, on the device, as n "won-gene masks" W_s (bit g of W_s set when
// gene g is taken from parent slot s), 9.4 MB that stay in L2; a cell's
// crossover is then OR_s(parent_s & W_s) -- the genes in visiting order,
// before the max_genes cut -- followed by keeping the first max_genes set
// genes in visiting order and the mutation flips.  The state after the
// crossover is one composed affine map of x0.
#include <string.h>

#include <map>
#include <mutex>
#include <utility>

#include "xk_internal.cuh"

// GenomeColor.positional weights (double) per gene and channel
__constant__ double c_evo_pos[18 * 3];

__device__ __forceinline__ uint32_t xk_lcg(uint32_t x) { return (x * 58321u + 11113u) % 65535u; }

// float -> unsigned int as the GPU converts: truncation, NaN -> 0
__device__ __forceinline__ uint32_t xk_f2u(float v) { return __float2uint_rz(v); }

// bit j of the result = bit (s + j) mod 18 of v (v < 2^18, s < 18), and back
__device__ __forceinline__ uint32_t xk_rot18(uint32_t v, uint32_t s)
{
    return ((v >> s) | (v << (18u - s))) & 0x3FFFFu;
}

__device__ __forceinline__ uint32_t xk_unrot18(uint32_t w, uint32_t s)
{
    return ((w << s) | (w >> (18u - s))) & 0x3FFFFu;
}

__device__ __forceinline__ int xk_ma_clamp(int v, int old, int fade_in, int fade_out)
{
    int m = v < old + fade_in ? v : old + fade_in;
    return m > old - fade_out ? m : old - fade_out;
}

// hsv2rgb(hue, 1, 1) with deferred hue (tools/color.py:8-60) of the modular
// genome colour's hue (rule >> 1) % 360: the float channels before EvoLife's
// energy weighting
__device__ __forceinline__ void xk_evo_hue_rgb(uint32_t hue, float *out)
{
    float hue_f = 0.0f;
    hue_f = __fadd_rn(hue_f, __fmul_rn(__fdiv_rn((float)hue, 360.0f), 6.0f));
    uint32_t hue_i = 0;
    hue_i += xk_f2u(hue_f);
    hue_f = __fsub_rn(hue_f, (float)hue_i);
    float sat = 0.0f;
    sat = __fadd_rn(sat, 1.0f);
    float val = 0.0f;
    val = __fadd_rn(val, 1.0f);
    float grad_p = 0.0f, grad_q = 0.0f, grad_t = 0.0f;
    grad_p = __fadd_rn(grad_p, __fmul_rn(val, __fsub_rn(1.0f, sat)));
    grad_q = __fadd_rn(grad_q, __fmul_rn(val, __fsub_rn(1.0f, __fmul_rn(sat, hue_f))));
    grad_t = __fadd_rn(grad_t, __fmul_rn(val, __fsub_rn(1.0f, __fmul_rn(sat, __fsub_rn(1.0f, hue_f)))));
    float r = __fmul_rn((float)((hue_i == 0) | (hue_i >= 5)), val);
    r = __fadd_rn(r, __fmul_rn((float)(hue_i == 1), grad_q));
    r = __fadd_rn(r, __fmul_rn((float)((hue_i == 2) | (hue_i == 3)), grad_p));
    r = __fadd_rn(r, __fmul_rn((float)(hue_i == 4), grad_t));
    float g = __fmul_rn((float)((hue_i == 0) | (hue_i >= 6)), grad_t);
    g = __fadd_rn(g, __fmul_rn((float)((hue_i == 1) | (hue_i == 2)), val));
    g = __fadd_rn(g, __fmul_rn((float)(hue_i == 3), grad_q));
    g = __fadd_rn(g, __fmul_rn((float)((hue_i == 4) | (hue_i == 5)), grad_p));
    float b = __fmul_rn((float)(((hue_i == 0) | (hue_i == 1)) | (hue_i >= 6)), grad_p);
    b = __fadd_rn(b, __fmul_rn((float)(hue_i == 2), grad_t));
    b = __fadd_rn(b, __fmul_rn((float)((hue_i == 3) | (hue_i == 4)), val));
    b = __fadd_rn(b, __fmul_rn((float)(hue_i == 5), grad_q));
    out[0] = r;
    out[1] = g;
    out[2] = b;
}

// the 360 hues' channels, computed once per device context by the same
// operations (xk_k_evo_hues) and read per cell
__global__ void xk_k_evo_hues(float4 *__restrict__ hues)
{
    const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= 360u) return;
    float c[3];
    xk_evo_hue_rgb(h, c);
    hues[h] = make_float4(c[0], c[1], c[2], 0.0f);
}

// modular genome colour with the energy weighting of EvoLife.color
// (evolife.py:431-444)
__device__ __forceinline__ void xk_evo_color_modular(const float4 *__restrict__ hues, uint32_t rule,
                                                     uint32_t energy, int *rgb)
{
    const float4 c = __ldg(hues + (rule >> 1) % 360u);
    const int e = (255 - (int)energy) * ((int)(rule > 0) * (int)(energy < 255));
    rgb[0] = (int)xk_f2u(__fmul_rn(c.x, (float)e));
    rgb[1] = (int)xk_f2u(__fmul_rn(c.y, (float)e));
    rgb[2] = (int)xk_f2u(__fmul_rn(c.z, (float)e));
}

// GenomeColor.positional (tools/color.py:63-104): double weights added into
// float variables, then normalised by the float maximum
__device__ __forceinline__ void xk_evo_color_positional(uint32_t rule, uint32_t energy, int *rgb)
{
    float red = 0.0f, green = 0.0f, blue = 0.0f;
#pragma unroll
    for (int i = 0; i < 18; ++i) {
        if ((rule >> i) & 1u) {
            red = __double2float_rn(__dadd_rn((double)red, c_evo_pos[3 * i]));
            green = __double2float_rn(__dadd_rn((double)green, c_evo_pos[3 * i + 1]));
            blue = __double2float_rn(__dadd_rn((double)blue, c_evo_pos[3 * i + 2]));
        }
    }
    float maxval = 0.0f;
    const float m01 = red > green ? red : green;
    maxval = __fadd_rn(maxval, m01 > blue ? m01 : blue);
    red = __fdiv_rn(red, maxval);
    green = __fdiv_rn(green, maxval);
    blue = __fdiv_rn(blue, maxval);
    const int e = (255 - (int)energy) * ((int)(rule > 0) * (int)(energy < 255));
    rgb[0] = (int)xk_f2u(__fmul_rn(red, (float)e));
    rgb[1] = (int)xk_f2u(__fmul_rn(green, (float)e));
    rgb[2] = (int)xk_f2u(__fmul_rn(blue, (float)e));
}

// The random draws of the crossover are u(x) = RN(x / 65535) of the 16-bit
// state x in [0, 65534]: a parent index trunc(RN(u(x) * n)) for n parents,
// the start gene trunc(RN(u(x) * 18)) % 8, and a mutation iff u(x) <= t.
// For each n (and 18) there is a multiplier K with floor(x * K / 2^32) equal
// to the float expression for every x -- found once per process on the host
// by trying multipliers near n * 2^32 / 65535 against all 65535 states with
// the same IEEE single-precision operations -- so a draw is one umulhi.  The
// mutation test is monotonic in x: x <= mut_x.
struct EvoParams {
    int32_t W, H;
    uint32_t death_speed, max_genes;
    int32_t mut_x;             // largest x with u(x) <= t (-1: none)
    int32_t mutation;          // mutation_prob > 0
    int32_t positional;
    int32_t color_kind;        // XK_COLOR_*
    int32_t fade_in, fade_out, smooth;
    uint32_t kmul[9];          // parent draw for 0..8 parents (0: none)
    uint32_t kstart;           // start-gene draw (n = 18)
    uint32_t jump_a, jump_c;   // the crossover's RNG advances as one map x -> (a x + c) % 65535
    const uint32_t *won;       // won-gene masks: n masks per x0, blocks of 65536 x0 per n
    const uint32_t *mut;       // mutation flips per x0 (mutation only)
    const float4 *hues;        // modular colour channels per hue
    uint8_t *frame;            // null, or the W x H RendererPlain frame (zoom 1, no offset)
    int32_t frame_smooth;      // its SMOOTH_FACTOR (0: none)
};

static float evo_u(uint32_t x) { return (float)x / 65535.0f; }

// K with floor(x * K / 2^32) == trunc(RN(u(x) * n)) for all x in [0, 65534]
static uint32_t evo_find_multiplier(uint32_t n)
{
    static uint32_t want[65535];
    for (uint32_t x = 0; x < 65535; ++x) want[x] = (uint32_t)(evo_u(x) * (float)n);
    const uint64_t base = ((uint64_t)n << 32) / 65535;
    for (uint64_t d = 0; d < 65536; ++d)
        for (int sign = 0; sign < 2; ++sign) {
            const int64_t k = (int64_t)base + (sign ? -(int64_t)d : (int64_t)d);
            if (k <= 0 || k > 0xFFFFFFFFLL) continue;
            bool ok = true;
            for (uint32_t x = 0; x < 65535 && ok; ++x)
                ok = (uint32_t)(((uint64_t)x * (uint64_t)k) >> 32) == want[x];
            if (ok) return (uint32_t)k;
        }
    return 0;   // not reached for n <= 18 (checked by the EvoLife GPU tests)
}

// The crossover advances the RNG once for the start gene and once (twice
// with mutation) per gene: 19 or 37 applications of x -> (58321 x + 11113)
// mod 65535, composed into one affine map.  For every 16-bit x the composed
// a x + c stays below 2^32 (a, c < 65535).
static void evo_jump(EvoParams &p)
{
    const uint64_t m = 65535;
    uint64_t a = 1, c = 0;
    const int steps = 1 + 18 * (p.mutation ? 2 : 1);
    for (int k = 0; k < steps; ++k) {
        a = (58321 * a) % m;
        c = (58321 * c + 11113) % m;
    }
    p.jump_a = (uint32_t)a;
    p.jump_c = (uint32_t)c;
}

static std::once_flag g_evo_once;
static uint32_t g_evo_k[9], g_evo_kstart;

static void evo_draws(EvoParams &p, float mut_thresh)
{
    std::call_once(g_evo_once, [] {
        g_evo_k[0] = 0;
        for (uint32_t n = 1; n <= 8; ++n) g_evo_k[n] = evo_find_multiplier(n);
        g_evo_kstart = evo_find_multiplier(18);
    });
    memcpy(p.kmul, g_evo_k, sizeof(p.kmul));
    p.kstart = g_evo_kstart;
    if (!(evo_u(0) <= mut_thresh)) {
        p.mut_x = -1;
        return;
    }
    uint32_t lo = 0, hi = 65534;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) / 2;
        if (evo_u(mid) <= mut_thresh) lo = mid;
        else hi = mid - 1;
    }
    p.mut_x = (int32_t)lo;
}

// ---------------------------------------------------------------------------
// crossover tables

struct EvoDraws {
    uint32_t kmul[9], kstart;
};

// won-gene masks of every (x0, n): thread t = x0 + 65536 (n - 1) replays the
// crossover's draws from x0 -- one advance for the start gene, then per
// visited gene one advance and a parent draw (and one more advance with
// mutation) -- and writes its n masks at 32768 n (n - 1) + n x0
__global__ void xk_k_evo_won(uint32_t *__restrict__ won, EvoDraws d, int mutation)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 65536u * 8u) return;
    const uint32_t x0 = t & 65535u, n = (t >> 16) + 1u;
    uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t x = xk_lcg(x0);
    const uint32_t start = __umulhi(x, d.kstart) % 8u;
    for (uint32_t j = 0; j < 18; ++j) {
        x = xk_lcg(x);
        const uint32_t win = __umulhi(x, d.kmul[n]);      // < n for every state
        const uint32_t gene = start + j < 18u ? start + j : start + j - 18u;
#pragma unroll
        for (uint32_t s = 0; s < 8; ++s) w[s] |= (uint32_t)(s == win) << gene;
        if (mutation) x = xk_lcg(x);
    }
    uint32_t *o = won + 32768u * n * (n - 1u) + x0 * n;
#pragma unroll
    for (uint32_t s = 0; s < 8; ++s)
        if (s < n) o[s] = w[s];
}

// mutation flips of every x0 (genes whose second draw is <= mut_x), in
// gene order
__global__ void xk_k_evo_mut(uint32_t *__restrict__ mut, int32_t mut_x, uint32_t kstart)
{
    const uint32_t x0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (x0 >= 65536u) return;
    uint32_t x = xk_lcg(x0);
    const uint32_t start = __umulhi(x, kstart) % 8u;
    uint32_t m = 0;
    for (uint32_t j = 0; j < 18; ++j) {
        x = xk_lcg(xk_lcg(x));
        const uint32_t gene = start + j < 18u ? start + j : start + j - 18u;
        m |= (uint32_t)((int32_t)x <= mut_x) << gene;
    }
    mut[x0] = m;
}

namespace {
struct EvoTables {
    float4 *hues = nullptr;
    uint32_t *won[2] = {nullptr, nullptr};     // without / with mutation
    std::map<int32_t, uint32_t *> mut;        // per mut_x
};
std::mutex g_evo_tab_mu;
std::map<std::pair<int, unsigned long long>, EvoTables> g_evo_tabs;   // per device and context
}  // namespace

// the tables for p's draws, built on first use in this device context (the
// stream is synchronised once so that every stream may use them)
static cudaError_t evo_tables(EvoParams &p, cudaStream_t s)
{
    std::lock_guard<std::mutex> lk(g_evo_tab_mu);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    EvoTables &t = g_evo_tabs[std::make_pair(dev, xk_context_id())];
    EvoDraws d;
    memcpy(d.kmul, p.kmul, sizeof(d.kmul));
    d.kstart = p.kstart;
    bool built = false;
    if (!t.hues) {
        if ((e = cudaMalloc(&t.hues, 360 * sizeof(float4))) != cudaSuccess) {
            t.hues = nullptr;
            return e;
        }
        xk_k_evo_hues<<<2, 192, 0, s>>>(t.hues);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        built = true;
    }
    p.hues = t.hues;
    uint32_t *&won = t.won[p.mutation ? 1 : 0];
    if (!won) {
        if ((e = cudaMalloc(&won, 65536u * 36u * sizeof(uint32_t))) != cudaSuccess) {
            won = nullptr;
            return e;
        }
        xk_k_evo_won<<<65536u * 8u / 256u, 256, 0, s>>>(won, d, p.mutation);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        built = true;
    }
    p.won = won;
    p.mut = nullptr;
    if (p.mutation) {
        auto it = t.mut.find(p.mut_x);
        if (it == t.mut.end()) {
            uint32_t *m = nullptr;
            if ((e = cudaMalloc(&m, 65536u * sizeof(uint32_t))) != cudaSuccess) return e;
            xk_k_evo_mut<<<65536u / 256u, 256, 0, s>>>(m, p.mut_x, p.kstart);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            it = t.mut.emplace(p.mut_x, m).first;
            built = true;
        }
        p.mut = it->second;
    }
    return built ? cudaStreamSynchronize(s) : cudaSuccess;
}

#define XK_EVO_BX 32
#define XK_EVO_BY 8
#ifndef XK_EVO_MINB
#define XK_EVO_MINB 8     // CTAs per SM the registers are cut for (32 per thread): latency hiding for
                          // the crossover's table lookups, which come from L2
#endif

// MUT: mutation_prob > 0 (the mutation flips, and the union of the parents'
// genomes they are masked with, exist only then)
template <bool MUT>
__global__ void __launch_bounds__(XK_EVO_BX * XK_EVO_BY, XK_EVO_MINB)
xk_k_evolife(const uint64_t *__restrict__ src, uint64_t *__restrict__ dst, int32_t *__restrict__ col,
             EvoParams p)
{
    const int x = blockIdx.x * XK_EVO_BX + threadIdx.x;
    const int y = blockIdx.y * XK_EVO_BY + threadIdx.y;
    if (x >= p.W || y >= p.H) return;   // no block-wide synchronisation below
    xk_grid_dep_wait();                 // launched as a dependent of the previous generation
    const int xl = x > 0 ? x - 1 : p.W - 1, xr = x < p.W - 1 ? x + 1 : 0;
    const int yu = y > 0 ? y - 1 : p.H - 1, yd = y < p.H - 1 ? y + 1 : 0;
    const int nxs[8] = {xl, xl, xl, x, x, xr, xr, xr};
    const int nys[8] = {yu, y, yd, yu, yd, yu, y, yd};
    // a neighbour's energy (bits 0-8) and rule (bits 9-26) are both in the
    // low 32-bit half of its cell: only that half is read
    const uint32_t *src_lo = reinterpret_cast<const uint32_t *>(src);
    uint32_t nr[8], nlo[8];
    uint32_t num_neighbors = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        nlo[k] = __ldg(src_lo + 2 * ((int64_t)nys[k] * p.W + nxs[k]));
        nr[k] = (nlo[k] >> 9) & 262143u;
        num_neighbors += (nlo[k] & 0x7FFFFFFu) != 0u;   // xmath.min(1, e + r): e + r != 0
    }
    const int64_t i = (int64_t)y * p.W + x;
    const uint64_t c = src[i];
    uint32_t energy = (uint32_t)(c & 511u);
    uint32_t rule = (uint32_t)((c >> 9) & 262143u);
    uint32_t rng = (uint32_t)((c >> 27) & 65535u);
    const uint32_t is_sustained = ((rule & 261120u) >> (num_neighbors + 9)) & 1u;
    // num_parents for every birth count 1..8 at once, bit-sliced: lane g of
    // the 4-bit counts (b3 b2 b1 b0) counts the neighbours whose rule has
    // bit g + 1 (a dead neighbour has rule 0).  Carry-save adder tree over
    // the eight 8-lane words.
    uint32_t m[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) m[k] = (nlo[k] >> 10) & 255u;
    const uint32_t s0 = m[0] ^ m[1] ^ m[2], c0 = (m[0] & m[1]) | (m[2] & (m[0] ^ m[1]));
    const uint32_t s1 = m[3] ^ m[4] ^ m[5], c1 = (m[3] & m[4]) | (m[5] & (m[3] ^ m[4]));
    const uint32_t s2 = m[6] ^ m[7], c2 = m[6] & m[7];
    const uint32_t b0 = s0 ^ s1 ^ s2, c3 = (s0 & s1) | (s2 & (s0 ^ s1));
    const uint32_t t0 = c0 ^ c1 ^ c2, d0 = (c0 & c1) | (c2 & (c0 ^ c1));
    const uint32_t b1 = t0 ^ c3, d1 = t0 & c3;
    const uint32_t b2 = d0 ^ d1, b3 = d0 & d1;
    // lane g has a fit when its count equals g + 1 (bit planes of g + 1 per
    // lane: 0x55, 0x66, 0x78, 0x80); num_fit = the largest such g + 1
    const uint32_t eq = ~(b0 ^ 0x55u) & ~(b1 ^ 0x66u) & ~(b2 ^ 0x78u) & ~(b3 ^ 0x80u) & 255u;
    const uint32_t num_fit = 32u - (uint32_t)__clz(eq);
    // parents: rules with the winning birth count, in neighbour order.  The
    // neighbours' birth bytes packed four to a word; bit num_fit - 1 of
    // each byte gathered into a nibble by one multiply (the products of the
    // four bits land on bits 24..27 without carries)
    uint32_t pmask = 0, any = 0;
    if (num_fit != 0) {
        const uint32_t f = num_fit - 1u;
        const uint32_t M0 = __byte_perm(__byte_perm(m[0], m[1], 0x0040), __byte_perm(m[2], m[3], 0x0040), 0x5410);
        const uint32_t M1 = __byte_perm(__byte_perm(m[4], m[5], 0x0040), __byte_perm(m[6], m[7], 0x0040), 0x5410);
        const uint32_t lo = (((M0 >> f) & 0x01010101u) * 0x01020408u) >> 24;
        const uint32_t hi = (((M1 >> f) & 0x01010101u) * 0x01020408u) >> 24;
        pmask = lo | (hi << 4);
    }
    if (MUT) {
#pragma unroll
        for (int k = 0; k < 8; ++k) any |= nr[k] * ((pmask >> k) & 1u);
    }
    const uint32_t n = __popc(pmask);
    const uint32_t old_rule = rule, old_energy = energy;
    // genome_crossover(main, 18, *genomes, max_genes, mutation_prob).  With
    // no parent, every gene is 0 (no winner, and a mutation needs a gene that
    // some parent has): only the RNG advances, by the composed map.
    uint32_t new_genome = 0;
    const uint32_t x0 = rng;
    rng = (p.jump_a * rng + p.jump_c) % 65535u;
    if (n != 0) {
        const uint32_t start_gene = __umulhi(xk_lcg(x0), p.kstart) % 8u;
        const uint32_t *w = p.won + 32768u * n * (n - 1) + x0 * n;
        uint32_t raw = 0, slot = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if ((pmask >> k) & 1u) raw |= nr[k] & __ldg(w + slot++);
        // the first max_genes genes taken, in visiting order (from
        // start_gene, wrapping at 18): keep the lowest set bits of the
        // rotated word
        uint32_t rot = xk_rot18(raw, start_gene);
        for (int e = __popc(rot) - (int)p.max_genes; e > 0; --e)
            rot &= ~(0x80000000u >> __clz(rot));
        new_genome = xk_unrot18(rot, start_gene);
        if (MUT) new_genome ^= __ldg(p.mut + x0) & any;
    }
    // the reference's selections by multiplication, as selects (the same
    // integers): a new genome replaces the rule and resets the energy, a
    // cell that does not live keeps neither
    rule = new_genome != 0 ? new_genome : rule;
    const bool is_live = old_energy < 255u && ((old_energy + old_rule) == 0u || is_sustained != 0u);
    const uint32_t new_energy = old_energy + ((old_energy + old_rule) != 0u ? p.death_speed : 0u);
    energy = rule == old_rule && is_live ? (uint16_t)new_energy : 0u;
    rule = is_live ? rule : 0u;
    if (p.color_kind != XK_COLOR_NONE) {
        int rgb[3];
        if (p.positional) xk_evo_color_positional(rule, energy, rgb);
        else xk_evo_color_modular(p.hues, rule, energy, rgb);
        if (p.color_kind == XK_COLOR_MOVING_AVERAGE) {
#pragma unroll
            for (int ch = 0; ch < 3; ++ch)
                rgb[ch] = xk_ma_clamp(rgb[ch] * p.smooth, col[3 * i + ch], p.fade_in, p.fade_out);
        }
        col[3 * i] = rgb[0];
        col[3 * i + 1] = rgb[1];
        col[3 * i + 2] = rgb[2];
        if (p.frame) {
            // the pixel of this cell as RendererPlain computes it at zoom 1
            // (render.cu): the colour as a float, / SMOOTH_FACTOR, truncated,
            // its low byte.  Below 2^24 in magnitude int -> float -> int is
            // exact, and so is a division by 1: with SMOOTH_FACTOR 1 (or none)
            // such a pixel is the colour's low byte
            const bool small = (((uint32_t)rgb[0] + (1u << 24)) | ((uint32_t)rgb[1] + (1u << 24)) |
                                ((uint32_t)rgb[2] + (1u << 24))) < (1u << 25);   // all three
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                const int c = rgb[ch];
                uint8_t px;
                if (p.frame_smooth <= 1 && small) {
                    px = (uint8_t)c;
                } else {
                    float v = (float)c;
                    if (p.frame_smooth > 0) v = __fdiv_rn(v, (float)p.frame_smooth);
                    px = (uint8_t)(int)v;
                }
                p.frame[3 * i + ch] = px;
            }
        }
    }
    // energy | rule << 9 | rng << 27 (fields masked, so + and | agree) as two halves
    const uint32_t rn = rng & 65535u;
    reinterpret_cast<uint2 *>(dst)[i] = make_uint2((energy & 511u) | ((rule & 262143u) << 9) | (rn << 27), rn >> 5);
}

cudaError_t xk_evolife_set_positional(const double *lut54)
{
    return cudaMemcpyToSymbol(c_evo_pos, lut54, 54 * sizeof(double));
}

cudaError_t xk_evolife_step(const uint64_t *src, uint64_t *dst, int32_t *col, const xk_desc &d,
                            float mut_thresh, cudaStream_t s, uint8_t *frame, int frame_smooth)
{
    EvoParams p;
    p.W = (int32_t)d.size[0];
    p.H = (int32_t)d.size[1];
    p.death_speed = d.death_speed;
    p.max_genes = d.max_genes;
    p.mutation = d.mutation_prob > 0.0;
    p.positional = d.positional;
    p.color_kind = d.color_kind;
    p.fade_in = d.fade_in;
    p.fade_out = d.fade_out;
    p.smooth = d.smooth;
    p.frame = frame;
    p.frame_smooth = frame_smooth;
    evo_draws(p, mut_thresh);
    evo_jump(p);
    cudaError_t e = evo_tables(p, s);
    if (e != cudaSuccess) return e;
    dim3 block(XK_EVO_BX, XK_EVO_BY);
    dim3 grid((p.W + XK_EVO_BX - 1) / XK_EVO_BX, (p.H + XK_EVO_BY - 1) / XK_EVO_BY);
    return p.mutation ? xk_launch_pdl(xk_k_evolife<true>, grid, block, 0, s, src, dst, col, p)
                      : xk_launch_pdl(xk_k_evolife<false>, grid, block, 0, s, src, dst, col, p);
}
