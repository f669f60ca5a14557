/*
 * oracle.c -- CPU restatement of Xentica's buffered-state CA generation step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the CUDA product
 * path never links, loads or calls it.  Only the tests, the smoke check and the
 * CPU-baseline leg of the benchmark use it, and only as the checker.
 *
 * It restates, in plain C on the reference's own memory layout, what the
 * reference's translator-generated kernels compute:
 *
 *   fld  : n * (N + 1) + 1 elements of the packed cell type
 *          (reference xentica/core/base.py:660-661): plane 0 is the main
 *          state, planes 1..N the emit buffers;
 *   col  : n int3 colours (base.py:659), rewritten by absorb.
 *
 * emit  (base.py:461-473): per cell, unpack main (properties.py:496-514), run
 *        the model's emit, pack each buffer and store it in plane
 *        rev_index_map[k] + 1 (base.py:226-230, properties.py:516-541).
 * absorb (base.py:475-487): per cell, index -> coords (lattice.py:146-170),
 *        neighbour k at coords + delta_k (neighborhood.py:122-148), torus wrap
 *        (border.py:104-117) or static off-board container value
 *        (border.py:144-151, properties.py:444-483), read the neighbour's
 *        buffer plane k + 1, run the model's absorb and the colour effect
 *        (color_effects.py:66-82, :106-130), pack and store main.
 * render (renderers.py:220-270): viewport pixel -> lattice coords with float
 *        zoom, view wrap, float accumulation over the projected axes.
 *
 * All loops are written the way the generated C computes them (same integer
 * types, promotions and float operation order), with OpenMP over cells; emit
 * and absorb only write cells they own, so the thread count cannot change a
 * result.  Build: see oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define XO_MAXDIM 16

typedef struct {
    int ndim;                   /* lattice dimensionality                     */
    int64_t size[XO_MAXDIM];    /* size per axis, axis 0 fastest              */
    int nbr;                    /* number of neighbours N                     */
    const int8_t *delta;        /* N x ndim neighbour offsets                 */
    const int32_t *rev;         /* rev_index_map, N entries                   */
    int torus;                  /* 1: TorusBorder, 0: StaticBorder            */
    uint64_t border_value;      /* StaticBorder whole-container value         */
} xo_topo;

typedef struct { int32_t fade_in, fade_out, smooth; int moving_average; } xo_color;

static int64_t xo_cells(const xo_topo *t)
{
    int64_t n = 1;
    for (int d = 0; d < t->ndim; ++d) n *= t->size[d];
    return n;
}

/* lattice.py:146-170 (index -> coords) */
static void xo_coords(const xo_topo *t, int64_t i, int64_t *x)
{
    for (int d = 0; d < t->ndim; ++d) {
        if (d < t->ndim - 1) { x[d] = i % t->size[d]; i /= t->size[d]; }
        else x[d] = i;
    }
}

/* Neighbour k of the cell at x: returns its index, or -1 when it is off the
 * board of a StaticBorder lattice (neighborhood.py:122-148, border.py:104-117,
 * lattice.py:206-221). */
static int64_t xo_neighbor(const xo_topo *t, const int64_t *x, int k)
{
    int64_t nx[XO_MAXDIM];
    int off = 0;
    for (int d = 0; d < t->ndim; ++d) {
        nx[d] = x[d] + t->delta[k * t->ndim + d];
        if (nx[d] < 0 || nx[d] >= t->size[d]) off = 1;
    }
    if (off) {
        if (!t->torus) return -1;
        for (int d = 0; d < t->ndim; ++d) nx[d] = (nx[d] + t->size[d]) % t->size[d];
    }
    int64_t idx = 0, stride = 1;
    for (int d = 0; d < t->ndim; ++d) { idx += nx[d] * stride; stride *= t->size[d]; }
    return idx;
}

static uint64_t xo_load(const void *fld, int esz, int64_t i)
{
    switch (esz) {
    case 1: return ((const uint8_t *)fld)[i];
    case 2: return ((const uint16_t *)fld)[i];
    case 4: return ((const uint32_t *)fld)[i];
    default: return ((const uint64_t *)fld)[i];
    }
}

static void xo_store(void *fld, int esz, int64_t i, uint64_t v)
{
    switch (esz) {
    case 1: ((uint8_t *)fld)[i] = (uint8_t)v; break;
    case 2: ((uint16_t *)fld)[i] = (uint16_t)v; break;
    case 4: ((uint32_t *)fld)[i] = (uint32_t)v; break;
    default: ((uint64_t *)fld)[i] = v; break;
    }
}

/* MovingAverage (color_effects.py:106-130) or plain ColorEffect (:66-82). */
static void xo_color_write(int32_t *col, int64_t i, int r, int g, int b, const xo_color *c)
{
    if (c->moving_average) {
        int v[3] = {r * c->smooth, g * c->smooth, b * c->smooth};
        for (int ch = 0; ch < 3; ++ch) {
            int old = col[3 * i + ch];
            int lo = old - c->fade_out, hi = old + c->fade_in;
            int m = v[ch] < hi ? v[ch] : hi;
            v[ch] = m > lo ? m : lo;
        }
        r = v[0]; g = v[1]; b = v[2];
    }
    col[3 * i] = r; col[3 * i + 1] = g; col[3 * i + 2] = b;
}

/* ------------------------------------------------------------------------ */
/* Life-like family: one IntegerProperty ``state`` of ``bits`` bits at shift 0,
 * emit broadcasts it (examples/game_of_life.py:42-53), absorb sums the
 * neighbour buffers into an ``unsigned int`` and applies
 *   state = ((B >> k) & 1) | ((S >> k) & 1) & state
 * which is GameOfLife's (B=8, S=12, game_of_life.py:55-70) and LifelikeCA's
 * (B = rule, S = rule >> 9, game_of_life.py:190-197) absorb.  The colour
 * of a cell is a per-state table (lut6: rgb of state 0, then of state 1),
 * e.g. state * 255 on every channel for GameOfLife (game_of_life.py:72-90). */
void xo_life_step(const xo_topo *t, void *fld, int esz, int bits,
                  uint32_t born, uint32_t sustain, int32_t *col,
                  const xo_color *cc, const int32_t *lut6, int threads)
{
    const int64_t n = xo_cells(t);
    const uint64_t mask = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
    /* emit: every buffer gets the unpacked state, re-packed with the mask */
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t s = xo_load(fld, esz, i) & mask;
        for (int k = 0; k < t->nbr; ++k)
            xo_store(fld, esz, i + n * (int64_t)(t->rev[k] + 1), s & mask);
    }
    /* absorb */
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t x[XO_MAXDIM];
        xo_coords(t, i, x);
        uint32_t alive = 0;
        for (int k = 0; k < t->nbr; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            uint64_t v = j < 0 ? t->border_value : xo_load(fld, esz, j + n * (int64_t)(k + 1));
            alive += (uint32_t)(v & mask);
        }
        uint64_t s = xo_load(fld, esz, i) & mask;
        uint64_t ns = (uint64_t)(((born >> alive) & 1u) | (((sustain >> alive) & 1u) & (uint32_t)s));
        const int32_t *rgb = lut6 + 3 * (ns & 1u);
        xo_color_write(col, i, rgb[0], rgb[1], rgb[2], cc);
        xo_store(fld, esz, i, ns & mask);
    }
}

/* ------------------------------------------------------------------------ */
/* ShiftingSands (examples/shifting_sands.py:15-47): a 1-bit ``state``; emit
 * writes it into one buffer and 0 into the others (the buffer that lands in
 * plane ``plane0``, 1..N, after the rev_index_map placement), absorb sums the
 * neighbours' buffers (the off-board container for an off-board neighbour)
 * into an int, the colour effect sees that int, and the state stores it
 * masked to 1 bit.  ``lut`` holds the rgb for every sum 0..N. */
void xo_shift_step(const xo_topo *t, void *fld, int esz, int plane0, int32_t *col,
                   const xo_color *cc, const int32_t *lut, int threads)
{
    const int64_t n = xo_cells(t);
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t s = xo_load(fld, esz, i) & 1u;
        for (int p = 1; p <= t->nbr; ++p) xo_store(fld, esz, i + n * (int64_t)p, p == plane0 ? s : 0u);
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t x[XO_MAXDIM];
        xo_coords(t, i, x);
        int new_val = 0;
        for (int k = 0; k < t->nbr; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            uint64_t v = j < 0 ? t->border_value : xo_load(fld, esz, j + n * (int64_t)(k + 1));
            new_val += (int)(v & 1u);
        }
        const int32_t *rgb = lut + 3 * new_val;
        xo_color_write(col, i, rgb[0], rgb[1], rgb[2], cc);
        xo_store(fld, esz, i, (uint64_t)new_val & 1u);
    }
}

/* ------------------------------------------------------------------------ */
/* GameOfLifeColor (examples/game_of_life.py:112-159): a uint32 cell packs
 * state (1 bit) | red << 1 | green << 9 | blue << 17, LSB first in
 * declaration order (properties.py:496-541).  emit copies every field into
 * every buffer (:125-131); absorb runs GameOfLife's absorb (:55-70) on the
 * states, then each channel becomes the sum over the neighbours' buffers of
 * (channel + 1) in an unsigned int, times the new state, stored into its
 * 8-bit field (:133-151); the colour (MovingAverage, :153-159) is state *
 * channel per channel.  An off-board neighbour reads as the whole border
 * container. */
void xo_lifecolor_step(const xo_topo *t, uint32_t *fld, int32_t *col, const xo_color *cc, int threads)
{
    const int64_t n = xo_cells(t);
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t v = fld[i];
        const uint32_t packed = (v & 1u) + (((v >> 1) & 255u) << 1) + (((v >> 9) & 255u) << 9) +
                                (((v >> 17) & 255u) << 17);
        for (int k = 0; k < t->nbr; ++k) fld[i + n * (int64_t)(t->rev[k] + 1)] = packed;
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t x[XO_MAXDIM];
        xo_coords(t, i, x);
        uint32_t alive = 0, rs = 0, gs = 0, bs = 0;
        for (int k = 0; k < t->nbr; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            uint32_t v = j < 0 ? (uint32_t)t->border_value : fld[j + n * (int64_t)(k + 1)];
            alive += v & 1u;
            rs += ((v >> 1) & 255u) + 1u;
            gs += ((v >> 9) & 255u) + 1u;
            bs += ((v >> 17) & 255u) + 1u;
        }
        const uint32_t s = fld[i] & 1u;
        const uint32_t ns = ((8u >> alive) & 1u) | (((12u >> alive) & 1u) & s);
        const uint32_t r = (uint8_t)(rs * ns), g = (uint8_t)(gs * ns), b = (uint8_t)(bs * ns);
        xo_color_write(col, i, (int)(ns * r), (int)(ns * g), (int)(ns * b), cc);
        fld[i] = (ns & 1u) + ((r & 255u) << 1) + ((g & 255u) << 9) + ((b & 255u) << 17);
    }
}

/* ------------------------------------------------------------------------ */
/* Mass transfer (3-D von Neumann, StaticBorder(WALL)): the model added for the
 * sand-transfer configuration, written in the reference DSL (see
 * tests/golden/ref_models.py:MassTransfer).  uint32 cell = mass.
 *   emit  : buffers[k].mass = (mass / 7) * (neighbors[k].main.mass != WALL)
 *   absorb: mass = mass - sum_k buffers[k].mass
 *                + sum_k nb_k * (nb_k != WALL),  nb_k = neighbors[k].buffer.mass
 *   color : v = min(mass * 32, 255) on every channel, plain ColorEffect. */
void xo_mass_step(const xo_topo *t, uint32_t *fld, int32_t *col, uint32_t wall,
                  int threads)
{
    const int64_t n = xo_cells(t);
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t x[XO_MAXDIM];
        xo_coords(t, i, x);
        uint32_t m = fld[i];
        for (int k = 0; k < t->nbr; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            uint32_t nm = j < 0 ? (uint32_t)t->border_value : fld[j];
            fld[i + n * (int64_t)(t->rev[k] + 1)] = (m / 7u) * (uint32_t)(nm != wall);
        }
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t x[XO_MAXDIM];
        xo_coords(t, i, x);
        uint32_t out = 0, in = 0;
        for (int k = 0; k < t->nbr; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            uint32_t nb = j < 0 ? (uint32_t)t->border_value : fld[j + n * (int64_t)(k + 1)];
            in += nb * (uint32_t)(nb != wall);
        }
        for (int k = 0; k < t->nbr; ++k) out += fld[i + n * (int64_t)(t->rev[k] + 1)];
        uint32_t m = fld[i] - out + in;
        uint32_t v32 = m * 32u;
        int c = (int)(v32 < 255u ? v32 : 255u);
        col[3 * i] = c; col[3 * i + 1] = c; col[3 * i + 2] = c;
        fld[i] = m;
    }
}

/* ------------------------------------------------------------------------ */
/* EvoLife (examples/evolife.py:20-128): uint64 cell = energy(9) | rule(18) << 9
 * | rng(16) << 27 (properties.py:496-541).  2-D Moore torus, N = 8.
 * RandomProperty: every read of main.rng advances x = (x * 58321 + 11113) %
 * 65535 (properties.py:638-660); genome_crossover (tools/genetics.py:7-56)
 * reads it once, then once (or twice with mutation) per gene. */
static inline uint32_t xo_lcg(uint32_t x) { return ((x * 58321u) + 11113u) % 65535u; }

typedef struct {
    uint32_t death_speed, max_genes;
    double mutation_prob;       /* > 0 adds the mutation draw per gene      */
    int positional;             /* 0: GenomeColor.modular, 1: .positional   */
    const double *pos_lut;      /* positional: 18 x 3 channel weights        */
} xo_evo;

/* hsv2rgb with Deferred operands (tools/color.py:8-60), GenomeColor.modular
 * (color.py:106-125): every intermediate is a float variable or expression. */
static void xo_evo_color_modular(uint32_t rule, uint32_t energy, int *rgb)
{
    float hue_f = 0.0f;
    hue_f += ((float)((rule >> 1) % 360u) / (float)360) * 6;
    uint32_t hue_i = 0;
    hue_i += (uint32_t)hue_f;
    hue_f -= (float)hue_i;
    float sat = 0.0f; sat += 1;
    float val = 0.0f; val += 1;
    float grad_p = 0.0f; grad_p += val * (1 - sat);
    float grad_q = 0.0f; grad_q += val * (1 - sat * hue_f);
    float grad_t = 0.0f; grad_t += val * (1 - sat * (1 - hue_f));
    float r = (float)((hue_i == 0) | (hue_i >= 5)) * val;
    r = r + (float)(hue_i == 1) * grad_q;
    r = r + (float)((hue_i == 2) | (hue_i == 3)) * grad_p;
    r = r + (float)(hue_i == 4) * grad_t;
    float g = (float)((hue_i == 0) | (hue_i >= 6)) * grad_t;
    g = g + (float)((hue_i == 1) | (hue_i == 2)) * val;
    g = g + (float)(hue_i == 3) * grad_q;
    g = g + (float)((hue_i == 4) | (hue_i == 5)) * grad_p;
    float b = (float)(((hue_i == 0) | (hue_i == 1)) | (hue_i >= 6)) * grad_p;
    b = b + (float)(hue_i == 2) * grad_t;
    b = b + (float)((hue_i == 3) | (hue_i == 4)) * val;
    b = b + (float)(hue_i == 5) * grad_q;
    int e = (255 - (int)energy) * ((int)(rule > 0) * (int)(energy < 255));
    rgb[0] = (int)(uint32_t)(r * (float)e);
    rgb[1] = (int)(uint32_t)(g * (float)e);
    rgb[2] = (int)(uint32_t)(b * (float)e);
}

/* float -> unsigned int conversion as the GPU does it: truncate, NaN and
 * negatives give 0 (the values here are never negative). */
static uint32_t xo_f2u(float v) { return (v != v || v <= 0.0f) ? 0u : (uint32_t)v; }

/* GenomeColor.positional (color.py:63-104): 18 hue-weighted genes summed in
 * double and stored into float variables, then normalised by their max. */
static void xo_evo_color_positional(uint32_t rule, uint32_t energy, const double *lut, int *rgb)
{
    float red = 0.0f, green = 0.0f, blue = 0.0f;
    for (int i = 0; i < 18; ++i) {
        int bit = (int)((rule >> i) & 1u);
        red = (float)((double)red + lut[3 * i] * bit);
        green = (float)((double)green + lut[3 * i + 1] * bit);
        blue = (float)((double)blue + lut[3 * i + 2] * bit);
    }
    float maxval = 0.0f;
    float m01 = red > green ? red : green;
    maxval += (m01 > blue ? m01 : blue);
    red /= maxval; green /= maxval; blue /= maxval;
    int e = (255 - (int)energy) * ((int)(rule > 0) * (int)(energy < 255));
    rgb[0] = (int)xo_f2u(red * (float)e);
    rgb[1] = (int)xo_f2u(green * (float)e);
    rgb[2] = (int)xo_f2u(blue * (float)e);
}

void xo_evolife_step(const xo_topo *t, uint64_t *fld, int32_t *col,
                     const xo_evo *p, const xo_color *cc, int threads)
{
    const int64_t n = xo_cells(t);
    /* emit (evolife.py:364-368): buffers get energy and rule; the buffer's rng
     * field is packed from an unset local and is never read back. */
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t c = fld[i];
        uint64_t v = (c & 511u) + (((c >> 9) & 262143u) << 9);
        for (int k = 0; k < t->nbr; ++k) fld[i + n * (int64_t)(t->rev[k] + 1)] = v;
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t x[XO_MAXDIM];
        xo_coords(t, i, x);
        uint32_t ne[8], nr[8], alive[8];
        uint32_t num_neighbors = 0;
        for (int k = 0; k < 8; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            uint64_t v = j < 0 ? t->border_value : fld[j + n * (int64_t)(k + 1)];
            ne[k] = (uint32_t)(v & 511u);
            nr[k] = (uint32_t)((v >> 9) & 262143u);
            uint32_t s = ne[k] + nr[k];
            alive[k] = 1u < s ? 1u : s;             /* xmath.min(1, e + r) */
            num_neighbors += alive[k];
        }
        uint64_t c = fld[i];
        uint32_t energy = (uint32_t)(c & 511u);
        uint32_t rule = (uint32_t)((c >> 9) & 262143u);
        uint32_t rng = (uint32_t)((c >> 27) & 65535u);
        /* is_sustained: ((rule & 261120) >> (k + 9)) & 1 (properties.py:572-585) */
        uint32_t is_sustained = ((rule & 261120u) >> (num_neighbors + 9)) & 1u;
        uint32_t fit[8];
        for (int gene = 0; gene < 8; ++gene) {
            uint32_t num_parents = 0;
            for (int k = 0; k < 8; ++k)
                num_parents += alive[k] * (((nr[k] & 510u) >> (gene + 1)) & 1u);
            fit[gene] = num_parents * (uint32_t)(num_parents == (uint32_t)(gene + 1));
        }
        uint32_t num_fit = fit[0];                  /* xmath.max, left fold */
        for (int gene = 1; gene < 8; ++gene) num_fit = num_fit > fit[gene] ? num_fit : fit[gene];
        uint32_t genome[8];
        for (int k = 0; k < 8; ++k) genome[k] = nr[k] * (((nr[k] & 510u) >> num_fit) & 1u);
        uint32_t old_rule = rule, old_energy = energy;
        /* genome_crossover(main, 18, *genomes, max_genes, mutation_prob) */
        rng = xo_lcg(rng);
        uint32_t start_gene = ((uint32_t)(((float)rng / (float)65535) * (float)18)) % 8u;
        uint32_t new_genome = 0, num_active = 0;
        for (uint32_t g = 0; g < 18; ++g) {
            uint32_t gene = (g + start_gene) % 18u;
            uint32_t gene_choose = 0, num_genomes = 0;
            for (int k = 0; k < 8; ++k) {
                gene_choose += (((genome[k] >> gene) & 1u) & (uint32_t)(genome[k] > 0)) << num_genomes;
                num_genomes += (uint32_t)(genome[k] > 0);
            }
            rng = xo_lcg(rng);
            uint32_t winner = (uint32_t)(((float)rng / (float)65535) * (float)num_genomes);
            uint32_t new_gene = (gene_choose >> winner) & 1u;
            num_active += new_gene;
            new_gene *= (uint32_t)(num_active <= p->max_genes);
            uint32_t mutated = 0;
            if (p->mutation_prob > 0) {
                rng = xo_lcg(rng);
                mutated = (uint32_t)((double)((float)rng / (float)65535) < p->mutation_prob)
                          * (uint32_t)(gene_choose > 0);
            }
            new_genome += (new_gene ^ mutated) << gene;
        }
        rule = new_genome + rule * (uint32_t)(new_genome == 0);
        uint32_t is_live = (uint32_t)(old_energy < 255u)
                           & ((uint32_t)((old_energy + old_rule) == 0) | is_sustained);
        uint32_t new_energy = old_energy + p->death_speed * (uint32_t)((old_energy + old_rule) != 0);
        /* main.energy was zeroed, so the second product vanishes */
        energy = (uint16_t)(new_energy * (uint32_t)(rule == old_rule));
        rule = old_rule * (uint32_t)(rule == old_rule) + rule * (uint32_t)(rule != old_rule);
        energy = (uint16_t)(energy * is_live);
        rule = rule * is_live;
        int rgb[3];
        if (p->positional) xo_evo_color_positional(rule, energy, p->pos_lut, rgb);
        else xo_evo_color_modular(rule, energy, rgb);
        xo_color_write(col, i, rgb[0], rgb[1], rgb[2], cc);
        fld[i] = ((uint64_t)energy & 511u) + (((uint64_t)rule & 262143u) << 9)
                 + (((uint64_t)rng & 65535u) << 27);
    }
}

/* ------------------------------------------------------------------------ */
/* NoiseTV (examples/noisetv.py:13-31): a uint16 cell holding one
 * RandomProperty; emit does nothing; absorb reads main.rng (one advance of
 * x = (x * 58321 + 11113) % 65535, properties.py:638-660) and the colour
 * reads its uniform (a second advance), (unsigned)((float)x / 65535 * 255)
 * on every channel; the cell stores x after both.  No neighbour is read. */
void xo_noise_step(const xo_topo *t, uint16_t *fld, int32_t *col, const xo_color *cc, int threads)
{
    const int64_t n = xo_cells(t);
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t x = fld[i];
        x = xo_lcg(xo_lcg(x));
        const float u = (float)x / 65535.0f;
        const int v = (int)(unsigned int)(u * 255.0f);
        xo_color_write(col, i, v, v, v, cc);
        fld[i] = (uint16_t)x;
    }
}

/* ------------------------------------------------------------------------ */
/* GraviCowboys (examples/gravicowboys.py): a uint64 cell packs energy (12
 * bits) | new_energy << 12 | gravity (float bits) << 24.  emit: new_energy =
 * energy; the smallest of the neighbours' gravities (a < b ? a : b in
 * neighbour order, then 0.0f + it); for each buffer k in order one unit goes
 * to neighbour k when its gravity equals that smallest and
 * (unsigned)(energy - sent) > 0; every buffer carries gravity + energy (a
 * float sum); new_energy -= sent, stored to the cell.  absorb: energy =
 * new_energy + the units received (16-bit), gravity = (the float sum of the
 * buffers' gravities in neighbour order) / 8.008 in double, rounded to float;
 * colour (MovingAverage) energy * 255 and (unsigned)(gravity * 108) twice.
 * An off-board neighbour reads as the whole border container. */
static inline float xo_bits_f(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t xo_f_bits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

/* float -> unsigned int as the GPU converts: truncation, NaN and negatives -> 0 */
static inline uint32_t xo_f2u_sat(float f)
{
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

void xo_gravity_step(const xo_topo *t, uint64_t *fld, int32_t *col, const xo_color *cc, int threads)
{
    const int64_t n = xo_cells(t);
    uint64_t *mains = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t x[XO_MAXDIM];
        xo_coords(t, i, x);
        const uint64_t v = fld[i];
        const uint32_t energy = (uint32_t)(v & 4095u);
        const float g = xo_bits_f((uint32_t)(v >> 24));
        uint16_t newe = (uint16_t)(1u * energy);
        float gk[64];
        for (int k = 0; k < t->nbr; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            const uint64_t w = j < 0 ? t->border_value : fld[j];
            gk[k] = xo_bits_f((uint32_t)(w >> 24));
        }
        float m = gk[0];
        for (int k = 1; k < t->nbr; ++k) m = m < gk[k] ? m : gk[k];
        const float lowest = 0.0f + m;
        uint32_t sent = 0;
        for (int k = 0; k < t->nbr; ++k) {
            const uint32_t towards = lowest == gk[k];
            const uint32_t left = (uint32_t)(energy - sent) > 0u;
            const uint32_t unit = towards * left * 1u;
            sent += unit;
            const uint64_t gb = xo_f_bits(g + (float)energy);
            fld[i + n * (int64_t)(t->rev[k] + 1)] = ((uint64_t)(unit & 4095u)) + (gb << 24);
        }
        newe = (uint16_t)((uint32_t)newe - sent);
        mains[i] = (v & 4095u) + ((uint64_t)(newe & 4095u) << 12) + (v & ~0xFFFFFFull);
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) fld[i] = mains[i];
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t x[XO_MAXDIM];
        xo_coords(t, i, x);
        uint32_t received = 0;
        float field = 0.0f;
        for (int k = 0; k < t->nbr; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            const uint64_t w = j < 0 ? t->border_value : fld[j + n * (int64_t)(k + 1)];
            received += (uint32_t)(w & 4095u);
        }
        for (int k = 0; k < t->nbr; ++k) {
            int64_t j = xo_neighbor(t, x, k);
            const uint64_t w = j < 0 ? t->border_value : fld[j + n * (int64_t)(k + 1)];
            field += xo_bits_f((uint32_t)(w >> 24));
        }
        const uint64_t v = fld[i];
        const uint32_t newe = (uint32_t)((v >> 12) & 4095u);
        const uint16_t energy = (uint16_t)(newe + received);
        const float g = (float)((double)field / 8.008);
        const int r = (int)energy * 255;
        const int gg = (int)xo_f2u_sat(g * 108.0f);
        xo_color_write(col, i, r, gg, gg, cc);
        fld[i] = ((uint64_t)(energy & 4095u)) + ((uint64_t)newe << 12) + ((uint64_t)xo_f_bits(g) << 24);
    }
    free(mains);
}

/* ------------------------------------------------------------------------ */
/* RendererPlain.render_code (renderers.py:220-270): pixel i of a width x
 * height viewport; axes (a0, a1) are projected, every other axis is summed
 * in nested-loop order (outer loop = lowest axis index). */
void xo_render(const xo_topo *t, const int32_t *col, int32_t *img, int width,
               int height, int zoom, int dx, int dy, int a0, int a1,
               int smooth, int threads)
{
    const int64_t npix = (int64_t)width * height;
    int rest[XO_MAXDIM], nrest = 0;
    int64_t projected = 1;
    for (int d = 0; d < t->ndim; ++d)
        if (d != a0 && d != a1) { rest[nrest++] = d; projected *= t->size[d]; }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < npix; ++i) {
        unsigned ui = (unsigned)i;
        int w0 = (int)t->size[a0], w1 = (int)t->size[a1];
        int xa = (int)(((float)(ui % (unsigned)width)) / (float)zoom) + dx;
        int xb = (int)(((float)(ui / (unsigned)width)) / (float)zoom) + dy;
        if (xa < 0) xa = w0 - (-xa % w0);
        if (xa >= w0) xa = xa % w0;
        if (xb < 0) xb = w1 - (-xb % w1);
        if (xb >= w1) xb = xb % w1;
        float r = 0, g = 0, b = 0;
        int64_t x[XO_MAXDIM] = {0};
        x[a0] = xa; x[a1] = xb;
        int64_t total = projected;
        for (int64_t q = 0; q < total; ++q) {
            /* innermost loop = highest summed axis */
            int64_t rem = q;
            for (int m = nrest - 1; m >= 0; --m) {
                x[rest[m]] = rem % t->size[rest[m]];
                rem /= t->size[rest[m]];
            }
            int64_t idx = 0, stride = 1;
            for (int d = 0; d < t->ndim; ++d) { idx += x[d] * stride; stride *= t->size[d]; }
            r += (float)col[3 * idx]; g += (float)col[3 * idx + 1]; b += (float)col[3 * idx + 2];
        }
        int num = (int)projected;
        if (smooth > 0) {
            img[3 * i] = (int)(r / (float)num / (float)smooth);
            img[3 * i + 1] = (int)(g / (float)num / (float)smooth);
            img[3 * i + 2] = (int)(b / (float)num / (float)smooth);
        } else {
            img[3 * i] = (int)(r / (float)num);
            img[3 * i + 1] = (int)(g / (float)num);
            img[3 * i + 2] = (int)(b / (float)num);
        }
    }
}
