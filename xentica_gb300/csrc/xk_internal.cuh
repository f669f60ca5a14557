// Internal declarations shared by the libxk translation units.
#pragma once

#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string>

#include "../../include/xk.h"

// ---------------------------------------------------------------------------
// error handling: every C-ABI function returns a status and records a message
void xk_set_error(const char *fmt, ...);
int xk_cuda_status(cudaError_t err, const char *what);

#define XK_CUDA(call)                                                         \
    do {                                                                      \
        cudaError_t xk_e_ = (call);                                           \
        if (xk_e_ != cudaSuccess) return xk_cuda_status(xk_e_, #call);        \
    } while (0)

#define XK_REQUIRE(cond, code, ...)                                           \
    do {                                                                      \
        if (!(cond)) { xk_set_error(__VA_ARGS__); return (code); }            \
    } while (0)

void xk_set_last_step_ms(double ms);

// ---------------------------------------------------------------------------
// Life-like bit-packed lattices: cell x of row y is bit (x & 31) of word
// y * wpr + (x >> 5); padding bits past the row's last cell are always 0.

// The rule as the coefficients of the multiplexer tree's first level.  The
// truth-table masks T[s][n] (0 or ~0: the next state of a cell in state s
// with n live neighbours) are paired by the count's bit 0, and
// `sel ? B : A` over masks A, B is the integer multiply-add sel * k + A with
// k = 0 (A == B), 1 (A = 0, B = ~0) or ~0 (A = ~0, B = 0), exactly, on the
// FMA pipe instead of the logic pipe.  Pair q < 4: A = T[0][2q],
// B = T[0][2q + 1]; q >= 4: the same for T[1][2(q - 4)].  a8/k8: the count-8
// pair (T[0][8], T[1][8]) selected by the cell's state.
struct LifeTable {
    uint32_t a[8], k[8];
    uint32_t a8, k8;
};

// The same rule over the count n9 of the 3 x 3 block including the cell
// (0..9; a live cell's n9 is its neighbour count + 1): dead D[n] = T[0][n],
// live L[n] = T[1][n - 1] (L[0] never occurs and repeats L[1]).  Pairs by
// the count's bit 0: q < 4 (D[2q], D[2q + 1]), q >= 4 (L[2(q - 4)],
// L[2(q - 4) + 1]); n9 of 8 or 9: D[8] for a dead cell, the pair (L[8], L[9])
// (a9, k9) for a live one.
struct LifeTable9 {
    uint32_t a[8], k[8];
    uint32_t d8, a9, k9;
};

__host__ __device__ inline uint32_t xk_mux_coef(uint32_t A, uint32_t B)
{
    return A == B ? 0u : (A ? 0xFFFFFFFFu : 1u);
}

LifeTable xk_life_table(uint32_t rule0, uint32_t rule1);

struct LifeGeo {
    int32_t W, H, wpr, rlast;  // width, height, words per row, bits in last word
    uint32_t lastmask;         // valid bits of a row's last word
    int32_t torus;             // 1: wrap; 0: off-board cells read as bfill
    uint32_t bfill;            // 0 or ~0: static border state replicated
    uint32_t div_wpr;          // xk_div_magic(wpr, H * wpr)
};

// n / d for every n < N as umulhi(n, m) with m = ceil(2^32 / d): exact when
// N * (m d - 2^32) < 2^32 (then n / d + n e / (d 2^32) stays below the next
// integer); 0 when that does not hold or d < 2, meaning a plain division
inline uint32_t xk_div_magic(uint64_t d, uint64_t N)
{
    if (d < 2 || d >= (1ull << 32)) return 0;
    const uint64_t m = ((1ull << 32) + d - 1) / d;
    const uint64_t e = m * d - (1ull << 32);
    return (e == 0 || N < (1ull << 32) / e) && N <= 0xFFFFFFFFull ? (uint32_t)m : 0u;
}

__device__ __forceinline__ uint32_t xk_divu(uint32_t n, uint32_t d, uint32_t m)
{
    return m ? __umulhi(n, m) : n / d;
}

LifeGeo xk_life_geo(int64_t W, int64_t H, int torus, int border_state);

// one lattice (or ensemble instance) for the resident kernel
struct LifeInst {
    int64_t off;               // first word in the state array
    int32_t W, H, wpr, rlast;
    uint32_t lastmask;
    uint32_t rule0, rule1;
    int32_t smem_words;        // shared memory the instance needs
};

// shared-memory words a resident lattice needs with `threads` threads
int64_t xk_life_resident_words(int W, int H, int threads);
// largest dynamic shared memory a CTA may use on this device
int xk_max_smem_optin();
// identity of the CUDA context current on this thread (unique for the
// process's lifetime; 0 when it cannot be told): device-side objects cached
// per context are looked up again after a context reset
unsigned long long xk_context_id();
// Raise a kernel's cudaFuncAttributeMaxDynamicSharedMemorySize (one value per
// function and device) to at least `bytes`; never lowers it.  A graph node
// keeps the shared memory of the launch it captured, and a node launched or
// replayed later (a profiler replays graph nodes one by one) is checked
// against the attribute as it is then: had a later, smaller launch lowered
// the attribute, that node would fail with cudaErrorLaunchFailure or an
// invalid-argument error.  Kept monotone, every captured node stays valid.
cudaError_t xk_smem_attr_at_least(const void *fn, int bytes);

// launchers (stream-ordered, no synchronisation)
cudaError_t xk_life_pack(const void *src, int esz, uint32_t *dst, const LifeGeo &g, cudaStream_t s);
cudaError_t xk_life_unpack(const uint32_t *src, void *dst, int esz, const LifeGeo &g, cudaStream_t s);
cudaError_t xk_life_step_global(const uint32_t *src, uint32_t *dst, const LifeGeo &g,
                                const LifeTable &t, cudaStream_t s);
// bytes_io: state is one byte per cell (LifeInst.off in bytes) instead of
// bit-packed words; `bad` (bytes_io only) is or-ed with 1 if a cell held a
// value other than 0/1
// rule_form (bit-packed state only): XK_RULE_CONWAY runs the instantiation
// with B3/S23 compiled in (every instance's rule must then be B3/S23)
// priority (one-byte torus state only): the launch's priority attribute
// (a graph instantiated with cudaGraphInstantiateFlagUseNodePriority keeps it)
#define XK_NO_PRIORITY (-1000000)
cudaError_t xk_life_step_resident(const LifeInst *inst, int ninst, void *state, int bytes_io,
                                  int generations, int torus, uint32_t bfill, unsigned int *bad,
                                  int threads, int smem_bytes, cudaStream_t s, int rule_form = 0,
                                  int priority = XK_NO_PRIORITY);
// torus, one byte per cell, in place: lattice k advances gens[k]
// generations (a device array of ninst counts)
cudaError_t xk_life_step_resident_each(const LifeInst *inst, const int32_t *gens, int ninst, void *state,
                                       unsigned int *bad, int threads, int smem_bytes, cudaStream_t s);
// torus, one byte per cell: lattices read from `in`, results written to
// `out` and, when `mirror` is not null, also to `mirror` (the same offsets);
// `in` and `out` may be device addresses of mapped host memory
cudaError_t xk_life_step_resident_io(const LifeInst *inst, int ninst, const uint8_t *in, uint8_t *out,
                                     uint8_t *mirror, int generations, unsigned int *bad, int threads,
                                     int smem_bytes, cudaStream_t s);
// CTAs of that kernel one SM holds at once with this block size and
// shared memory (1 when the query fails)
int xk_life_resident_ctas_per_sm(int threads, int smem_bytes);
// threads and dynamic shared memory of the resident kernel for one lattice;
// rows_per_band: target band length (controls the number of warps)
int xk_life_resident_config(int W, int H, int rows_per_band, int *threads, int *smem_bytes);
cudaError_t xk_life_colors(const uint32_t *bits, int32_t *col, const LifeGeo &g,
                           const int32_t *lut6, int smooth, cudaStream_t s);
cudaError_t xk_life_color_step(const uint32_t *bits, int32_t *col, const LifeGeo &g,
                               const int32_t *lut6, int fade_in, int fade_out, int smooth,
                               int plain, cudaStream_t s);

// 3-D von Neumann Life-like on a torus, bit-packed along x; row (y, z) is row
// z * H + y (pack/unpack with xk_life_geo(W, H * D, 1, 0))
struct Life3Geo {
    int32_t W, H, D, wpr, rlast;
    uint32_t lastmask;
    uint32_t div_wpr, div_h;   // xk_div_magic(wpr, H * D * wpr), xk_div_magic(H, H * D)
};
cudaError_t xk_life_step3d_vn(const uint32_t *src, uint32_t *dst, const Life3Geo &g,
                              const LifeTable &t, cudaStream_t s);

// one lattice (W <= 1024) on a thread-block cluster of C CTAs, R rows each,
// in place on its bit-packed words (cluster.cu); config returns 0 when no
// cluster of (up to) C CTAs whose lane groups walk bands of about `band` rows
// fits
LifeTable9 xk_life_table9(uint32_t rule0, uint32_t rule1);
// Rule forms of the single-lattice kernels: a rule loaded at run time, or
// Conway's Life B3/S23 fixed at compile time (the reference's default
// LifelikeCA rule and its GameOfLife model)
#define XK_RULE_TABLE 0
#define XK_RULE_CONWAY 1
// the rule form a single-lattice kernel compiles for (rule0: dead-cell table,
// rule1: live-cell table): XK_RULE_CONWAY for B3/S23, else XK_RULE_TABLE
int xk_rule_form(uint32_t rule0, uint32_t rule1);
int xk_life_cluster_config(const LifeGeo &g, int C, int band, int *C_out, int *R, int *threads);
// sync: how the CTAs of the cluster order their halo exchange every
// generation -- XK_SYNC_BARRIER a cluster barrier; XK_SYNC_NEIGHBOUR mbarriers
// of the two neighbouring CTAs only (bands of 1, 2 and 4 rows);
// XK_SYNC_SPLIT a cluster barrier whose arrive and wait enclose the bands'
// inner rows (every CTA's bands exactly 4 or 8 rows); XK_SYNC_ASYNC the
// neighbour form with the rows sent by asynchronous remote stores that
// complete a transaction count on the receiver's mbarrier (bands of 1 row, or
// every CTA's bands exactly 2, 4 or 8 rows): xk_life_cluster_has_sync
#define XK_SYNC_BARRIER 0
#define XK_SYNC_NEIGHBOUR 1
#define XK_SYNC_SPLIT 2
#define XK_SYNC_ASYNC 3
cudaError_t xk_life_step_cluster(uint32_t *bits, const LifeGeo &g, uint32_t rule0, uint32_t rule1,
                                 int generations, int C, int R, int threads, cudaStream_t s, int sync = 0);
int xk_life_cluster_has_sync(const LifeGeo &g, int C, int R, int threads, int sync);
// a CTA of the neighbour form gave up waiting since the last call (clears it)
bool xk_cluster_take_wait_failure();

// T (1..8) generations per launch of a 2-D lattice of any size (W >= 64),
// tiles with a T-generation halo in shared memory, src -> dst (life_tb.cu)
int xk_life_tb_supported(const LifeGeo &g);
cudaError_t xk_life_step_tb(const uint32_t *src, uint32_t *dst, const LifeGeo &g, const LifeTable9 &t,
                            int T, cudaStream_t s);

// byte-per-cell lattices (N-D, any neighbourhood; and the plain 2-D form)
struct NdGeo {
    int32_t ndim, nbr, torus;
    int64_t size[XK_MAXDIM];
    int8_t delta[XK_MAXNBR][XK_MAXDIM];
    uint32_t border_state;      // 0/1 state of off-board cells
};
cudaError_t xk_nd_pack(const void *src, int esz, uint8_t *dst, int64_t n, cudaStream_t s);
cudaError_t xk_nd_unpack(const uint8_t *src, void *dst, int esz, int64_t n, cudaStream_t s);
cudaError_t xk_life_step_nd(const uint8_t *src, uint8_t *dst, const NdGeo &g, uint32_t rule0,
                            uint32_t rule1, cudaStream_t s);
cudaError_t xk_life_step_bytes2d(const uint8_t *src, uint8_t *dst, int W, int H,
                                 uint32_t rule0, uint32_t rule1, cudaStream_t s);
// shifting family (shift.cu): one generation (any topology and border), or
// `generations` at once on a torus
cudaError_t xk_shift_step_nd(const uint8_t *src, uint8_t *dst, const NdGeo &g, int i0, cudaStream_t s);
cudaError_t xk_shift_jump(const uint8_t *src, uint8_t *dst, const NdGeo &g, int i0, int64_t generations,
                          cudaStream_t s);
cudaError_t xk_nd_colors(const uint8_t *st, int32_t *col, int64_t n, const int32_t *lut6,
                         int smooth, cudaStream_t s);
cudaError_t xk_nd_color_step(const uint8_t *st, int32_t *col, int64_t n, const int32_t *lut6,
                             int fade_in, int fade_out, int smooth, int plain, cudaStream_t s);

// RendererPlain over an int3 colour array of an N-D lattice
struct RenderGeo {
    int32_t ndim, a0, a1;
    int64_t size[XK_MAXDIM];
    int32_t smooth;             // 0: no SMOOTH_FACTOR division
};
// smallest and largest of `count` colour values into the device ints out[0],
// out[1] (render.cu)
cudaError_t xk_colors_minmax(const int32_t *col, int64_t count, int *out, cudaStream_t s);
cudaError_t xk_render_colors(const int32_t *col, int32_t *img, const RenderGeo &g, int width,
                             int height, int zoom, int dx, int dy, cudaStream_t s);
// the same frame as bytes (the int's low byte, as the reference's
// render() converts it)
cudaError_t xk_render_colors_u8(const int32_t *col, uint8_t *img, const RenderGeo &g, int width,
                                int height, int zoom, int dx, int dy, cudaStream_t s);

int xk_sm_count();

// generic interpreter (vm.cu)
struct VmGeo {
    int32_t ndim, nbr, torus, esz;
    int64_t n;
    int64_t size[XK_MAXDIM];
    int8_t delta[XK_MAXNBR][XK_MAXDIM];
    uint64_t border;             // static border: the whole off-board container
    int32_t color_kind, fade_in, fade_out, smooth;
};
cudaError_t xk_vm_run(const xk_vm_ins *code, int ncode, const uint64_t *consts,
                      const uint64_t *params, uint8_t *fld, int32_t *col, const VmGeo &g,
                      cudaStream_t s);

// EvoLife family (evolife.cu)
cudaError_t xk_evolife_set_positional(const double *lut54);
// frame: null, or a W x H uint8 RGB frame written as RendererPlain renders the
// new colours at zoom 1 with no offset (frame_smooth: its SMOOTH_FACTOR, 0
// for none)
cudaError_t xk_evolife_step(const uint64_t *src, uint64_t *dst, int32_t *col, const xk_desc &d,
                            float mut_thresh, cudaStream_t s, uint8_t *frame = nullptr,
                            int frame_smooth = 0);

// Life with inherited colour channels (lifecolor.cu): one generation, the
// colours updated, and (frame) the zoom-1 frame as for EvoLife
cudaError_t xk_lifecolor_step(const uint32_t *src, uint32_t *dst, int32_t *col, const xk_desc &d,
                              cudaStream_t s, uint8_t *frame = nullptr, int frame_smooth = 0);

// per-cell noise (noise.cu): `generations` generations of every cell in one
// launch, in place (1 when the zoom-1 frame of a 2-D lattice is written)
cudaError_t xk_noise_step(uint16_t *cells, int32_t *col, const xk_desc &d, int64_t n, int generations,
                          cudaStream_t s, uint8_t *frame = nullptr, int frame_smooth = 0);
// one GraviCowboys generation, cells ping-pong (gravity.cu)
cudaError_t xk_gravity_step(const uint64_t *src, uint64_t *dst, int32_t *col, const xk_desc &d,
                            cudaStream_t s, uint8_t *frame, int frame_smooth);

// Programmatic dependent launch for kernels that run once per generation: the
// launch may begin while the previous kernel in the stream finishes, and the
// kernel calls xk_grid_dep_wait() before its first global-memory access
// (which returns once that kernel has completed and its writes are
// visible).  XK_PDL=0 in the environment launches plainly.
__device__ __forceinline__ void xk_grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline bool xk_pdl_enabled()
{
    const char *v = getenv("XK_PDL");
    return !(v && v[0] == '0');
}

template <typename... KArgs, typename... Args>
cudaError_t xk_launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                          Args... args)
{
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = &attr;
    cfg.numAttrs = xk_pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Bernoulli seeds (seed.cu): cells[off .. off + n) of a lattice =
// RandomState(seed).random_sample(n) < p, bit for bit
struct XkSeedJob {
    int64_t off, n;
    uint32_t seed, pad;
    double p;
};
cudaError_t xk_seed_bernoulli(const XkSeedJob *jobs, int count, uint8_t *cells, cudaStream_t s);

// mass-transfer family (mass.cu)
// Mass-transfer state on the device: rows of W cells at a pitch of W rounded
// up to a multiple of 4 (so a row starts on 16 bytes, as the tensor copies
// need); the padding cells hold 0.
inline int64_t xk_mass_pitch(int64_t W) { return (W + 3) / 4 * 4; }
// small: the lattice's total mass is below 2^30 (then every cell stays below
// it for good), which allows the fast-only kernel
// proj (only where xk_mass_fuses_projection()): also add the new state's
// column colour sums into proj (W x H, zero on entry); with frame_prev, also
// write the zoom-1 frame of the previous generation from its sums proj_prev
// and zero proj_prev
cudaError_t xk_mass_step(const uint32_t *src, uint32_t *dst, unsigned long long *total,
                         const xk_desc &d, bool small, cudaStream_t s, uint32_t *proj = nullptr,
                         uint32_t *proj_prev = nullptr, uint8_t *frame_prev = nullptr);
bool xk_mass_fuses_projection(const xk_desc &d);
// the W x H zoom-1 RendererPlain frame (axes (0, 1), no smoothing) from
// column colour sums
cudaError_t xk_mass_frame(const uint32_t *proj, uint8_t *frame, const xk_desc &d, cudaStream_t s);
// total of n cells into *out (64-bit)
cudaError_t xk_mass_sum(const uint32_t *src, int64_t n, unsigned long long *out, cudaStream_t s);
// true when a mass-transfer CTA gave up waiting for a tensor copy since the
// last call (the flag is cleared)
bool xk_mass_take_wait_failure();
// column colour sums over z; with `frame`, also the W x H RendererPlain frame
// over axes (0, 1) at zoom 1, no offset, as uint8 RGB
cudaError_t xk_mass_project(const uint32_t *src, uint32_t *proj, const xk_desc &d, cudaStream_t s,
                            uint8_t *frame = nullptr);
cudaError_t xk_mass_colors(const uint32_t *src, int32_t *col, const xk_desc &d, cudaStream_t s);
cudaError_t xk_mass_render(const uint32_t *proj, int32_t *img, const xk_desc &d, int width,
                           int height, int zoom, int dx, int dy, cudaStream_t s);
cudaError_t xk_mass_render_u8(const uint32_t *proj, uint8_t *img, const xk_desc &d, int width,
                              int height, int zoom, int dx, int dy, cudaStream_t s);
