/*
 * xk.h -- C-ABI of libxk, the GB300 (sm_103a) engine behind the xentica_gb300
 * Python API.
 *
 * Plain C: pointers, sizes and status codes only.  The library owns device
 * memory; callers own host buffers and the library copies.  Every function
 * returns XK_OK (0) or a negative status; xk_last_error() gives the message of
 * the last failure on the calling thread.  A handle is not thread-safe (the
 * Python layer serialises each model with a lock, as the reference does at
 * xentica/core/base.py:669,716,748); each handle owns one CUDA stream.
 *
 * Each entry point names the reference interface it replaces.  The reference
 * is pure Python over PyCUDA; "replaces" means the PyCUDA calls its
 * CellularAutomaton makes for the same job.
 */
#ifndef XK_H
#define XK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XK_ABI_VERSION 1
#define XK_MAXDIM 8
#define XK_MAXNBR 32

enum {
    XK_OK = 0,
    XK_ERR_ARG = -1,          /* invalid argument or descriptor            */
    XK_ERR_CUDA = -2,         /* CUDA runtime failure                      */
    XK_ERR_OOM = -3,          /* device allocation failed / over budget    */
    XK_ERR_UNSUPPORTED = -4,  /* no kernel for this configuration          */
    XK_ERR_STATE = -5,        /* call out of order (e.g. step before upload) */
    XK_ERR_TIMEOUT = -6,      /* a bounded device-side wait gave up        */
    XK_ERR_INVARIANT = -7     /* a conserved quantity changed              */
};

/* XK_FAMILY_SHIFT: ShiftingSands' family (examples/shifting_sands.py:15-47),
 * a 1-bit state that moves in from neighbour rule0 each generation.
 * XK_FAMILY_LIFECOLOR: Conway's Life whose cells carry three 8-bit colour
 * channels inherited from their neighbours (GameOfLifeColor,
 * examples/game_of_life.py:112-159): a 2-D Moore lattice of uint32 cells,
 * torus or static border, MovingAverage colours or none.
 * XK_FAMILY_NOISE: per-cell noise (NoiseTV, examples/noisetv.py:13-31), one
 * 16-bit RandomProperty per cell advanced twice a generation, any lattice.
 * XK_FAMILY_GRAVITY: energy flowing down a gravity field (GraviCowboys,
 * examples/gravicowboys.py:20-71): a 2-D Moore lattice of uint64 cells
 * (energy 12 bits | new_energy 12 bits | float gravity), torus or static
 * border, MovingAverage colours or none. */
enum { XK_FAMILY_LIFE = 1, XK_FAMILY_EVOLIFE = 2, XK_FAMILY_MASS = 3, XK_FAMILY_VM = 4,
       XK_FAMILY_SHIFT = 5, XK_FAMILY_LIFECOLOR = 6, XK_FAMILY_NOISE = 7, XK_FAMILY_GRAVITY = 8 };
enum { XK_COLOR_NONE = 0, XK_COLOR_PLAIN = 1, XK_COLOR_MOVING_AVERAGE = 2 };

/* Model descriptor filled by the translator (xentica_gb300/core/templates.py)
 * from the traced model: the template family plus its rule parameters. */
typedef struct xk_desc {
    int32_t abi_version;               /* XK_ABI_VERSION                          */
    int32_t family;                    /* XK_FAMILY_*                             */
    int32_t ndim;                      /* lattice dimensions                      */
    int32_t nbr;                       /* neighbours per cell                     */
    int64_t size[XK_MAXDIM];           /* cells per axis, axis 0 fastest          */
    int8_t delta[XK_MAXNBR][XK_MAXDIM];/* neighbour offsets                       */
    int32_t torus;                     /* 1 TorusBorder, 0 StaticBorder           */
    int32_t state_bytes;               /* reference packed cell size: 1,2,4,8     */
    uint64_t border_value;             /* StaticBorder packed off-board value     */
    int32_t color_kind;                /* XK_COLOR_*                              */
    int32_t fade_in, fade_out, smooth; /* MovingAverage constants                 */
    int32_t proj_axis0, proj_axis1;    /* RendererPlain projection axes           */
    int32_t render_smooth;             /* render divisor (SMOOTH_FACTOR) or 0     */
    /* XK_FAMILY_LIFE: the next state of a cell in state s (0/1) with k live
     * neighbours is bit k of rule0 (s == 0) or rule1 (s == 1).  For the
     * reference's Life-like absorb ``is_born | is_sustain & state``
     * (examples/game_of_life.py:65-70, :190-197): rule0 = B, rule1 = B | S. */
    uint32_t rule0, rule1;
    int32_t color_lut[6];              /* rgb of state 0, rgb of state 1          */
    int32_t color_history_free;        /* colour is a function of state alone     */
    /* XK_FAMILY_EVOLIFE */
    uint32_t death_speed, max_genes;
    double mutation_prob;
    int32_t positional;                /* 0 GenomeColor.modular, 1 .positional    */
    double palette[54];                /* positional: rgb weight of each of 18 genes */
    /* XK_FAMILY_MASS */
    uint32_t wall;                     /* StaticBorder value = off-board mass     */
    int32_t reserved[8];
} xk_desc;

typedef struct xk_model xk_model;

/* Replaces GPUKernels/GPUArrays construction (SourceModule + to_gpu,
 * xentica/core/base.py:527-569, :664): allocate the device state. */
int xk_model_create(const xk_desc *desc, xk_model **out);
void xk_model_destroy(xk_model *m);

/* Replaces gpuarray.to_gpu(init_cells) / cells.get() (base.py:558-559,
 * tests reading gpu.arrays.cells.get()[:cells_num]): main plane in the
 * reference layout, desc->state_bytes per cell. */
int xk_upload(xk_model *m, const void *host_main, int64_t ncells);
int xk_download(xk_model *m, void *host_main, int64_t ncells);

/* Replaces gpu.arrays.colors (int3 per cell, base.py:558, :659). */
int xk_upload_colors(xk_model *m, const int32_t *host_col, int64_t ncells);
/* Smallest and largest value of the last xk_upload_colors (out[0], out[1];
 * 0, 0 before any): what a host needs to decide xk_set_color_mode without a
 * pass of its own over the colours. */
int xk_colors_range(const xk_model *m, int32_t out[2]);
int xk_download_colors(xk_model *m, int32_t *host_col, int64_t ncells);

/* Interactive rule of the Life-like family: the values the reference passes
 * as kernel arguments at every step (base.py:717, :722). */
int xk_life_set_rule(xk_model *m, uint32_t rule0, uint32_t rule1, const int32_t color_lut[6]);

/* Colour bookkeeping of the Life-like family: with history_free = 1 the
 * colour after a step is a function of the state alone (the MovingAverage
 * clamp can never bind), so steps skip the colour pass and colours are
 * computed when read; 0 updates colours every generation like the reference's
 * absorb (color_effects.py:106-130). */
int xk_set_color_mode(xk_model *m, int32_t history_free);

/* Replaces CellularAutomaton.step (base.py:703-728): nsteps generations of
 * emit + absorb + colour, fused.  Returns once the work is queued on the
 * model's stream, as the reference's step() returns after its asynchronous
 * launches (mass-transfer steps wait, to read their kernels' give-up flag);
 * xk_download, xk_sync and xk_last_step_ms wait for it, and errors of the
 * queued work are reported there.  XK_ERR_TIMEOUT: a mass-transfer kernel
 * gave up waiting for one of its tensor copies (a bounded wait; the state is
 * then unspecified). */
int xk_step(xk_model *m, int64_t nsteps);

/* Replaces CellularAutomaton.render (base.py:730-753): width*height*3 int32. */
int xk_render(xk_model *m, int32_t *host_img, int32_t width, int32_t height,
              int32_t zoom, int32_t dx, int32_t dy);

/* Replaces the viewer loop's step() + render() pair (base.py:703-753, called
 * once per frame by the Moire bridge): nsteps generations, each followed by a
 * RendererPlain frame of the viewport as uint8 RGB -- what render() returns,
 * img.get().astype(np.uint8) -- written to frames + g * width * height * 3
 * for generation g.  frames_on_device = 0: `frames` is host memory (frames
 * pass through a ring of 4 device frames and are copied on a second stream
 * while the next generations run; page-locked memory makes the copies
 * asynchronous); 1: `frames` is a device buffer of nsteps frames.
 * last_step_ms covers every generation, render and copy. */
int xk_step_frames(xk_model *m, int64_t nsteps, int32_t width, int32_t height, int32_t zoom,
                   int32_t dx, int32_t dy, uint8_t *frames, int32_t frames_on_device);

/* Launch plan of a 2-D Life-like model whose colours follow from its state:
 * which kernel family runs its multi-generation steps, chosen by timing on
 * the first step (or by xk_model_plan before it).  The reference has one
 * kernel shape for every model (base.py:254-283); these exist so that a host
 * can cache the choice per device, library build and lattice and re-apply it
 * without timing.  plan[0]: XK_PLAN_*; CLUSTER: plan[1] = CTAs asked for
 * (1..16), plan[2] = rows per lane group, plan[3] = how the CTAs order
 * their row exchange each generation: 0 a cluster barrier, 1 each CTA waits
 * only for its two neighbours' rows (mbarriers; bands of 1, 2 or 4 rows), 2
 * a cluster barrier whose arrival comes before the bands' inner rows and
 * whose wait after them (every CTA's bands exactly 4 or 8 rows), 3 as 1 with
 * the rows sent by asynchronous remote stores counted in bytes on the
 * receiver's mbarrier (bands of 1 row, or every CTA's bands exactly 2, 4 or
 * 8 rows); TEMPORAL: plan[3] =
 * generations per launch (2..8).  xk_model_plan gives kind -1 for models
 * without plans.  A bounded wait of the neighbour or async form that gave up makes
 * the next xk_download return XK_ERR_TIMEOUT. */
enum { XK_PLAN_GLOBAL = 0, XK_PLAN_RESIDENT = 1, XK_PLAN_CLUSTER = 2, XK_PLAN_TEMPORAL = 3 };
int xk_model_plan(xk_model *m, int32_t plan[4]);
int xk_model_set_plan(xk_model *m, const int32_t plan[4]);
/* Rule form the 2-D Life-like kernels of a model run with its current rule:
 * 1 (Conway's B3/S23, compiled into the kernels: fewer instructions per
 * word), 0 (any other rule, read from a table at run time), -1 for models
 * without 2-D Life-like kernels.  A plan is timed with this form, so a
 * cache of plans keys on it.  No reference counterpart (the reference
 * compiles every rule into its generated source, base.py:538-541, or passes
 * it as a kernel argument, game_of_life.py:183-203). */
int32_t xk_model_rule_form(const xk_model *m);

/* Mass family: total mass after each of the last xk_step's generations
 * (count = that nsteps); the invariant the configuration checks. */
int xk_mass_totals(xk_model *m, uint64_t *host_totals, int64_t count);

/* Generic interpreter family (XK_FAMILY_VM): models no hand-written template
 * implements run their traced emit and absorb programs, compiled to typed
 * register instructions by xentica_gb300/core/vm.py, with the reference's
 * execution model -- replaces the emit and absorb kernels the reference
 * generates for the model (base.py:461-487) and their launches in step()
 * (base.py:703-728).  The model keeps the reference's layout: N + 1 planes of
 * state_bytes-wide containers and int32 x 3 colours. */
typedef struct xk_vm_ins {
    uint8_t op, ty;               /* opcode and C type (codes of core/vm.py)   */
    uint16_t dst, a, b, c;        /* registers, or constant / parameter slot,
                                     load kind / neighbour / plane            */
    uint16_t reserved;
} xk_vm_ins;
#define XK_VM_MAX_REGS 256
#define XK_VM_MAX_PARAMS 64
/* which: 0 emit, 1 absorb.  Every instruction is checked against the model
 * (registers < nregs <= XK_VM_MAX_REGS, slots, planes, neighbours). */
int xk_vm_load(xk_model *m, int32_t which, const xk_vm_ins *code, int32_t ncode,
               const uint64_t *consts, int32_t nconsts, int32_t nregs);
/* Interactive parameter values (64-bit register images), bound at the next
 * step, as the reference passes them per launch (base.py:717, :722). */
int xk_vm_set_params(xk_model *m, const uint64_t *values, int32_t count);

/* Wait for all work queued on the model's stream. */
int xk_sync(xk_model *m);

/* Device time of the last xk_step / batch step, in milliseconds (CUDA events
 * on the launching stream); after an xk_step it waits for that step. */
double xk_last_step_ms(void);

/* ------------------------------------------------------------------------ */
/* Ensemble: many independent Life-like instances (LifelikeCA with an
 * interactive rule, examples/game_of_life.py:183-203) on 2-D tori, advanced
 * together.  The reference has no batch API: its equivalent is one
 * CellularAutomaton per instance, each calling step() (base.py:703-728). */
typedef struct xk_batch xk_batch;

/* width/height per instance (any positive sizes), rule = golly integer
 * (born bits 0-8, sustain bits 9-17, xentica/tools/rules.py:5-21), applied
 * as LifelikeCA's absorb does: next = born[k] | sustain[k] & state. */
int xk_batch_create(int32_t count, const int32_t *width, const int32_t *height,
                    const uint32_t *rule, xk_batch **out);
void xk_batch_destroy(xk_batch *b);
/* One byte per cell (0/1), instances concatenated in creation order. */
int xk_batch_upload(xk_batch *b, const uint8_t *host_cells, int64_t total_cells);
int xk_batch_download(xk_batch *b, uint8_t *host_cells, int64_t total_cells);
/* Batched form: every instance resident in shared memory for all
 * generations, one graph launch. */
int xk_batch_step(xk_batch *b, int32_t generations);
/* Plain form: one launch per instance per generation, reference layout
 * (one byte per cell), for comparison. */
int xk_batch_step_plain(xk_batch *b, int32_t generations);
/* End to end: host_in -> `generations` -> host_out (host_in == host_out is
 * allowed); the result is also left as the batch's device state.  When both
 * buffers are page-locked (xk_host_register, cudaHostAlloc), lattices whose
 * CTA fills an SM are copied in and out by the copy engines around their
 * launches and every other lattice is read and written by its kernel over
 * the host link; pageable buffers are copied in overlapped chunks
 * (XK_E2E=chunks in the environment forces that form). */
int xk_batch_run(xk_batch *b, const uint8_t *host_in, uint8_t *host_out,
                 int64_t total_cells, int32_t generations);
/* Seed every instance on the device: cell j of instance i =
 * (RandomState(seeds[i]).random_sample(W_i * H_i)[j] < p[i]), bit for bit
 * NumPy's legacy MT19937 stream (the draw a seed pattern makes through
 * xentica/seeds/random.py:22-54 LocalRandom.numpy; the reference's seeds are
 * host NumPy arrays packed by xentica/core/base.py:510-524), so a huge
 * ensemble needs no host array.  One CTA per instance; last_step_ms is the
 * device time. */
int xk_batch_seed_bernoulli(xk_batch *b, const uint32_t *seeds, const double *p);
/* Autotune the batched kernel's CTA shapes for this batch, timed on the
 * device over `generations` (the state is restored): one band length (rows
 * per lane group) for every lattice, then per lattice size (W, H) holding at
 * least 3 % of the cells a band length of its own where that makes the whole
 * batch at least 2 % faster (confirmed by repeated timing).
 * *chosen_rows_per_band is the common band; xk_batch_size_bands reads the
 * per-size choices. */
int xk_batch_tune(xk_batch *b, int32_t generations, int32_t *chosen_rows_per_band);
/* Set the common band length (rows per lane group, 1..1024) the tuner would
 * choose, e.g. from a cached tuning result, without timing (this clears the
 * per-size choices); and read it back. */
int xk_batch_set_band(xk_batch *b, int32_t rows_per_band);
int32_t xk_batch_band(const xk_batch *b);
/* Per-size band lengths: `count` triples (W, H, band) replace the per-size
 * choices (W x H lattices use `band` instead of the common one); and read
 * them back (returns how many there are, writing at most `capacity`
 * triples).  No reference counterpart (tuning state). */
int xk_batch_set_size_bands(xk_batch *b, const int32_t *triples, int32_t count);
int32_t xk_batch_size_bands(const xk_batch *b, int32_t *triples, int32_t capacity);
int64_t xk_batch_total_cells(const xk_batch *b);
/* Kernel launches one xk_batch_step makes (one per instance class, plus
 * per-generation launches for instances too large for a CTA). */
int64_t xk_batch_launches(const xk_batch *b, int32_t generations);
/* Membership changes between steps.  The reference adds or drops an
 * instance by creating or discarding a CellularAutomaton
 * (base.py:591-690); here an ensemble changes in place.  xk_batch_add appends
 * a lattice (cells one byte each from host_cells, or all 0 when NULL) and
 * returns its index (>= 0) or a negative status; xk_batch_remove drops
 * lattice `index` (later lattices move down by one; the last lattice cannot
 * be removed).  Both keep every other lattice's cells, re-plan the launch
 * classes and capture a new graph at the next step. */
int xk_batch_add(xk_batch *b, int32_t width, int32_t height, uint32_t rule,
                 const uint8_t *host_cells);
int xk_batch_remove(xk_batch *b, int32_t index);
int32_t xk_batch_count(const xk_batch *b);

/* Ensemble step that allocates nothing.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc (a host framework owns every
 * device allocation, or nothing may be allocated after start-up): d_cells is
 * the caller's device buffer of concatenated lattices (one byte per cell,
 * 0/1), advanced in place by `generations` on `stream` (a cudaStream_t, NULL
 * for the default stream); the call returns when the work is done.  The only
 * other device memory used is a file-scope array sized for
 * XK_NOALLOC_MAX_LATTICES lattice descriptors of 40 bytes plus a 256-byte
 * flag slot (164,096 bytes, about 160 KB), held by every device that loads
 * the library until exit.  Every call shares it, so calls whose GPU work
 * overlaps race; the first call on a device (and the first after its context
 * was reset) looks the array up (cudaGetSymbolAddress) and should come
 * before any stream capture.  More
 * lattices, or lattices wider than 1024 cells or too large for one CTA, are
 * rejected with an error. */
#define XK_NOALLOC_MAX_LATTICES 4096
int xk_batch_step_noalloc(uint8_t *d_cells, int32_t count, const int32_t *width,
                          const int32_t *height, const uint32_t *rule, int32_t generations,
                          void *stream);

/* ---- Serving: continuous batching of independent simulation requests ------
 * No reference counterpart: the reference runs one model per Python object
 * (xentica/core/base.py:591-728, stepped by the caller) and has no request
 * loop.  A server owns a device arena of `budget_bytes` and a pinned host
 * arena of `host_bytes` (each one allocation at creation), a worker thread and
 * its CUDA streams.  Requests are admitted first come, first served, when their
 * device bytes and result bytes fit and fewer than `max_active` run; each
 * active request advances in rounds, a new round starting as soon as its
 * previous one finished, so requests admitted while others run share the GPU
 * with them.  Large 2-D, 3-D and mass-transfer lattices run rounds of
 * `quantum` generations on their own streams.  2-D lattices that fit one CTA
 * run together, one resident-kernel launch per shape class over its idle
 * members (up to 4 such rounds of a class in flight), each member running
 * about quantum x 2^18 cell-generations per round (at least `quantum`
 * generations, at most 65536).  Kernels of requests with less work (cells x
 * generations) run at a greater stream priority.  Results wait in the pinned arena until
 * xk_serve_result collects them.  A request computes exactly what it
 * computes alone. */
enum { XK_SERVE_LIFE2D = 1, XK_SERVE_LIFE3D_VN = 2, XK_SERVE_MASS3D = 3 };
enum {
    XK_REQ_PENDING = 0,      /* queued, waiting for memory or a slot          */
    XK_REQ_ACTIVE = 1,       /* on the device                                 */
    XK_REQ_DONE = 2,         /* result ready for xk_serve_result              */
    XK_REQ_CANCELLED = 3,
    XK_REQ_FAILED = 4
};

typedef struct xk_request {
    int32_t kind;            /* XK_SERVE_*                                            */
    int32_t reserved0;       /* 0                                                     */
    int64_t size[3];         /* cells per axis, axis 0 fastest; size[2] = 1 for 2-D   */
    uint32_t rule;           /* LIFE2D: B bits 0-8, S bits 9-17 (golly int, Moore,
                                torus, LifelikeCA semantics); LIFE3D_VN: B bits 0-6,
                                S bits 7-13 (6 von Neumann neighbours, torus);
                                next = B(k) | S(k) & state.  MASS3D: unused (0)      */
    int32_t reserved1;       /* 0                                                     */
    int64_t generations;     /* >= 0                                                  */
} xk_request;
/* Cells are one byte (0/1) for the Life kinds and uint32 mass for MASS3D
 * (the mass-transfer model: StaticBorder wall 2**32-1), axis 0 fastest. */

typedef struct xk_request_info {
    int32_t status;          /* XK_REQ_*                                               */
    int32_t reserved;
    int64_t generations_done;
    double submit_s, admit_s, done_s;   /* seconds since server start; -1 not yet   */
    uint64_t mass_total;     /* MASS3D: total mass after the last generation          */
} xk_request_info;

typedef struct xk_serve_stats {
    int64_t submitted, admitted, completed, cancelled, rejected, failed;
    int64_t pending, active;
    int64_t device_bytes_in_use, device_bytes_peak, budget_bytes;
    int64_t cell_updates;    /* cells x generations of completed requests             */
    int64_t rounds, launches;/* worker rounds that launched work; kernel launches     */
    double elapsed_s;
} xk_serve_stats;

typedef struct xk_server xk_server;

int xk_serve_create(int64_t budget_bytes, int64_t host_bytes, int32_t max_active,
                    int32_t quantum, xk_server **out);
/* Cancels pending and active requests, waits for in-flight work, frees all. */
int xk_serve_destroy(xk_server *srv);
/* Device bytes a request is admitted with (validates it; host only). */
int xk_serve_request_bytes(const xk_request *req, int64_t *bytes);
/* Copies the cells; returns the request id.  Malformed requests and requests
 * larger than the whole budget are rejected (XK_ERR_ARG / XK_ERR_OOM). */
int xk_serve_submit(xk_server *srv, const xk_request *req, const void *host_cells, int64_t *id);
int xk_serve_info(xk_server *srv, int64_t id, xk_request_info *info);
/* Waits until the request is DONE, CANCELLED or FAILED, or the timeout
 * passes (XK_ERR_TIMEOUT); info may be NULL. */
int xk_serve_wait(xk_server *srv, int64_t id, double timeout_s, xk_request_info *info);
/* Copies a DONE request's cells to host_out and forgets the request. */
int xk_serve_result(xk_server *srv, int64_t id, void *host_out, int64_t cells);
/* Pending: dropped at once; active: stops at its next round boundary. */
int xk_serve_cancel(xk_server *srv, int64_t id);
int xk_serve_stats_get(xk_server *srv, xk_serve_stats *st);

/* The server's arena allocator on its own (host only, no CUDA): first-fit
 * offsets in [0, capacity), 256-byte granules, neighbours merged on free. */
typedef struct xk_arena xk_arena;
int xk_arena_create(int64_t capacity, xk_arena **out);
int xk_arena_alloc(xk_arena *a, int64_t bytes, int64_t *offset);   /* XK_ERR_OOM: no fit */
int xk_arena_free(xk_arena *a, int64_t offset);
int xk_arena_stats(xk_arena *a, int64_t *in_use, int64_t *largest_free, int32_t *free_ranges);
int xk_arena_destroy(xk_arena *a);

/* Select the CUDA device for handles created afterwards on this thread. */
int xk_set_device(int32_t device);
/* Page-lock (pin) caller-owned host memory for fast copies and for kernels
 * to read and write (mapped, portable), and release it. */
int xk_host_register(void *ptr, int64_t bytes);
int xk_host_unregister(void *ptr);

/* Named NVTX range around a region of host code, for profilers that filter
 * kernels by range (ncu --nvtx-include "name/"); no reference counterpart. */
int xk_range_push(const char *name);
int xk_range_pop(void);

/* Last error message of the calling thread ("" if none). */
const char *xk_last_error(void);
/* Name and SM count of the current device, for logs. */
int xk_device_info(char *buf, int32_t len);

#ifdef __cplusplus
}
#endif
#endif /* XK_H */
