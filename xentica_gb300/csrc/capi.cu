// C-ABI of single models (include/xk.h): device state, layout conversion and
// generation stepping for the kernel families.
#include <math.h>
#include <stdlib.h>
#include <stdarg.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>

#include <cudaTypedefs.h>   // PFN_cuCtxGetCurrent, PFN_cuCtxGetId
#include <nvtx3/nvToolsExt.h>

#include "xk_internal.cuh"

// ---------------------------------------------------------------------------
// errors

static thread_local char g_err[1024] = "";
static std::mutex g_ms_mu;
static double g_last_ms = 0.0;

void xk_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int xk_cuda_status(cudaError_t err, const char *what)
{
    xk_set_error("CUDA error in %s: %s", what, cudaGetErrorString(err));
    return err == cudaErrorMemoryAllocation ? XK_ERR_OOM : XK_ERR_CUDA;
}

// the model whose last xk_step returned without waiting for the device: its
// step's time is read from its events when asked for
static xk_model *g_pending_model = nullptr;
static float pending_step_ms(xk_model *m);

void xk_set_last_step_ms(double ms)
{
    std::lock_guard<std::mutex> lk(g_ms_mu);
    g_last_ms = ms;
    g_pending_model = nullptr;
}

static void set_pending_step(xk_model *m)
{
    std::lock_guard<std::mutex> lk(g_ms_mu);
    g_pending_model = m;
}

// a model going away: its pending step time is resolved first
static void settle_pending_step(xk_model *m)
{
    std::lock_guard<std::mutex> lk(g_ms_mu);
    if (g_pending_model == m) {
        g_last_ms = pending_step_ms(m);
        g_pending_model = nullptr;
    }
}

extern "C" double xk_last_step_ms(void)
{
    std::lock_guard<std::mutex> lk(g_ms_mu);
    if (g_pending_model) {
        g_last_ms = pending_step_ms(g_pending_model);
        g_pending_model = nullptr;
    }
    return g_last_ms;
}

extern "C" const char *xk_last_error(void) { return g_err; }

int xk_sm_count()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return sms;
}

int xk_max_smem_optin()
{
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    return v;
}

unsigned long long xk_context_id()
{
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = (PFN_cuCtxGetCurrent_v4000)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = (PFN_cuCtxGetId_v12000)f;
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx ||
        get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

cudaError_t xk_smem_attr_at_least(const void *fn, int bytes)
{
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, fn);
    if (e != cudaSuccess) return e;
    if (a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

extern "C" int xk_device_info(char *buf, int32_t len)
{
    int dev = 0;
    XK_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp p;
    XK_CUDA(cudaGetDeviceProperties(&p, dev));
    snprintf(buf, len, "%s sm_%d%d SMs=%d smem_optin=%zu", p.name, p.major, p.minor,
             p.multiProcessorCount, (size_t)p.sharedMemPerBlockOptin);
    return XK_OK;
}

// ---------------------------------------------------------------------------
// model object

enum { LAYOUT_BITS2D = 1, LAYOUT_BYTES = 2, LAYOUT_CELLS64 = 3, LAYOUT_MASS = 4, LAYOUT_VM = 5, LAYOUT_LCOLOR = 6,
       LAYOUT_NOISE = 7, LAYOUT_GRAVITY = 8 };

// largest float t with (double)u < p  <=>  u <= t for every float u
static float below_threshold(double p)
{
    float t = (float)p;
    if ((double)t >= p) t = nextafterf(t, -INFINITY);
    return t;
}

// frames of xk_step_frames in flight between rendering and the host copy
constexpr int kFrameRing = 4;

struct xk_model {
    xk_desc d;
    int64_t n = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int layout = 0;
    LifeGeo lg;
    NdGeo ng;
    uint32_t *bits[2] = {nullptr, nullptr};
    uint8_t *bytes[2] = {nullptr, nullptr};
    uint64_t *cells64[2] = {nullptr, nullptr};  // EvoLife, GraviCowboys: reference layout, ping-pong
    float mut_thresh = 0.f;
    uint32_t *cells32[2] = {nullptr, nullptr};  // mass transfer, colour Life: reference layout, ping-pong
    uint16_t *cells16 = nullptr;                // noise: reference layout, updated in place
    int *col_range_d = nullptr;                 // device scratch of xk_upload_colors' range
    int32_t col_range[2] = {0, 0};              // smallest and largest colour value of the last upload
    uint32_t *proj = nullptr;                   // mass: colour sum of every (x, y) column
    uint32_t *proj2 = nullptr;                  // mass: the second buffer of xk_step_frames
    int proj_valid = 0;
    unsigned long long *totals = nullptr;       // mass: total after each generation
    int64_t totals_cap = 0, totals_count = 0;
    bool mass_small = false;                    // mass: uploaded total below 2^30
    int cur = 0;
    void *stage = nullptr;       // reference-layout staging + validity flag
    int32_t *col = nullptr;      // colours (3 int32 per cell) when materialised
    int32_t *img = nullptr;
    int64_t img_cap = 0;
    LifeInst *d_inst = nullptr;  // the lattice as a one-instance resident batch
    int resident = 0, res_threads = 0, res_smem = 0;
    int cl_tuned = 0, cl_C = 0, cl_R = 0, cl_threads = 0;   // cluster plan (cl_C = 0: none)
    int cl_want = 0, cl_band = 0;    // the cluster size and band length the plan was made from
    int cl_sync = 0;                 // the cluster plan's synchronisation form (XK_SYNC_*)
    int tb_T = 0;                // temporally blocked global kernel: generations per launch (0: none)
    uint32_t rule0 = 0, rule1 = 0;
    int32_t lut[6] = {0, 0, 0, 0, 0, 0};
    uint8_t *fld = nullptr;      // interpreter: the reference's N + 1 planes
    xk_vm_ins *vm_code[2] = {nullptr, nullptr};     // emit, absorb
    uint64_t *vm_consts[2] = {nullptr, nullptr};
    int vm_ncode[2] = {0, 0};
    uint64_t *vm_params = nullptr;                  // XK_VM_MAX_PARAMS slots
    VmGeo vg;
    int hf = 0;                  // colour is a function of the state alone
    int derived = 0;             // colours currently implied by the state
    int uploaded = 0;
    // xk_step_frames to host memory: device frame ring and its copy stream
    uint8_t *ring = nullptr;
    int64_t ring_cap = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t rendered[kFrameRing] = {}, copied[kFrameRing] = {};
};

static int64_t cells_of(const xk_desc &d)
{
    int64_t n = 1;
    for (int i = 0; i < d.ndim; ++i) n *= d.size[i];
    return n;
}

static bool is_moore2d(const xk_desc &d)
{
    if (d.ndim != 2 || d.nbr != 8) return false;
    // Moore 2-D neighbour order of the reference: product([-1,0,1], repeat=2)
    // without (0,0); any order works for a totalistic count, but every offset
    // must appear once
    int seen = 0;
    for (int k = 0; k < 8; ++k) {
        int dx = d.delta[k][0], dy = d.delta[k][1];
        if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || (dx == 0 && dy == 0)) return false;
        seen |= 1 << ((dy + 1) * 3 + (dx + 1));
    }
    return seen == (0x1FF & ~(1 << 4));
}

int xk_life_resident_config(int W, int H, int rows_per_band, int *threads, int *smem_bytes)
{
    const int wpr = (W + 31) / 32;
    if (wpr > 32) return 0;
    int P = 1;
    while (P < wpr) P <<= 1;
    const int gpw = 32 / P;
    const int groups = (H + rows_per_band - 1) / rows_per_band;
    int warps = (groups + gpw - 1) / gpw;
    if (warps > 32) warps = 32;
    if (warps < 1) warps = 1;
    const int64_t words = xk_life_resident_words(W, H, warps * 32);
    const int64_t bytes = words * 4;
    if (words < 0 || bytes > xk_max_smem_optin()) return 0;
    *threads = warps * 32;
    *smem_bytes = (int)bytes;
    return 1;
}

static int resident_plan_for(xk_model *m)
{
    return xk_life_resident_config(m->lg.W, m->lg.H, 8, &m->res_threads, &m->res_smem);
}

// Multi-generation steps of a 2-D lattice run in one launch on the resident
// kernel (one CTA) or on a cluster of 2..16 CTAs (cluster.cu).  On the first
// such step the candidates (cluster sizes, and bands of 1, 2 or 4 rows per
// lane group) are timed over 32 generations on the ping-pong partner buffer
// (the state is not touched) and the fastest is kept; lattices too large for
// one CTA take the fastest cluster that fits, else the per-generation global
// kernel.  XK_CLUSTER=0 disables clusters and XK_CLUSTER=n asks for a cluster
// of (up to) n CTAs, with bands of XK_CLUSTER_BAND rows (default 2).
static int tune_cluster(xk_model *m)
{
    m->cl_tuned = 1;
    m->cl_C = 0;
    m->cl_sync = 0;
    m->tb_T = 0;
    const char *tenv = getenv("XK_TB");
    if (tenv && tenv[0]) {
        // a fixed temporal-blocking depth (1: the per-generation kernel)
        const int T = atoi(tenv);
        if (T >= 2 && T <= 8 && xk_life_tb_supported(m->lg)) m->tb_T = T;
        return XK_OK;
    }
    const char *env = getenv("XK_CLUSTER");
    if (env && env[0]) {
        const int want = atoi(env);
        const char *benv = getenv("XK_CLUSTER_BAND");
        const int band = benv && benv[0] ? atoi(benv) : 2;
        int C = 0, R = 0, th = 0;
        if (want > 0 && xk_life_cluster_config(m->lg, want, band, &C, &R, &th)) {
            m->cl_C = C;
            m->cl_R = R;
            m->cl_threads = th;
            m->cl_want = want;
            m->cl_band = band;
            const char *senv = getenv("XK_CLUSTER_SYNC");
            const int sync = !senv ? XK_SYNC_BARRIER
                             : strcmp(senv, "p2p") == 0 ? XK_SYNC_NEIGHBOUR
                             : strcmp(senv, "split") == 0 ? XK_SYNC_SPLIT
                             : strcmp(senv, "async") == 0 ? XK_SYNC_ASYNC : XK_SYNC_BARRIER;
            m->cl_sync = xk_life_cluster_has_sync(m->lg, C, R, th, sync) ? sync : XK_SYNC_BARRIER;
        }
        return XK_OK;
    }
    const size_t bytes = (size_t)m->lg.H * m->lg.wpr * 4;
    uint32_t *scratch = m->bits[1 - m->cur];
    XK_CUDA(cudaMemcpyAsync(scratch, m->bits[m->cur], bytes, cudaMemcpyDeviceToDevice, m->stream));
    const int G = 32;
    const int rf = xk_rule_form(m->rule0, m->rule1);
    // device time of `run` (G generations): one untimed run, then the best
    // of three timed ones
    auto time_it = [&](auto run, float *best_ms) -> cudaError_t {
        cudaError_t e = run();
        *best_ms = 1e30f;
        for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
            float ms = 0.f;
            e = cudaEventRecord(m->ev0, m->stream);
            if (e == cudaSuccess) e = run();
            if (e == cudaSuccess) e = cudaEventRecord(m->ev1, m->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(m->ev1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, m->ev0, m->ev1);
            if (e == cudaSuccess) *best_ms = std::min(*best_ms, ms);
        }
        return e;
    };
    float best = 1e30f;
    if (m->resident) {
        XK_CUDA(time_it([&]() {
            return xk_life_step_resident(m->d_inst, 1, scratch, 0, G, m->lg.torus, m->lg.bfill, nullptr,
                                         m->res_threads, m->res_smem, m->stream, rf);
        }, &best));
    }
    if (xk_life_tb_supported(m->lg)) {
        // temporal blocking, 2..8 generations per launch, ping-pong through
        // a temporary partner of the scratch copy
        uint32_t *tmp = nullptr;
        XK_CUDA(cudaMalloc(&tmp, bytes));
        const LifeTable9 t9 = xk_life_table9(m->rule0, m->rule1);
        cudaError_t e = cudaSuccess;
        const LifeTable t = xk_life_table(m->rule0, m->rule1);
        // depth 1: the per-generation kernel, what runs when no plan is kept
        static const int depths[] = {1, 2, 4, 8};
        for (int T : depths) {
            if (T == 1 && m->resident) continue;
            float ms = 0.f;
            e = time_it([&]() {
                uint32_t *a = scratch, *b = tmp;
                cudaError_t r = cudaSuccess;
                for (int g = 0; g < G && r == cudaSuccess; g += T) {
                    r = T == 1 ? xk_life_step_global(a, b, m->lg, t, m->stream)
                               : xk_life_step_tb(a, b, m->lg, t9, T, m->stream);
                    std::swap(a, b);
                }
                return r;
            }, &ms);
            if (e != cudaSuccess) break;
            if (ms < best) {
                best = ms;
                m->tb_T = T == 1 ? 0 : T;
            }
        }
        cudaFree(tmp);
        XK_CUDA(e);
    }
    // clusters: sizes, band lengths and the synchronisation forms
    static const int cand[] = {16, 8, 4, 2};
    static const int bands[] = {1, 2, 4, 8};
    for (int k = 0; k < 64; ++k) {
        const int want = cand[k / 16], band = bands[(k / 4) % 4], sync = k % 4;
        int C = 0, R = 0, th = 0;
        if (!xk_life_cluster_config(m->lg, want, band, &C, &R, &th)) continue;
        if (!xk_life_cluster_has_sync(m->lg, C, R, th, sync)) continue;
        float ms = 0.f;
        XK_CUDA(time_it([&]() {
            return xk_life_step_cluster(scratch, m->lg, m->rule0, m->rule1, G, C, R, th, m->stream, sync);
        }, &ms));
        if (xk_cluster_take_wait_failure()) {
            xk_set_error("cluster step: a CTA gave up waiting for its neighbours' rows");
            return XK_ERR_TIMEOUT;
        }
        if (ms < best) {
            best = ms;
            m->cl_C = C;
            m->cl_R = R;
            m->cl_threads = th;
            m->cl_want = want;
            m->cl_band = band;
            m->cl_sync = sync;
            m->tb_T = 0;
        }
    }
    return XK_OK;
}

static void free_model(xk_model *m)
{
    if (!m) return;
    for (int i = 0; i < 2; ++i) {
        if (m->bits[i]) cudaFree(m->bits[i]);
        if (m->bytes[i]) cudaFree(m->bytes[i]);
        if (m->cells64[i]) cudaFree(m->cells64[i]);
        if (m->cells32[i]) cudaFree(m->cells32[i]);
    }
    if (m->cells16) cudaFree(m->cells16);
    if (m->col_range_d) cudaFree(m->col_range_d);
    for (int i = 0; i < 2; ++i) {
        if (m->vm_code[i]) cudaFree(m->vm_code[i]);
        if (m->vm_consts[i]) cudaFree(m->vm_consts[i]);
    }
    if (m->fld) cudaFree(m->fld);
    if (m->vm_params) cudaFree(m->vm_params);
    if (m->proj) cudaFree(m->proj);
    if (m->proj2) cudaFree(m->proj2);
    if (m->totals) cudaFree(m->totals);
    if (m->stage) cudaFree(m->stage);
    if (m->col) cudaFree(m->col);
    if (m->img) cudaFree(m->img);
    if (m->ring) cudaFree(m->ring);
    for (int k = 0; k < kFrameRing; ++k) {
        if (m->rendered[k]) cudaEventDestroy(m->rendered[k]);
        if (m->copied[k]) cudaEventDestroy(m->copied[k]);
    }
    if (m->copy_stream) cudaStreamDestroy(m->copy_stream);
    if (m->d_inst) cudaFree(m->d_inst);
    if (m->ev0) cudaEventDestroy(m->ev0);
    if (m->ev1) cudaEventDestroy(m->ev1);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

static int upload_inst(xk_model *m)
{
    LifeInst in;
    memset(&in, 0, sizeof(in));
    in.off = 0;
    in.W = m->lg.W;
    in.H = m->lg.H;
    in.wpr = m->lg.wpr;
    in.rlast = m->lg.rlast;
    in.lastmask = m->lg.lastmask;
    in.rule0 = m->rule0;
    in.rule1 = m->rule1;
    in.smem_words = m->res_smem / 4;
    XK_CUDA(cudaMemcpyAsync(m->d_inst, &in, sizeof(in), cudaMemcpyHostToDevice, m->stream));
    return XK_OK;
}

extern "C" int xk_model_create(const xk_desc *desc, xk_model **out)
{
    XK_REQUIRE(desc && out, XK_ERR_ARG, "xk_model_create: null argument");
    *out = nullptr;
    const xk_desc &d = *desc;
    XK_REQUIRE(d.abi_version == XK_ABI_VERSION, XK_ERR_ARG, "ABI version %d, library has %d",
               d.abi_version, XK_ABI_VERSION);
    XK_REQUIRE(d.ndim >= 1 && d.ndim <= XK_MAXDIM, XK_ERR_ARG, "ndim %d outside 1..%d", d.ndim,
               XK_MAXDIM);
    XK_REQUIRE(d.nbr >= 1 && d.nbr <= XK_MAXNBR - 1, XK_ERR_ARG, "%d neighbours outside 1..%d",
               d.nbr, XK_MAXNBR - 1);
    for (int i = 0; i < d.ndim; ++i)
        XK_REQUIRE(d.size[i] >= 1 && d.size[i] <= (1LL << 31) - 1, XK_ERR_ARG,
                   "size[%d] = %lld out of range", i, (long long)d.size[i]);
    XK_REQUIRE(d.state_bytes == 1 || d.state_bytes == 2 || d.state_bytes == 4 || d.state_bytes == 8,
               XK_ERR_ARG, "state_bytes %d", d.state_bytes);
    const int64_t n = cells_of(d);
    XK_REQUIRE(n <= (1LL << 40), XK_ERR_ARG, "lattice of %lld cells too large", (long long)n);
    XK_REQUIRE(d.family == XK_FAMILY_LIFE || d.family == XK_FAMILY_EVOLIFE ||
                   d.family == XK_FAMILY_MASS || d.family == XK_FAMILY_VM || d.family == XK_FAMILY_SHIFT ||
                   d.family == XK_FAMILY_LIFECOLOR || d.family == XK_FAMILY_NOISE ||
                   d.family == XK_FAMILY_GRAVITY,
               XK_ERR_UNSUPPORTED, "model family %d has no kernel in this library", d.family);
    if (d.family == XK_FAMILY_NOISE)
        XK_REQUIRE(d.state_bytes == 2 &&
                       (d.color_kind == XK_COLOR_NONE || d.color_kind == XK_COLOR_MOVING_AVERAGE),
                   XK_ERR_ARG, "noise needs 16-bit cells and MovingAverage colours (or none)");
    if (d.family == XK_FAMILY_LIFECOLOR)
        XK_REQUIRE(is_moore2d(d) && d.state_bytes == 4 &&
                       (d.color_kind == XK_COLOR_NONE || d.color_kind == XK_COLOR_MOVING_AVERAGE),
                   XK_ERR_ARG, "colour Life needs a 2-D Moore lattice of 32-bit cells and MovingAverage "
                   "colours (or none)");
    if (d.family == XK_FAMILY_GRAVITY)
        XK_REQUIRE(is_moore2d(d) && d.state_bytes == 8 &&
                       (d.color_kind == XK_COLOR_NONE || d.color_kind == XK_COLOR_MOVING_AVERAGE),
                   XK_ERR_ARG, "GraviCowboys needs a 2-D Moore lattice of 64-bit cells and MovingAverage "
                   "colours (or none)");
    if (d.family == XK_FAMILY_SHIFT)
        XK_REQUIRE(d.rule0 < (uint32_t)d.nbr, XK_ERR_ARG, "shifting family: neighbour %u of %d",
                   d.rule0, d.nbr);
    if (d.family == XK_FAMILY_MASS)
        XK_REQUIRE(d.ndim == 3 && d.nbr == 6 && !d.torus && d.state_bytes == 4, XK_ERR_ARG,
                   "mass transfer needs a 3-D von Neumann lattice of 32-bit cells with a wall");
    if (d.family == XK_FAMILY_LIFE)
        XK_REQUIRE(d.rule0 >> (d.nbr + 1) == 0 && d.rule1 >> (d.nbr + 1) == 0, XK_ERR_ARG,
                   "rule tables have bits above %d neighbours", d.nbr);
    if (d.family == XK_FAMILY_EVOLIFE)
        XK_REQUIRE(is_moore2d(d) && d.torus && d.state_bytes == 8, XK_ERR_ARG,
                   "EvoLife needs a 2-D Moore torus of 64-bit cells");

    xk_model *m = new (std::nothrow) xk_model();
    XK_REQUIRE(m, XK_ERR_OOM, "host allocation failed");
    m->d = d;
    m->n = n;
    m->rule0 = d.rule0;
    m->rule1 = d.rule1;
    memcpy(m->lut, d.color_lut, sizeof(m->lut));
    m->hf = d.color_history_free;
    int rc = XK_OK;
#define XK_TRY(call)                                                          \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) { rc = xk_cuda_status(e_, #call); goto fail; } \
    } while (0)
    XK_TRY(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    XK_TRY(cudaEventCreate(&m->ev0));
    XK_TRY(cudaEventCreate(&m->ev1));
    {
        const int border_state = (int)(d.border_value & 1u);
        if (d.family == XK_FAMILY_VM) {
            m->layout = LAYOUT_VM;
            const size_t bytes = (size_t)(d.nbr + 1) * n * d.state_bytes + 16;
            XK_TRY(cudaMalloc(&m->fld, bytes));
            XK_TRY(cudaMemsetAsync(m->fld, 0, bytes, m->stream));
            XK_TRY(cudaMalloc(&m->vm_params, XK_VM_MAX_PARAMS * sizeof(uint64_t)));
            XK_TRY(cudaMemsetAsync(m->vm_params, 0, XK_VM_MAX_PARAMS * sizeof(uint64_t), m->stream));
            memset(&m->vg, 0, sizeof(m->vg));
            m->vg.ndim = d.ndim;
            m->vg.nbr = d.nbr;
            m->vg.torus = d.torus;
            m->vg.esz = d.state_bytes;
            m->vg.n = n;
            for (int i = 0; i < d.ndim; ++i) m->vg.size[i] = d.size[i];
            memcpy(m->vg.delta, d.delta, sizeof(m->vg.delta));
            m->vg.border = d.border_value;
            m->vg.color_kind = d.color_kind;
            m->vg.fade_in = d.fade_in;
            m->vg.fade_out = d.fade_out;
            m->vg.smooth = d.smooth;
        } else if (d.family == XK_FAMILY_MASS) {
            m->layout = LAYOUT_MASS;
            // pitched rows (xk_mass_pitch); padding cells stay 0
            const size_t bytes = (size_t)xk_mass_pitch(d.size[0]) * d.size[1] * d.size[2] * 4;
            XK_TRY(cudaMalloc(&m->cells32[0], bytes));
            XK_TRY(cudaMalloc(&m->cells32[1], bytes));
            XK_TRY(cudaMemsetAsync(m->cells32[0], 0, bytes, m->stream));
            XK_TRY(cudaMemsetAsync(m->cells32[1], 0, bytes, m->stream));
            XK_TRY(cudaMalloc(&m->proj, (size_t)d.size[0] * d.size[1] * 4));
        } else if (d.family == XK_FAMILY_NOISE) {
            m->layout = LAYOUT_NOISE;
            XK_TRY(cudaMalloc(&m->cells16, (size_t)n * 2));
            XK_TRY(cudaMemsetAsync(m->cells16, 0, (size_t)n * 2, m->stream));
        } else if (d.family == XK_FAMILY_LIFECOLOR) {
            m->layout = LAYOUT_LCOLOR;
            XK_TRY(cudaMalloc(&m->cells32[0], (size_t)n * 4));
            XK_TRY(cudaMalloc(&m->cells32[1], (size_t)n * 4));
            XK_TRY(cudaMemsetAsync(m->cells32[0], 0, (size_t)n * 4, m->stream));
        } else if (d.family == XK_FAMILY_GRAVITY) {
            m->layout = LAYOUT_GRAVITY;
            XK_TRY(cudaMalloc(&m->cells64[0], (size_t)n * 8));
            XK_TRY(cudaMalloc(&m->cells64[1], (size_t)n * 8));
            XK_TRY(cudaMemsetAsync(m->cells64[0], 0, (size_t)n * 8, m->stream));
        } else if (d.family == XK_FAMILY_EVOLIFE) {
            m->layout = LAYOUT_CELLS64;
            XK_TRY(cudaMalloc(&m->cells64[0], (size_t)n * 8));
            XK_TRY(cudaMalloc(&m->cells64[1], (size_t)n * 8));
            XK_TRY(cudaMemsetAsync(m->cells64[0], 0, (size_t)n * 8, m->stream));
            XK_TRY(xk_evolife_set_positional(d.palette));
            m->mut_thresh = below_threshold(d.mutation_prob);
        } else if (d.family == XK_FAMILY_LIFE && is_moore2d(d)) {
            m->layout = LAYOUT_BITS2D;
            m->lg = xk_life_geo(d.size[0], d.size[1], d.torus, border_state);
            const size_t words = (size_t)m->lg.H * m->lg.wpr;
            XK_TRY(cudaMalloc(&m->bits[0], (words + 4) * 4));
            XK_TRY(cudaMalloc(&m->bits[1], (words + 4) * 4));
            XK_TRY(cudaMemsetAsync(m->bits[0], 0, (words + 4) * 4, m->stream));
            XK_TRY(cudaMalloc(&m->d_inst, sizeof(LifeInst)));
            m->resident = resident_plan_for(m);
        } else {
            m->layout = LAYOUT_BYTES;
            memset(&m->ng, 0, sizeof(m->ng));
            m->ng.ndim = d.ndim;
            m->ng.nbr = d.nbr;
            m->ng.torus = d.torus;
            m->ng.border_state = (uint32_t)border_state;
            for (int i = 0; i < d.ndim; ++i) m->ng.size[i] = d.size[i];
            memcpy(m->ng.delta, d.delta, sizeof(m->ng.delta));
            const size_t bytes = ((size_t)n + 15) / 16 * 16 + 16;
            XK_TRY(cudaMalloc(&m->bytes[0], bytes));
            XK_TRY(cudaMalloc(&m->bytes[1], bytes));
            XK_TRY(cudaMemsetAsync(m->bytes[0], 0, bytes, m->stream));
        }
        if (m->layout != LAYOUT_CELLS64 && m->layout != LAYOUT_MASS && m->layout != LAYOUT_VM &&
            m->layout != LAYOUT_LCOLOR && m->layout != LAYOUT_NOISE && m->layout != LAYOUT_GRAVITY)
            XK_TRY(cudaMalloc(&m->stage, (size_t)n * d.state_bytes + 16));
        XK_TRY(cudaMalloc(&m->col, (size_t)n * 3 * sizeof(int32_t)));
        XK_TRY(cudaMemsetAsync(m->col, 0, (size_t)n * 3 * sizeof(int32_t), m->stream));
    }
    if (m->layout == LAYOUT_BITS2D) {
        rc = upload_inst(m);
        if (rc != XK_OK) goto fail;
    }
    XK_TRY(cudaStreamSynchronize(m->stream));
#undef XK_TRY
    *out = m;
    return XK_OK;
fail:
    free_model(m);
    return rc;
}

extern "C" void xk_model_destroy(xk_model *m)
{
    if (m) settle_pending_step(m);
    if (m && m->stream) cudaStreamSynchronize(m->stream);
    free_model(m);
}

extern "C" int xk_upload(xk_model *m, const void *host_main, int64_t ncells)
{
    XK_REQUIRE(m && host_main, XK_ERR_ARG, "xk_upload: null argument");
    XK_REQUIRE(ncells == m->n, XK_ERR_ARG, "xk_upload: %lld cells given, model has %lld",
               (long long)ncells, (long long)m->n);
    const int esz = m->d.state_bytes;
    if (m->layout == LAYOUT_CELLS64 || m->layout == LAYOUT_MASS || m->layout == LAYOUT_VM ||
        m->layout == LAYOUT_LCOLOR || m->layout == LAYOUT_NOISE || m->layout == LAYOUT_GRAVITY) {
        void *dst = m->layout == LAYOUT_MASS || m->layout == LAYOUT_LCOLOR ? (void *)m->cells32[m->cur]
                    : m->layout == LAYOUT_NOISE ? (void *)m->cells16
                    : m->layout == LAYOUT_VM ? (void *)m->fld : (void *)m->cells64[m->cur];
        if (m->layout == LAYOUT_MASS) {
            // W cells per row into rows of the pitch; the padding keeps its 0s
            const int64_t W = m->d.size[0];
            XK_CUDA(cudaMemcpy2DAsync(dst, (size_t)xk_mass_pitch(W) * 4, host_main, (size_t)W * 4,
                                      (size_t)W * 4, (size_t)(m->n / W), cudaMemcpyHostToDevice,
                                      m->stream));
        } else {
            XK_CUDA(cudaMemcpyAsync(dst, host_main, (size_t)m->n * esz, cudaMemcpyHostToDevice,
                                    m->stream));
        }
        if (m->layout == LAYOUT_MASS) {
            // the total decides the kernel for good: mass is conserved
            if (m->totals_cap < 1) {
                XK_CUDA(cudaMalloc(&m->totals, sizeof(unsigned long long)));
                m->totals_cap = 1;
            }
            unsigned long long tot = 0;
            XK_CUDA(xk_mass_sum((const uint32_t *)dst, xk_mass_pitch(m->d.size[0]) * (m->n / m->d.size[0]),
                                m->totals, m->stream));
            XK_CUDA(cudaMemcpyAsync(&tot, m->totals, sizeof(tot), cudaMemcpyDeviceToHost, m->stream));
            XK_CUDA(cudaStreamSynchronize(m->stream));
            m->mass_small = tot < (1ull << 30);
            m->totals_count = 0;
        }
        XK_CUDA(cudaStreamSynchronize(m->stream));
        m->proj_valid = 0;
        m->uploaded = 1;
        return XK_OK;
    }
    XK_CUDA(cudaMemcpyAsync(m->stage, host_main, (size_t)m->n * esz, cudaMemcpyHostToDevice,
                            m->stream));
    unsigned int *bad;
    if (m->layout == LAYOUT_BITS2D) {
        XK_CUDA(xk_life_pack(m->stage, esz, m->bits[m->cur], m->lg, m->stream));
        bad = (unsigned int *)(m->bits[m->cur] + (int64_t)m->lg.H * m->lg.wpr);
    } else {
        XK_CUDA(xk_nd_pack(m->stage, esz, m->bytes[m->cur], m->n, m->stream));
        bad = (unsigned int *)(m->bytes[m->cur] + ((m->n + 15) / 16) * 16);
    }
    unsigned int hbad = 0;
    XK_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, m->stream));
    XK_CUDA(cudaStreamSynchronize(m->stream));
    XK_REQUIRE(hbad == 0, XK_ERR_ARG,
               "Life-like kernel needs every cell state to be 0 or 1; the upload has other values");
    m->uploaded = 1;
    return XK_OK;
}

extern "C" int xk_download(xk_model *m, void *host_main, int64_t ncells)
{
    XK_REQUIRE(m && host_main, XK_ERR_ARG, "xk_download: null argument");
    XK_REQUIRE(ncells == m->n, XK_ERR_ARG, "xk_download: %lld cells given, model has %lld",
               (long long)ncells, (long long)m->n);
    const int esz = m->d.state_bytes;
    if (m->layout == LAYOUT_CELLS64 || m->layout == LAYOUT_MASS || m->layout == LAYOUT_VM ||
        m->layout == LAYOUT_LCOLOR || m->layout == LAYOUT_NOISE || m->layout == LAYOUT_GRAVITY) {
        const void *src = m->layout == LAYOUT_MASS || m->layout == LAYOUT_LCOLOR ? (const void *)m->cells32[m->cur]
                          : m->layout == LAYOUT_NOISE ? (const void *)m->cells16
                          : m->layout == LAYOUT_VM ? (const void *)m->fld
                                                   : (const void *)m->cells64[m->cur];
        if (m->layout == LAYOUT_MASS) {
            const int64_t W = m->d.size[0];
            XK_CUDA(cudaMemcpy2DAsync(host_main, (size_t)W * 4, src, (size_t)xk_mass_pitch(W) * 4,
                                      (size_t)W * 4, (size_t)(m->n / W), cudaMemcpyDeviceToHost,
                                      m->stream));
        } else {
            XK_CUDA(cudaMemcpyAsync(host_main, src, (size_t)m->n * esz, cudaMemcpyDeviceToHost,
                                    m->stream));
        }
        XK_CUDA(cudaStreamSynchronize(m->stream));
        return XK_OK;
    }
    if (m->layout == LAYOUT_BITS2D)
        XK_CUDA(xk_life_unpack(m->bits[m->cur], m->stage, esz, m->lg, m->stream));
    else
        XK_CUDA(xk_nd_unpack(m->bytes[m->cur], m->stage, esz, m->n, m->stream));
    XK_CUDA(cudaMemcpyAsync(host_main, m->stage, (size_t)m->n * esz, cudaMemcpyDeviceToHost,
                            m->stream));
    XK_CUDA(cudaStreamSynchronize(m->stream));
    // the neighbour form of the cluster kernel records bounded waits that
    // gave up; the steps do not synchronise, so it is checked here
    if (m->layout == LAYOUT_BITS2D && xk_cluster_take_wait_failure()) {
        xk_set_error("cluster step: a CTA gave up waiting for its neighbours' rows; the cells are "
                     "not valid");
        return XK_ERR_TIMEOUT;
    }
    return XK_OK;
}

// write the colours implied by the state into m->col
static int materialize_colors(xk_model *m)
{
    if (m->layout == LAYOUT_VM || m->layout == LAYOUT_LCOLOR || m->layout == LAYOUT_NOISE ||
        m->layout == LAYOUT_GRAVITY)
        return XK_OK;   // the steps write the colours
    if (m->layout == LAYOUT_MASS) {
        XK_CUDA(xk_mass_colors(m->cells32[m->cur], m->col, m->d, m->stream));
        return XK_OK;
    }
    if (!m->derived) return XK_OK;
    const int smooth = m->d.color_kind == XK_COLOR_MOVING_AVERAGE ? m->d.smooth : 1;
    if (m->layout == LAYOUT_BITS2D)
        XK_CUDA(xk_life_colors(m->bits[m->cur], m->col, m->lg, m->lut, smooth, m->stream));
    else
        XK_CUDA(xk_nd_colors(m->bytes[m->cur], m->col, m->n, m->lut, smooth, m->stream));
    m->derived = 0;
    return XK_OK;
}

extern "C" int xk_upload_colors(xk_model *m, const int32_t *host_col, int64_t ncells)
{
    XK_REQUIRE(m && host_col, XK_ERR_ARG, "xk_upload_colors: null argument");
    XK_REQUIRE(ncells == m->n, XK_ERR_ARG, "xk_upload_colors: cell count mismatch");
    // mass transfer: the colour is a function of the state, recomputed from
    // it whenever it is read, so uploaded colours would never be seen
    if (m->layout == LAYOUT_MASS) return XK_OK;
    XK_CUDA(cudaMemcpyAsync(m->col, host_col, (size_t)m->n * 3 * sizeof(int32_t),
                            cudaMemcpyHostToDevice, m->stream));
    // the range of the uploaded values, for the host's colour bookkeeping
    // (xk_colors_range), reduced on the device while the copy is fresh
    if (!m->col_range_d) XK_CUDA(cudaMalloc(&m->col_range_d, 2 * sizeof(int)));
    XK_CUDA(xk_colors_minmax(m->col, m->n * 3, m->col_range_d, m->stream));
    XK_CUDA(cudaMemcpyAsync(m->col_range, m->col_range_d, 2 * sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    XK_CUDA(cudaStreamSynchronize(m->stream));
    m->derived = 0;
    return XK_OK;
}

extern "C" int xk_colors_range(const xk_model *m, int32_t out[2])
{
    XK_REQUIRE(m && out, XK_ERR_ARG, "xk_colors_range: null argument");
    out[0] = m->col_range[0];
    out[1] = m->col_range[1];
    return XK_OK;
}

extern "C" int xk_download_colors(xk_model *m, int32_t *host_col, int64_t ncells)
{
    XK_REQUIRE(m && host_col, XK_ERR_ARG, "xk_download_colors: null argument");
    XK_REQUIRE(ncells == m->n, XK_ERR_ARG, "xk_download_colors: cell count mismatch");
    int rc = materialize_colors(m);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaMemcpyAsync(host_col, m->col, (size_t)m->n * 3 * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, m->stream));
    XK_CUDA(cudaStreamSynchronize(m->stream));
    return XK_OK;
}

extern "C" int xk_life_set_rule(xk_model *m, uint32_t rule0, uint32_t rule1,
                                const int32_t color_lut[6])
{
    XK_REQUIRE(m, XK_ERR_ARG, "xk_life_set_rule: null model");
    XK_REQUIRE(m->d.family == XK_FAMILY_LIFE, XK_ERR_STATE, "not a Life-like model");
    XK_REQUIRE(rule0 >> (m->d.nbr + 1) == 0 && rule1 >> (m->d.nbr + 1) == 0, XK_ERR_ARG,
               "rule tables have bits above %d neighbours", m->d.nbr);
    if (color_lut && memcmp(color_lut, m->lut, sizeof(m->lut)) != 0) {
        // colours shown until the next step follow the table they were made with
        int rc = materialize_colors(m);
        if (rc != XK_OK) return rc;
        memcpy(m->lut, color_lut, sizeof(m->lut));
    }
    if (rule0 != m->rule0 || rule1 != m->rule1) {
        m->rule0 = rule0;
        m->rule1 = rule1;
        if (m->layout == LAYOUT_BITS2D) return upload_inst(m);
    }
    return XK_OK;
}

extern "C" int xk_set_color_mode(xk_model *m, int32_t history_free)
{
    XK_REQUIRE(m, XK_ERR_ARG, "xk_set_color_mode: null model");
    if (!history_free) {
        int rc = materialize_colors(m);
        if (rc != XK_OK) return rc;
    }
    m->hf = history_free ? 1 : 0;
    return XK_OK;
}

static int life_color_step(xk_model *m)
{
    if (m->d.color_kind == XK_COLOR_NONE) return XK_OK;
    const int plain = m->d.color_kind == XK_COLOR_PLAIN;
    if (m->layout == LAYOUT_BITS2D)
        XK_CUDA(xk_life_color_step(m->bits[m->cur], m->col, m->lg, m->lut, m->d.fade_in,
                                   m->d.fade_out, m->d.smooth, plain, m->stream));
    else
        XK_CUDA(xk_nd_color_step(m->bytes[m->cur], m->col, m->n, m->lut, m->d.fade_in,
                                 m->d.fade_out, m->d.smooth, plain, m->stream));
    return XK_OK;
}

// A call of `nsteps` generations in three parts: what must exist before the
// timed region (totals buffer, materialised colours, the cluster plan), the
// stream-ordered launches of generations [first, first + count) of the call,
// and the bookkeeping after the last one.
static bool colors_free_of(const xk_model *m)
{
    return m->hf || m->d.color_kind == XK_COLOR_NONE;
}

static int step_prepare(xk_model *m, int64_t nsteps)
{
    if (m->layout == LAYOUT_MASS) {
        if (nsteps > m->totals_cap) {
            if (m->totals) cudaFree(m->totals);
            m->totals = nullptr;
            m->totals_cap = 0;
            XK_CUDA(cudaMalloc(&m->totals, (size_t)nsteps * sizeof(unsigned long long)));
            m->totals_cap = nsteps;
        }
        XK_CUDA(cudaMemsetAsync(m->totals, 0, (size_t)nsteps * sizeof(unsigned long long), m->stream));
        return XK_OK;
    }
    if (m->layout == LAYOUT_VM || m->layout == LAYOUT_CELLS64 || m->layout == LAYOUT_LCOLOR ||
        m->layout == LAYOUT_NOISE || m->layout == LAYOUT_GRAVITY)
        return XK_OK;
    const bool colors_free = colors_free_of(m);
    if (!colors_free) {
        int rc = materialize_colors(m);
        if (rc != XK_OK) return rc;
    }
    if (m->layout == LAYOUT_BITS2D && colors_free && !m->cl_tuned) {
        int rc = tune_cluster(m);
        if (rc != XK_OK) return rc;
    }
    return XK_OK;
}

// XK_SHIFT_JUMP=0 in the environment steps the shifting family one
// generation per launch even where one gather would do (for comparison)
static bool shift_jump_enabled()
{
    const char *v = getenv("XK_SHIFT_JUMP");
    return !(v && v[0] == '0');
}

// frame (EvoLife, count == 1 only): the generation's zoom-1 frame written by
// the step kernel itself; proj (mass transfer, count == 1 only): the step
// kernel also adds the new state's column colour sums into it, and with
// frame_prev writes the previous generation's frame from proj_prev
static int step_enqueue(xk_model *m, int64_t first, int64_t count, uint8_t *frame = nullptr,
                        uint32_t *proj = nullptr, uint32_t *proj_prev = nullptr, uint8_t *frame_prev = nullptr)
{
    if (m->layout == LAYOUT_VM) {
        for (int64_t g = 0; g < count; ++g)
            for (int w = 0; w < 2; ++w)
                XK_CUDA(xk_vm_run(m->vm_code[w], m->vm_ncode[w], m->vm_consts[w], m->vm_params,
                                  m->fld, m->col, m->vg, m->stream));
        return XK_OK;
    }
    if (m->layout == LAYOUT_MASS) {
        for (int64_t g = 0; g < count; ++g) {
            XK_CUDA(xk_mass_step(m->cells32[m->cur], m->cells32[1 - m->cur], m->totals + first + g,
                                 m->d, m->mass_small, m->stream, proj, proj_prev, frame_prev));
            m->cur = 1 - m->cur;
        }
        return XK_OK;
    }
    if (m->layout == LAYOUT_CELLS64) {
        for (int64_t g = 0; g < count; ++g) {
            XK_CUDA(xk_evolife_step(m->cells64[m->cur], m->cells64[1 - m->cur], m->col, m->d,
                                    m->mut_thresh, m->stream, frame, m->d.render_smooth));
            m->cur = 1 - m->cur;
        }
        return XK_OK;
    }
    if (m->layout == LAYOUT_NOISE) {
        // cells are independent: up to 1024 generations per launch (one with a frame)
        for (int64_t g = 0; g < count;) {
            const int gens = frame ? 1 : (int)std::min<int64_t>(1024, count - g);
            XK_CUDA(xk_noise_step(m->cells16, m->col, m->d, m->n, gens, m->stream, frame, m->d.render_smooth));
            g += gens;
        }
        return XK_OK;
    }
    if (m->layout == LAYOUT_GRAVITY) {
        for (int64_t g = 0; g < count; ++g) {
            XK_CUDA(xk_gravity_step(m->cells64[m->cur], m->cells64[1 - m->cur], m->col, m->d, m->stream,
                                    frame, m->d.render_smooth));
            m->cur = 1 - m->cur;
        }
        return XK_OK;
    }
    if (m->layout == LAYOUT_LCOLOR) {
        for (int64_t g = 0; g < count; ++g) {
            XK_CUDA(xk_lifecolor_step(m->cells32[m->cur], m->cells32[1 - m->cur], m->col, m->d, m->stream,
                                      frame, m->d.render_smooth));
            m->cur = 1 - m->cur;
        }
        return XK_OK;
    }
    const bool colors_free = colors_free_of(m);
    if (m->layout == LAYOUT_BITS2D && colors_free && m->cl_C) {
        // whole lattice in the shared memory of a cluster; long runs are cut
        // into launches of at most 4096 generations
        int64_t left = count;
        while (left > 0) {
            const int g = (int)(left > 4096 ? 4096 : left);
            XK_CUDA(xk_life_step_cluster(m->bits[m->cur], m->lg, m->rule0, m->rule1, g, m->cl_C, m->cl_R,
                                         m->cl_threads, m->stream, m->cl_sync));
            left -= g;
        }
    } else if (m->d.family == XK_FAMILY_SHIFT && m->d.torus && colors_free && shift_jump_enabled()) {
        // every generation moves the states by the same offset: one gather
        XK_CUDA(xk_shift_jump(m->bytes[m->cur], m->bytes[1 - m->cur], m->ng, (int)m->rule0, count,
                              m->stream));
        m->cur = 1 - m->cur;
    } else if (m->layout == LAYOUT_BITS2D && colors_free && m->tb_T > 1) {
        // temporal blocking: launches of tb_T generations, the rest in one
        // shorter launch; ping-pong between the two word buffers
        const LifeTable9 t9 = xk_life_table9(m->rule0, m->rule1);
        int64_t left = count;
        while (left > 0) {
            const int T = (int)(left >= m->tb_T ? m->tb_T : left);
            XK_CUDA(xk_life_step_tb(m->bits[m->cur], m->bits[1 - m->cur], m->lg, t9, T, m->stream));
            m->cur = 1 - m->cur;
            left -= T;
        }
    } else if (m->layout == LAYOUT_BITS2D && m->resident && colors_free) {
        // whole lattice in shared memory; long runs are cut into launches of
        // at most 4096 generations
        int64_t left = count;
        while (left > 0) {
            const int g = (int)(left > 4096 ? 4096 : left);
            XK_CUDA(xk_life_step_resident(m->d_inst, 1, m->bits[m->cur], 0, g, m->lg.torus,
                                          m->lg.bfill, nullptr, m->res_threads, m->res_smem,
                                          m->stream, xk_rule_form(m->rule0, m->rule1)));
            left -= g;
        }
    } else {
        const LifeTable t = xk_life_table(m->rule0, m->rule1);
        for (int64_t s = 0; s < count; ++s) {
            if (m->layout == LAYOUT_BITS2D) {
                if (m->resident)
                    XK_CUDA(xk_life_step_resident(m->d_inst, 1, m->bits[m->cur], 0, 1, m->lg.torus,
                                                  m->lg.bfill, nullptr, m->res_threads,
                                                  m->res_smem, m->stream,
                                                  xk_rule_form(m->rule0, m->rule1)));
                else {
                    XK_CUDA(xk_life_step_global(m->bits[m->cur], m->bits[1 - m->cur], m->lg, t,
                                                m->stream));
                    m->cur = 1 - m->cur;
                }
            } else {
                if (m->d.family == XK_FAMILY_SHIFT)
                    XK_CUDA(xk_shift_step_nd(m->bytes[m->cur], m->bytes[1 - m->cur], m->ng, (int)m->rule0,
                                             m->stream));
                else
                    XK_CUDA(xk_life_step_nd(m->bytes[m->cur], m->bytes[1 - m->cur], m->ng, m->rule0,
                                            m->rule1, m->stream));
                m->cur = 1 - m->cur;
            }
            if (!colors_free) {
                int rc = life_color_step(m);
                if (rc != XK_OK) return rc;
            }
        }
    }
    // history-free colours are implied by the state from here on
    if (colors_free && m->d.color_kind != XK_COLOR_NONE) m->derived = 1;
    return XK_OK;
}

static int step_finish(xk_model *m, int64_t nsteps)
{
    if (m->layout == LAYOUT_MASS) {
        m->totals_count = nsteps;
        m->proj_valid = 0;
        if (xk_mass_take_wait_failure()) {
            xk_set_error("mass-transfer step: a CTA gave up waiting for a tensor copy");
            return XK_ERR_TIMEOUT;
        }
    }
    return XK_OK;
}

// device time between a model's step events (waits for the step)
static float pending_step_ms(xk_model *m)
{
    float ms = 0.f;
    if (cudaEventSynchronize(m->ev1) != cudaSuccess || cudaEventElapsedTime(&ms, m->ev0, m->ev1) != cudaSuccess) {
        cudaGetLastError();
        return 0.f;
    }
    return ms;
}

extern "C" int xk_step(xk_model *m, int64_t nsteps)
{
    XK_REQUIRE(m, XK_ERR_ARG, "xk_step: null model");
    XK_REQUIRE(nsteps >= 0, XK_ERR_ARG, "xk_step: negative step count");
    XK_REQUIRE(m->uploaded, XK_ERR_STATE, "xk_step before xk_upload");
    if (nsteps == 0) return XK_OK;
    int rc = step_prepare(m, nsteps);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaEventRecord(m->ev0, m->stream));
    rc = step_enqueue(m, 0, nsteps);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaEventRecord(m->ev1, m->stream));
    if (m->layout == LAYOUT_MASS) {
        // the mass kernels' give-up flag is read after the step
        XK_CUDA(cudaEventSynchronize(m->ev1));
        float ms = 0.f;
        XK_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
        xk_set_last_step_ms(ms);
    } else {
        // returns once the work is queued, as the reference's step() does
        // (its launches are asynchronous); xk_last_step_ms waits for it
        set_pending_step(m);
    }
    return step_finish(m, nsteps);
}

// ---------------------------------------------------------------------------
// launch plans of 2-D Life-like models (the autotuner's choice), for a cache

static bool plan_applies(const xk_model *m)
{
    return m->layout == LAYOUT_BITS2D && colors_free_of(m);
}

extern "C" int xk_model_plan(xk_model *m, int32_t plan[4])
{
    XK_REQUIRE(m && plan, XK_ERR_ARG, "xk_model_plan: null argument");
    XK_REQUIRE(m->uploaded, XK_ERR_STATE, "xk_model_plan before xk_upload");
    if (!plan_applies(m)) {
        plan[0] = -1;
        plan[1] = plan[2] = plan[3] = 0;
        return XK_OK;
    }
    if (!m->cl_tuned) {
        int rc = tune_cluster(m);
        if (rc != XK_OK) return rc;
    }
    if (m->cl_C) {
        plan[0] = XK_PLAN_CLUSTER;
        plan[1] = m->cl_want;
        plan[2] = m->cl_band;
        plan[3] = m->cl_sync;
    } else if (m->tb_T > 1) {
        plan[0] = XK_PLAN_TEMPORAL;
        plan[1] = plan[2] = 0;
        plan[3] = m->tb_T;
    } else {
        plan[0] = m->resident ? XK_PLAN_RESIDENT : XK_PLAN_GLOBAL;
        plan[1] = plan[2] = plan[3] = 0;
    }
    return XK_OK;
}

extern "C" int32_t xk_model_rule_form(const xk_model *m)
{
    if (!m || m->layout != LAYOUT_BITS2D) return -1;
    return xk_rule_form(m->rule0, m->rule1);
}

extern "C" int xk_model_set_plan(xk_model *m, const int32_t plan[4])
{
    XK_REQUIRE(m && plan, XK_ERR_ARG, "xk_model_set_plan: null argument");
    XK_REQUIRE(plan_applies(m), XK_ERR_STATE,
               "xk_model_set_plan: only 2-D Life-like models with colours implied by the state "
               "have launch plans");
    int C = 0, R = 0, th = 0;
    switch (plan[0]) {
    case XK_PLAN_GLOBAL:
        XK_REQUIRE(!m->resident, XK_ERR_ARG, "xk_model_set_plan: this lattice fits one CTA");
        break;
    case XK_PLAN_RESIDENT:
        XK_REQUIRE(m->resident, XK_ERR_ARG, "xk_model_set_plan: the lattice does not fit one CTA");
        break;
    case XK_PLAN_CLUSTER:
        XK_REQUIRE(plan[1] >= 1 && plan[1] <= 16 && plan[2] >= 1 &&
                       xk_life_cluster_config(m->lg, plan[1], plan[2], &C, &R, &th),
                   XK_ERR_ARG, "xk_model_set_plan: no cluster of %d CTAs with bands of %d rows",
                   plan[1], plan[2]);
        XK_REQUIRE(plan[3] >= XK_SYNC_BARRIER && plan[3] <= XK_SYNC_ASYNC &&
                       xk_life_cluster_has_sync(m->lg, C, R, th, plan[3]),
                   XK_ERR_ARG, "xk_model_set_plan: cluster synchronisation form %d does not apply "
                   "(1: bands of 1, 2 or 4 rows; 2: every CTA's bands 4 or 8 rows; 3: bands of "
                   "1 row, or every CTA's bands 2, 4 or 8 rows)", plan[3]);
        break;
    case XK_PLAN_TEMPORAL:
        XK_REQUIRE(plan[3] >= 2 && plan[3] <= 8 && xk_life_tb_supported(m->lg), XK_ERR_ARG,
                   "xk_model_set_plan: temporal depth %d (2..8, width >= 64)", plan[3]);
        break;
    default:
        XK_REQUIRE(false, XK_ERR_ARG, "xk_model_set_plan: unknown plan kind %d", plan[0]);
    }
    m->cl_tuned = 1;
    m->cl_C = C;
    m->cl_R = R;
    m->cl_threads = th;
    m->cl_want = plan[0] == XK_PLAN_CLUSTER ? plan[1] : 0;
    m->cl_band = plan[0] == XK_PLAN_CLUSTER ? plan[2] : 0;
    m->cl_sync = plan[0] == XK_PLAN_CLUSTER ? plan[3] : 0;
    m->tb_T = plan[0] == XK_PLAN_TEMPORAL ? plan[3] : 0;
    return XK_OK;
}

// RendererPlain of the current state into `img` (int32 or the uint8 frame),
// stream-ordered on the model's stream
static int render_enqueue(xk_model *m, void *img, bool bytes, int32_t width, int32_t height,
                          int32_t zoom, int32_t dx, int32_t dy)
{
    if (m->layout == LAYOUT_MASS && m->d.proj_axis0 == 0 && m->d.proj_axis1 == 1 &&
        m->d.render_smooth == 0) {
        if (bytes && !m->proj_valid && zoom == 1 && dx == 0 && dy == 0 && width == m->d.size[0] &&
            height == m->d.size[1]) {
            // the whole lattice at zoom 1: the projection writes the frame
            XK_CUDA(xk_mass_project(m->cells32[m->cur], m->proj, m->d, m->stream, (uint8_t *)img));
            m->proj_valid = 1;
            return XK_OK;
        }
        if (!m->proj_valid) {
            XK_CUDA(xk_mass_project(m->cells32[m->cur], m->proj, m->d, m->stream));
            m->proj_valid = 1;
        }
        if (bytes)
            XK_CUDA(xk_mass_render_u8(m->proj, (uint8_t *)img, m->d, width, height, zoom, dx, dy,
                                      m->stream));
        else
            XK_CUDA(xk_mass_render(m->proj, (int32_t *)img, m->d, width, height, zoom, dx, dy,
                                   m->stream));
        return XK_OK;
    }
    int rc = materialize_colors(m);
    if (rc != XK_OK) return rc;
    RenderGeo g;
    memset(&g, 0, sizeof(g));
    g.ndim = m->d.ndim;
    g.a0 = m->d.proj_axis0;
    g.a1 = m->d.proj_axis1;
    for (int i = 0; i < m->d.ndim; ++i) g.size[i] = m->d.size[i];
    g.smooth = m->d.render_smooth;
    if (bytes)
        XK_CUDA(xk_render_colors_u8(m->col, (uint8_t *)img, g, width, height, zoom, dx, dy, m->stream));
    else
        XK_CUDA(xk_render_colors(m->col, (int32_t *)img, g, width, height, zoom, dx, dy, m->stream));
    return XK_OK;
}

// The mass-transfer frames of xk_step_frames at zoom 1: generation g adds its
// column colour sums into one of two buffers (zero on entry) and writes
// generation g - 1's frame from the other, zeroing it, so no launch comes
// between two generations; the last frame comes from a small kernel after
// the loop.  Host frames go through the device ring as in xk_step_frames.
static int mass_frames_enqueue(xk_model *m, int64_t nsteps, uint8_t *frames, bool on_device, size_t fb)
{
    const size_t pbytes = (size_t)m->d.size[0] * m->d.size[1] * 4;
    if (!m->proj2) XK_CUDA(cudaMalloc(&m->proj2, pbytes));
    uint32_t *P[2] = {m->proj, m->proj2};
    XK_CUDA(cudaMemsetAsync(P[0], 0, pbytes, m->stream));
    XK_CUDA(cudaMemsetAsync(P[1], 0, pbytes, m->stream));
    auto slot = [&](int64_t g) {
        return on_device ? frames + (size_t)g * fb : m->ring + (size_t)(g % kFrameRing) * fb;
    };
    // frame g is about to be written: its ring slot's previous copy must be done
    auto claim = [&](int64_t g) -> int {
        if (!on_device && g >= kFrameRing)
            XK_CUDA(cudaStreamWaitEvent(m->stream, m->copied[g % kFrameRing], 0));
        return XK_OK;
    };
    // frame g is complete: copy it out
    auto release = [&](int64_t g) -> int {
        if (on_device) return XK_OK;
        const int k = (int)(g % kFrameRing);
        XK_CUDA(cudaEventRecord(m->rendered[k], m->stream));
        XK_CUDA(cudaStreamWaitEvent(m->copy_stream, m->rendered[k], 0));
        XK_CUDA(cudaMemcpyAsync(frames + (size_t)g * fb, slot(g), fb, cudaMemcpyDeviceToHost, m->copy_stream));
        XK_CUDA(cudaEventRecord(m->copied[k], m->copy_stream));
        return XK_OK;
    };
    for (int64_t g = 0; g < nsteps; ++g) {
        if (g > 0) {
            int rc = claim(g - 1);
            if (rc != XK_OK) return rc;
        }
        int rc = step_enqueue(m, g, 1, nullptr, P[g & 1], P[(g + 1) & 1], g > 0 ? slot(g - 1) : nullptr);
        if (rc != XK_OK) return rc;
        if (g > 0 && (rc = release(g - 1)) != XK_OK) return rc;
    }
    int rc = claim(nsteps - 1);
    if (rc != XK_OK) return rc;
    uint32_t *last = P[(nsteps - 1) & 1];
    XK_CUDA(xk_mass_frame(last, slot(nsteps - 1), m->d, m->stream));
    if ((rc = release(nsteps - 1)) != XK_OK) return rc;
    // m->proj holds the current state's column sums from here on
    if (last != m->proj) std::swap(m->proj, m->proj2);
    m->proj_valid = 1;
    return XK_OK;
}

extern "C" int xk_step_frames(xk_model *m, int64_t nsteps, int32_t width, int32_t height,
                              int32_t zoom, int32_t dx, int32_t dy, uint8_t *frames,
                              int32_t frames_on_device)
{
    XK_REQUIRE(m && frames, XK_ERR_ARG, "xk_step_frames: null argument");
    XK_REQUIRE(nsteps >= 0, XK_ERR_ARG, "xk_step_frames: negative step count");
    XK_REQUIRE(width > 0 && height > 0 && zoom > 0, XK_ERR_ARG,
               "xk_step_frames: bad viewport %dx%d zoom %d", width, height, zoom);
    XK_REQUIRE(m->uploaded, XK_ERR_STATE, "xk_step_frames before xk_upload");
    if (nsteps == 0) return XK_OK;
    const size_t fb = (size_t)width * height * 3;
    int rc = step_prepare(m, nsteps);
    if (rc != XK_OK) return rc;
    if (!frames_on_device) {
        // a ring of device frames, each copied to the host on its own stream
        // while the next generations run
        if ((int64_t)fb * kFrameRing > m->ring_cap) {
            if (m->ring) cudaFree(m->ring);
            m->ring = nullptr;
            m->ring_cap = 0;
            XK_CUDA(cudaMalloc(&m->ring, fb * kFrameRing));
            m->ring_cap = (int64_t)fb * kFrameRing;
        }
        if (!m->copy_stream) {
            XK_CUDA(cudaStreamCreateWithFlags(&m->copy_stream, cudaStreamNonBlocking));
            for (int k = 0; k < kFrameRing; ++k) {
                XK_CUDA(cudaEventCreateWithFlags(&m->rendered[k], cudaEventDisableTiming));
                XK_CUDA(cudaEventCreateWithFlags(&m->copied[k], cudaEventDisableTiming));
            }
        }
    }
    // EvoLife or colour Life viewed whole at zoom 1: the step kernel writes the frame
    const bool fused = (m->layout == LAYOUT_CELLS64 || m->layout == LAYOUT_LCOLOR || m->layout == LAYOUT_NOISE ||
                        m->layout == LAYOUT_GRAVITY) &&
                       m->d.color_kind != XK_COLOR_NONE &&
                       m->d.ndim == 2 && m->d.proj_axis0 == 0 && m->d.proj_axis1 == 1 && zoom == 1 &&
                       dx == 0 && dy == 0 && width == m->d.size[0] && height == m->d.size[1];
    // mass transfer viewed whole at zoom 1 along z: the step kernel sums the
    // column colours as it writes the cells (no second pass over the state)
    const bool mass_fused = m->layout == LAYOUT_MASS && m->d.proj_axis0 == 0 && m->d.proj_axis1 == 1 &&
                            m->d.render_smooth == 0 && zoom == 1 && dx == 0 && dy == 0 &&
                            width == m->d.size[0] && height == m->d.size[1] && xk_mass_fuses_projection(m->d);
    XK_CUDA(cudaEventRecord(m->ev0, m->stream));
    if (mass_fused) {
        rc = mass_frames_enqueue(m, nsteps, frames, frames_on_device != 0, fb);
        if (rc != XK_OK) return rc;
    }
    for (int64_t g = 0; g < nsteps && !mass_fused; ++g) {
        const int k = (int)(g % kFrameRing);
        uint8_t *dst = frames_on_device ? frames + (size_t)g * fb : m->ring + (size_t)k * fb;
        if (!frames_on_device && g >= kFrameRing)
            XK_CUDA(cudaStreamWaitEvent(m->stream, m->copied[k], 0));
        rc = step_enqueue(m, g, 1, fused ? dst : nullptr);
        if (rc != XK_OK) return rc;
        m->proj_valid = 0;
        if (!fused) {
            rc = render_enqueue(m, dst, true, width, height, zoom, dx, dy);
            if (rc != XK_OK) return rc;
        }
        if (frames_on_device) continue;
        uint8_t *slot = dst;
        XK_CUDA(cudaEventRecord(m->rendered[k], m->stream));
        XK_CUDA(cudaStreamWaitEvent(m->copy_stream, m->rendered[k], 0));
        XK_CUDA(cudaMemcpyAsync(frames + (size_t)g * fb, slot, fb, cudaMemcpyDeviceToHost,
                                m->copy_stream));
        XK_CUDA(cudaEventRecord(m->copied[k], m->copy_stream));
    }
    if (!frames_on_device) {
        const int last = (int)((nsteps - 1) % kFrameRing);
        XK_CUDA(cudaStreamWaitEvent(m->stream, m->copied[last], 0));
    }
    XK_CUDA(cudaEventRecord(m->ev1, m->stream));
    XK_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    XK_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    xk_set_last_step_ms(ms);
    return step_finish(m, nsteps);
}

extern "C" int xk_render(xk_model *m, int32_t *host_img, int32_t width, int32_t height,
                         int32_t zoom, int32_t dx, int32_t dy)
{
    XK_REQUIRE(m && host_img, XK_ERR_ARG, "xk_render: null argument");
    XK_REQUIRE(width > 0 && height > 0 && zoom > 0, XK_ERR_ARG, "xk_render: bad viewport %dx%d zoom %d",
               width, height, zoom);
    const int64_t npx = (int64_t)width * height;
    if (npx * 3 > m->img_cap) {
        if (m->img) cudaFree(m->img);
        m->img = nullptr;
        XK_CUDA(cudaMalloc(&m->img, (size_t)npx * 3 * sizeof(int32_t)));
        m->img_cap = npx * 3;
    }
    int rc = render_enqueue(m, m->img, false, width, height, zoom, dx, dy);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaMemcpyAsync(host_img, m->img, (size_t)npx * 3 * sizeof(int32_t),
                            cudaMemcpyDeviceToHost, m->stream));
    XK_CUDA(cudaStreamSynchronize(m->stream));
    return XK_OK;
}

extern "C" int xk_mass_totals(xk_model *m, uint64_t *host_totals, int64_t count)
{
    XK_REQUIRE(m && host_totals, XK_ERR_ARG, "xk_mass_totals: null argument");
    XK_REQUIRE(m->d.family == XK_FAMILY_MASS, XK_ERR_STATE, "not a mass-transfer model");
    XK_REQUIRE(count == m->totals_count, XK_ERR_ARG,
               "xk_mass_totals: %lld totals asked, the last step recorded %lld", (long long)count,
               (long long)m->totals_count);
    if (count == 0) return XK_OK;
    XK_CUDA(cudaMemcpyAsync(host_totals, m->totals, (size_t)count * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, m->stream));
    XK_CUDA(cudaStreamSynchronize(m->stream));
    return XK_OK;
}

extern "C" int xk_sync(xk_model *m)
{
    XK_REQUIRE(m, XK_ERR_ARG, "xk_sync: null model");
    XK_CUDA(cudaStreamSynchronize(m->stream));
    return XK_OK;
}

extern "C" int xk_set_device(int32_t device)
{
    XK_CUDA(cudaSetDevice(device));
    return XK_OK;
}

extern "C" int xk_host_register(void *ptr, int64_t bytes)
{
    XK_REQUIRE(ptr && bytes > 0, XK_ERR_ARG, "xk_host_register: bad buffer");
    XK_CUDA(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterMapped | cudaHostRegisterPortable));
    return XK_OK;
}

extern "C" int xk_host_unregister(void *ptr)
{
    XK_REQUIRE(ptr, XK_ERR_ARG, "xk_host_unregister: null pointer");
    XK_CUDA(cudaHostUnregister(ptr));
    return XK_OK;
}

extern "C" int xk_range_push(const char *name)
{
    XK_REQUIRE(name, XK_ERR_ARG, "xk_range_push: null name");
    nvtxRangePushA(name);
    return XK_OK;
}

extern "C" int xk_range_pop(void)
{
    nvtxRangePop();
    return XK_OK;
}

// opcodes and type codes of the interpreter (csrc/vm.cu, core/vm.py)
static bool vm_check(const xk_model *m, const xk_vm_ins &in, int nconsts, int nregs, int pc)
{
    const int op = in.op;
    auto reg = [&](int r) { return r >= 0 && r < nregs; };
    if (in.ty > 8) return false;
    switch (op) {
    case 1: return reg(in.dst) && in.a < nconsts;                      // const
    case 2: return reg(in.dst) && in.a < XK_VM_MAX_PARAMS;             // param
    case 3:                                                            // load
        if (!reg(in.dst) || in.a > 3 || in.c > m->d.nbr) return false;
        return in.a < 2 || in.b < m->d.nbr;
    case 4: case 30: case 31: case 32: case 41: case 42: case 50: case 51:
        return reg(in.dst) && reg(in.a);
    case 5: return reg(in.dst) && reg(in.a) && in.b <= 8;               // cvt
    case 40: return reg(in.dst) && reg(in.a) && reg(in.b) && reg(in.c); // select
    case 60: return reg(in.a) && in.b <= m->d.nbr;                     // store
    case 61: return reg(in.a) && reg(in.b) && reg(in.c);               // colour
    default:
        if (op >= 10 && op <= 25) return reg(in.dst) && reg(in.a) && reg(in.b);
        (void)pc;
        return false;
    }
}

extern "C" int xk_vm_load(xk_model *m, int32_t which, const xk_vm_ins *code, int32_t ncode,
                          const uint64_t *consts, int32_t nconsts, int32_t nregs)
{
    XK_REQUIRE(m && (code || ncode == 0) && consts, XK_ERR_ARG, "xk_vm_load: null argument");
    XK_REQUIRE(m->layout == LAYOUT_VM, XK_ERR_STATE, "xk_vm_load: not an interpreter model");
    XK_REQUIRE(which == 0 || which == 1, XK_ERR_ARG, "xk_vm_load: program %d", which);
    XK_REQUIRE(ncode >= 0 && nconsts >= 1 && nregs >= 1 && nregs <= XK_VM_MAX_REGS, XK_ERR_ARG,
               "xk_vm_load: %d instructions, %d constants, %d registers", ncode, nconsts, nregs);
    for (int pc = 0; pc < ncode; ++pc)
        XK_REQUIRE(vm_check(m, code[pc], nconsts, nregs, pc), XK_ERR_ARG,
                   "xk_vm_load: instruction %d (opcode %d) is malformed", pc, code[pc].op);
    if (m->vm_code[which]) cudaFree(m->vm_code[which]);
    if (m->vm_consts[which]) cudaFree(m->vm_consts[which]);
    m->vm_code[which] = nullptr;
    m->vm_consts[which] = nullptr;
    m->vm_ncode[which] = 0;
    if (ncode > 0) {
        XK_CUDA(cudaMalloc(&m->vm_code[which], (size_t)ncode * sizeof(xk_vm_ins)));
        XK_CUDA(cudaMemcpyAsync(m->vm_code[which], code, (size_t)ncode * sizeof(xk_vm_ins),
                                cudaMemcpyHostToDevice, m->stream));
    }
    XK_CUDA(cudaMalloc(&m->vm_consts[which], (size_t)nconsts * sizeof(uint64_t)));
    XK_CUDA(cudaMemcpyAsync(m->vm_consts[which], consts, (size_t)nconsts * sizeof(uint64_t),
                            cudaMemcpyHostToDevice, m->stream));
    XK_CUDA(cudaStreamSynchronize(m->stream));
    m->vm_ncode[which] = ncode;
    return XK_OK;
}

extern "C" int xk_vm_set_params(xk_model *m, const uint64_t *values, int32_t count)
{
    XK_REQUIRE(m && (values || count == 0), XK_ERR_ARG, "xk_vm_set_params: null argument");
    XK_REQUIRE(m->layout == LAYOUT_VM, XK_ERR_STATE, "xk_vm_set_params: not an interpreter model");
    XK_REQUIRE(count >= 0 && count <= XK_VM_MAX_PARAMS, XK_ERR_ARG, "xk_vm_set_params: %d values",
               count);
    if (count == 0) return XK_OK;
    XK_CUDA(cudaMemcpyAsync(m->vm_params, values, (size_t)count * sizeof(uint64_t),
                            cudaMemcpyHostToDevice, m->stream));
    XK_CUDA(cudaStreamSynchronize(m->stream));
    return XK_OK;
}
