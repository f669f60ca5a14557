// Serving loop (include/xk.h, xk_serve_*): continuous batching of independent
// simulation requests on one GPU.
//
// Memory: one device arena (the HBM budget) and one pinned host arena (result
// staging), each allocated once; requests take ranges of both at admission
// (XkArena, first fit) and give the device range back when their result has
// been copied out, the host range when the caller collects the result.
//
// Execution: a worker thread owns every CUDA call after creation.  Each pass
// it (1) retires finished work by polling events, (2) admits queued requests
// first come, first served while their bytes fit and fewer than max_active run,
// (3) starts the next round of every request whose previous round finished,
// and (4) starts the result copy of requests
// that reached their generation count.  Rounds of different requests are
// independent, so a request admitted while others run starts computing at
// once and its kernels overlap theirs on the device.
//
// Paths per request:
//   resident  2-D Life-like lattices that fit one CTA (and at most
//             XK_SERVE_RESIDENT_MAX cells): grouped by CTA shape; a group round
//             is one launch of the resident kernel over the group's idle
//             members (one CTA each, each with its own generation count, about
//             quantum x 2^18 cell-generations), in one of XK_SERVE_GROUP_SLOTS
//             slots, so members admitted while a round runs start at once;
//   global2d  larger 2-D lattices: packed to 32 cells per word once, one
//             bit-sliced launch per generation on the request's stream;
//   life3d    3-D von Neumann Life-like: bit-packed along x like global2d, one
//             launch per generation;
//   mass3d    mass transfer: uint32 ping-pong with the per-generation totals
//             (the fast-only kernel when the submitted total is below 2^30).
// The other paths run rounds of `quantum` generations.  Full rounds of the
// per-request paths are captured once as a CUDA graph (per ping-pong parity)
// and replayed, so a round costs the worker one launch.  Streams carry a
// priority: resident rounds the device's greatest, other requests one level
// lower per factor of 4 of work above 2^26 cell-generations, so the block
// scheduler serves short requests ahead of the kernels of long ones.
// A request's cells see exactly the arithmetic they see alone: every kernel
// touches only its own request's range.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <vector>

#include "arena.h"
#include "xk_internal.cuh"

#define XK_SERVE_MAX_QUANTUM 4096

namespace {

enum Path { PATH_RESIDENT = 0, PATH_GLOBAL2D = 1, PATH_LIFE3D = 2, PATH_MASS3D = 3 };

struct Req {
    int64_t id = 0;
    xk_request r;
    int64_t n = 0;             // cells
    int64_t esz = 1;           // host bytes per cell
    int64_t dev_need = 0, host_need = 0;
    std::vector<uint8_t> input;
    int status = XK_REQ_PENDING;
    int path = PATH_RESIDENT;
    int64_t dev_off = -1, host_off = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    bool ev_pending = false;   // upload, own round or result copy in flight
    bool in_group = false;     // member of its resident group's round in flight
    bool draining = false;     // the pending event is the result copy
    bool cancel = false;
    int64_t done = 0, chunk = 0;
    int64_t last_chunk = 0;    // generations of the last finished round
    int cur = 0;               // ping-pong buffer holding the state
    int group = -1;            // resident group index
    LifeGeo lg;                // bit-packed rows (3-D: H * D rows)
    Life3Geo g3;
    LifeTable lt;
    LifeTable9 lt9;
    int tb_T = 0;              // global2d: generations per temporally blocked launch (0: one per launch)
    xk_desc md;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};   // full round from buffer 0 / 1
    uint32_t rule0 = 0, rule1 = 0;
    int threads = 0, smem = 0;
    double t_submit = -1, t_admit = -1, t_done = -1;
    uint64_t mass_total = 0;
    bool mass_small = false;   // initial total below 2^30
};

// rounds of one resident group that may be in flight at once: a member
// admitted while earlier members run starts in a free slot at once
#define XK_SERVE_GROUP_SLOTS 4

// one round of a resident group: its members, their instance records and
// generation counts (pinned staging, device copy), its stream and event
struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    bool in_flight = false;
    LifeInst *h_inst = nullptr;   // pinned, max_active entries
    LifeInst *d_inst = nullptr;
    int32_t *h_gens = nullptr;    // pinned, max_active entries
    int32_t *d_gens = nullptr;
    bool owned = false;           // arrays allocated for this slot (not carved from the pool)
    std::vector<Req *> members;
};

struct Group {
    int threads = 0, smem = 0;
    Slot slot[XK_SERVE_GROUP_SLOTS];
};

int64_t rnd(int64_t b) { return XkArena::round(b); }

uint32_t life2d_rule0(uint32_t r) { return r & 511u; }
uint32_t life2d_rule1(uint32_t r) { return (r & 511u) | ((r >> 9) & 511u); }
uint32_t life3d_rule0(uint32_t r) { return r & 127u; }
uint32_t life3d_rule1(uint32_t r) { return (r & 127u) | ((r >> 7) & 127u); }

}  // namespace

// device/host bytes of a request (validates it)
// cells of a mass-transfer request's device buffers: rows at the pitch of
// xk_mass_pitch (padding cells hold 0)
static int64_t mass_pitched_cells(const xk_request &r)
{
    return xk_mass_pitch(r.size[0]) * r.size[1] * r.size[2];
}

static int request_layout(const xk_request *q, int64_t *n_out, int64_t *esz_out, int64_t *dev,
                          int64_t *host)
{
    XK_REQUIRE(q, XK_ERR_ARG, "serve: null request");
    XK_REQUIRE(q->kind == XK_SERVE_LIFE2D || q->kind == XK_SERVE_LIFE3D_VN ||
                   q->kind == XK_SERVE_MASS3D,
               XK_ERR_ARG, "serve: unknown request kind %d", q->kind);
    XK_REQUIRE(q->reserved0 == 0 && q->reserved1 == 0, XK_ERR_ARG, "serve: reserved fields not 0");
    XK_REQUIRE(q->generations >= 0, XK_ERR_ARG, "serve: negative generation count %lld",
               (long long)q->generations);
    for (int i = 0; i < 3; ++i)
        XK_REQUIRE(q->size[i] >= 1 && q->size[i] <= (1 << 20), XK_ERR_ARG,
                   "serve: size[%d] = %lld out of [1, 2^20]", i, (long long)q->size[i]);
    const int64_t n = q->size[0] * q->size[1] * q->size[2];
    XK_REQUIRE(n < (1LL << 31), XK_ERR_ARG, "serve: %lld cells (limit 2^31 - 1)", (long long)n);
    if (q->kind == XK_SERVE_LIFE2D) {
        XK_REQUIRE(q->size[2] == 1, XK_ERR_ARG, "serve: 2-D request with size[2] = %lld",
                   (long long)q->size[2]);
        XK_REQUIRE((q->rule >> 18) == 0, XK_ERR_ARG, "serve: 2-D rule %u has bits above 17", q->rule);
        const int64_t words = (q->size[0] + 31) / 32 * q->size[1];
        *dev = rnd(n + 16) + 2 * rnd(words * 4);
        *esz_out = 1;
    } else if (q->kind == XK_SERVE_LIFE3D_VN) {
        XK_REQUIRE((q->rule >> 14) == 0, XK_ERR_ARG, "serve: 3-D rule %u has bits above 13", q->rule);
        const int64_t words = (q->size[0] + 31) / 32 * q->size[1] * q->size[2];
        *dev = rnd(n + 16) + 2 * rnd(words * 4);
        *esz_out = 1;
    } else {
        XK_REQUIRE(q->rule == 0, XK_ERR_ARG, "serve: mass-transfer requests take rule 0");
        *dev = 2 * rnd(4 * mass_pitched_cells(*q)) + rnd(8 * XK_SERVE_MAX_QUANTUM);
        *esz_out = 4;
    }
    *host = rnd(n * *esz_out) + XK_ARENA_ALIGN;
    *n_out = n;
    return XK_OK;
}

struct xk_server {
    int device = 0;
    int64_t budget = 0, host_bytes = 0;
    int max_active = 0;
    int64_t quantum = 0;
    int tb_depth = 8;          // generations per launch of large 2-D requests (XK_SERVE_TB)
    int64_t round_work = 0;    // cell-generations of a resident member's round (quantum x 2^18)
    int prio_least = 0, prio_greatest = 0;   // the device's stream priority range
    // resident-group slot arrays, allocated once at creation (a group created
    // while requests run then costs no page-locked allocation on the worker):
    // slot_pool slots of slot_bytes each, pinned and on the device
    uint8_t *slot_host = nullptr, *slot_dev = nullptr;
    int slot_pool = 0, slot_used = 0;
    int64_t slot_bytes = 0;
    int64_t resident_max = 1 << 18;
    // rows per lane group of resident lattices: 1 gives a lattice as many
    // threads as a CTA holds, so each generation is as short as it can be (a
    // request's latency is its generation count times that); XK_SERVE_BAND
    int resident_band = 1;
    uint8_t *dev_base = nullptr;
    uint8_t *host_base = nullptr;
    unsigned int *bad = nullptr;
    std::unique_ptr<XkArena> dev_arena, host_arena;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stop = false;
    bool failed = false;
    std::string fail_msg;
    int64_t next_id = 1;
    std::map<int64_t, std::unique_ptr<Req>> reqs;
    std::vector<Req *> pending;   // FIFO
    std::vector<Req *> active;    // admitted, not yet finished
    std::vector<Group> groups;
    std::chrono::steady_clock::time_point t0;
    xk_serve_stats st;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

// ---------------------------------------------------------------------------
// worker helpers (called with srv->mu held, on the worker thread)

static void release_device(xk_server *s, Req *q)
{
    if (q->dev_off >= 0) s->dev_arena->release(q->dev_off);
    q->dev_off = -1;
    s->st.device_bytes_in_use = s->dev_arena->in_use();
    for (auto &g : q->graph)
        if (g) cudaGraphExecDestroy(g);
    q->graph[0] = q->graph[1] = nullptr;
    if (q->stream) cudaStreamDestroy(q->stream);
    if (q->ev) cudaEventDestroy(q->ev);
    q->stream = nullptr;
    q->ev = nullptr;
}

static bool graphs_enabled()
{
    const char *v = getenv("XK_GRAPHS");
    return !(v && v[0] == '0');
}

static void drop_active(xk_server *s, Req *q)
{
    s->active.erase(std::find(s->active.begin(), s->active.end(), q));
}

// resident groups: same block size, shared memory in the same 8 KB bucket; a
// group launches with the largest shared memory of the members it has seen
static int group_for(xk_server *s, int threads, int smem)
{
    const int bucket = (smem + 8191) / 8192;
    for (size_t g = 0; g < s->groups.size(); ++g)
        if (s->groups[g].threads == threads && (s->groups[g].smem + 8191) / 8192 == bucket) {
            s->groups[g].smem = std::max(s->groups[g].smem, smem);
            return (int)g;
        }
    s->groups.emplace_back();
    Group &g = s->groups.back();
    g.threads = threads;
    g.smem = smem;
    // resident lattices are the smallest requests: their rounds take the
    // device's greatest stream priority
    for (Slot &sl : g.slot) {
        XK_CUDA(cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, s->prio_greatest));
        XK_CUDA(cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
        const size_t inst_bytes = sizeof(LifeInst) * s->max_active;
        if (s->slot_used < s->slot_pool) {
            const int64_t at = (int64_t)s->slot_used++ * s->slot_bytes;
            sl.h_inst = (LifeInst *)(s->slot_host + at);
            sl.d_inst = (LifeInst *)(s->slot_dev + at);
            sl.h_gens = (int32_t *)(s->slot_host + at + inst_bytes);
            sl.d_gens = (int32_t *)(s->slot_dev + at + inst_bytes);
            continue;
        }
        sl.owned = true;
        XK_CUDA(cudaMallocHost(&sl.h_inst, inst_bytes));
        XK_CUDA(cudaMalloc(&sl.d_inst, inst_bytes));
        XK_CUDA(cudaMallocHost(&sl.h_gens, sizeof(int32_t) * s->max_active));
        XK_CUDA(cudaMalloc(&sl.d_gens, sizeof(int32_t) * s->max_active));
    }
    return (int)s->groups.size() - 1;
}

// stream priority of a request: the less work (cell-generations) it asks
// for, the greater its priority, so that short requests are not queued
// behind the kernels of long ones; one priority level per factor of 4 of work
// above 2^26
static int request_priority(const xk_server *s, const Req *q)
{
    const double work = (double)q->n * (double)std::max<int64_t>(1, q->r.generations);
    const int levels = s->prio_least - s->prio_greatest;
    int step = 0;
    for (double w = work; w >= (double)(1LL << 26) && step < levels; w /= 4.0) ++step;
    return s->prio_greatest + step;
}

// generations of the next round of a resident member: the round's work is
// about round_work cell-generations (so small lattices run many generations
// per round), at least `quantum`, at most 65536 generations (a round of the
// tiniest lattice stays a few milliseconds, so cancellation and the other
// members of its slot are not held up) and at most what is left
static int64_t resident_chunk(const xk_server *s, const Req *q)
{
    const int64_t left = q->r.generations - q->done;
    int64_t chunk = std::max<int64_t>(s->quantum, s->round_work / std::max<int64_t>(1, q->n));
    chunk = std::min<int64_t>(chunk, std::max<int64_t>(s->quantum, 1 << 16));
    return std::min(chunk, left);
}

static int admit(xk_server *s, Req *q, bool *admitted)
{
    *admitted = false;
    const int64_t doff = s->dev_arena->alloc(q->dev_need);
    if (doff < 0) return XK_OK;
    const int64_t hoff = s->host_arena->alloc(q->host_need);
    if (hoff < 0) {
        s->dev_arena->release(doff);
        return XK_OK;
    }
    q->dev_off = doff;
    q->host_off = hoff;
    s->st.device_bytes_in_use = s->dev_arena->in_use();
    s->st.device_bytes_peak = std::max(s->st.device_bytes_peak, s->st.device_bytes_in_use);
    XK_CUDA(cudaStreamCreateWithPriority(&q->stream, cudaStreamNonBlocking, request_priority(s, q)));
    XK_CUDA(cudaEventCreateWithFlags(&q->ev, cudaEventDisableTiming));
    uint8_t *base = s->dev_base + doff;
    const xk_request &r = q->r;
    // pageable source: the call returns once the bytes are staged
    if (r.kind == XK_SERVE_MASS3D) {
        const int64_t W = r.size[0];
        XK_CUDA(cudaMemsetAsync(base, 0, (size_t)(4 * mass_pitched_cells(r)), q->stream));
        XK_CUDA(cudaMemcpy2DAsync(base, (size_t)xk_mass_pitch(W) * 4, q->input.data(), (size_t)W * 4,
                                  (size_t)W * 4, (size_t)(q->n / W), cudaMemcpyHostToDevice, q->stream));
    } else {
        XK_CUDA(cudaMemcpyAsync(base, q->input.data(), (size_t)(q->n * q->esz), cudaMemcpyHostToDevice,
                                q->stream));
    }
    if (r.kind == XK_SERVE_LIFE2D) {
        q->rule0 = life2d_rule0(r.rule);
        q->rule1 = life2d_rule1(r.rule);
        int threads = 0, smem = 0;
        const bool fits = q->n <= s->resident_max &&
                          xk_life_resident_config((int)r.size[0], (int)r.size[1], s->resident_band, &threads,
                                                  &smem);
        if (fits) {
            q->path = PATH_RESIDENT;
            q->threads = threads;
            q->smem = smem;
            const int g = group_for(s, threads, smem);
            if (g < 0) return g;
            q->group = g;
        } else {
            q->path = PATH_GLOBAL2D;
            q->lg = xk_life_geo(r.size[0], r.size[1], 1, 0);
            q->lt = xk_life_table(q->rule0, q->rule1);
            q->lt9 = xk_life_table9(q->rule0, q->rule1);
            q->tb_T = xk_life_tb_supported(q->lg) ? s->tb_depth : 0;
            uint32_t *w0 = (uint32_t *)(base + rnd(q->n + 16));
            XK_CUDA(xk_life_pack(base, 1, w0, q->lg, q->stream));
            s->st.launches++;
            q->cur = 0;
        }
    } else if (r.kind == XK_SERVE_LIFE3D_VN) {
        q->path = PATH_LIFE3D;
        q->rule0 = life3d_rule0(r.rule);
        q->rule1 = life3d_rule1(r.rule);
        q->lg = xk_life_geo(r.size[0], r.size[1] * r.size[2], 1, 0);
        q->lt = xk_life_table(q->rule0, q->rule1);
        q->g3.W = (int32_t)r.size[0];
        q->g3.H = (int32_t)r.size[1];
        q->g3.D = (int32_t)r.size[2];
        q->g3.wpr = q->lg.wpr;
        q->g3.rlast = q->lg.rlast;
        q->g3.lastmask = q->lg.lastmask;
        q->g3.div_wpr = xk_div_magic((uint64_t)q->g3.wpr,
                                     (uint64_t)q->g3.H * (uint64_t)q->g3.D * (uint64_t)q->g3.wpr);
        q->g3.div_h = xk_div_magic((uint64_t)q->g3.H, (uint64_t)q->g3.H * (uint64_t)q->g3.D);
        uint32_t *w0 = (uint32_t *)(base + rnd(q->n + 16));
        XK_CUDA(xk_life_pack(base, 1, w0, q->lg, q->stream));
        s->st.launches++;
        q->cur = 0;
    } else {
        q->path = PATH_MASS3D;
        memset(&q->md, 0, sizeof(q->md));
        q->md.abi_version = XK_ABI_VERSION;
        q->md.family = XK_FAMILY_MASS;
        q->md.ndim = 3;
        q->md.nbr = 6;
        for (int i = 0; i < 3; ++i) q->md.size[i] = r.size[i];
        q->md.state_bytes = 4;
        q->md.border_value = 0xFFFFFFFFu;
        q->md.wall = 0xFFFFFFFFu;
        q->cur = 0;
    }
    XK_CUDA(cudaEventRecord(q->ev, q->stream));
    q->ev_pending = true;
    q->chunk = 0;
    std::vector<uint8_t>().swap(q->input);
    q->status = XK_REQ_ACTIVE;
    q->t_admit = s->now();
    s->st.admitted++;
    *admitted = true;
    return XK_OK;
}

// the launches of `chunk` generations of a request on its own stream (direct
// or into a graph being captured); flips q->cur per generation
static int enqueue_round(xk_server *s, Req *q, int64_t chunk)
{
    uint8_t *base = s->dev_base + q->dev_off;
    if (q->path == PATH_GLOBAL2D || q->path == PATH_LIFE3D) {
        uint32_t *w[2];
        w[0] = (uint32_t *)(base + rnd(q->n + 16));
        w[1] = (uint32_t *)((uint8_t *)w[0] + rnd((int64_t)q->lg.wpr * q->lg.H * 4));
        if (q->path == PATH_GLOBAL2D && q->tb_T > 1) {
            // temporal blocking: tb_T generations per launch
            for (int64_t g = 0; g < chunk;) {
                const int T = (int)std::min<int64_t>(q->tb_T, chunk - g);
                XK_CUDA(xk_life_step_tb(w[q->cur], w[1 - q->cur], q->lg, q->lt9, T, q->stream));
                q->cur ^= 1;
                g += T;
            }
            return XK_OK;
        }
        for (int64_t g = 0; g < chunk; ++g) {
            if (q->path == PATH_GLOBAL2D)
                XK_CUDA(xk_life_step_global(w[q->cur], w[1 - q->cur], q->lg, q->lt, q->stream));
            else
                XK_CUDA(xk_life_step3d_vn(w[q->cur], w[1 - q->cur], q->g3, q->lt, q->stream));
            q->cur ^= 1;
        }
    } else {
        const int64_t pn = mass_pitched_cells(q->r);
        uint32_t *m[2] = {(uint32_t *)base, (uint32_t *)(base + rnd(4 * pn))};
        unsigned long long *tot = (unsigned long long *)(base + 2 * rnd(4 * pn));
        XK_CUDA(cudaMemsetAsync(tot, 0, (size_t)chunk * 8, q->stream));
        for (int64_t g = 0; g < chunk; ++g) {
            XK_CUDA(xk_mass_step(m[q->cur], m[1 - q->cur], tot + g, q->md, q->mass_small, q->stream));
            q->cur ^= 1;
        }
    }
    return XK_OK;
}

// ping-pong flips of a round of `chunk` generations: one per launch (a
// temporally blocked launch covers up to tb_T generations)
static int64_t round_flips(const Req *q, int64_t chunk)
{
    if (q->path == PATH_GLOBAL2D && q->tb_T > 1) return (chunk + q->tb_T - 1) / q->tb_T;
    return chunk;
}

// next round of a request on its own stream; full rounds of requests with at
// least two of them left are captured once per parity and replayed
static int launch_round(xk_server *s, Req *q)
{
    const int64_t chunk = std::min(s->quantum, q->r.generations - q->done);
    const int c0 = q->cur;
    const bool full = chunk == s->quantum && graphs_enabled();
    if (full && !q->graph[c0] && q->r.generations - q->done >= 2 * s->quantum) {
        XK_CUDA(cudaStreamBeginCapture(q->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_round(s, q, chunk);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(q->stream, &graph);
        if (rc != XK_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        XK_CUDA(e);
        e = cudaGraphInstantiate(&q->graph[c0], graph, 0);
        cudaGraphDestroy(graph);
        XK_CUDA(e);
        q->cur = c0;
    }
    if (full && q->graph[c0]) {
        XK_CUDA(cudaGraphLaunch(q->graph[c0], q->stream));
        q->cur = c0 ^ (int)(round_flips(q, chunk) & 1);
    } else {
        int rc = enqueue_round(s, q, chunk);
        if (rc != XK_OK) return rc;
    }
    s->st.launches += round_flips(q, chunk);
    XK_CUDA(cudaEventRecord(q->ev, q->stream));
    q->ev_pending = true;
    q->chunk = chunk;
    return XK_OK;
}

// one round of every idle member of resident group g, in a free slot: one
// launch over all of them, each member advancing its own generation count
static int launch_group(xk_server *s, int gi)
{
    Group &g = s->groups[gi];
    Slot *sl = nullptr;
    for (Slot &c : g.slot)
        if (!c.in_flight) {
            sl = &c;
            break;
        }
    if (!sl) return XK_OK;
    sl->members.clear();
    for (Req *q : s->active)
        if (q->path == PATH_RESIDENT && q->group == gi && !q->ev_pending && !q->in_group &&
            !q->draining && !q->cancel && q->done < q->r.generations)
            sl->members.push_back(q);
    if (sl->members.empty()) return XK_OK;
    for (size_t k = 0; k < sl->members.size(); ++k) {
        Req *q = sl->members[k];
        q->chunk = resident_chunk(s, q);
        LifeInst &in = sl->h_inst[k];
        memset(&in, 0, sizeof(in));
        in.off = q->dev_off;
        in.W = (int32_t)q->r.size[0];
        in.H = (int32_t)q->r.size[1];
        in.wpr = (in.W + 31) / 32;
        in.rlast = in.W - 32 * (in.wpr - 1);
        in.lastmask = in.rlast == 32 ? 0xFFFFFFFFu : ((1u << in.rlast) - 1u);
        in.rule0 = q->rule0;
        in.rule1 = q->rule1;
        in.smem_words = q->smem / 4;
        sl->h_gens[k] = (int32_t)q->chunk;
    }
    const size_t n = sl->members.size();
    XK_CUDA(cudaMemcpyAsync(sl->d_inst, sl->h_inst, sizeof(LifeInst) * n, cudaMemcpyHostToDevice,
                            sl->stream));
    XK_CUDA(cudaMemcpyAsync(sl->d_gens, sl->h_gens, sizeof(int32_t) * n, cudaMemcpyHostToDevice,
                            sl->stream));
    XK_CUDA(xk_life_step_resident_each(sl->d_inst, sl->d_gens, (int)n, s->dev_base, s->bad, g.threads,
                                       g.smem, sl->stream));
    s->st.launches++;
    XK_CUDA(cudaEventRecord(sl->ev, sl->stream));
    sl->in_flight = true;
    for (Req *q : sl->members) q->in_group = true;
    return XK_OK;
}

// copy a finished request's state (and mass total) to its pinned slot
static int start_result_copy(xk_server *s, Req *q)
{
    uint8_t *base = s->dev_base + q->dev_off;
    uint8_t *hst = s->host_base + q->host_off;
    const void *src = base;
    if (q->path == PATH_GLOBAL2D || q->path == PATH_LIFE3D) {
        uint32_t *w0 = (uint32_t *)(base + rnd(q->n + 16));
        uint32_t *w = q->cur ? (uint32_t *)((uint8_t *)w0 + rnd((int64_t)q->lg.wpr * q->lg.H * 4)) : w0;
        XK_CUDA(xk_life_unpack(w, base, 1, q->lg, q->stream));
        s->st.launches++;
    } else if (q->path == PATH_MASS3D) {
        const int64_t pn = mass_pitched_cells(q->r);
        src = base + (q->cur ? rnd(4 * pn) : 0);
        if (q->r.generations > 0) {
            const unsigned long long *tot = (const unsigned long long *)(base + 2 * rnd(4 * pn));
            XK_CUDA(cudaMemcpyAsync(hst + rnd(q->n * q->esz), tot + (q->last_chunk - 1), 8,
                                    cudaMemcpyDeviceToHost, q->stream));
        }
        const int64_t W = q->r.size[0];
        XK_CUDA(cudaMemcpy2DAsync(hst, (size_t)W * 4, src, (size_t)xk_mass_pitch(W) * 4, (size_t)W * 4,
                                  (size_t)(q->n / W), cudaMemcpyDeviceToHost, q->stream));
        XK_CUDA(cudaEventRecord(q->ev, q->stream));
        q->ev_pending = true;
        q->draining = true;
        return XK_OK;
    }
    XK_CUDA(cudaMemcpyAsync(hst, src, (size_t)(q->n * q->esz), cudaMemcpyDeviceToHost, q->stream));
    XK_CUDA(cudaEventRecord(q->ev, q->stream));
    q->ev_pending = true;
    q->draining = true;
    return XK_OK;
}

static void finish(xk_server *s, Req *q, int status)
{
    if (status == XK_REQ_DONE && q->path == PATH_MASS3D && q->r.generations > 0)
        memcpy(&q->mass_total, s->host_base + q->host_off + rnd(q->n * q->esz), 8);
    release_device(s, q);
    if (status != XK_REQ_DONE && q->host_off >= 0) {
        s->host_arena->release(q->host_off);
        q->host_off = -1;
    }
    q->status = status;
    q->t_done = s->now();
    if (status == XK_REQ_DONE) {
        s->st.completed++;
        s->st.cell_updates += q->n * q->r.generations;
    } else if (status == XK_REQ_CANCELLED) {
        s->st.cancelled++;
    } else {
        s->st.failed++;
    }
    drop_active(s, q);
}

// one pass of the worker; *busy: GPU work in flight or queued requests
static int worker_pass(xk_server *s, bool *busy)
{
    // (1) retire
    for (Group &g : s->groups)
        for (Slot &sl : g.slot) {
            if (!sl.in_flight) continue;
            cudaError_t e = cudaEventQuery(sl.ev);
            if (e == cudaErrorNotReady) continue;
            XK_CUDA(e);
            sl.in_flight = false;
            for (Req *q : sl.members) {
                q->in_group = false;
                q->done += q->chunk;
                q->last_chunk = q->chunk;
                q->chunk = 0;
            }
            sl.members.clear();
        }
    std::vector<Req *> snapshot = s->active;
    for (Req *q : snapshot) {
        if (q->ev_pending) {
            cudaError_t e = cudaEventQuery(q->ev);
            if (e == cudaErrorNotReady) continue;
            XK_CUDA(e);
            q->ev_pending = false;
            if (q->draining) {
                finish(s, q, XK_REQ_DONE);
                continue;
            }
            q->done += q->chunk;
            if (q->chunk) q->last_chunk = q->chunk;
            q->chunk = 0;
        }
        if (q->in_group) continue;
        if (q->cancel) {
            finish(s, q, XK_REQ_CANCELLED);
            continue;
        }
        if (q->done >= q->r.generations) {
            int rc = start_result_copy(s, q);
            if (rc != XK_OK) return rc;
        }
    }
    if (s->active.size() < snapshot.size()) s->cv_done.notify_all();
    // (2) admit, first come first served
    while (!s->pending.empty() && (int)s->active.size() < s->max_active) {
        Req *q = s->pending.front();
        bool ok = false;
        int rc = admit(s, q, &ok);
        if (rc != XK_OK) return rc;
        if (!ok) break;
        s->pending.erase(s->pending.begin());
        s->active.push_back(q);
    }
    // (3) rounds
    bool launched = false;
    for (Req *q : s->active) {
        if (q->path == PATH_RESIDENT || q->ev_pending || q->draining || q->cancel ||
            q->done >= q->r.generations)
            continue;
        int rc = launch_round(s, q);
        if (rc != XK_OK) return rc;
        launched = true;
    }
    for (size_t gi = 0; gi < s->groups.size(); ++gi) {
        const int64_t before = s->st.launches;
        int rc = launch_group(s, (int)gi);
        if (rc != XK_OK) return rc;
        launched |= s->st.launches != before;
    }
    if (launched) s->st.rounds++;
    *busy = !s->active.empty() || !s->pending.empty();
    return XK_OK;
}

static void worker_main(xk_server *s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        if (s->stop && s->pending.empty()) {
            bool idle = true;
            for (Req *q : s->active) idle &= !(q->ev_pending || q->in_group);
            if (idle) break;
        }
        bool busy = false;
        int rc = worker_pass(s, &busy);
        if (rc != XK_OK) {
            s->failed = true;
            s->fail_msg = xk_last_error();
            for (auto &kv : s->reqs) {
                Req *q = kv.second.get();
                if (q->status == XK_REQ_PENDING || q->status == XK_REQ_ACTIVE) {
                    q->status = XK_REQ_FAILED;
                    s->st.failed++;
                }
            }
            s->pending.clear();
            s->active.clear();
            s->cv_done.notify_all();
            break;
        }
        if (busy)
            s->cv_work.wait_for(lk, std::chrono::microseconds(20));
        else
            s->cv_work.wait(lk, [s] { return s->stop || !s->pending.empty(); });
    }
    for (auto &g : s->groups)
        for (Slot &sl : g.slot)
            if (sl.stream) cudaStreamSynchronize(sl.stream);
    for (Req *q : s->active)
        if (q->stream) cudaStreamSynchronize(q->stream);
}

// ---------------------------------------------------------------------------
// C-ABI

extern "C" int xk_serve_request_bytes(const xk_request *req, int64_t *bytes)
{
    XK_REQUIRE(bytes, XK_ERR_ARG, "xk_serve_request_bytes: null argument");
    int64_t n, esz, dev, host;
    int rc = request_layout(req, &n, &esz, &dev, &host);
    if (rc != XK_OK) return rc;
    *bytes = dev;
    return XK_OK;
}

static void free_server(xk_server *s)
{
    for (auto &g : s->groups)
        for (Slot &sl : g.slot) {
            if (sl.stream) cudaStreamDestroy(sl.stream);
            if (sl.ev) cudaEventDestroy(sl.ev);
            if (!sl.owned) continue;
            if (sl.h_inst) cudaFreeHost(sl.h_inst);
            if (sl.d_inst) cudaFree(sl.d_inst);
            if (sl.h_gens) cudaFreeHost(sl.h_gens);
            if (sl.d_gens) cudaFree(sl.d_gens);
        }
    if (s->slot_host) cudaFreeHost(s->slot_host);
    if (s->slot_dev) cudaFree(s->slot_dev);
    for (auto &kv : s->reqs) {
        if (kv.second->stream) cudaStreamDestroy(kv.second->stream);
        if (kv.second->ev) cudaEventDestroy(kv.second->ev);
    }
    if (s->dev_base) cudaFree(s->dev_base);
    if (s->host_base) cudaFreeHost(s->host_base);
    if (s->bad) cudaFree(s->bad);
    delete s;
}

extern "C" int xk_serve_create(int64_t budget_bytes, int64_t host_bytes, int32_t max_active,
                               int32_t quantum, xk_server **out)
{
    XK_REQUIRE(out, XK_ERR_ARG, "xk_serve_create: null argument");
    *out = nullptr;
    XK_REQUIRE(budget_bytes >= XK_ARENA_ALIGN, XK_ERR_ARG, "xk_serve_create: budget %lld bytes",
               (long long)budget_bytes);
    XK_REQUIRE(max_active >= 1 && max_active <= 65536, XK_ERR_ARG,
               "xk_serve_create: max_active %d out of [1, 65536]", max_active);
    XK_REQUIRE(quantum >= 1 && quantum <= XK_SERVE_MAX_QUANTUM, XK_ERR_ARG,
               "xk_serve_create: quantum %d out of [1, %d]", quantum, XK_SERVE_MAX_QUANTUM);
    if (host_bytes <= 0) host_bytes = std::min<int64_t>(budget_bytes, 8LL << 30);
    xk_server *s = new (std::nothrow) xk_server();
    XK_REQUIRE(s, XK_ERR_OOM, "host allocation failed");
    memset(&s->st, 0, sizeof(s->st));
    s->budget = budget_bytes;
    s->host_bytes = host_bytes;
    s->max_active = max_active;
    s->quantum = quantum;
    s->round_work = (int64_t)quantum << 18;
    if (const char *e = getenv("XK_SERVE_TB")) {
        const int T = atoi(e);
        s->tb_depth = T >= 2 && T <= 8 ? T : 0;
    }
    if (const char *e = getenv("XK_SERVE_RESIDENT_MAX")) s->resident_max = atoll(e);
    if (const char *e = getenv("XK_SERVE_BAND")) s->resident_band = std::max(1, std::min(1024, atoi(e)));
    // room for the slots of up to 64 resident groups, at most 64 MB
    s->slot_bytes = XkArena::round((int64_t)(sizeof(LifeInst) + sizeof(int32_t)) * max_active);
    s->slot_pool = (int)std::min<int64_t>(64 * XK_SERVE_GROUP_SLOTS, (64LL << 20) / s->slot_bytes);
    cudaError_t e;
    if ((e = cudaGetDevice(&s->device)) != cudaSuccess ||
        (s->slot_pool > 0 &&
         ((e = cudaMallocHost(&s->slot_host, (size_t)(s->slot_bytes * s->slot_pool))) != cudaSuccess ||
          (e = cudaMalloc(&s->slot_dev, (size_t)(s->slot_bytes * s->slot_pool))) != cudaSuccess)) ||
        (e = cudaDeviceGetStreamPriorityRange(&s->prio_least, &s->prio_greatest)) != cudaSuccess ||
        (e = cudaMalloc(&s->dev_base, (size_t)budget_bytes)) != cudaSuccess ||
        (e = cudaMallocHost(&s->host_base, (size_t)host_bytes)) != cudaSuccess ||
        (e = cudaMalloc(&s->bad, sizeof(unsigned int))) != cudaSuccess ||
        (e = cudaMemset(s->bad, 0, sizeof(unsigned int))) != cudaSuccess) {
        int rc = xk_cuda_status(e, "xk_serve_create");
        if (e == cudaErrorMemoryAllocation) rc = XK_ERR_OOM;
        free_server(s);
        return rc;
    }
    s->dev_arena.reset(new XkArena(budget_bytes));
    s->host_arena.reset(new XkArena(host_bytes));
    s->st.budget_bytes = s->dev_arena->capacity();
    s->t0 = std::chrono::steady_clock::now();
    s->worker = std::thread(worker_main, s);
    *out = s;
    return XK_OK;
}

extern "C" int xk_serve_destroy(xk_server *s)
{
    if (!s) return XK_OK;
    cudaSetDevice(s->device);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (Req *q : s->pending) {
            q->status = XK_REQ_CANCELLED;
            s->st.cancelled++;
        }
        s->pending.clear();
        for (Req *q : s->active) q->cancel = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    s->cv_done.notify_all();
    free_server(s);
    return XK_OK;
}

extern "C" int xk_serve_submit(xk_server *s, const xk_request *req, const void *host_cells,
                               int64_t *id)
{
    XK_REQUIRE(s && req && host_cells && id, XK_ERR_ARG, "xk_serve_submit: null argument");
    *id = 0;
    std::unique_ptr<Req> q(new (std::nothrow) Req());
    XK_REQUIRE(q, XK_ERR_OOM, "host allocation failed");
    q->r = *req;
    int rc = request_layout(req, &q->n, &q->esz, &q->dev_need, &q->host_need);
    if (rc != XK_OK) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->st.rejected++;
        return rc;
    }
    if (q->dev_need > s->dev_arena->capacity() || q->host_need > s->host_arena->capacity()) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->st.rejected++;
        xk_set_error("serve: request needs %lld device / %lld host bytes, the server has %lld / %lld",
                     (long long)q->dev_need, (long long)q->host_need,
                     (long long)s->dev_arena->capacity(), (long long)s->host_arena->capacity());
        return XK_ERR_OOM;
    }
    const uint8_t *src = (const uint8_t *)host_cells;
    if (req->kind != XK_SERVE_MASS3D) {
        for (int64_t i = 0; i < q->n; ++i)
            if (src[i] > 1) {
                std::lock_guard<std::mutex> lk(s->mu);
                s->st.rejected++;
                xk_set_error("serve: cell %lld holds %u, Life-like cells are 0 or 1", (long long)i,
                             (unsigned)src[i]);
                return XK_ERR_ARG;
            }
    } else {
        // the initial total: the result's total when no generation runs, and
        // below 2^30 the fast-only kernel (mass is conserved, so every cell
        // stays below 2^30)
        const uint32_t *m = (const uint32_t *)host_cells;
        uint64_t total = 0;
        for (int64_t i = 0; i < q->n; ++i) total += m[i];
        q->mass_small = total < (1ull << 30);
        if (req->generations == 0) q->mass_total = total;
    }
    q->input.assign(src, src + q->n * q->esz);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->failed) {
            xk_set_error("serve: server failed: %s", s->fail_msg.c_str());
            return XK_ERR_CUDA;
        }
        XK_REQUIRE(!s->stop, XK_ERR_STATE, "serve: server is shutting down");
        q->id = s->next_id++;
        q->t_submit = s->now();
        *id = q->id;
        s->pending.push_back(q.get());
        s->reqs[q->id] = std::move(q);
        s->st.submitted++;
    }
    s->cv_work.notify_one();
    return XK_OK;
}

static void fill_info(const Req *q, xk_request_info *info)
{
    memset(info, 0, sizeof(*info));
    info->status = q->status;
    info->generations_done = q->status == XK_REQ_DONE ? q->r.generations : q->done;
    info->submit_s = q->t_submit;
    info->admit_s = q->t_admit;
    info->done_s = q->t_done;
    info->mass_total = q->mass_total;
}

extern "C" int xk_serve_info(xk_server *s, int64_t id, xk_request_info *info)
{
    XK_REQUIRE(s && info, XK_ERR_ARG, "xk_serve_info: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    XK_REQUIRE(it != s->reqs.end(), XK_ERR_ARG, "serve: unknown request %lld", (long long)id);
    fill_info(it->second.get(), info);
    return XK_OK;
}

extern "C" int xk_serve_wait(xk_server *s, int64_t id, double timeout_s, xk_request_info *info)
{
    XK_REQUIRE(s, XK_ERR_ARG, "xk_serve_wait: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    XK_REQUIRE(it != s->reqs.end(), XK_ERR_ARG, "serve: unknown request %lld", (long long)id);
    Req *q = it->second.get();
    auto final_state = [q] {
        return q->status == XK_REQ_DONE || q->status == XK_REQ_CANCELLED || q->status == XK_REQ_FAILED;
    };
    const auto limit = std::chrono::steady_clock::now() +
                       std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                           std::chrono::duration<double>(timeout_s < 0 ? 1e9 : timeout_s));
    if (!s->cv_done.wait_until(lk, limit, final_state)) {
        if (info) fill_info(q, info);
        xk_set_error("serve: request %lld not finished after %.3f s", (long long)id, timeout_s);
        return XK_ERR_TIMEOUT;
    }
    if (info) fill_info(q, info);
    if (q->status == XK_REQ_FAILED) {
        xk_set_error("serve: request %lld failed: %s", (long long)id, s->fail_msg.c_str());
        return XK_ERR_CUDA;
    }
    return XK_OK;
}

extern "C" int xk_serve_result(xk_server *s, int64_t id, void *host_out, int64_t cells)
{
    XK_REQUIRE(s && host_out, XK_ERR_ARG, "xk_serve_result: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    XK_REQUIRE(it != s->reqs.end(), XK_ERR_ARG, "serve: unknown request %lld", (long long)id);
    Req *q = it->second.get();
    XK_REQUIRE(q->status == XK_REQ_DONE, XK_ERR_STATE, "serve: request %lld is not done (status %d)",
               (long long)id, q->status);
    XK_REQUIRE(cells == q->n, XK_ERR_ARG, "serve: request %lld has %lld cells, %lld asked",
               (long long)id, (long long)q->n, (long long)cells);
    memcpy(host_out, s->host_base + q->host_off, (size_t)(q->n * q->esz));
    s->host_arena->release(q->host_off);
    s->reqs.erase(it);
    s->cv_work.notify_one();
    return XK_OK;
}

extern "C" int xk_serve_cancel(xk_server *s, int64_t id)
{
    XK_REQUIRE(s, XK_ERR_ARG, "xk_serve_cancel: null server");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(id);
        XK_REQUIRE(it != s->reqs.end(), XK_ERR_ARG, "serve: unknown request %lld", (long long)id);
        Req *q = it->second.get();
        if (q->status == XK_REQ_PENDING) {
            s->pending.erase(std::find(s->pending.begin(), s->pending.end(), q));
            q->status = XK_REQ_CANCELLED;
            q->t_done = s->now();
            s->st.cancelled++;
            s->cv_done.notify_all();
        } else if (q->status == XK_REQ_ACTIVE) {
            q->cancel = true;
        }
    }
    s->cv_work.notify_one();
    return XK_OK;
}

extern "C" int xk_serve_stats_get(xk_server *s, xk_serve_stats *st)
{
    XK_REQUIRE(s && st, XK_ERR_ARG, "xk_serve_stats_get: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *st = s->st;
    st->pending = (int64_t)s->pending.size();
    st->active = (int64_t)s->active.size();
    st->elapsed_s = s->now();
    return XK_OK;
}

// ---------------------------------------------------------------------------
// the allocator alone (host only)

struct xk_arena {
    XkArena a;
    explicit xk_arena(int64_t cap) : a(cap) {}
};

extern "C" int xk_arena_create(int64_t capacity, xk_arena **out)
{
    XK_REQUIRE(out && capacity >= XK_ARENA_ALIGN, XK_ERR_ARG, "xk_arena_create: bad argument");
    *out = new (std::nothrow) xk_arena(capacity);
    XK_REQUIRE(*out, XK_ERR_OOM, "host allocation failed");
    return XK_OK;
}

extern "C" int xk_arena_alloc(xk_arena *a, int64_t bytes, int64_t *offset)
{
    XK_REQUIRE(a && offset && bytes >= 0, XK_ERR_ARG, "xk_arena_alloc: bad argument");
    *offset = a->a.alloc(bytes);
    XK_REQUIRE(*offset >= 0, XK_ERR_OOM, "arena: no free range of %lld bytes (largest %lld)",
               (long long)bytes, (long long)a->a.largest_free());
    return XK_OK;
}

extern "C" int xk_arena_free(xk_arena *a, int64_t offset)
{
    XK_REQUIRE(a, XK_ERR_ARG, "xk_arena_free: null arena");
    XK_REQUIRE(a->a.release(offset), XK_ERR_ARG, "arena: %lld is not an allocation",
               (long long)offset);
    return XK_OK;
}

extern "C" int xk_arena_stats(xk_arena *a, int64_t *in_use, int64_t *largest_free,
                              int32_t *free_ranges)
{
    XK_REQUIRE(a && in_use && largest_free && free_ranges, XK_ERR_ARG, "xk_arena_stats: null argument");
    *in_use = a->a.in_use();
    *largest_free = a->a.largest_free();
    *free_ranges = a->a.free_ranges();
    return XK_OK;
}

extern "C" int xk_arena_destroy(xk_arena *a)
{
    delete a;
    return XK_OK;
}
