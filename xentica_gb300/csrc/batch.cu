// Ensembles of independent Life-like lattices (include/xk.h, xk_batch_*).
//
// Every instance keeps the reference's one-byte-per-cell layout in HBM,
// concatenated in creation order.  The batched form advances all of them with
// the resident kernel: one CTA per instance loads it (packing to 32 cells per
// word), runs every generation of the call out of shared memory and stores it
// back, so HBM sees two bytes per cell per call however many generations run.
// Instances are grouped into classes with the same CTA shape (threads,
// shared memory); each class is one launch, classes run concurrently on their
// own streams, and the whole fork/join is captured once per generation count
// as a CUDA graph.  Instances too wide or too large for one CTA take the plain
// path below.
//
// The plain form is the reference's execution model on the same GPU: one
// launch per instance per generation over the byte layout.
//
// End to end (xk_batch_run, host buffers in and out): on page-locked buffers,
// classes whose CTA has its SM to itself are staged by the copy engines
// around grouped launches on high-priority streams while every other class
// reads and writes the host buffers from its kernel (run_mapped); pageable
// buffers go through index-order chunks whose uploads, launches and
// downloads overlap (run_pipelined).  Seeds: xk_batch_seed_bernoulli draws
// every instance's cells on the device (seed.cu).
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <new>
#include <vector>

#include "xk_internal.cuh"

namespace {

struct Class {
    int threads = 0, smem = 0;
    int first = 0, count = 0;      // range in the sorted instance table
    int priority = 0;              // launch priority: larger CTAs (longer runs) first
    cudaStream_t stream = nullptr;
};

}  // namespace

struct xk_batch {
    int n = 0;
    std::vector<int32_t> W, H;
    std::vector<uint32_t> rule;
    std::vector<int64_t> off;      // byte offset of each instance
    int64_t total = 0;
    uint8_t *cells = nullptr;      // current state, bytes
    uint8_t *scratch = nullptr;    // plain-form ping-pong partner
    unsigned int *bad = nullptr;   // value-check flag of the resident kernel
    LifeInst *d_inst = nullptr;
    std::vector<LifeInst> h_inst;  // sorted by class, largest first
    std::vector<Class> classes;
    std::vector<int> big;          // instances run with the plain kernel
    int rows_per_band = 8;
    // band length of the lattices of one size (W, H), overriding
    // rows_per_band (the tuner's per-size choices)
    std::map<std::pair<int, int>, int> size_band;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr;
    std::vector<cudaEvent_t> joins;
    std::map<int, cudaGraphExec_t> graphs;
    // end-to-end pipeline (xk_batch_run): instances cut into chunks of
    // consecutive lattices; per chunk and class a run of descriptors
    std::vector<int> cls_of;       // class of each instance (-1: plain path)
    std::vector<int> chunk_first;  // chunk k = instances [chunk_first[k], chunk_first[k + 1])
    std::vector<std::vector<std::pair<int, int>>> seg;   // [chunk][class] -> (first, count)
    LifeInst *d_pipe = nullptr;
    cudaStream_t out_stream = nullptr;
    std::vector<cudaStream_t> pipe_streams;  // one per chunk: its class launches
    std::vector<cudaEvent_t> pev;  // per chunk: input landed, generations done
    // end to end on page-locked buffers: classes whose CTA has its SM to
    // itself run from device memory in groups (staged by the copy engines);
    // the others read and write the host buffers from the kernel (mapped)
    bool e2e_planned = false;
    std::vector<int> stage_cls, stage_first, stage_count;   // groups, as runs of h_inst
    std::vector<int> mapped_cls;
    std::vector<cudaStream_t> stage_streams;               // high priority
    std::vector<cudaEvent_t> sev;                          // per group: landed, done
    cudaEvent_t staged_in = nullptr;
};

static void destroy_graphs(xk_batch *b)
{
    for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

static void free_pipeline(xk_batch *b)
{
    for (auto e : b->pev) cudaEventDestroy(e);
    b->pev.clear();
    for (auto st : b->pipe_streams) cudaStreamDestroy(st);
    b->pipe_streams.clear();
    for (auto e : b->sev) cudaEventDestroy(e);
    b->sev.clear();
    for (auto st : b->stage_streams) cudaStreamDestroy(st);
    b->stage_streams.clear();
    if (b->staged_in) cudaEventDestroy(b->staged_in);
    b->staged_in = nullptr;
    b->stage_cls.clear();
    b->stage_first.clear();
    b->stage_count.clear();
    b->mapped_cls.clear();
    b->e2e_planned = false;
    if (b->d_pipe) cudaFree(b->d_pipe);
    b->d_pipe = nullptr;
    b->seg.clear();
    b->chunk_first.clear();
}

static void free_batch(xk_batch *b)
{
    if (!b) return;
    destroy_graphs(b);
    free_pipeline(b);
    if (b->out_stream) cudaStreamDestroy(b->out_stream);
    for (auto &c : b->classes)
        if (c.stream) cudaStreamDestroy(c.stream);
    for (auto e : b->joins) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->cells) cudaFree(b->cells);
    if (b->scratch) cudaFree(b->scratch);
    if (b->bad) cudaFree(b->bad);
    if (b->d_inst) cudaFree(b->d_inst);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

static inline uint32_t rule0_of(uint32_t golly) { return golly & 511u; }
static inline uint32_t rule1_of(uint32_t golly) { return (golly & 511u) | ((golly >> 9) & 511u); }

// band length of a W x H lattice: its size's override, else rows_per_band
static int band_for(const xk_batch *b, int W, int H)
{
    auto it = b->size_band.find(std::make_pair(W, H));
    return it == b->size_band.end() ? b->rows_per_band : it->second;
}

// (re)build the class table for the current band lengths
static int plan_classes(xk_batch *b)
{
    destroy_graphs(b);
    free_pipeline(b);
    b->cls_of.assign(b->n, -1);
    for (auto &c : b->classes)
        if (c.stream) cudaStreamDestroy(c.stream);
    for (auto e : b->joins) cudaEventDestroy(e);
    b->classes.clear();
    b->joins.clear();
    b->big.clear();
    struct Item {
        int idx, threads, smem;
        int64_t cells;
    };
    std::vector<Item> items;
    for (int i = 0; i < b->n; ++i) {
        int threads = 0, smem = 0;
        if (xk_life_resident_config(b->W[i], b->H[i], band_for(b, b->W[i], b->H[i]), &threads, &smem))
            items.push_back({i, threads, smem, (int64_t)b->W[i] * b->H[i]});
        else
            b->big.push_back(i);
    }
    // classes: same block size, shared memory rounded up to 8 KB buckets
    std::sort(items.begin(), items.end(), [](const Item &a, const Item &c) {
        if (a.threads != c.threads) return a.threads > c.threads;
        if (a.smem != c.smem) return a.smem > c.smem;
        return a.cells > c.cells;
    });
    b->h_inst.clear();
    for (size_t k = 0; k < items.size(); ++k) {
        const Item &it = items[k];
        const int bucket = (it.smem + 8191) / 8192 * 8192;
        if (b->classes.empty() || b->classes.back().threads != it.threads ||
            (b->classes.back().smem + 8191) / 8192 * 8192 != bucket) {
            Class c;
            c.threads = it.threads;
            c.smem = it.smem;   // the first (largest) member sets the allocation
            c.first = (int)k;
            b->classes.push_back(c);
        }
        Class &c = b->classes.back();
        b->cls_of[it.idx] = (int)b->classes.size() - 1;
        c.smem = std::max(c.smem, it.smem);
        c.count++;
        LifeInst in;
        memset(&in, 0, sizeof(in));
        in.off = b->off[it.idx];
        in.W = b->W[it.idx];
        in.H = b->H[it.idx];
        in.wpr = (in.W + 31) / 32;
        in.rlast = in.W - 32 * (in.wpr - 1);
        in.lastmask = in.rlast == 32 ? 0xFFFFFFFFu : ((1u << in.rlast) - 1u);
        in.rule0 = rule0_of(b->rule[it.idx]);
        in.rule1 = rule1_of(b->rule[it.idx]);
        in.smem_words = it.smem / 4;
        b->h_inst.push_back(in);
    }
    // classes come sorted by block size, largest first; their CTAs run longest,
    // so their launches (xk_batch_step, direct or in the graph) carry the
    // greater priorities and the block scheduler dispatches them first
    // (longest work first packs the SMs best).  The streams themselves keep
    // the default priority: the end-to-end schedule (xk_batch_run) launches
    // the classes that share their SMs on them behind its high-priority
    // staged groups.
    int prio_least = 0, prio_greatest = 0;
    XK_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
    for (size_t k = 0; k < b->classes.size(); ++k)
        b->classes[k].priority = prio_greatest + std::min<int>((int)k, prio_least - prio_greatest);
    for (auto &c : b->classes) {
        XK_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        cudaEvent_t e;
        XK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->joins.push_back(e);
    }
    if (b->d_inst) cudaFree(b->d_inst);
    b->d_inst = nullptr;
    if (!b->h_inst.empty()) {
        XK_CUDA(cudaMalloc(&b->d_inst, b->h_inst.size() * sizeof(LifeInst)));
        XK_CUDA(cudaMemcpy(b->d_inst, b->h_inst.data(), b->h_inst.size() * sizeof(LifeInst),
                           cudaMemcpyHostToDevice));
    }
    return XK_OK;
}

extern "C" int xk_batch_create(int32_t count, const int32_t *width, const int32_t *height,
                               const uint32_t *rule, xk_batch **out)
{
    XK_REQUIRE(out && width && height && rule, XK_ERR_ARG, "xk_batch_create: null argument");
    *out = nullptr;
    XK_REQUIRE(count > 0, XK_ERR_ARG, "xk_batch_create: count %d", count);
    xk_batch *b = new (std::nothrow) xk_batch();
    XK_REQUIRE(b, XK_ERR_OOM, "host allocation failed");
    b->n = count;
    b->W.assign(width, width + count);
    b->H.assign(height, height + count);
    b->rule.assign(rule, rule + count);
    b->off.resize(count);
    for (int i = 0; i < count; ++i) {
        if (b->W[i] < 1 || b->H[i] < 1 || (int64_t)b->W[i] * b->H[i] > (1LL << 31)) {
            xk_set_error("instance %d has size %dx%d", i, b->W[i], b->H[i]);
            free_batch(b);
            return XK_ERR_ARG;
        }
        if (b->rule[i] >> 18) {
            xk_set_error("instance %d rule %u has bits above 17", i, b->rule[i]);
            free_batch(b);
            return XK_ERR_ARG;
        }
        b->off[i] = b->total;
        b->total += (int64_t)b->W[i] * b->H[i];
    }
    int rc = XK_OK;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&b->ev0)) != cudaSuccess || (e = cudaEventCreate(&b->ev1)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaMalloc(&b->cells, (size_t)b->total + 16)) != cudaSuccess ||
        (e = cudaMalloc(&b->bad, sizeof(unsigned int))) != cudaSuccess ||
        (e = cudaMemset(b->cells, 0, (size_t)b->total + 16)) != cudaSuccess ||
        (e = cudaMemset(b->bad, 0, sizeof(unsigned int))) != cudaSuccess) {
        rc = xk_cuda_status(e, "xk_batch_create");
        free_batch(b);
        return rc;
    }
    rc = plan_classes(b);
    if (rc != XK_OK) {
        free_batch(b);
        return rc;
    }
    *out = b;
    return XK_OK;
}

extern "C" void xk_batch_destroy(xk_batch *b)
{
    if (b && b->stream) cudaStreamSynchronize(b->stream);
    free_batch(b);
}

extern "C" int64_t xk_batch_total_cells(const xk_batch *b) { return b ? b->total : -1; }

extern "C" int xk_batch_upload(xk_batch *b, const uint8_t *host_cells, int64_t total_cells)
{
    XK_REQUIRE(b && host_cells, XK_ERR_ARG, "xk_batch_upload: null argument");
    XK_REQUIRE(total_cells == b->total, XK_ERR_ARG, "xk_batch_upload: %lld cells, batch has %lld",
               (long long)total_cells, (long long)b->total);
    XK_CUDA(cudaMemcpyAsync(b->cells, host_cells, (size_t)b->total, cudaMemcpyHostToDevice, b->stream));
    XK_CUDA(cudaStreamSynchronize(b->stream));
    return XK_OK;
}

extern "C" int xk_batch_download(xk_batch *b, uint8_t *host_cells, int64_t total_cells)
{
    XK_REQUIRE(b && host_cells, XK_ERR_ARG, "xk_batch_download: null argument");
    XK_REQUIRE(total_cells == b->total, XK_ERR_ARG, "xk_batch_download: %lld cells, batch has %lld",
               (long long)total_cells, (long long)b->total);
    XK_CUDA(cudaMemcpyAsync(host_cells, b->cells, (size_t)b->total, cudaMemcpyDeviceToHost, b->stream));
    XK_CUDA(cudaStreamSynchronize(b->stream));
    return XK_OK;
}

// plain per-generation launches for one instance (also used for instances
// the resident kernel cannot hold)
static int plain_instance(xk_batch *b, int i, int generations, cudaStream_t s)
{
    if (!b->scratch) XK_CUDA(cudaMalloc(&b->scratch, (size_t)b->total + 16));
    uint8_t *a = b->cells + b->off[i], *c = b->scratch + b->off[i];
    const uint32_t r0 = rule0_of(b->rule[i]), r1 = rule1_of(b->rule[i]);
    for (int g = 0; g < generations; ++g) {
        XK_CUDA(xk_life_step_bytes2d(a, c, b->W[i], b->H[i], r0, r1, s));
        std::swap(a, c);
    }
    if (generations & 1)
        XK_CUDA(cudaMemcpyAsync(b->cells + b->off[i], a, (size_t)b->W[i] * b->H[i],
                                cudaMemcpyDeviceToDevice, s));
    return XK_OK;
}

// record the batched step (fork, one launch per class, join) on b->stream
static int enqueue_batched(xk_batch *b, int generations)
{
    XK_CUDA(cudaEventRecord(b->fork, b->stream));
    for (size_t k = 0; k < b->classes.size(); ++k) {
        const Class &c = b->classes[k];
        XK_CUDA(cudaStreamWaitEvent(c.stream, b->fork, 0));
        XK_CUDA(xk_life_step_resident(b->d_inst + c.first, c.count, b->cells, 1, generations, 1, 0u,
                                      b->bad, c.threads, c.smem, c.stream, XK_RULE_TABLE, c.priority));
        XK_CUDA(cudaEventRecord(b->joins[k], c.stream));
    }
    for (int i : b->big) {
        int rc = plain_instance(b, i, generations, b->stream);
        if (rc != XK_OK) return rc;
    }
    for (size_t k = 0; k < b->classes.size(); ++k) XK_CUDA(cudaStreamWaitEvent(b->stream, b->joins[k], 0));
    return XK_OK;
}

// XK_GRAPHS=0 in the environment launches the class kernels directly on their
// streams instead of through a captured graph (same kernels, same order) --
// for tools that cannot follow graph launches
static bool graphs_enabled()
{
    const char *v = getenv("XK_GRAPHS");
    return !(v && v[0] == '0');
}

static int set_class_attributes(xk_batch *b)
{
    for (const Class &c : b->classes)
        XK_CUDA(xk_life_step_resident(b->d_inst + c.first, 0, b->cells, 1, 0, 1, 0u, b->bad,
                                      c.threads, c.smem, b->stream));
    return XK_OK;
}

// enqueue one batched step of `generations` on b->stream (graph or direct)
static int launch_batched(xk_batch *b, int generations);

static int graph_for(xk_batch *b, int generations, cudaGraphExec_t *exec)
{
    auto it = b->graphs.find(generations);
    if (it != b->graphs.end()) {
        *exec = it->second;
        return XK_OK;
    }
    if (!b->big.empty() && !b->scratch) XK_CUDA(cudaMalloc(&b->scratch, (size_t)b->total + 16));
    // kernel attributes are set outside capture
    int arc = set_class_attributes(b);
    if (arc != XK_OK) return arc;
    XK_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_batched(b, generations);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
    if (rc != XK_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    XK_CUDA(e);
    cudaGraphExec_t g = nullptr;
    e = cudaGraphInstantiate(&g, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    XK_CUDA(e);
    b->graphs[generations] = g;
    *exec = g;
    return XK_OK;
}

static int launch_batched(xk_batch *b, int generations)
{
    if (generations <= 0) return XK_OK;
    if (!graphs_enabled()) {
        if (!b->big.empty() && !b->scratch) XK_CUDA(cudaMalloc(&b->scratch, (size_t)b->total + 16));
        int rc = set_class_attributes(b);
        if (rc != XK_OK) return rc;
        return enqueue_batched(b, generations);
    }
    cudaGraphExec_t g;
    int rc = graph_for(b, generations, &g);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaGraphLaunch(g, b->stream));
    return XK_OK;
}

static int check_bad(xk_batch *b)
{
    unsigned int hbad = 0;
    XK_CUDA(cudaMemcpyAsync(&hbad, b->bad, sizeof(hbad), cudaMemcpyDeviceToHost, b->stream));
    XK_CUDA(cudaStreamSynchronize(b->stream));
    if (hbad) {
        XK_CUDA(cudaMemsetAsync(b->bad, 0, sizeof(unsigned int), b->stream));
        XK_CUDA(cudaStreamSynchronize(b->stream));
        xk_set_error("ensemble cells must hold 0 or 1; the uploaded state has other values");
        return XK_ERR_ARG;
    }
    return XK_OK;
}

extern "C" int xk_batch_step(xk_batch *b, int32_t generations)
{
    XK_REQUIRE(b, XK_ERR_ARG, "xk_batch_step: null batch");
    XK_REQUIRE(generations >= 0, XK_ERR_ARG, "xk_batch_step: negative generations");
    if (generations == 0) return XK_OK;
    if (graphs_enabled()) {
        cudaGraphExec_t g;
        int rc = graph_for(b, generations, &g);   // instantiate outside the timed region
        if (rc != XK_OK) return rc;
    }
    XK_CUDA(cudaEventRecord(b->ev0, b->stream));
    int rc = launch_batched(b, generations);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaEventRecord(b->ev1, b->stream));
    XK_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    XK_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    xk_set_last_step_ms(ms);
    return check_bad(b);
}

extern "C" int xk_batch_seed_bernoulli(xk_batch *b, const uint32_t *seeds, const double *p)
{
    XK_REQUIRE(b && seeds && p, XK_ERR_ARG, "xk_batch_seed_bernoulli: null argument");
    std::vector<XkSeedJob> jobs(b->n);
    for (int i = 0; i < b->n; ++i) {
        jobs[i].off = b->off[i];
        jobs[i].n = (int64_t)b->W[i] * b->H[i];
        jobs[i].seed = seeds[i];
        jobs[i].pad = 0;
        jobs[i].p = p[i];
    }
    // the longest streams first: their CTAs start in the first wave
    std::stable_sort(jobs.begin(), jobs.end(),
                     [](const XkSeedJob &a, const XkSeedJob &c) { return a.n > c.n; });
    XkSeedJob *d_jobs = nullptr;
    XK_CUDA(cudaMallocAsync(&d_jobs, jobs.size() * sizeof(XkSeedJob), b->stream));
    cudaError_t e = cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(XkSeedJob),
                                    cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev0, b->stream);
    if (e == cudaSuccess) e = xk_seed_bernoulli(d_jobs, b->n, b->cells, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev1, b->stream);
    cudaFreeAsync(d_jobs, b->stream);
    XK_CUDA(e);
    XK_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    XK_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    xk_set_last_step_ms(ms);
    return XK_OK;
}

extern "C" int xk_batch_step_plain(xk_batch *b, int32_t generations)
{
    XK_REQUIRE(b, XK_ERR_ARG, "xk_batch_step_plain: null batch");
    XK_REQUIRE(generations >= 0, XK_ERR_ARG, "xk_batch_step_plain: negative generations");
    XK_CUDA(cudaEventRecord(b->ev0, b->stream));
    // generation-major order, like a host loop calling step() on every model
    if (!b->scratch) XK_CUDA(cudaMalloc(&b->scratch, (size_t)b->total + 16));
    for (int g = 0; g < generations; ++g) {
        uint8_t *src = (g & 1) ? b->scratch : b->cells;
        uint8_t *dst = (g & 1) ? b->cells : b->scratch;
        for (int i = 0; i < b->n; ++i)
            XK_CUDA(xk_life_step_bytes2d(src + b->off[i], dst + b->off[i], b->W[i], b->H[i],
                                         rule0_of(b->rule[i]), rule1_of(b->rule[i]), b->stream));
    }
    if (generations & 1)
        XK_CUDA(cudaMemcpyAsync(b->cells, b->scratch, (size_t)b->total, cudaMemcpyDeviceToDevice,
                                b->stream));
    XK_CUDA(cudaEventRecord(b->ev1, b->stream));
    XK_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    XK_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    xk_set_last_step_ms(ms);
    return XK_OK;
}

// Chunks for the end-to-end pipeline: about XK_PIPE_CHUNKS runs of
// consecutive lattices with equal cell counts, and per chunk and class the
// descriptors of its lattices (built on the first pipelined run after the
// class table changed).
#define XK_PIPE_CHUNKS 8

static int plan_pipeline(xk_batch *b)
{
    int K = XK_PIPE_CHUNKS;
    if (const char *e = getenv("XK_PIPE_CHUNKS")) K = std::max(1, atoi(e));
    K = std::min(K, b->n);
    b->chunk_first.assign(1, 0);
    const int64_t per = (b->total + K - 1) / K;
    int64_t acc = 0;
    for (int i = 0; i < b->n; ++i) {
        acc += (int64_t)b->W[i] * b->H[i];
        if (acc >= per * (int64_t)b->chunk_first.size() && i + 1 < b->n &&
            (int)b->chunk_first.size() < K)
            b->chunk_first.push_back(i + 1);
    }
    b->chunk_first.push_back(b->n);
    const int nk = (int)b->chunk_first.size() - 1, nc = (int)b->classes.size();
    std::vector<LifeInst> table;
    b->seg.assign(nk, std::vector<std::pair<int, int>>(nc, {0, 0}));
    for (int k = 0; k < nk; ++k)
        for (int c = 0; c < nc; ++c) {
            const int first = (int)table.size();
            for (int i = b->chunk_first[k]; i < b->chunk_first[k + 1]; ++i)
                if (b->cls_of[i] == c) {
                    const Class &cl = b->classes[c];
                    // the class table holds this instance's descriptor
                    for (int j = cl.first; j < cl.first + cl.count; ++j)
                        if (b->h_inst[j].off == b->off[i]) {
                            table.push_back(b->h_inst[j]);
                            break;
                        }
                }
            b->seg[k][c] = {first, (int)table.size() - first};
        }
    if (!table.empty()) {
        XK_CUDA(cudaMalloc(&b->d_pipe, table.size() * sizeof(LifeInst)));
        XK_CUDA(cudaMemcpy(b->d_pipe, table.data(), table.size() * sizeof(LifeInst),
                           cudaMemcpyHostToDevice));
    }
    if (!b->out_stream) XK_CUDA(cudaStreamCreateWithFlags(&b->out_stream, cudaStreamNonBlocking));
    b->pev.assign((size_t)nk * 2, nullptr);
    for (auto &e : b->pev) XK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->pipe_streams.assign(nk, nullptr);
    for (auto &st : b->pipe_streams) XK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    return XK_OK;
}

// End to end with the copies overlapped: chunk k's upload (b->stream), its
// lattices' generations (stream k, after the upload, classes largest first)
// and its download (out_stream, after its generations) run while other
// chunks are in other stages; chunk k + 1's launches fill the SMs while
// chunk k's last lattices finish.  Lattices only the plain path runs make
// the call take the serial form.
static int run_pipelined(xk_batch *b, const uint8_t *host_in, uint8_t *host_out, int generations)
{
    if (b->chunk_first.empty()) {
        int rc = plan_pipeline(b);
        if (rc != XK_OK) return rc;
    }
    const int nk = (int)b->chunk_first.size() - 1, nc = (int)b->classes.size();
    XK_CUDA(cudaEventRecord(b->ev0, b->stream));
    XK_CUDA(cudaStreamWaitEvent(b->out_stream, b->ev0, 0));
    for (int k = 0; k < nk; ++k) {
        const int i0 = b->chunk_first[k], i1 = b->chunk_first[k + 1];
        const int64_t lo = b->off[i0], hi = b->off[i1 - 1] + (int64_t)b->W[i1 - 1] * b->H[i1 - 1];
        cudaEvent_t in_done = b->pev[(size_t)k * 2], done = b->pev[(size_t)k * 2 + 1];
        cudaStream_t st = b->pipe_streams[k];
        XK_CUDA(cudaMemcpyAsync(b->cells + lo, host_in + lo, (size_t)(hi - lo),
                                cudaMemcpyHostToDevice, b->stream));
        XK_CUDA(cudaEventRecord(in_done, b->stream));
        XK_CUDA(cudaStreamWaitEvent(st, in_done, 0));
        for (int c = 0; c < nc; ++c) {
            const auto sg = b->seg[k][c];
            if (sg.second == 0) continue;
            const Class &cl = b->classes[c];
            XK_CUDA(xk_life_step_resident(b->d_pipe + sg.first, sg.second, b->cells, 1, generations,
                                          1, 0u, b->bad, cl.threads, cl.smem, st));
        }
        XK_CUDA(cudaEventRecord(done, st));
        XK_CUDA(cudaStreamWaitEvent(b->out_stream, done, 0));
        XK_CUDA(cudaMemcpyAsync(host_out + lo, b->cells + lo, (size_t)(hi - lo),
                                cudaMemcpyDeviceToHost, b->out_stream));
    }
    XK_CUDA(cudaEventRecord(b->fork, b->out_stream));
    XK_CUDA(cudaStreamWaitEvent(b->stream, b->fork, 0));
    XK_CUDA(cudaEventRecord(b->ev1, b->stream));
    XK_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    XK_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    xk_set_last_step_ms(ms);
    return check_bad(b);
}

// Device address of a host range [p, p + bytes) when all of it is mapped
// page-locked memory (cudaHostRegister / cudaHostAlloc), else null.
static uint8_t *mapped_host(const void *p, int64_t bytes)
{
    cudaPointerAttributes a0, a1;
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess ||
        cudaPointerGetAttributes(&a1, (const uint8_t *)p + bytes - 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer ||
        (uint8_t *)a1.devicePointer != (uint8_t *)a0.devicePointer + bytes - 1)
        return nullptr;
    return (uint8_t *)a0.devicePointer;
}

#define XK_STAGE_GROUP 16   // lattices per staged launch
#define XK_STAGE_STREAMS 12

static int plan_e2e(xk_batch *b)
{
    int lo = 0, hi = 0;
    XK_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (int c = 0; c < (int)b->classes.size(); ++c) {
        const Class &cl = b->classes[c];
        if (xk_life_resident_ctas_per_sm(cl.threads, cl.smem) > 1) {
            b->mapped_cls.push_back(c);
            continue;
        }
        for (int j = 0; j < cl.count; j += XK_STAGE_GROUP) {
            b->stage_cls.push_back(c);
            b->stage_first.push_back(cl.first + j);
            b->stage_count.push_back(std::min(XK_STAGE_GROUP, cl.count - j));
        }
    }
    if (!b->stage_cls.empty()) {
        b->stage_streams.assign(XK_STAGE_STREAMS, nullptr);
        for (auto &st : b->stage_streams)
            XK_CUDA(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, hi));
        b->sev.assign(2 * b->stage_cls.size(), nullptr);
        for (auto &e : b->sev) XK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    XK_CUDA(cudaEventCreateWithFlags(&b->staged_in, cudaEventDisableTiming));
    if (!b->out_stream) XK_CUDA(cudaStreamCreateWithFlags(&b->out_stream, cudaStreamNonBlocking));
    b->e2e_planned = true;
    return XK_OK;
}

// queue the staged groups: per-lattice uploads on b->stream, one launch per
// group on the high-priority streams, per-lattice downloads on out_stream
static int enqueue_staged(xk_batch *b, const uint8_t *host_in, uint8_t *host_out, int generations)
{
    for (size_t g = 0; g < b->stage_cls.size(); ++g) {
        const Class &cl = b->classes[b->stage_cls[g]];
        const int first = b->stage_first[g], count = b->stage_count[g];
        for (int j = first; j < first + count; ++j) {
            const LifeInst &in = b->h_inst[j];
            XK_CUDA(cudaMemcpyAsync(b->cells + in.off, host_in + in.off, (size_t)in.W * in.H,
                                    cudaMemcpyHostToDevice, b->stream));
        }
        cudaEvent_t landed = b->sev[2 * g], done = b->sev[2 * g + 1];
        cudaStream_t st = b->stage_streams[g % b->stage_streams.size()];
        XK_CUDA(cudaEventRecord(landed, b->stream));
        XK_CUDA(cudaStreamWaitEvent(st, landed, 0));
        XK_CUDA(xk_life_step_resident_io(b->d_inst + first, count, b->cells, b->cells, nullptr, generations,
                                         b->bad, cl.threads, cl.smem, st));
        XK_CUDA(cudaEventRecord(done, st));
        XK_CUDA(cudaStreamWaitEvent(b->out_stream, done, 0));
        for (int j = first; j < first + count; ++j) {
            const LifeInst &in = b->h_inst[j];
            XK_CUDA(cudaMemcpyAsync(host_out + in.off, b->cells + in.off, (size_t)in.W * in.H,
                                    cudaMemcpyDeviceToHost, b->out_stream));
        }
    }
    return XK_OK;
}

// join the end-to-end streams on b->stream and time the run
static int finish_e2e(xk_batch *b)
{
    XK_CUDA(cudaEventRecord(b->fork, b->out_stream));
    XK_CUDA(cudaStreamWaitEvent(b->stream, b->fork, 0));
    for (int c : b->mapped_cls) XK_CUDA(cudaStreamWaitEvent(b->stream, b->joins[c], 0));
    XK_CUDA(cudaEventRecord(b->ev1, b->stream));
    XK_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    XK_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    xk_set_last_step_ms(ms);
    return check_bad(b);
}

// End to end on page-locked buffers.  A CTA that has its SM to itself (the
// largest lattices) would leave the SM idle while it read and wrote the host
// link, so those lattices are copied in by the copy engines in launch order,
// run from device memory in groups on high-priority streams, and copied out
// as each group ends.  Every other CTA shares its SM, which keeps computing
// while one CTA waits: those read their cells from host_in and write results
// to host_out (and to the batch's device state) from the kernel; they are
// launched after the staged groups, on streams of lower priority, so the
// largest lattices are dispatched first.
static int run_mapped(xk_batch *b, const uint8_t *host_in, uint8_t *host_out, const uint8_t *din,
                      uint8_t *dout, int generations)
{
    if (!b->e2e_planned) {
        int rc = plan_e2e(b);
        if (rc != XK_OK) return rc;
    }
    int rc = set_class_attributes(b);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaEventRecord(b->ev0, b->stream));
    XK_CUDA(cudaStreamWaitEvent(b->out_stream, b->ev0, 0));
    rc = enqueue_staged(b, host_in, host_out, generations);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaEventRecord(b->staged_in, b->stream));
    // the mapped classes start with the run, queued behind the staged
    // groups' launches (XK_E2E_RELEASE=landed: once the staged uploads have
    // landed, 1-3 % slower)
    const char *rel = getenv("XK_E2E_RELEASE");
    const bool landed = rel && !strcmp(rel, "landed");
    for (int c : b->mapped_cls) {
        const Class &cl = b->classes[c];
        XK_CUDA(cudaStreamWaitEvent(cl.stream, landed ? b->staged_in : b->ev0, 0));
        XK_CUDA(xk_life_step_resident_io(b->d_inst + cl.first, cl.count, din, dout, b->cells, generations,
                                         b->bad, cl.threads, cl.smem, cl.stream));
        XK_CUDA(cudaEventRecord(b->joins[c], cl.stream));
    }
    return finish_e2e(b);
}

extern "C" int xk_batch_run(xk_batch *b, const uint8_t *host_in, uint8_t *host_out,
                            int64_t total_cells, int32_t generations)
{
    XK_REQUIRE(b && host_in && host_out, XK_ERR_ARG, "xk_batch_run: null argument");
    XK_REQUIRE(total_cells == b->total, XK_ERR_ARG, "xk_batch_run: %lld cells, batch has %lld",
               (long long)total_cells, (long long)b->total);
    XK_REQUIRE(generations >= 0, XK_ERR_ARG, "xk_batch_run: negative generations");
    if (generations > 0 && b->big.empty() && !b->classes.empty()) {
        // XK_E2E=chunks in the environment takes the chunked copies for
        // page-locked buffers too
        const char *form = getenv("XK_E2E");
        const bool chunks = form && !strcmp(form, "chunks");
        uint8_t *din = chunks ? nullptr : mapped_host(host_in, b->total);
        uint8_t *dout = din ? mapped_host(host_out, b->total) : nullptr;
        if (din && dout) return run_mapped(b, host_in, host_out, din, dout, generations);
        return run_pipelined(b, host_in, host_out, generations);
    }
    if (generations > 0 && graphs_enabled()) {
        cudaGraphExec_t g;
        int rc = graph_for(b, generations, &g);
        if (rc != XK_OK) return rc;
    }
    XK_CUDA(cudaEventRecord(b->ev0, b->stream));
    XK_CUDA(cudaMemcpyAsync(b->cells, host_in, (size_t)b->total, cudaMemcpyHostToDevice, b->stream));
    int rc = launch_batched(b, generations);
    if (rc != XK_OK) return rc;
    XK_CUDA(cudaMemcpyAsync(host_out, b->cells, (size_t)b->total, cudaMemcpyDeviceToHost, b->stream));
    XK_CUDA(cudaEventRecord(b->ev1, b->stream));
    XK_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    XK_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    xk_set_last_step_ms(ms);
    return check_bad(b);
}

extern "C" int xk_batch_set_band(xk_batch *b, int32_t rows_per_band)
{
    XK_REQUIRE(b, XK_ERR_ARG, "xk_batch_set_band: null batch");
    XK_REQUIRE(rows_per_band >= 1 && rows_per_band <= 1024, XK_ERR_ARG,
               "xk_batch_set_band: rows per band must be 1..1024, got %d", (int)rows_per_band);
    if (rows_per_band == b->rows_per_band && b->size_band.empty()) return XK_OK;
    const int old = b->rows_per_band;
    std::map<std::pair<int, int>, int> old_sizes;
    old_sizes.swap(b->size_band);
    b->rows_per_band = rows_per_band;
    const int rc = plan_classes(b);
    if (rc != XK_OK) {
        b->rows_per_band = old;
        b->size_band.swap(old_sizes);
        plan_classes(b);
    }
    return rc;
}

extern "C" int32_t xk_batch_band(const xk_batch *b)
{
    return b ? b->rows_per_band : 0;
}

extern "C" int xk_batch_set_size_bands(xk_batch *b, const int32_t *triples, int32_t count)
{
    XK_REQUIRE(b && (triples || count == 0), XK_ERR_ARG, "xk_batch_set_size_bands: null argument");
    XK_REQUIRE(count >= 0 && count <= 4096, XK_ERR_ARG,
               "xk_batch_set_size_bands: count %d out of [0, 4096]", (int)count);
    std::map<std::pair<int, int>, int> sizes;
    for (int k = 0; k < count; ++k) {
        const int W = triples[3 * k], H = triples[3 * k + 1], band = triples[3 * k + 2];
        XK_REQUIRE(W >= 1 && H >= 1 && band >= 1 && band <= 1024, XK_ERR_ARG,
                   "xk_batch_set_size_bands: entry %d (%d x %d, band %d) out of range", k, W, H, band);
        sizes[std::make_pair(W, H)] = band;
    }
    if (sizes == b->size_band) return XK_OK;
    sizes.swap(b->size_band);
    const int rc = plan_classes(b);
    if (rc != XK_OK) {
        b->size_band.swap(sizes);
        plan_classes(b);
    }
    return rc;
}

extern "C" int32_t xk_batch_size_bands(const xk_batch *b, int32_t *triples, int32_t capacity)
{
    if (!b) return -1;
    int32_t k = 0;
    for (const auto &kv : b->size_band) {
        if (triples && k < capacity) {
            triples[3 * k] = kv.first.first;
            triples[3 * k + 1] = kv.first.second;
            triples[3 * k + 2] = kv.second;
        }
        ++k;
    }
    return k;
}

// device time of one graph launch of the current plan (the graph is built,
// and run once untimed, first)
static int time_plan(xk_batch *b, int generations, float *ms)
{
    int rc = plan_classes(b);
    if (rc != XK_OK) return rc;
    if ((rc = launch_batched(b, generations)) != XK_OK) return rc;
    XK_CUDA(cudaEventRecord(b->ev0, b->stream));
    if ((rc = launch_batched(b, generations)) != XK_OK) return rc;
    XK_CUDA(cudaEventRecord(b->ev1, b->stream));
    XK_CUDA(cudaEventSynchronize(b->ev1));
    XK_CUDA(cudaEventElapsedTime(ms, b->ev0, b->ev1));
    return XK_OK;
}

// Band lengths by timing the whole batch (on a copy of the state, so tuning
// never changes the cells).  (1) One band for every lattice: the candidates
// are timed in turn, three rounds (a clock that changes during tuning then
// biases no candidate), best of the three per candidate.  (2) Per lattice
// size, largest shares of the cells first, for every size holding at least 3
// % of them: each candidate that gives that size another CTA shape is timed
// (best of two) against the current plan; one that looks at least 3 % faster
// is timed again, alternating with the current plan three more times, and
// kept only when its best time stays at least 2 % below the current plan's
// (a graph launch of the whole batch varies by a few per cent from run to
// run, so smaller gains are not told apart from noise).
extern "C" int xk_batch_tune(xk_batch *b, int32_t generations, int32_t *chosen)
{
    XK_REQUIRE(b && chosen, XK_ERR_ARG, "xk_batch_tune: null argument");
    XK_REQUIRE(generations > 0, XK_ERR_ARG, "xk_batch_tune: generations must be positive");
    static const int cand[] = {2, 4, 8, 16, 32};
    const int ncand = (int)(sizeof(cand) / sizeof(cand[0]));
    uint8_t *keep = nullptr;
    XK_CUDA(cudaMalloc(&keep, (size_t)b->total + 16));
    XK_CUDA(cudaMemcpyAsync(keep, b->cells, (size_t)b->total, cudaMemcpyDeviceToDevice, b->stream));
    const int old_rpb = b->rows_per_band;
    std::map<std::pair<int, int>, int> old_sizes;
    old_sizes.swap(b->size_band);
    int rc = XK_OK;
    float best[8];
    for (int c = 0; c < ncand; ++c) best[c] = 1e30f;
    for (int round = 0; round < 3 && rc == XK_OK; ++round)
        for (int c = 0; c < ncand && rc == XK_OK; ++c) {
            b->rows_per_band = cand[c];
            float t = 0.f;
            if ((rc = time_plan(b, generations, &t)) == XK_OK) best[c] = std::min(best[c], t);
        }
    int bc = 0;
    for (int c = 1; c < ncand; ++c)
        if (best[c] < best[bc]) bc = c;
    b->rows_per_band = cand[bc];
    if (rc == XK_OK) {
        std::map<std::pair<int, int>, int64_t> cells;
        int64_t all = 0;
        for (int i = 0; i < b->n; ++i) {
            cells[std::make_pair(b->W[i], b->H[i])] += (int64_t)b->W[i] * b->H[i];
            all += (int64_t)b->W[i] * b->H[i];
        }
        std::vector<std::pair<int64_t, std::pair<int, int>>> order;
        for (const auto &kv : cells)
            if (kv.second * 100 >= all * 3) order.push_back(std::make_pair(kv.second, kv.first));
        std::sort(order.rbegin(), order.rend());
        for (const auto &o : order) {
            if (rc != XK_OK) break;
            const int W = o.second.first, H = o.second.second;
            int th0 = 0, sm0 = 0;
            if (!xk_life_resident_config(W, H, band_for(b, W, H), &th0, &sm0)) continue;
            float cur = 1e30f;
            for (int rep = 0; rep < 2 && rc == XK_OK; ++rep) {
                float t = 0.f;
                if ((rc = time_plan(b, generations, &t)) == XK_OK) cur = std::min(cur, t);
            }
            std::vector<int> seen_threads{th0};
            for (int c = 0; c < ncand && rc == XK_OK; ++c) {
                int th = 0, sm = 0;
                if (!xk_life_resident_config(W, H, cand[c], &th, &sm)) continue;
                if (std::find(seen_threads.begin(), seen_threads.end(), th) != seen_threads.end()) continue;
                seen_threads.push_back(th);
                const int before = band_for(b, W, H);
                const bool had = b->size_band.count(std::make_pair(W, H)) > 0;
                auto set_trial = [&](bool on) {
                    if (on) b->size_band[std::make_pair(W, H)] = cand[c];
                    else if (had) b->size_band[std::make_pair(W, H)] = before;
                    else b->size_band.erase(std::make_pair(W, H));
                };
                set_trial(true);
                float t = 1e30f;
                for (int rep = 0; rep < 2 && rc == XK_OK; ++rep) {
                    float u = 0.f;
                    if ((rc = time_plan(b, generations, &u)) == XK_OK) t = std::min(t, u);
                }
                bool keep = rc == XK_OK && t < cur * 0.97f;
                if (keep) {
                    // confirm: the current plan and the trial alternately
                    float base = cur;
                    for (int rep = 0; rep < 3 && rc == XK_OK; ++rep) {
                        float u = 0.f;
                        set_trial(false);
                        if ((rc = time_plan(b, generations, &u)) != XK_OK) break;
                        base = std::min(base, u);
                        set_trial(true);
                        if ((rc = time_plan(b, generations, &u)) != XK_OK) break;
                        t = std::min(t, u);
                    }
                    keep = rc == XK_OK && t < base * 0.98f;
                    cur = keep ? t : base;
                }
                if (keep) {
                    set_trial(true);
                } else if (had) {
                    b->size_band[std::make_pair(W, H)] = before;
                } else {
                    b->size_band.erase(std::make_pair(W, H));
                }
            }
        }
    }
    cudaMemcpyAsync(b->cells, keep, (size_t)b->total, cudaMemcpyDeviceToDevice, b->stream);
    cudaStreamSynchronize(b->stream);
    cudaFree(keep);
    if (rc != XK_OK) {
        b->rows_per_band = old_rpb;
        b->size_band.swap(old_sizes);
        plan_classes(b);
        return rc;
    }
    rc = plan_classes(b);
    *chosen = b->rows_per_band;
    return rc;
}

extern "C" int64_t xk_batch_launches(const xk_batch *b, int32_t generations)
{
    if (!b) return -1;
    return (int64_t)b->classes.size() + (int64_t)b->big.size() * generations +
           (int64_t)b->big.size() * (generations & 1);
}

// ---------------------------------------------------------------------------
// membership changes: the device state is rebuilt as one buffer in the new
// order (kept lattices copied device to device), then the classes are
// re-planned, so the next step captures a new graph

static int rebuild_cells(xk_batch *b, const std::vector<int64_t> &src_off, const std::vector<int64_t> &len,
                         int64_t new_total)
{
    uint8_t *cells = nullptr;
    XK_CUDA(cudaMalloc(&cells, (size_t)new_total + 16));
    cudaError_t e = cudaMemsetAsync(cells, 0, (size_t)new_total + 16, b->stream);
    int64_t at = 0;
    for (size_t k = 0; k < len.size() && e == cudaSuccess; ++k) {
        if (src_off[k] >= 0 && len[k] > 0)
            e = cudaMemcpyAsync(cells + at, b->cells + src_off[k], (size_t)len[k], cudaMemcpyDeviceToDevice,
                                b->stream);
        at += len[k];
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        cudaFree(cells);
        return xk_cuda_status(e, "rebuilding the ensemble's cells");
    }
    cudaFree(b->cells);
    b->cells = cells;
    if (b->scratch) cudaFree(b->scratch);   // the plain form's partner, sized anew on use
    b->scratch = nullptr;
    return XK_OK;
}

extern "C" int xk_batch_add(xk_batch *b, int32_t width, int32_t height, uint32_t rule,
                            const uint8_t *host_cells)
{
    XK_REQUIRE(b, XK_ERR_ARG, "xk_batch_add: null batch");
    XK_REQUIRE(width >= 1 && height >= 1 && (int64_t)width * height <= (1LL << 31), XK_ERR_ARG,
               "xk_batch_add: size %dx%d", width, height);
    XK_REQUIRE(rule >> 18 == 0, XK_ERR_ARG, "xk_batch_add: rule %u has bits above 17", rule);
    XK_CUDA(cudaStreamSynchronize(b->stream));
    const int64_t n = (int64_t)width * height;
    std::vector<int64_t> src(b->n + 1), len(b->n + 1);
    for (int i = 0; i < b->n; ++i) {
        src[i] = b->off[i];
        len[i] = (int64_t)b->W[i] * b->H[i];
    }
    src[b->n] = -1;          // the new lattice: zeros, then its cells
    len[b->n] = n;
    int rc = rebuild_cells(b, src, len, b->total + n);
    if (rc != XK_OK) return rc;
    if (host_cells) {
        XK_CUDA(cudaMemcpyAsync(b->cells + b->total, host_cells, (size_t)n, cudaMemcpyHostToDevice,
                                b->stream));
        XK_CUDA(cudaStreamSynchronize(b->stream));
    }
    b->W.push_back(width);
    b->H.push_back(height);
    b->rule.push_back(rule);
    b->off.push_back(b->total);
    b->total += n;
    b->n += 1;
    rc = plan_classes(b);
    return rc == XK_OK ? b->n - 1 : rc;
}

extern "C" int xk_batch_remove(xk_batch *b, int32_t index)
{
    XK_REQUIRE(b, XK_ERR_ARG, "xk_batch_remove: null batch");
    XK_REQUIRE(index >= 0 && index < b->n, XK_ERR_ARG, "xk_batch_remove: index %d of %d lattices",
               index, b->n);
    XK_REQUIRE(b->n > 1, XK_ERR_ARG, "xk_batch_remove: an ensemble keeps at least one lattice");
    XK_CUDA(cudaStreamSynchronize(b->stream));
    std::vector<int64_t> src, len;
    int64_t new_total = 0;
    for (int i = 0; i < b->n; ++i) {
        if (i == index) continue;
        src.push_back(b->off[i]);
        len.push_back((int64_t)b->W[i] * b->H[i]);
        new_total += len.back();
    }
    int rc = rebuild_cells(b, src, len, new_total);
    if (rc != XK_OK) return rc;
    b->W.erase(b->W.begin() + index);
    b->H.erase(b->H.begin() + index);
    b->rule.erase(b->rule.begin() + index);
    b->n -= 1;
    b->off.assign(b->n, 0);
    b->total = 0;
    for (int i = 0; i < b->n; ++i) {
        b->off[i] = b->total;
        b->total += (int64_t)b->W[i] * b->H[i];
    }
    return plan_classes(b);
}

extern "C" int32_t xk_batch_count(const xk_batch *b) { return b ? b->n : -1; }
