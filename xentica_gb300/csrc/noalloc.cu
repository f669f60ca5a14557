// xk_batch_step_noalloc: the ensemble step for callers that cannot allocate
// device memory.
//
// Some callers cannot call cudaMalloc: code running inside another
// framework's memory pool (which owns every device allocation), code that
// must not allocate after start-up (real-time or graph-replay loops), and
// environments that hand a plugin preallocated buffers only.  They own the
// cell buffer already; what the resident kernel additionally needs -- the
// per-lattice descriptor table it reads and the flag it raises on bad cell
// values -- lives here in a fixed, file-scope device array instead of in
// memory the library allocates.
//
// Limits and sharing:
//   * at most XK_NOALLOC_MAX_LATTICES lattices per call, every one small
//     enough for one CTA (width <= 1024, fits in shared memory); larger
//     requests are rejected with XK_ERR_ARG / XK_ERR_UNSUPPORTED;
//   * the array exists once per device (each device that loads the library
//     holds it until the process exits) and every call shares it: calls that
//     overlap on the GPU (different streams, or different host threads)
//     race on it.  Calls from several host threads are serialised by a
//     mutex, but the caller must not let two calls' GPU work overlap;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current); make that first call
//     before any stream capture.  The address is kept per device together
//     with the identity of the CUDA context it was taken in, and looked up
//     again when the device's context has changed (after cudaDeviceReset, or
//     a host framework resetting the primary context, the module is loaded
//     anew and the old address is stale).
#include <string.h>

#include <algorithm>
#include <mutex>

#include "xk_internal.cuh"

// 4096 descriptors of 40 bytes plus the 256-byte flag slot: 164,096 bytes
// (about 160 KB) on every device that loads the library
static_assert(sizeof(LifeInst) == 40, "LifeInst layout changed: update the scratch size notes");
#define XK_NOALLOC_SCRATCH_BYTES (XK_NOALLOC_MAX_LATTICES * sizeof(LifeInst) + 256)

// the only device memory this entry point uses besides the caller's cells:
// [0, 256) validity flag, then the descriptor table
static __device__ __align__(256) unsigned char g_noalloc_scratch[XK_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};   // context id the address belongs to
// host staging, reused by every call (guarded by g_mu)
LifeInst g_inst[XK_NOALLOC_MAX_LATTICES];
int g_order[XK_NOALLOC_MAX_LATTICES];
int g_threads[XK_NOALLOC_MAX_LATTICES];
int g_smem[XK_NOALLOC_MAX_LATTICES];
LifeInst g_sorted[XK_NOALLOC_MAX_LATTICES];

}  // namespace

extern "C" int xk_batch_step_noalloc(uint8_t *d_cells, int32_t count, const int32_t *width,
                                     const int32_t *height, const uint32_t *rule,
                                     int32_t generations, void *stream)
{
    XK_REQUIRE(d_cells && width && height && rule, XK_ERR_ARG,
               "xk_batch_step_noalloc: null argument");
    XK_REQUIRE(count > 0 && count <= XK_NOALLOC_MAX_LATTICES, XK_ERR_ARG,
               "xk_batch_step_noalloc: %d lattices, the limit is %d", count,
               XK_NOALLOC_MAX_LATTICES);
    XK_REQUIRE(generations >= 0, XK_ERR_ARG, "xk_batch_step_noalloc: negative generations");
    std::lock_guard<std::mutex> lk(g_mu);
    int dev = 0;
    XK_CUDA(cudaGetDevice(&dev));
    XK_REQUIRE(dev >= 0 && dev < kMaxDevices, XK_ERR_ARG, "device %d out of range", dev);
    XK_CUDA(cudaSetDevice(dev));   // makes the device's primary context current
    const unsigned long long ctx = xk_context_id();
    if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
        // once per device (and per context of it), with that device current:
        // the device address of the file-scope array (its name is only a
        // host-side stand-in)
        void *addr = nullptr;
        XK_CUDA(cudaGetSymbolAddress(&addr, g_noalloc_scratch));
        g_scratch_addr[dev] = addr;
        g_scratch_ctx[dev] = ctx;
    }
    unsigned int *bad = (unsigned int *)g_scratch_addr[dev];
    LifeInst *d_inst = (LifeInst *)((unsigned char *)g_scratch_addr[dev] + 256);
    cudaStream_t s = (cudaStream_t)stream;
    int64_t off = 0;
    for (int i = 0; i < count; ++i) {
        XK_REQUIRE(width[i] >= 1 && height[i] >= 1 && (int64_t)width[i] * height[i] <= (1LL << 31),
                   XK_ERR_ARG, "lattice %d has size %dx%d", i, width[i], height[i]);
        XK_REQUIRE(rule[i] >> 18 == 0, XK_ERR_ARG, "lattice %d rule %u has bits above 17", i,
                   rule[i]);
        XK_REQUIRE(xk_life_resident_config(width[i], height[i], 8, &g_threads[i], &g_smem[i]),
                   XK_ERR_UNSUPPORTED,
                   "lattice %d (%dx%d) does not fit one CTA; use xk_batch_step", i, width[i],
                   height[i]);
        LifeInst &in = g_inst[i];
        memset(&in, 0, sizeof(in));
        in.off = off;
        in.W = width[i];
        in.H = height[i];
        in.wpr = (in.W + 31) / 32;
        in.rlast = in.W - 32 * (in.wpr - 1);
        in.lastmask = in.rlast == 32 ? 0xFFFFFFFFu : ((1u << in.rlast) - 1u);
        in.rule0 = rule[i] & 511u;
        in.rule1 = (rule[i] & 511u) | ((rule[i] >> 9) & 511u);
        in.smem_words = g_smem[i] / 4;
        off += (int64_t)in.W * in.H;
        g_order[i] = i;
    }
    if (generations == 0) return XK_OK;
    // group lattices with the same CTA shape so each group is one launch
    std::sort(g_order, g_order + count, [](int a, int b) {
        if (g_threads[a] != g_threads[b]) return g_threads[a] > g_threads[b];
        return g_smem[a] > g_smem[b];
    });
    for (int k = 0; k < count; ++k) g_sorted[k] = g_inst[g_order[k]];
    XK_CUDA(cudaMemcpyAsync(d_inst, g_sorted, (size_t)count * sizeof(LifeInst),
                            cudaMemcpyHostToDevice, s));
    XK_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned int), s));
    int first = 0;
    while (first < count) {
        const int threads = g_threads[g_order[first]];
        int smem = 0, last = first;
        while (last < count && g_threads[g_order[last]] == threads) {
            smem = std::max(smem, g_smem[g_order[last]]);
            ++last;
        }
        XK_CUDA(xk_life_step_resident(d_inst + first, last - first, d_cells, 1, generations, 1, 0u,
                                      bad, threads, smem, s));
        first = last;
    }
    unsigned int hbad = 0;
    XK_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, s));
    XK_CUDA(cudaStreamSynchronize(s));
    XK_REQUIRE(hbad == 0, XK_ERR_ARG,
               "ensemble cells must hold 0 or 1; the state has other values");
    return XK_OK;
}
