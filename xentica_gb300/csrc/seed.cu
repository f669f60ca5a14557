// Bernoulli seeds on the device: cell j of lattice i is
//   RandomState(seed_i).random_sample(n_i)[j] < p_i
// bit for bit as NumPy's legacy generator draws it (the ensemble's seeded
// initial states), so huge ensembles need no host arrays and no host time.
//
// NumPy's RandomState with a 32-bit integer seed is MT19937 (Matsumoto and
// Nishimura, 1998) initialised by the Knuth linear recurrence
//   mt[0] = seed,  mt[i] = 1812433253 * (mt[i-1] ^ (mt[i-1] >> 30)) + i,
// and random_sample takes two consecutive tempered outputs a, b per double:
//   ((a >> 5) * 2^26 + (b >> 6)) / 2^53.
// One twist regenerates the 624-word state, element i from old words i and
// i + 1 and word i + 397 (old for i < 227, otherwise the new word i - 227);
// the last element uses the new word 0.  That splits a twist into three
// phases with no dependency inside a phase: [0, 227), [227, 454), [454, 624).
// One CTA per lattice runs the phases on 256 threads with the old and new
// state double-buffered in shared memory, then tempers the 624 outputs in
// pairs: 312 cells per twist, written as consecutive bytes.
#include "xk_internal.cuh"

#define XK_MT_N 624
#define XK_MT_M 397
#define XK_MT_SPLIT (XK_MT_N - XK_MT_M)    // 227

__device__ __forceinline__ uint32_t xk_mt_next(uint32_t cur, uint32_t nxt, uint32_t far)
{
    const uint32_t y = (cur & 0x80000000u) | (nxt & 0x7FFFFFFFu);
    return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908B0DFu : 0u);
}

__device__ __forceinline__ uint32_t xk_mt_temper(uint32_t y)
{
    y ^= y >> 11;
    y ^= (y << 7) & 0x9D2C5680u;
    y ^= (y << 15) & 0xEFC60000u;
    y ^= y >> 18;
    return y;
}

__global__ void __launch_bounds__(256)
xk_k_seed_bernoulli(const XkSeedJob *__restrict__ jobs, uint8_t *__restrict__ cells)
{
    __shared__ uint32_t buf[2][XK_MT_N];
    const XkSeedJob job = jobs[blockIdx.x];
    const int t = threadIdx.x;
    if (job.n <= 0) return;
    uint32_t *A = buf[0], *B = buf[1];
    if (t == 0) {
        uint32_t s = job.seed;
        for (int i = 0; i < XK_MT_N; ++i) {
            A[i] = s;
            s = 1812433253u * (s ^ (s >> 30)) + (uint32_t)(i + 1);
        }
    }
    __syncthreads();
    uint8_t *out = cells + job.off;
    const double p = job.p;
    const int64_t twists = (job.n + XK_MT_N / 2 - 1) / (XK_MT_N / 2);
    for (int64_t r = 0; r < twists; ++r) {
        if (t < XK_MT_SPLIT) B[t] = xk_mt_next(A[t], A[t + 1], A[t + XK_MT_M]);
        __syncthreads();
        if (t < XK_MT_SPLIT) {
            const int i = XK_MT_SPLIT + t;
            B[i] = xk_mt_next(A[i], A[i + 1], B[i - XK_MT_SPLIT]);
        }
        __syncthreads();
        if (t < XK_MT_N - 2 * XK_MT_SPLIT) {
            const int i = 2 * XK_MT_SPLIT + t;
            B[i] = xk_mt_next(A[i], i + 1 < XK_MT_N ? A[i + 1] : B[0], B[i - XK_MT_SPLIT]);
        }
        __syncthreads();
        // 312 doubles from this twist; the next twist reads B and writes A,
        // which nothing reads any more
        const int64_t base = r * (XK_MT_N / 2);
        for (int k = t; k < XK_MT_N / 2; k += blockDim.x) {
            const int64_t idx = base + k;
            if (idx < job.n) {
                const uint32_t a = xk_mt_temper(B[2 * k]) >> 5, b = xk_mt_temper(B[2 * k + 1]) >> 6;
                const double d = ((double)a * 67108864.0 + (double)b) / 9007199254740992.0;
                out[idx] = d < p ? 1 : 0;
            }
        }
        uint32_t *tmp = A;
        A = B;
        B = tmp;
    }
}

cudaError_t xk_seed_bernoulli(const XkSeedJob *jobs, int count, uint8_t *cells, cudaStream_t s)
{
    if (count <= 0) return cudaSuccess;
    xk_k_seed_bernoulli<<<count, 256, 0, s>>>(jobs, cells);
    return cudaGetLastError();
}
