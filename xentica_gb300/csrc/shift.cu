// The "shifting" family (ShiftingSands, examples/shifting_sands.py:15-47):
// a 1-bit state; emit copies it into one buffer and 0 into every other;
// absorb sets the state to the sum of the neighbours' buffers.  Of those
// buffers only one can hold a state, the one neighbour i0 sends towards this
// cell, so on a torus a generation moves every cell's state by -delta[i0]:
// new(x) = old(x + delta[i0]).  On a static border every off-board neighbour's
// buffer reads as the border's whole container (xentica/core/properties.py:
// 444-483), so an edge cell adds the border state once per off-board
// neighbour; the sum is masked to the 1-bit field when stored
// (properties.py:496-541).
//
// Layout: the reference's main plane, one byte per cell, ping-pong.  On a
// torus with colours implied by the state, G generations are one gather:
// new(x) = old(x + G delta[i0]) with each axis taken modulo its size.
#include "xk_internal.cuh"

__global__ void xk_k_shift_nd(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst, NdGeo g,
                              int i0, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t x[XK_MAXDIM];
    int64_t rem = i;
    for (int d = 0; d < g.ndim; ++d) {
        if (d < g.ndim - 1) { x[d] = rem % g.size[d]; rem /= g.size[d]; }
        else x[d] = rem;
    }
    uint32_t sum = 0;
    for (int k = 0; k < g.nbr; ++k) {
        int64_t idx = 0, stride = 1;
        bool off = false;
        for (int d = 0; d < g.ndim; ++d) {
            int64_t c = x[d] + g.delta[k][d];
            if (c < 0 || c >= g.size[d]) {
                off = true;
                c = (c + g.size[d]) % g.size[d];
            }
            idx += c * stride;
            stride *= g.size[d];
        }
        if (off && !g.torus) sum += g.border_state;
        else if (k == i0) sum += src[idx];
    }
    dst[i] = (uint8_t)(sum & 1u);
}

struct ShiftJump {
    int64_t off[XK_MAXDIM];   // per axis: (G delta[i0]) mod size, in [0, size)
};

__global__ void xk_k_shift_jump(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst, NdGeo g,
                                ShiftJump j, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t rem = i, idx = 0, stride = 1;
    for (int d = 0; d < g.ndim; ++d) {
        int64_t x;
        if (d < g.ndim - 1) { x = rem % g.size[d]; rem /= g.size[d]; }
        else x = rem;
        x += j.off[d];
        if (x >= g.size[d]) x -= g.size[d];
        idx += x * stride;
        stride *= g.size[d];
    }
    dst[i] = src[idx];
}

cudaError_t xk_shift_step_nd(const uint8_t *src, uint8_t *dst, const NdGeo &g, int i0, cudaStream_t s)
{
    int64_t n = 1;
    for (int d = 0; d < g.ndim; ++d) n *= g.size[d];
    xk_k_shift_nd<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, g, i0, n);
    return cudaGetLastError();
}

cudaError_t xk_shift_jump(const uint8_t *src, uint8_t *dst, const NdGeo &g, int i0, int64_t generations,
                          cudaStream_t s)
{
    int64_t n = 1;
    ShiftJump j;
    for (int d = 0; d < XK_MAXDIM; ++d) j.off[d] = 0;
    for (int d = 0; d < g.ndim; ++d) {
        n *= g.size[d];
        const int64_t size = g.size[d];
        int64_t o = ((generations % size) * ((int64_t)g.delta[i0][d] % size)) % size;
        if (o < 0) o += size;
        j.off[d] = o;
    }
    xk_k_shift_jump<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, g, j, n);
    return cudaGetLastError();
}
