// RendererPlain for sm_103a (reference xentica/core/renderers.py:220-270).
//
// Pixel i of a width x height viewport looks at lattice coordinates
//   xa = (int)((float)(i % width) / (float)zoom) + dx
//   xb = (int)((float)(i / width) / (float)zoom) + dy
// on the projection axes (a0, a1), wrapped onto the board with the reference's
// two-step rule, then sums the colours of every cell along the other axes in
// float (outer loop = lowest axis), and stores r / num (/ SMOOTH_FACTOR) as an
// int.  Same operations, same order, same float rounding.  The uint8
// instantiation stores the int's low byte: the frame the reference's render()
// returns (img.get().astype(np.uint8), base.py:753).
#include <climits>

#include "xk_internal.cuh"

template <typename T>
__global__ void xk_k_render(const int32_t *__restrict__ col, T *__restrict__ img,
                            RenderGeo g, int width, int height, int zoom, int dx, int dy)
{
    const int64_t ip = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= (int64_t)width * height) return;
    const unsigned i = (unsigned)ip;
    const int w0 = (int)g.size[g.a0], w1 = (int)g.size[g.a1];
    int xa = (int)(__fdiv_rn((float)(i % (unsigned)width), (float)zoom)) + dx;
    int xb = (int)(__fdiv_rn((float)(i / (unsigned)width), (float)zoom)) + dy;
    if (xa < 0) xa = w0 - (-xa % w0);
    if (xa >= w0) xa = xa % w0;
    if (xb < 0) xb = w1 - (-xb % w1);
    if (xb >= w1) xb = xb % w1;
    int rest[XK_MAXDIM];
    int nrest = 0;
    int64_t projected = 1;
    for (int d = 0; d < g.ndim; ++d)
        if (d != g.a0 && d != g.a1) { rest[nrest++] = d; projected *= g.size[d]; }
    int64_t stride[XK_MAXDIM];
    int64_t s = 1;
    for (int d = 0; d < g.ndim; ++d) { stride[d] = s; s *= g.size[d]; }
    const int64_t base = xa * stride[g.a0] + xb * stride[g.a1];
    float r = 0.f, gg = 0.f, b = 0.f;
    for (int64_t q = 0; q < projected; ++q) {
        int64_t rem = q, idx = base;
        for (int m = nrest - 1; m >= 0; --m) {
            const int d = rest[m];
            idx += (rem % g.size[d]) * stride[d];
            rem /= g.size[d];
        }
        r = __fadd_rn(r, (float)col[3 * idx]);
        gg = __fadd_rn(gg, (float)col[3 * idx + 1]);
        b = __fadd_rn(b, (float)col[3 * idx + 2]);
    }
    const float num = (float)(int)projected;
    float vr = __fdiv_rn(r, num), vg = __fdiv_rn(gg, num), vb = __fdiv_rn(b, num);
    if (g.smooth > 0) {
        const float sf = (float)g.smooth;
        vr = __fdiv_rn(vr, sf);
        vg = __fdiv_rn(vg, sf);
        vb = __fdiv_rn(vb, sf);
    }
    img[3 * ip] = (T)(int)vr;
    img[3 * ip + 1] = (T)(int)vg;
    img[3 * ip + 2] = (T)(int)vb;
}

// The same for a 2-D lattice viewed on axes (0, 1), where nothing is
// projected: one cell per pixel, the sum over projected cells is the cell's
// colour and the division by their number (1) is exact, as is the division
// of a coordinate below 2^24 by a zoom of 1, so both are skipped; the rest
// are the same operations.
template <typename T>
__global__ void xk_k_render2d(const int32_t *__restrict__ col, T *__restrict__ img, int w0, int w1,
                              int smooth, int width, int height, int zoom, int dx, int dy)
{
    const int64_t ip = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= (int64_t)width * height) return;
    const unsigned i = (unsigned)ip;
    const unsigned px = i % (unsigned)width, py = i / (unsigned)width;
    int xa, xb;
    if (zoom == 1) {
        xa = (int)px + dx;
        xb = (int)py + dy;
    } else {
        xa = (int)(__fdiv_rn((float)px, (float)zoom)) + dx;
        xb = (int)(__fdiv_rn((float)py, (float)zoom)) + dy;
    }
    if (xa < 0) xa = w0 - (-xa % w0);
    if (xa >= w0) xa = xa % w0;
    if (xb < 0) xb = w1 - (-xb % w1);
    if (xb >= w1) xb = xb % w1;
    const int32_t *c = col + 3 * ((int64_t)xb * w0 + xa);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        float v = (float)__ldg(c + ch);
        if (smooth > 0) v = __fdiv_rn(v, (float)smooth);
        img[3 * ip + ch] = (T)(int)v;
    }
}

template <typename T>
static cudaError_t render_any(const int32_t *col, T *img, const RenderGeo &g, int width, int height,
                              int zoom, int dx, int dy, cudaStream_t s)
{
    const int64_t n = (int64_t)width * height;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (g.ndim == 2 && g.a0 == 0 && g.a1 == 1 && (zoom != 1 || (width <= (1 << 24) && height <= (1 << 24))))
        xk_k_render2d<T><<<blocks, 256, 0, s>>>(col, img, (int)g.size[0], (int)g.size[1], g.smooth, width,
                                                height, zoom, dx, dy);
    else
        xk_k_render<T><<<blocks, 256, 0, s>>>(col, img, g, width, height, zoom, dx, dy);
    return cudaGetLastError();
}

cudaError_t xk_render_colors(const int32_t *col, int32_t *img, const RenderGeo &g, int width,
                             int height, int zoom, int dx, int dy, cudaStream_t s)
{
    return render_any<int32_t>(col, img, g, width, height, zoom, dx, dy, s);
}

cudaError_t xk_render_colors_u8(const int32_t *col, uint8_t *img, const RenderGeo &g, int width,
                                int height, int zoom, int dx, int dy, cudaStream_t s)
{
    return render_any<uint8_t>(col, img, g, width, height, zoom, dx, dy, s);
}

// smallest and largest of `count` colour values (out[0], out[1]), for the
// colour bookkeeping after an upload
__global__ void xk_k_colors_range(const int32_t *__restrict__ col, int64_t count, int *__restrict__ out)
{
    int lo = INT_MAX, hi = INT_MIN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int v = col[i];
        lo = v < lo ? v : lo;
        hi = v > hi ? v : hi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_down_sync(0xFFFFFFFFu, lo, o));
        hi = max(hi, __shfl_down_sync(0xFFFFFFFFu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(out, lo);
        atomicMax(out + 1, hi);
    }
}

cudaError_t xk_colors_minmax(const int32_t *col, int64_t count, int *out, cudaStream_t s)
{
    const int init[2] = {INT_MAX, INT_MIN};
    cudaError_t e = cudaMemcpyAsync(out, init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    xk_k_colors_range<<<304, 256, 0, s>>>(col, count, out);
    return cudaGetLastError();
}
