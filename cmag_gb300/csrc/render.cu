// render.cu -- headless replacement of the Demo colour buffers and point view.
//
// The reference fills an OpenGL colour VBO (fluidSystem.cpp:97-114 colorRamp and
// :165-181, poiseuilleFlowSystem.cpp:152-166, PeristalsisSystem.cpp:409-442
// Coloring) and draws the position VBO as points.  Here the colours are a device
// float4 array with the reference's values, and the point view is an RGB image
// (x right, y up) splatted on the device and written by the host as a PPM file.
#include <cuda_runtime.h>

#include "kernels.h"

namespace cmag {

namespace {

// colorRamp, fluidSystem.cpp:97-114: seven-stop ramp, linear between stops
__device__ void color_ramp(float t, float *r)
{
    const float c[7][3] = {{1.0f, 0.0f, 0.0f}, {1.0f, 0.5f, 0.0f}, {1.0f, 1.0f, 0.0f},
                           {0.0f, 1.0f, 0.0f}, {0.0f, 1.0f, 1.0f}, {0.0f, 0.0f, 1.0f},
                           {1.0f, 0.0f, 1.0f}};
    t = __fmul_rn(t, 6.0f);
    const int i = (int)t;
    const float u = __fsub_rn(t, floorf(t));
    for (int k = 0; k < 3; ++k) r[k] = __fadd_rn(c[i][k], __fmul_rn(u, __fsub_rn(c[i + 1][k], c[i][k])));
}

__global__ void k_color(DevParams p, const float4 *__restrict__ pos, uint32_t fluid,
                        uint32_t type_one, float4 *__restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    if (p.system == CMAG_PERISTALSIS) {  // PeristalsisSystem.cpp:423-437
        const float4 q = pos[i];
        if (q.w != 0.0f) out[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        else if (q.x < p.ox + 4.0f * p.r) out[i] = make_float4(255.0f, 0.0f, 0.0f, 1.0f);
        else out[i] = make_float4(255.0f, 255.0f, 255.0f, 1.0f);
        return;
    }
    float t = 0.7f;
    if (p.system == CMAG_DAMBREAK) {  // fluidSystem.cpp:171-176
        if (i < type_one) t = 0.2f;
        if (i < fluid) t = 0.5f;
    } else {                          // poiseuilleFlowSystem.cpp:157-161
        if (i < fluid) t = 0.5f;
        if (i % p.gx == 0 && i < fluid) t = 0.2f;
    }
    float r[3];
    color_ramp(t, r);
    out[i] = make_float4(r[0], r[1], r[2], 1.0f);
}

// Points projected on x-y: each pixel shows the particle with the largest index
// that lands in it (its colour is looked up after the scatter).
__global__ void k_splat(const float4 *__restrict__ pos, uint32_t n, float x0, float y0,
                        float inv_px, uint32_t w, uint32_t h, uint32_t *__restrict__ owner)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 q = pos[i];
    const float fx = (q.x - x0) * inv_px, fy = (q.y - y0) * inv_px;
    if (!(fx >= 0.0f && fy >= 0.0f && fx < (float)w && fy < (float)h)) return;
    const uint32_t px = (uint32_t)fx, py = h - 1u - (uint32_t)fy;
    atomicMax(owner + (size_t)py * w + px, i + 1u);
}

__global__ void k_shade(const uint32_t *__restrict__ owner, const float4 *__restrict__ color,
                        uint32_t npix, float scale, uint8_t *__restrict__ rgb)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npix) return;
    const uint32_t o = owner[k];
    uint8_t r = 0, g = 0, b = 0;
    if (o) {
        const float4 c = color[o - 1u];
        r = (uint8_t)fminf(fmaxf(c.x * scale, 0.0f), 255.0f);
        g = (uint8_t)fminf(fmaxf(c.y * scale, 0.0f), 255.0f);
        b = (uint8_t)fminf(fmaxf(c.z * scale, 0.0f), 255.0f);
    }
    rgb[3 * (size_t)k] = r;
    rgb[3 * (size_t)k + 1] = g;
    rgb[3 * (size_t)k + 2] = b;
}

}  // namespace

void launch_colors(const DevParams &p, const float4 *pos, uint32_t fluid, uint32_t type_one,
                   float4 *out, cudaStream_t st)
{
    if (p.n == 0) return;
    k_color<<<(p.n + 255) / 256, 256, 0, st>>>(p, pos, fluid, type_one, out);
}

void launch_render(const float4 *pos, const float4 *color, uint32_t n, float x0, float y0,
                   float inv_px, uint32_t w, uint32_t h, float scale, uint32_t *owner,
                   uint8_t *rgb, cudaStream_t st)
{
    const uint32_t npix = w * h;
    cudaMemsetAsync(owner, 0, sizeof(uint32_t) * (size_t)npix, st);
    if (n) k_splat<<<(n + 255) / 256, 256, 0, st>>>(pos, n, x0, y0, inv_px, w, h, owner);
    k_shade<<<(npix + 255) / 256, 256, 0, st>>>(owner, color, npix, scale, rgb);
}

}  // namespace cmag
