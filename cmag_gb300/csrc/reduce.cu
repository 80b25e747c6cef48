// reduce.cu -- device reductions over the fluid particles (front, height,
// averages), replacing the Report harnesses' host-side work:
//   XFrontTest.h:75-86 / YFrontTest.h:79-90: D2H copy + host thrust::sort for
//     the largest x / y of a fluid particle;
//   density.h:51-67, forces.h:56-82: D2H copies + host loops averaging density
//     and forces over fluid particles.
#include <cuda_runtime.h>

#include "kernels.h"

namespace cmag {

namespace {

__device__ __forceinline__ bool is_fluid(int32_t system, float w)
{
    return system == CMAG_DAMBREAK ? w == (float)CMAG_FLUID : w == 0.0f;
}

// order-preserving float <-> uint mapping for atomicMin/atomicMax
__device__ __forceinline__ uint32_t fkey(float f)
{
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// out[0..2] min keys, out[3..5] max keys (initialised to 0xffffffff / 0)
__global__ void __launch_bounds__(256) k_extent(int32_t system, const float4 *__restrict__ pos,
                                                uint32_t n, uint32_t *out)
{
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = pos[i];
        if (!is_fluid(system, q.w)) continue;
        lo[0] = fminf(lo[0], q.x); lo[1] = fminf(lo[1], q.y); lo[2] = fminf(lo[2], q.z);
        hi[0] = fmaxf(hi[0], q.x); hi[1] = fmaxf(hi[1], q.y); hi[2] = fmaxf(hi[2], q.z);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k) {
            atomicMin(&out[k], fkey(lo[k]));
            atomicMax(&out[3 + k], fkey(hi[k]));
        }
}

// sums[0..3] (double) and the count of fluid particles
__global__ void __launch_bounds__(256) k_fluid_sum(int32_t system, const float4 *__restrict__ type_src,
                                                   const float4 *__restrict__ a, uint32_t n,
                                                   double *sums, unsigned long long *count)
{
    double s[4] = {0, 0, 0, 0};
    unsigned long long c = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!is_fluid(system, type_src[i].w)) continue;
        float4 v = a[i];
        s[0] += v.x; s[1] += v.y; s[2] += v.z; s[3] += v.w;
        ++c;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 4; ++k) atomicAdd(&sums[k], s[k]);
        atomicAdd(count, c);
    }
}

// Per-scene extents of a batch: out[6 s .. 6 s + 5] as in k_extent.  Scenes are
// contiguous, so a warp almost always holds one scene and reduces before its
// atomics; a warp that straddles scenes falls back to one atomic per lane.
__global__ void __launch_bounds__(256) k_extent_batch(BatchView bv, const float4 *__restrict__ pos,
                                                      uint32_t *out)
{
    const uint32_t n = bv.n_total, stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        const uint32_t s = valid ? bv.scene_of[i] : 0xffffffffu;
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        bool fluid = false;
        if (valid) {
            q = pos[i];
            fluid = is_fluid(bv.scenes[s].system, q.w);
        }
        float lo[3] = {fluid ? q.x : 3.4e38f, fluid ? q.y : 3.4e38f, fluid ? q.z : 3.4e38f};
        float hi[3] = {fluid ? q.x : -3.4e38f, fluid ? q.y : -3.4e38f, fluid ? q.z : -3.4e38f};
        const uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);
        const bool uniform = __all_sync(0xffffffffu, s == s0 || !valid);
        if (uniform) {
            const bool any = __any_sync(0xffffffffu, fluid);
            if (!any) continue;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                for (int o = 16; o > 0; o >>= 1) {
                    lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
                    hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
                }
            if ((threadIdx.x & 31) == 0)
                for (int k = 0; k < 3; ++k) {
                    atomicMin(&out[6 * s0 + k], fkey(lo[k]));
                    atomicMax(&out[6 * s0 + 3 + k], fkey(hi[k]));
                }
        } else if (fluid) {
            for (int k = 0; k < 3; ++k) {
                atomicMin(&out[6 * s + k], fkey(lo[k]));
                atomicMax(&out[6 * s + 3 + k], fkey(hi[k]));
            }
        }
    }
}

uint32_t blocks_for(uint32_t n)
{
    uint32_t b = (n + 255) / 256;
    return b < 1 ? 1 : (b > 1216 ? 1216 : b);
}

// *flag |= 1 when some element's z differs from z (a NaN differs from everything).
__global__ void __launch_bounds__(256)
    k_z_differs(const float4 *__restrict__ a, uint32_t n, float z, uint32_t *__restrict__ flag)
{
    bool differs = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        differs |= a[i].z != z;
    if (__any_sync(0xffffffffu, differs) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// flags[slot] |= 1 when a particle of a checked slot (expect[slot].y != 0) has a z
// other than expect[slot].x (a NaN differs from everything).
__global__ void __launch_bounds__(256)
    k_z_differs_slots(const float4 *__restrict__ a, const uint16_t *__restrict__ slot_of, uint32_t n,
                      const float2 *__restrict__ expect, uint32_t *__restrict__ flags)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t s = slot_of[i];
        const float2 e = __ldg(expect + s);
        if (e.y != 0.0f && a[i].z != e.x) atomicOr(flags + s, 1u);
    }
}

}  // namespace

void launch_fluid_extent(int32_t system, const float4 *pos, uint32_t n, uint32_t *out6,
                         cudaStream_t st)
{
    k_extent<<<blocks_for(n), 256, 0, st>>>(system, pos, n, out6);
}

void launch_fluid_extents_batch(const BatchView &bv, const float4 *pos, uint32_t *out, cudaStream_t st)
{
    k_extent_batch<<<blocks_for(bv.n_total), 256, 0, st>>>(bv, pos, out);
}

void launch_fluid_sum(int32_t system, const float4 *type_src, const float4 *a, uint32_t n,
                      double *sums4, unsigned long long *count, cudaStream_t st)
{
    k_fluid_sum<<<blocks_for(n), 256, 0, st>>>(system, type_src, a, n, sums4, count);
}

void launch_z_differs(const float4 *a, uint32_t n, float z, uint32_t *flag, cudaStream_t st)
{
    cudaMemsetAsync(flag, 0, sizeof(uint32_t), st);
    if (n) k_z_differs<<<blocks_for(n), 256, 0, st>>>(a, n, z, flag);
}

void launch_z_differs_slots(const float4 *a, const uint16_t *slot_of, uint32_t n, const float2 *expect,
                            uint32_t *flags, uint32_t slots, cudaStream_t st)
{
    cudaMemsetAsync(flags, 0, sizeof(uint32_t) * (size_t)slots, st);
    if (n) k_z_differs_slots<<<blocks_for(n), 256, 0, st>>>(a, slot_of, n, expect, flags);
}

}  // namespace cmag
