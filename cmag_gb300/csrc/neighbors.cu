// neighbors.cu -- density and force neighbour loops over cell-ordered particles.
//
// Reference kernels (one thread per particle, 7^3 cell lookups each):
//   density  calculateDamBreakDensityD fluid_kernel.cu:130-169 (+ sumDensity :99-128)
//            calculatePoiseuilleDensityD poiseuilleFlowKernel.cu:141-182
//            computeDensityVariationD PeristalsisDensity.cu:39-79
//   force    calcAndApplyAccelerationD fluid_kernel.cu:245-292 (+ :172-243)
//            calculatePoiseuilleAccelerationD poiseuilleFlowKernel.cu:267-309 (+ :184-265)
//            computeViscousForceD + computePressureForceD
//            PeristalsisViscousForce.cu:198-242, PeristalsisPressureForce.cu:51-91
//
// Here a group of G lanes shares one particle.  The (2c+1)^2 rows of the cell box
// (just the particle's own z layer for planar 2-D scenes) are walked as runs of
// consecutive cells: a run's particles are one contiguous sorted range
// [off[a], off[b+1]), read with coalesced float4 loads, the G lanes striding
// through it.  Runs wrap at most once per row; a wrapped run carries the
// periodic image shift of its unmasked cell coordinates, as the reference's
// per-cell shift (poiseuilleFlowKernel.cu:121-127, PeristalsisUtil.cu:4-11).
// When every interaction vanishes beyond q = 2 (all families except the
// reference DamBreak wall force, which has no cut-off), rows and runs are trimmed
// to the support sphere.  Partial sums are combined by warp shuffles.
#include <cuda_runtime.h>

#include "kernels.h"

namespace cmag {

namespace {

// Walk the neighbour runs of a particle at (px,py,pz) in cell g, calling
// visit(begin, end, sx, sy, sz) with the sorted range and image shift.
template <class Visit>
__device__ __forceinline__ void for_each_run(const DevParams &p, const uint32_t *__restrict__ off,
                                             float px, float py, float pz, int3 g, Visit &&visit)
{
    const int c = p.cell_count;
    const int zlo = p.planar ? 0 : -c, zhi = p.planar ? 0 : c;
    // margin (in cells) that covers rounding of the cell assignment
    const float marg = 1e-3f;
    for (int dz = zlo; dz <= zhi; ++dz) {
        const int zu = g.z + dz;
        float dzm = 0.0f;
        if (p.trim && dz != 0) {
            float face = (dz > 0) ? (p.oz + (float)zu * p.csz) - pz : pz - (p.oz + (float)(zu + 1) * p.csz);
            dzm = fmaxf(face - marg * p.csz, 0.0f);
        }
        const uint32_t zrow = ((uint32_t)zu & (p.gz - 1u)) * p.gy;
        const float sz = (float)eval_shift(zu, p.gz) * p.wsz;
        for (int dy = -c; dy <= c; ++dy) {
            const int yu = g.y + dy;
            int xa = g.x - c, xb = g.x + c;
            if (p.trim) {
                float dym = 0.0f;
                if (dy != 0) {
                    float face = (dy > 0) ? (p.oy + (float)yu * p.csy) - py
                                          : py - (p.oy + (float)(yu + 1) * p.csy);
                    dym = fmaxf(face - marg * p.csy, 0.0f);
                }
                float r2 = p.support2 - dym * dym - dzm * dzm;
                if (r2 < 0.0f) continue;
                float R = sqrtf(r2) + marg * p.csx;
                int ta = __float2int_rd((px - R - p.ox) / p.csx);
                int tb = __float2int_rd((px + R - p.ox) / p.csx);
                xa = max(xa, ta);
                xb = min(xb, tb);
                if (xa > xb) continue;
            }
            // the offset table covers cells [scan_base, scan_base + scan_cells)
            // (one z layer for planar scenes); rows outside it hold no particles
            const uint32_t row = (zrow + ((uint32_t)yu & (p.gy - 1u))) * p.gx - p.scan_base;
            if (row >= p.scan_cells) continue;
            const float sy = (float)eval_shift(yu, p.gy) * p.wsy;
            const uint32_t xma = (uint32_t)xa & (p.gx - 1u);
            const uint32_t len = (uint32_t)(xb - xa);
            if (xma + len < p.gx) {
                visit(__ldg(off + row + xma), __ldg(off + row + xma + len + 1),
                      (float)eval_shift(xa, p.gx) * p.wsx, sy, sz);
            } else {
                visit(__ldg(off + row + xma), __ldg(off + row + p.gx),
                      (float)eval_shift(xa, p.gx) * p.wsx, sy, sz);
                const uint32_t xmb = (uint32_t)xb & (p.gx - 1u);
                visit(__ldg(off + row), __ldg(off + row + xmb + 1),
                      (float)eval_shift(xb, p.gx) * p.wsx, sy, sz);
            }
        }
    }
}

template <int G>
__device__ __forceinline__ float group_sum(float v)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o, G);
    return v;
}

// ---------------------------------------------------------------- density --
template <int G>
__global__ void __launch_bounds__(256)
    k_density(DevParams p, const float4 *__restrict__ spos, const uint32_t *__restrict__ off,
              float4 *__restrict__ meas)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool active = i < p.n;
    const float4 pi = active ? spos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    // Poiseuille walls keep rest density (poiseuilleFlowKernel.cu:154-158)
    const bool pinned = p.system == CMAG_POISEUILLE && pi.w == 1.0f;
    float sum = 0.0f;
    if (active && !pinned) {
        const int3 g = grid_pos(p, pi.x, pi.y, pi.z);
        for_each_run(p, off, pi.x, pi.y, pi.z, g,
                     [&](uint32_t b, uint32_t e, float sx, float sy, float sz) {
                         for (uint32_t j = b + lane; j < e; j += G) {
                             const float4 pj = __ldg(spos + j);
                             const float rx = pi.x - (pj.x + sx), ry = pi.y - (pj.y + sy),
                                         rz = pi.z - (pj.z + sz);
                             const float d2 = rx * rx + ry * ry + rz * rz;
                             if (d2 < p.support2) sum += kernel_w(p, sqrtf(d2) * p.inv_h);
                         }
                     });
    }
    sum = group_sum<G>(sum);
    if (active && lane == 0) {
        float rho, pr;
        if (pinned) {
            rho = p.rho0;
            pr = p.p_wall;
        } else {
            rho = sum * p.mass;
            pr = eos_pressure(p, rho);
        }
        meas[i] = make_float4(rho, pr, 0.0f, p.system == CMAG_PERISTALSIS ? pi.w : 0.0f);
    }
}

// ------------------------------------------------------------------ force --
template <int G, int SYS>
__global__ void __launch_bounds__(256)
    k_force(DevParams p, const float4 *__restrict__ spos, const float4 *__restrict__ svel,
            const float4 *__restrict__ meas, const uint32_t *__restrict__ idx,
            const uint32_t *__restrict__ off, float4 *__restrict__ out_a,
            float4 *__restrict__ out_b)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    bool active = i < p.n;
    const float4 pi = active ? spos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    // DamBreak: fluid particles only (fluid_kernel.cu:258)
    if (SYS == CMAG_DAMBREAK && pi.w != (float)CMAG_FLUID) active = false;
    float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
    if (active) {
        const float4 vi = svel[i];
        const float4 mi = meas[i];
        const float rho = mi.x;
        const float pterm = mi.y / (rho * rho);
        const int3 g = grid_pos(p, pi.x, pi.y, pi.z);
        for_each_run(p, off, pi.x, pi.y, pi.z, g, [&](uint32_t b, uint32_t e, float sx, float sy,
                                                      float sz) {
            for (uint32_t j = b + lane; j < e; j += G) {
                if (j == i) continue;
                const float4 pj = __ldg(spos + j);
                const float rx = pi.x - (pj.x + sx), ry = pi.y - (pj.y + sy),
                            rz = pi.z - (pj.z + sz);
                const float d2 = rx * rx + ry * ry + rz * rz;
                if (SYS == CMAG_DAMBREAK) {
                    if (pj.w != (float)CMAG_FLUID) {
                        // Lennard-Jones wall force (fluid_kernel.cu:199-207)
                        if (p.lj_cutoff && !(d2 < p.support2)) continue;
                        const float a2 = (p.lj_a * p.lj_a) / d2;
                        const float a6 = a2 * a2 * a2;
                        const float s = p.lj_D * (a6 * a6 - a6) / d2;
                        ax += s * rx; ay += s * ry; az += s * rz;
                        continue;
                    }
                    if (!(d2 < p.support2)) continue;
                    // pressure + Monaghan viscosity (fluid_kernel.cu:221-237)
                    const float dist = sqrtf(d2);
                    const float temp = kernel_dw(p, dist * p.inv_h);
                    const float4 vj = __ldg(svel + j);
                    const float4 mj = __ldg(meas + j);
                    const float vij = (vi.x - vj.x) * rx + (vi.y - vj.y) * ry + (vi.z - vj.z) * rz;
                    float art = 0.0f;
                    if (vij < 0.0f) {
                        const float nu = 2.0f * p.av_alpha * p.h * p.c0 / (rho + mj.x);
                        art = -nu * vij / (d2 + p.av_eps2);
                    }
                    const float s = -p.mass * (pterm + mj.y / (mj.x * mj.x) + art) * temp / dist;
                    ax += s * rx; ay += s * ry; az += s * rz;
                } else if (SYS == CMAG_POISEUILLE) {
                    if (!(d2 < p.support2)) continue;
                    // pressure + Morris viscosity with wall extrapolation
                    // (poiseuilleFlowKernel.cu:184-208, 236-245)
                    const float dist = sqrtf(d2);
                    const float temp = kernel_dw(p, dist * p.inv_h);
                    const float4 vj = __ldg(svel + j);
                    const float4 mj = __ldg(meas + j);
                    float vx, vy, vz;
                    if (pj.w == 1.0f && (pj.y > p.wall_top || pj.y < p.wall_bottom)) {
                        const bool top = pj.y > p.wall_top;
                        const float da = top ? p.wall_top - pi.y : pi.y - p.wall_bottom;
                        const float db = top ? pj.y - p.wall_top : p.wall_bottom - pj.y;
                        const float beta = fminf(1000.0f, 1.0f + db / da);
                        vx = beta * vi.x; vy = beta * vi.y; vz = beta * vi.z;
                    } else {
                        vx = vi.x - vj.x; vy = vi.y - vj.y; vz = vi.z - vj.z;
                    }
                    const float sp = -p.mass * (pterm + mj.y / (mj.x * mj.x)) * temp / dist;
                    const float sv = p.mass * (2.0f * p.mu) * temp / (rho * mj.x * dist);
                    ax += sp * rx + sv * vx; ay += sp * ry + sv * vy; az += sp * rz + sv * vz;
                } else {
                    if (!(d2 < p.support2)) continue;
                    // viscous (PeristalsisViscousForce.cu:206-213) and pressure
                    // (PeristalsisPressureForce.cu:39-43) from one pass
                    const float dist = sqrtf(d2);
                    const float temp = kernel_dw(p, dist * p.inv_h);
                    const float4 vj = __ldg(svel + j);
                    const float4 mj = __ldg(meas + j);
                    const float sv = p.mass * temp * (2.0f * p.mu) / (rho * mj.x * dist);
                    ax += sv * (vi.x - vj.x); ay += sv * (vi.y - vj.y); az += sv * (vi.z - vj.z);
                    const float sp = -p.mass * temp * (pterm + mj.y / (mj.x * mj.x)) / dist;
                    bx += sp * rx; by += sp * ry; bz += sp * rz;
                }
            }
        });
    }
    ax = group_sum<G>(ax); ay = group_sum<G>(ay); az = group_sum<G>(az);
    if (SYS == CMAG_PERISTALSIS) {
        bx = group_sum<G>(bx); by = group_sum<G>(by); bz = group_sum<G>(bz);
    }
    if (active && lane == 0) {
        const uint32_t o = idx[i];
        if (o >= p.n) return;  // only after a failed sort (reported by the sort itself)
        out_a[o] = make_float4(ax, ay, az, 0.0f);
        if (SYS == CMAG_PERISTALSIS) out_b[o] = make_float4(bx, by, bz, 0.0f);
    }
}

template <int G>
void density_g(const DevParams &p, const float4 *spos, const uint32_t *off, float4 *meas,
               cudaStream_t st)
{
    uint64_t threads = (uint64_t)p.n * G;
    uint32_t blocks = (uint32_t)((threads + 255) / 256);
    k_density<G><<<blocks, 256, 0, st>>>(p, spos, off, meas);
}

template <int G>
void force_g(const DevParams &p, const float4 *spos, const float4 *svel, const float4 *meas,
             const uint32_t *idx, const uint32_t *off, float4 *a, float4 *b, cudaStream_t st)
{
    uint64_t threads = (uint64_t)p.n * G;
    uint32_t blocks = (uint32_t)((threads + 255) / 256);
    if (p.system == CMAG_DAMBREAK)
        k_force<G, CMAG_DAMBREAK><<<blocks, 256, 0, st>>>(p, spos, svel, meas, idx, off, a, b);
    else if (p.system == CMAG_POISEUILLE)
        k_force<G, CMAG_POISEUILLE><<<blocks, 256, 0, st>>>(p, spos, svel, meas, idx, off, a, b);
    else
        k_force<G, CMAG_PERISTALSIS><<<blocks, 256, 0, st>>>(p, spos, svel, meas, idx, off, a, b);
}

}  // namespace

void launch_density(const DevParams &p, int group, const float4 *spos, const uint32_t *off,
                    float4 *meas, cudaStream_t st)
{
    if (p.n == 0) return;
    switch (group) {
    case 1: density_g<1>(p, spos, off, meas, st); break;
    case 2: density_g<2>(p, spos, off, meas, st); break;
    case 4: density_g<4>(p, spos, off, meas, st); break;
    case 16: density_g<16>(p, spos, off, meas, st); break;
    default: density_g<8>(p, spos, off, meas, st); break;
    }
}

void launch_force(const DevParams &p, int group, const float4 *spos, const float4 *svel,
                  const float4 *meas, const uint32_t *idx, const uint32_t *off, float4 *out_a,
                  float4 *out_b, cudaStream_t st)
{
    if (p.n == 0) return;
    switch (group) {
    case 1: force_g<1>(p, spos, svel, meas, idx, off, out_a, out_b, st); break;
    case 2: force_g<2>(p, spos, svel, meas, idx, off, out_a, out_b, st); break;
    case 4: force_g<4>(p, spos, svel, meas, idx, off, out_a, out_b, st); break;
    case 16: force_g<16>(p, spos, svel, meas, idx, off, out_a, out_b, st); break;
    default: force_g<8>(p, spos, svel, meas, idx, off, out_a, out_b, st); break;
    }
}

}  // namespace cmag
