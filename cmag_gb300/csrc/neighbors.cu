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
// The particles of each neighbour row are visited as runs of consecutive sorted
// particles (neighbor_walk.cuh: lanes per particle, periodic image shifts, runs
// trimmed to the support circle when every interaction vanishes beyond q = 2,
// which holds for all families except the reference DamBreak wall force).  Partial
// sums of a particle's lanes meet in a shuffle reduction.  The density kernel also stores, per particle,
// p/rho^2 and rho (DamBreak) or 1/rho (the others), so the force loop needs no
// division per pair.
//
// Every fused multiply-add is written out (__fmaf_rn and the paired forms); the
// library is compiled with -fmad=false, so no other multiply and add are fused.
// Results therefore do not depend on how the compiler schedules a particular
// template variant: a scene gives the same bits alone and inside a batch.
#include <cuda_runtime.h>

#include "kernels.h"
#include "neighbor_walk.cuh"

namespace cmag {

namespace {

using walk::for_each_candidate;
using walk::for_each_run;
using walk::frac_cell;
using walk::rel;

// Un-normalised Wendland sum over candidates [b, e) of one run, two candidates
// per step in paired FP32 (FFMA2/FMUL2/FADD2: two FP32 operations per issued
// instruction on sm_100+), scalar tail.  Adds (1 - q/2)^4 (2q + 1) for q < 2.
template <int SYS>
__device__ __forceinline__ void wendland_run(const DevParams &p, const float4 *__restrict__ spos,
                                             uint32_t b, uint32_t e, float4 pi, float sx, float sy,
                                             float sz, float2 &acc)
{
    const float2 px = make_float2(pi.x, pi.x), py = make_float2(pi.y, pi.y),
                 pz = make_float2(pi.z, pi.z);
    const float2 m1 = make_float2(-1.0f, -1.0f), half = make_float2(-0.5f, -0.5f),
                 one = make_float2(1.0f, 1.0f), two = make_float2(2.0f, 2.0f),
                 ih = make_float2(p.inv_h, p.inv_h);
    uint32_t j = b;
    for (; j + 1 < e; j += 2) {
        const float4 a = __ldg(spos + j), c = __ldg(spos + j + 1);
        float2 ax = make_float2(a.x, c.x), ay = make_float2(a.y, c.y), az = make_float2(a.z, c.z);
        if (SYS != CMAG_DAMBREAK) ax = __fadd2_rn(ax, make_float2(sx, sx));
        if (SYS == CMAG_PERISTALSIS) {
            ay = __fadd2_rn(ay, make_float2(sy, sy));
            az = __fadd2_rn(az, make_float2(sz, sz));
        }
        const float2 rx = __ffma2_rn(ax, m1, px), ry = __ffma2_rn(ay, m1, py), rz = __ffma2_rn(az, m1, pz);
        const float2 d2 = __ffma2_rn(rz, rz, __ffma2_rn(ry, ry, __fmul2_rn(rx, rx)));
        const float2 rs = make_float2(rsqrtf(fmaxf(d2.x, 1e-30f)), rsqrtf(fmaxf(d2.y, 1e-30f)));
        float2 q = __fmul2_rn(__fmul2_rn(d2, rs), ih);
        q = make_float2(fminf(q.x, 2.0f), fminf(q.y, 2.0f));
        const float2 t = __ffma2_rn(q, half, one);
        const float2 t2 = __fmul2_rn(t, t);
        float2 w = __fmul2_rn(__fmul2_rn(t2, t2), __ffma2_rn(q, two, one));
        w.x = (d2.x < p.support2) ? w.x : 0.0f;
        w.y = (d2.y < p.support2) ? w.y : 0.0f;
        acc = __fadd2_rn(acc, w);
    }
    if (j < e) {  // the same operations as one half of a pair step
        const float3 r = rel<SYS>(pi, __ldg(spos + j), sx, sy, sz);
        const float d2 = __fmaf_rn(r.z, r.z, __fmaf_rn(r.y, r.y, __fmul_rn(r.x, r.x)));
        const float q = fminf(__fmul_rn(__fmul_rn(d2, rsqrtf(fmaxf(d2, 1e-30f))), p.inv_h), 2.0f);
        const float t = __fmaf_rn(q, -0.5f, 1.0f), t2 = __fmul_rn(t, t);
        const float w = __fmul_rn(__fmul_rn(t2, t2), __fmaf_rn(q, 2.0f, 1.0f));
        acc.x = __fadd_rn(acc.x, (d2 < p.support2) ? w : 0.0f);
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
// 256 threads, 6 blocks per SM: at most 42 registers, no spills
template <int SYS, bool PLANAR, bool TRIM, int G, bool BATCH>
__global__ void __launch_bounds__(256, 6)
    k_density(DevParams pv, BatchView bv, const float4 *__restrict__ spos,
              const uint32_t *__restrict__ off_all, float4 *__restrict__ meas,
              float2 *__restrict__ aux)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = (BATCH ? bv.first : 0u) + t / G;
    const int lane = (int)(t % G);
    const bool active = t / G < (BATCH ? bv.count : pv.n);
    // a batch reads its scene's parameters; the scene's cells start at table_base
    const DevParams &p = BATCH ? bv.scenes[active ? bv.scene_of[i] : bv.scene_of[bv.first]] : pv;
    const uint32_t *off = off_all + p.table_base;
    const float4 pi = active ? spos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    // Poiseuille walls keep rest density (poiseuilleFlowKernel.cu:154-158)
    const bool pinned = SYS == CMAG_POISEUILLE && pi.w == 1.0f;
    float sum = 0.0f;
    if (active && !pinned) {
        const int3 g = grid_pos(p, pi.x, pi.y, pi.z);
        if (p.kernel == CMAG_KERNEL_WENDLAND) {
            float2 acc = make_float2(0.0f, 0.0f);
            for_each_run<SYS, PLANAR, TRIM, G>(
                p, off, lane, g, frac_cell(p, pi),
                [&](uint32_t b, uint32_t e, float sx, float sy, float sz) {
                    wendland_run<SYS>(p, spos, b, e, pi, sx, sy, sz, acc);
                });
            sum = p.w_norm * (acc.x + acc.y);
        } else {
            for_each_candidate<SYS, PLANAR, TRIM, G>(
                p, off, lane, g, frac_cell(p, pi), [&](uint32_t j, float sx, float sy, float sz) {
                    const float3 r = rel<SYS>(pi, __ldg(spos + j), sx, sy, sz);
                    const float d2 = __fmaf_rn(r.z, r.z, __fmaf_rn(r.y, r.y, __fmul_rn(r.x, r.x)));
                    // evaluated for every candidate and selected: no divergent branch
                    const float w = kernel_w(p, fminf(d2 * rsqrtf(fmaxf(d2, 1e-30f)) * p.inv_h, 2.0f));
                    sum += (d2 < p.support2) ? w : 0.0f;
                });
        }
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
        meas[i] = make_float4(rho, pr, 0.0f, SYS == CMAG_PERISTALSIS ? pi.w : 0.0f);
        const float inv_rho = 1.0f / rho;
        aux[i] = make_float2(pr * inv_rho * inv_rho, SYS == CMAG_DAMBREAK ? rho : inv_rho);
    }
}

// ---------------------------------------------- no-slip into moving walls --
// The closest point (xa, ya) of one Peristalsis wall interface
// y_w(x) = base + sgn A sin(K ((x - ox) - c t)) to a fluid particle at (x0, y0),
// by Newton's method on f(x) = (x0 - x) + (y0 - y_w(x)) y_w'(x) (the reference's
// commented-out BottomF/TopF + rtnewt, PeristalsisViscousForce.cu:4-66), with the
// interface's slope there, 1 / (distance of the particle) and the wall's vertical
// velocity.  Each wall particle's velocity is then extrapolated so that the fluid
// velocity relative to the wall vanishes on the interface:
// v_i - v_j -> beta (v_i - v_w), beta = min(beta_max, 1 + d_j / d_i), d_j the wall
// particle's distance from the interface's tangent (the commented-out
// getVelocityDiff, PeristalsisViscousForce.cu:68-138, which took v_w = 0).
struct WallSide {
    float xa, ya, slope, inv_norm, inv_da, vw;
};

__device__ __forceinline__ WallSide wall_side(const DevParams &p, float amp, float t, bool moving,
                                              float sgn, float base, float x0, float y0)
{
    const float K = p.wave_k;
    float x = x0;
#pragma unroll 1
    for (int it = 0; it < 8; ++it) {
        float s, c;
        sincosf(K * ((x - p.ox) - p.wave_speed * t), &s, &c);
        const float yw = base + sgn * amp * s;
        const float d1 = sgn * amp * K * c, d2 = -sgn * amp * K * K * s;
        const float f = (x0 - x) + (y0 - yw) * d1;
        const float df = -1.0f - d1 * d1 + (y0 - yw) * d2;
        const float dx = f / df;
        x -= dx;
        if (!(fabsf(dx) >= 1e-3f * p.r)) break;
    }
    if (!(fabsf(x - x0) < 4.0f * p.h)) x = x0;  // no convergence: the vertical distance
    float s, c;
    sincosf(K * ((x - p.ox) - p.wave_speed * t), &s, &c);
    WallSide w;
    w.xa = x;
    w.ya = base + sgn * amp * s;
    w.slope = sgn * amp * K * c;
    w.inv_norm = rsqrtf(1.0f + w.slope * w.slope);
    const float da = sqrtf((x0 - x) * (x0 - x) + (y0 - w.ya) * (y0 - w.ya));
    w.inv_da = 1.0f / fmaxf(da, 1e-6f * p.r);
    w.vw = moving ? -sgn * amp * K * p.wave_speed * c : 0.0f;  // d y_w / dt
    return w;
}

// ------------------------------------------------------------------ force --
// 256 threads, 4 blocks per SM: at most 64 registers
template <int SYS, bool PLANAR, bool TRIM, int G, bool BATCH>
__global__ void __launch_bounds__(256, 4)
    k_force(DevParams pv, BatchView bv, const float4 *__restrict__ spos,
            const float4 *__restrict__ svel, const float2 *__restrict__ aux,
            const uint32_t *__restrict__ idx, const uint32_t *__restrict__ off_all,
            float4 *__restrict__ out_a, float4 *__restrict__ out_b,
            const PhaseState *__restrict__ ph_all)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = (BATCH ? bv.first : 0u) + t / G;
    const int lane = (int)(t % G);
    const uint32_t n_all = BATCH ? bv.n_total : pv.n;
    bool active = t / G < (BATCH ? bv.count : pv.n);
    const DevParams &p = BATCH ? bv.scenes[active ? bv.scene_of[i] : bv.scene_of[bv.first]] : pv;
    const uint32_t *off = off_all + p.table_base;
    const float4 pi = active ? spos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    // DamBreak: fluid particles only (fluid_kernel.cu:258)
    if (SYS == CMAG_DAMBREAK && pi.w != (float)CMAG_FLUID) active = false;
    float ax = 0.f, ay = 0.f, az = 0.f, bx = 0.f, by = 0.f, bz = 0.f;
    if (active) {
        const float4 vi = svel[i];
        const float2 ai = aux[i];
        const float pterm = ai.x;
        const int3 g = grid_pos(p, pi.x, pi.y, pi.z);
        // Peristalsis no-slip walls: the interfaces as seen by this fluid particle
        const bool noslip = SYS == CMAG_PERISTALSIS && p.wall_noslip && pi.w == 0.0f;
        WallSide wb{}, wt{};
        if (noslip) {
            const PhaseState &ph = ph_all[BATCH ? bv.scene_of[i] : 0u];
            const float amp = ph.is_bc ? ph.configure_height : p.amplitude;
            const float tw = ph.is_bc ? 0.0f : ph.t;
            wb = wall_side(p, amp, tw, !ph.is_bc, 1.0f, -p.half_fluid_h, pi.x, pi.y);
            wt = wall_side(p, amp, tw, !ph.is_bc, -1.0f, p.half_fluid_h, pi.x, pi.y);
        }
        for_each_candidate<SYS, PLANAR, TRIM, G>(
            p, off, lane, g, frac_cell(p, pi), [&](uint32_t j, float sx, float sy, float sz) {
                if (j == i) return;
                const float4 pj = __ldg(spos + j);
                const float3 rv = rel<SYS>(pi, pj, sx, sy, sz);
                const float rx = rv.x, ry = rv.y, rz = rv.z;
                const float d2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, rx * rx));
                // a coincident pair has no direction (the reference's terms turn into
                // NaN there: 0 * inf); it contributes nothing
                if (d2 == 0.0f) return;
                if (SYS == CMAG_DAMBREAK) {
                    if (pj.w != (float)CMAG_FLUID) {
                        // Lennard-Jones wall force (fluid_kernel.cu:199-207)
                        if (TRIM && !(d2 < p.support2)) return;
                        const float inv_d2 = __frcp_rn(d2);
                        const float a2 = p.lj_a2 * inv_d2;
                        const float a6 = a2 * a2 * a2;
                        const float s = p.lj_D * __fmaf_rn(a6, a6, -a6) * inv_d2;
                        ax = __fmaf_rn(s, rx, ax); ay = __fmaf_rn(s, ry, ay); az = __fmaf_rn(s, rz, az);
                        return;
                    }
                    if (!(d2 < p.support2)) return;
                    // pressure + Monaghan viscosity (fluid_kernel.cu:221-237)
                    const float inv_d = rsqrtf(d2);
                    const float temp = kernel_dw(p, d2 * inv_d * p.inv_h);
                    const float2 aj = __ldg(aux + j);
                    float s = pterm + aj.x;
                    const float4 vj = __ldg(svel + j);
                    const float vij =
                        __fmaf_rn(vi.z - vj.z, rz, __fmaf_rn(vi.y - vj.y, ry, (vi.x - vj.x) * rx));
                    if (vij < 0.0f) {
                        const float nu = __fdividef(p.av_coeff, ai.y + aj.y);
                        s -= __fdividef(nu * vij, d2 + p.av_eps2);
                    }
                    s *= -p.mass * temp * inv_d;
                    ax = __fmaf_rn(s, rx, ax); ay = __fmaf_rn(s, ry, ay); az = __fmaf_rn(s, rz, az);
                } else if (SYS == CMAG_POISEUILLE) {
                    if (!(d2 < p.support2)) return;
                    // pressure + Morris viscosity with wall extrapolation
                    // (poiseuilleFlowKernel.cu:184-208, 236-245)
                    const float inv_d = rsqrtf(d2);
                    const float temp = kernel_dw(p, d2 * inv_d * p.inv_h);
                    const float2 aj = __ldg(aux + j);
                    const float4 vj = __ldg(svel + j);
                    float vx, vy, vz;
                    if (pj.w == 1.0f && (pj.y > p.wall_top || pj.y < p.wall_bottom)) {
                        const bool top = pj.y > p.wall_top;
                        const float da = top ? p.wall_top - pi.y : pi.y - p.wall_bottom;
                        const float db = top ? pj.y - p.wall_top : p.wall_bottom - pj.y;
                        const float beta = fminf(1000.0f, 1.0f + __fdividef(db, da));
                        vx = beta * vi.x; vy = beta * vi.y; vz = beta * vi.z;
                    } else {
                        vx = vi.x - vj.x; vy = vi.y - vj.y; vz = vi.z - vj.z;
                    }
                    const float sp = -p.mass * (pterm + aj.x) * temp * inv_d;
                    const float sv = p.visc_coeff * temp * ai.y * aj.y * inv_d;
                    ax = __fmaf_rn(sv, vx, __fmaf_rn(sp, rx, ax));
                    ay = __fmaf_rn(sv, vy, __fmaf_rn(sp, ry, ay));
                    az = __fmaf_rn(sv, vz, __fmaf_rn(sp, rz, az));
                } else {
                    if (!(d2 < p.support2)) return;
                    // viscous (PeristalsisViscousForce.cu:206-213) and pressure
                    // (PeristalsisPressureForce.cu:39-43) from one pass
                    const float inv_d = rsqrtf(d2);
                    const float temp = kernel_dw(p, d2 * inv_d * p.inv_h);
                    const float2 aj = __ldg(aux + j);
                    const float4 vj = __ldg(svel + j);
                    const float sv = p.visc_coeff * temp * ai.y * aj.y * inv_d;
                    float dvx = vi.x - vj.x, dvy = vi.y - vj.y, dvz = vi.z - vj.z;
                    if (noslip && pj.w != 0.0f) {
                        const WallSide &w = pj.w > 0.0f ? wb : wt;
                        const float db = fabsf(w.slope * (pj.x + sx - w.xa) - (pj.y + sy - w.ya)) * w.inv_norm;
                        const float beta = fminf(p.wall_beta_max, 1.0f + db * w.inv_da);
                        dvx = beta * vi.x;
                        dvy = beta * (vi.y - w.vw);
                        dvz = beta * vi.z;
                    }
                    ax = __fmaf_rn(sv, dvx, ax);
                    ay = __fmaf_rn(sv, dvy, ay);
                    az = __fmaf_rn(sv, dvz, az);
                    const float sp = -p.mass * temp * (pterm + aj.x) * inv_d;
                    bx = __fmaf_rn(sp, rx, bx); by = __fmaf_rn(sp, ry, by); bz = __fmaf_rn(sp, rz, bz);
                }
            });
    }
    if (G > 1) {
        ax = group_sum<G>(ax); ay = group_sum<G>(ay); az = group_sum<G>(az);
        if (SYS == CMAG_PERISTALSIS) {
            bx = group_sum<G>(bx); by = group_sum<G>(by); bz = group_sum<G>(bz);
        }
    }
    if (active && lane == 0) {
        const uint32_t o = idx[i];
        if (o >= n_all) return;  // only after a failed sort (reported by the sort itself)
        out_a[o] = make_float4(ax, ay, az, 0.0f);
        if (SYS == CMAG_PERISTALSIS) out_b[o] = make_float4(bx, by, bz, 0.0f);
    }
}

template <int SYS, bool PLANAR, bool TRIM, int G>
void launch_pair(bool force, const DevParams &p, const BatchView &bv, const float4 *spos,
                 const float4 *svel, float4 *meas, float2 *aux, const uint32_t *idx,
                 const uint32_t *off, float4 *a, float4 *b, const PhaseState *ph, cudaStream_t st)
{
    const uint64_t threads = (uint64_t)(bv.scenes ? bv.count : p.n) * G;
    const uint32_t blocks = (uint32_t)((threads + 255) / 256);
    if (bv.scenes) {
        if (force)
            k_force<SYS, PLANAR, TRIM, G, true><<<blocks, 256, 0, st>>>(p, bv, spos, svel, aux, idx, off, a, b, ph);
        else
            k_density<SYS, PLANAR, TRIM, G, true><<<blocks, 256, 0, st>>>(p, bv, spos, off, meas, aux);
    } else {
        if (force)
            k_force<SYS, PLANAR, TRIM, G, false><<<blocks, 256, 0, st>>>(p, bv, spos, svel, aux, idx, off, a, b, ph);
        else
            k_density<SYS, PLANAR, TRIM, G, false><<<blocks, 256, 0, st>>>(p, bv, spos, off, meas, aux);
    }
}

struct PairArgs {
    bool force;
    const float4 *spos, *svel;
    float4 *meas;
    float2 *aux;
    const uint32_t *idx, *off;
    float4 *a, *b;
    const PhaseState *ph;
};

template <int SYS, bool PLANAR, bool TRIM>
void dispatch_g(int group, const DevParams &p, const BatchView &bv, const PairArgs &x, cudaStream_t st)
{
    switch (group) {
    case 2: launch_pair<SYS, PLANAR, TRIM, 2>(x.force, p, bv, x.spos, x.svel, x.meas, x.aux, x.idx, x.off, x.a, x.b, x.ph, st); break;
    case 4: launch_pair<SYS, PLANAR, TRIM, 4>(x.force, p, bv, x.spos, x.svel, x.meas, x.aux, x.idx, x.off, x.a, x.b, x.ph, st); break;
    default: launch_pair<SYS, PLANAR, TRIM, 1>(x.force, p, bv, x.spos, x.svel, x.meas, x.aux, x.idx, x.off, x.a, x.b, x.ph, st); break;
    }
}

template <int SYS>
void dispatch(int group, const DevParams &p, const BatchView &bv, const PairArgs &x, cudaStream_t st)
{
    if (p.planar) {
        if (p.trim) dispatch_g<SYS, true, true>(group, p, bv, x, st);
        else dispatch_g<SYS, true, false>(group, p, bv, x, st);
    } else {
        if (p.trim) dispatch_g<SYS, false, true>(group, p, bv, x, st);
        else dispatch_g<SYS, false, false>(group, p, bv, x, st);
    }
}

// p: the scene's parameters, or for a batch launch group the parameters of any
// scene of the group (family, planar and trim select the kernel variant)
void dispatch_sys(int group, const DevParams &p, const BatchView &bv, const PairArgs &x,
                  cudaStream_t st)
{
    if ((bv.scenes ? bv.count : p.n) == 0) return;
    if (p.system == CMAG_DAMBREAK) dispatch<CMAG_DAMBREAK>(group, p, bv, x, st);
    else if (p.system == CMAG_POISEUILLE) dispatch<CMAG_POISEUILLE>(group, p, bv, x, st);
    else dispatch<CMAG_PERISTALSIS>(group, p, bv, x, st);
}

}  // namespace

void launch_density(const DevParams &p, const BatchView &bv, int group, const float4 *spos,
                    const uint32_t *off, float4 *meas, float2 *aux, cudaStream_t st)
{
    dispatch_sys(group, p, bv, PairArgs{false, spos, nullptr, meas, aux, nullptr, off, nullptr, nullptr, nullptr}, st);
}

void launch_force(const DevParams &p, const BatchView &bv, int group, const float4 *spos,
                  const float4 *svel, const float2 *aux, const uint32_t *idx, const uint32_t *off,
                  float4 *out_a, float4 *out_b, const PhaseState *ph, cudaStream_t st)
{
    dispatch_sys(group, p, bv,
                 PairArgs{true, spos, svel, nullptr, const_cast<float2 *>(aux), idx, off, out_a, out_b, ph}, st);
}

}  // namespace cmag
