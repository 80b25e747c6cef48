// force.cu -- the force pass over cell-ordered particles.
//
// Reference kernels (one thread per particle, 7^3 cell lookups each):
//   calcAndApplyAccelerationD fluid_kernel.cu:245-292 (+ :172-243)
//   calculatePoiseuilleAccelerationD poiseuilleFlowKernel.cu:267-309 (+ :184-265)
//   computeViscousForceD + computePressureForceD
//   PeristalsisViscousForce.cu:198-242, PeristalsisPressureForce.cu:51-91
//
// Each particle either walks its neighbour cells as runs of consecutive sorted
// particles (neighbor_walk.cuh; lanes per particle split the rows) or reads the
// interaction list the density pass recorded (the same pairs in the same order).
// Fused multiply-adds are written out (the library is compiled with -fmad=false).
#include <cuda_runtime.h>

#include "kernels.h"
#include "neighbor_walk.cuh"

namespace cmag {

namespace {

using walk::for_each_candidate;
using walk::frac_cell;
using walk::group_sum;
using walk::rel;

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
// 256 threads, as many blocks per SM as each family fits without (large) spills,
// to hide the gathers' latency: planar DamBreak and Poiseuille 6 (40 registers),
// planar Peristalsis and 3-D DamBreak and Poiseuille 5 (48), 3-D Peristalsis 4
// (64: its two 3-D force sums).  A single 3-D scene's list-driven force runs at 4
// (56 registers): the registers hold more of the pair steps in flight than the
// fifth block's warps (3-D dam break 0.167 -> 0.163 ms; 6 blocks spill, 0.220 ms).
template <int SYS, bool PLANAR, bool TRIM, int G, bool BATCH, bool LIST>
__global__ void __launch_bounds__(256, SYS == CMAG_PERISTALSIS ? (PLANAR ? 5 : 4)
                                                               : (PLANAR ? 6 : ((LIST && !BATCH) ? 4 : 5)))
    k_force(DevParams pv, BatchView bv, const float4 *__restrict__ spos,
            const float4 *__restrict__ svel, const float2 *__restrict__ aux,
            const uint32_t *__restrict__ idx, const uint32_t *__restrict__ off_all,
            float4 *__restrict__ out_a, float4 *__restrict__ out_b,
            const PhaseState *__restrict__ ph_all, NeighborList nl)
{
    pdl_entry();
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
        const float nmass = -p.mass;               // pressure factor
        const float visc_i = p.visc_coeff * ai.y;  // viscous factor of particle i
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
        auto pair = [&](uint32_t j, const float4 &pj, float sx, float sy, float sz) {
                if (j == i) return;
                const float3 rv = rel<SYS>(pi, pj, sx, sy, sz);
                // planar scenes: every particle has the same z and no z velocity, so
                // each z term is an exact zero and is left out (same bits)
                const float rx = rv.x, ry = rv.y, rz = PLANAR ? 0.0f : rv.z;
                const float d2 = PLANAR ? __fmaf_rn(ry, ry, rx * rx)
                                        : __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, rx * rx));
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
                        ax = __fmaf_rn(s, rx, ax); ay = __fmaf_rn(s, ry, ay);
                        if (!PLANAR) az = __fmaf_rn(s, rz, az);
                        return;
                    }
                    if (!(d2 < p.support2)) return;
                    // pressure + Monaghan viscosity (fluid_kernel.cu:221-237)
                    const float inv_d = rsqrtf(d2);
                    const float g = kernel_dw_over_r(p, d2 * inv_d, inv_d);  // dW/dr / r
                    const float2 aj = __ldg(aux + j);
                    float s = pterm + aj.x;
                    const float4 vj = __ldg(svel + j);
                    const float vxy = __fmaf_rn(vi.y - vj.y, ry, (vi.x - vj.x) * rx);
                    const float vij = PLANAR ? vxy : __fmaf_rn(vi.z - vj.z, rz, vxy);
                    if (vij < 0.0f) {
                        // viscosity 2 alpha h c0 v_ij / ((rho_i + rho_j)(r^2 + eps^2))
                        s -= __fdividef(p.av_coeff * vij, (ai.y + aj.y) * (d2 + p.av_eps2));
                    }
                    s *= nmass * g;
                    ax = __fmaf_rn(s, rx, ax); ay = __fmaf_rn(s, ry, ay);
                    if (!PLANAR) az = __fmaf_rn(s, rz, az);
                } else if (SYS == CMAG_POISEUILLE) {
                    if (!(d2 < p.support2)) return;
                    // pressure + Morris viscosity with wall extrapolation
                    // (poiseuilleFlowKernel.cu:184-208, 236-245)
                    const float inv_d = rsqrtf(d2);
                    const float g = kernel_dw_over_r(p, d2 * inv_d, inv_d);
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
                    const float sp = nmass * g * (pterm + aj.x);
                    const float sv = visc_i * aj.y * g;
                    ax = __fmaf_rn(sv, vx, __fmaf_rn(sp, rx, ax));
                    ay = __fmaf_rn(sv, vy, __fmaf_rn(sp, ry, ay));
                    if (!PLANAR) az = __fmaf_rn(sv, vz, __fmaf_rn(sp, rz, az));
                } else {
                    if (!(d2 < p.support2)) return;
                    // viscous (PeristalsisViscousForce.cu:206-213) and pressure
                    // (PeristalsisPressureForce.cu:39-43) from one pass
                    const float inv_d = rsqrtf(d2);
                    const float g = kernel_dw_over_r(p, d2 * inv_d, inv_d);
                    const float2 aj = __ldg(aux + j);
                    const float4 vj = __ldg(svel + j);
                    const float sv = visc_i * aj.y * g;
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
                    if (!PLANAR) az = __fmaf_rn(sv, dvz, az);
                    const float sp = nmass * g * (pterm + aj.x);
                    bx = __fmaf_rn(sp, rx, bx); by = __fmaf_rn(sp, ry, by);
                    if (!PLANAR) bz = __fmaf_rn(sp, rz, bz);
                }
            };
        // DamBreak list entries j0, j1, fluid or wall: the pair terms of both in paired
        // FP32, each operation the scalar pair's (same bits), added in list order.
        // Wall entries take the Lennard-Jones term; it is computed only when a lane
        // of the warp has one, so wall neighbours do not split the warp between the
        // paired and the scalar path.
        auto dam_pair2 = [&](uint32_t j0, const float4 &q0, uint32_t j1, const float4 &q1) {
            const float2 rx = __fadd2_rn(make_float2(pi.x, pi.x), make_float2(-q0.x, -q1.x));
            const float2 ry = __fadd2_rn(make_float2(pi.y, pi.y), make_float2(-q0.y, -q1.y));
            const float2 rz = __fadd2_rn(make_float2(pi.z, pi.z), make_float2(-q0.z, -q1.z));
            const float2 dxy = __ffma2_rn(ry, ry, __fmul2_rn(rx, rx));
            const float2 d2 = PLANAR ? dxy : __ffma2_rn(rz, rz, dxy);
            const bool w0 = q0.w != (float)CMAG_FLUID, w1 = q1.w != (float)CMAG_FLUID;
            // a coincident entry (d2 = 0) has no direction: the scalar path skips it.
            // Entries beyond the support (lists kept over several steps hold them)
            // stay on the paired path: 1 - q/2 is clamped at 0 there, which zeroes
            // their pressure and viscosity terms, and their wall term is masked
            // unless the wall force has no cut-off.
            if (!(d2.x > 0.0f && d2.y > 0.0f)) {
                pair(j0, q0, 0.0f, 0.0f, 0.0f);
                pair(j1, q1, 0.0f, 0.0f, 0.0f);
                return;
            }
            const bool in0 = !TRIM || d2.x < p.support2, in1 = !TRIM || d2.y < p.support2;
            float2 slj = make_float2(0.0f, 0.0f);
            if (__any_sync(__activemask(), w0 || w1)) {  // Lennard-Jones (fluid_kernel.cu:199-207)
                const float2 inv_d2 = make_float2(__frcp_rn(d2.x), __frcp_rn(d2.y));
                const float2 a2 = __fmul2_rn(make_float2(p.lj_a2, p.lj_a2), inv_d2);
                const float2 a6 = __fmul2_rn(__fmul2_rn(a2, a2), a2);
                slj = __fmul2_rn(__fmul2_rn(make_float2(p.lj_D, p.lj_D),
                                            __ffma2_rn(a6, a6, make_float2(-a6.x, -a6.y))),
                                 inv_d2);
            }
            const float2 inv_d = make_float2(rsqrtf(d2.x), rsqrtf(d2.y));
            float2 t = __ffma2_rn(__fmul2_rn(d2, inv_d), make_float2(p.nhalf_inv_h, p.nhalf_inv_h),
                                  make_float2(1.0f, 1.0f));
            t = make_float2(fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f));  // 0 beyond the support
            const float2 g = __fmul2_rn(make_float2(p.dwr_norm, p.dwr_norm), __fmul2_rn(__fmul2_rn(t, t), t));
            const float2 a0 = __ldg(aux + j0), a1 = __ldg(aux + j1);
            const float4 v0 = __ldg(svel + j0), v1 = __ldg(svel + j1);
            float2 sp = __fadd2_rn(make_float2(pterm, pterm), make_float2(a0.x, a1.x));
            const float2 dvx = __fadd2_rn(make_float2(vi.x, vi.x), make_float2(-v0.x, -v1.x));
            const float2 dvy = __fadd2_rn(make_float2(vi.y, vi.y), make_float2(-v0.y, -v1.y));
            const float2 vxy = __ffma2_rn(dvy, ry, __fmul2_rn(dvx, rx));
            const float2 vij = PLANAR ? vxy
                                      : __ffma2_rn(__fadd2_rn(make_float2(vi.z, vi.z), make_float2(-v0.z, -v1.z)), rz, vxy);
            {
                // Monaghan viscosity of approaching fluid pairs, evaluated for both and
                // selected (no divergent branch; the selected values are the scalar
                // pair's)
                const float av0 = __fdividef(p.av_coeff * vij.x, (ai.y + a0.y) * (d2.x + p.av_eps2));
                const float av1 = __fdividef(p.av_coeff * vij.y, (ai.y + a1.y) * (d2.y + p.av_eps2));
                sp.x = (vij.x < 0.0f && !w0) ? sp.x - av0 : sp.x;
                sp.y = (vij.y < 0.0f && !w1) ? sp.y - av1 : sp.y;
            }
            sp = __fmul2_rn(sp, __fmul2_rn(make_float2(nmass, nmass), g));
            const float s0 = w0 ? (in0 ? slj.x : 0.0f) : sp.x, s1 = w1 ? (in1 ? slj.y : 0.0f) : sp.y;
            ax = __fmaf_rn(s0, rx.x, ax); ay = __fmaf_rn(s0, ry.x, ay);
            if (!PLANAR) az = __fmaf_rn(s0, rz.x, az);
            ax = __fmaf_rn(s1, rx.y, ax); ay = __fmaf_rn(s1, ry.y, ay);
            if (!PLANAR) az = __fmaf_rn(s1, rz.y, az);
        };
        // Peristalsis list entries j0, j1 (image shifts s0, s1): both pair terms in
        // paired FP32, each operation the scalar pair's (same bits), added in order
        auto peri_pair2 = [&](uint32_t j0, const float4 &q0, float3 s0, uint32_t j1, const float4 &q1,
                              float3 s1) {
            const float2 tx = __fadd2_rn(make_float2(q0.x, q1.x), make_float2(s0.x, s1.x));
            const float2 ty = __fadd2_rn(make_float2(q0.y, q1.y), make_float2(s0.y, s1.y));
            const float2 tz = __fadd2_rn(make_float2(q0.z, q1.z), make_float2(s0.z, s1.z));
            const float2 rx = __fadd2_rn(make_float2(pi.x, pi.x), make_float2(-tx.x, -tx.y));
            const float2 ry = __fadd2_rn(make_float2(pi.y, pi.y), make_float2(-ty.x, -ty.y));
            const float2 rz = __fadd2_rn(make_float2(pi.z, pi.z), make_float2(-tz.x, -tz.y));
            const float2 dxy = __ffma2_rn(ry, ry, __fmul2_rn(rx, rx));
            const float2 d2 = PLANAR ? dxy : __ffma2_rn(rz, rz, dxy);
            // coincident entries take the scalar path; entries beyond the support
            // stay here with 1 - q/2 clamped at 0 (all their terms vanish)
            if (!(d2.x > 0.0f && d2.y > 0.0f)) {
                pair(j0, q0, s0.x, s0.y, s0.z);
                pair(j1, q1, s1.x, s1.y, s1.z);
                return;
            }
            const float2 inv_d = make_float2(rsqrtf(d2.x), rsqrtf(d2.y));
            float2 t = __ffma2_rn(__fmul2_rn(d2, inv_d), make_float2(p.nhalf_inv_h, p.nhalf_inv_h),
                                  make_float2(1.0f, 1.0f));
            t = make_float2(fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f));
            const float2 g = __fmul2_rn(make_float2(p.dwr_norm, p.dwr_norm), __fmul2_rn(__fmul2_rn(t, t), t));
            const float2 a0 = __ldg(aux + j0), a1 = __ldg(aux + j1);
            const float4 v0 = __ldg(svel + j0), v1 = __ldg(svel + j1);
            const float2 sv = __fmul2_rn(__fmul2_rn(make_float2(visc_i, visc_i), make_float2(a0.y, a1.y)), g);
            const float2 dvx = __fadd2_rn(make_float2(vi.x, vi.x), make_float2(-v0.x, -v1.x));
            const float2 dvy = __fadd2_rn(make_float2(vi.y, vi.y), make_float2(-v0.y, -v1.y));
            const float2 sp = __fmul2_rn(__fmul2_rn(make_float2(nmass, nmass), g),
                                         __fadd2_rn(make_float2(pterm, pterm), make_float2(a0.x, a1.x)));
            ax = __fmaf_rn(sv.x, dvx.x, ax); ay = __fmaf_rn(sv.x, dvy.x, ay);
            bx = __fmaf_rn(sp.x, rx.x, bx); by = __fmaf_rn(sp.x, ry.x, by);
            ax = __fmaf_rn(sv.y, dvx.y, ax); ay = __fmaf_rn(sv.y, dvy.y, ay);
            bx = __fmaf_rn(sp.y, rx.y, bx); by = __fmaf_rn(sp.y, ry.y, by);
            if (!PLANAR) {
                az = __fmaf_rn(sv.x, vi.z - v0.z, az); bz = __fmaf_rn(sp.x, rz.x, bz);
                az = __fmaf_rn(sv.y, vi.z - v1.z, az); bz = __fmaf_rn(sp.y, rz.y, bz);
            }
        };
        // a Poiseuille wall particle beyond the extrapolation lines
        auto extrapolated = [&](const float4 &q) {
            return q.w == 1.0f && (q.y > p.wall_top || q.y < p.wall_bottom);
        };
        // Poiseuille list entries j0, j1 (x image shifts sx0, sx1): both pair terms in
        // paired FP32, each operation the scalar pair's (same bits), added in order.
        // A wall entry beyond an extrapolation line takes beta v_i for v_i - v_j
        // (computed only when a lane of the warp has one).
        auto poi_pair2 = [&](uint32_t j0, const float4 &q0, float sx0, uint32_t j1, const float4 &q1,
                             float sx1) {
            const float2 tx = __fadd2_rn(make_float2(q0.x, q1.x), make_float2(sx0, sx1));
            const float2 rx = __fadd2_rn(make_float2(pi.x, pi.x), make_float2(-tx.x, -tx.y));
            const float2 ry = __fadd2_rn(make_float2(pi.y, pi.y), make_float2(-q0.y, -q1.y));
            const float2 rz = __fadd2_rn(make_float2(pi.z, pi.z), make_float2(-q0.z, -q1.z));
            const float2 dxy = __ffma2_rn(ry, ry, __fmul2_rn(rx, rx));
            const float2 d2 = PLANAR ? dxy : __ffma2_rn(rz, rz, dxy);
            // coincident entries take the scalar path; entries beyond the support
            // stay here with 1 - q/2 clamped at 0 (all their terms vanish)
            if (!(d2.x > 0.0f && d2.y > 0.0f)) {
                pair(j0, q0, sx0, 0.0f, 0.0f);
                pair(j1, q1, sx1, 0.0f, 0.0f);
                return;
            }
            const float2 inv_d = make_float2(rsqrtf(d2.x), rsqrtf(d2.y));
            float2 t = __ffma2_rn(__fmul2_rn(d2, inv_d), make_float2(p.nhalf_inv_h, p.nhalf_inv_h),
                                  make_float2(1.0f, 1.0f));
            t = make_float2(fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f));
            const float2 g = __fmul2_rn(make_float2(p.dwr_norm, p.dwr_norm), __fmul2_rn(__fmul2_rn(t, t), t));
            const float2 a0 = __ldg(aux + j0), a1 = __ldg(aux + j1);
            const float4 v0 = __ldg(svel + j0), v1 = __ldg(svel + j1);
            float2 vx = __fadd2_rn(make_float2(vi.x, vi.x), make_float2(-v0.x, -v1.x));
            float2 vy = __fadd2_rn(make_float2(vi.y, vi.y), make_float2(-v0.y, -v1.y));
            float vz0 = vi.z - v0.z, vz1 = vi.z - v1.z;
            const bool e0 = extrapolated(q0), e1 = extrapolated(q1);
            if (__any_sync(__activemask(), e0 || e1)) {  // poiseuilleFlowKernel.cu:184-208
                auto beta_of = [&](const float4 &q) {
                    const bool top = q.y > p.wall_top;
                    const float da = top ? p.wall_top - pi.y : pi.y - p.wall_bottom;
                    const float db = top ? q.y - p.wall_top : p.wall_bottom - q.y;
                    return fminf(1000.0f, 1.0f + __fdividef(db, da));
                };
                if (e0) {
                    const float b = beta_of(q0);
                    vx.x = b * vi.x; vy.x = b * vi.y; vz0 = b * vi.z;
                }
                if (e1) {
                    const float b = beta_of(q1);
                    vx.y = b * vi.x; vy.y = b * vi.y; vz1 = b * vi.z;
                }
            }
            const float2 sp = __fmul2_rn(__fmul2_rn(make_float2(nmass, nmass), g),
                                         __fadd2_rn(make_float2(pterm, pterm), make_float2(a0.x, a1.x)));
            const float2 sv = __fmul2_rn(__fmul2_rn(make_float2(visc_i, visc_i), make_float2(a0.y, a1.y)), g);
            ax = __fmaf_rn(sv.x, vx.x, __fmaf_rn(sp.x, rx.x, ax));
            ay = __fmaf_rn(sv.x, vy.x, __fmaf_rn(sp.x, ry.x, ay));
            ax = __fmaf_rn(sv.y, vx.y, __fmaf_rn(sp.y, rx.y, ax));
            ay = __fmaf_rn(sv.y, vy.y, __fmaf_rn(sp.y, ry.y, ay));
            if (!PLANAR) {
                az = __fmaf_rn(sv.x, vz0, __fmaf_rn(sp.x, rz.x, az));
                az = __fmaf_rn(sv.y, vz1, __fmaf_rn(sp.y, rz.y, az));
            }
        };
        // image shift of a list entry (2 bits per axis above the index); the code of
        // an unshifted entry decodes to exact zeros
        auto entry_shift = [&](uint32_t en) {
            const uint32_t cd = en >> kListIndexBits;
            return make_float3((float)((int)(cd & 3u) - 1) * p.wsx, (float)((int)((cd >> 2) & 3u) - 1) * p.wsy,
                               PLANAR ? 0.0f : (float)((int)((cd >> 4) & 3u) - 1) * p.wsz);
        };
        constexpr uint32_t kNoShift = 1u | (1u << 2) | (1u << 4);
        const uint32_t cnt = LIST ? __ldg(nl.count + i) : 0u;
        if (LIST && cnt <= nl.cap) {
            // the density pass's list: the walk's interacting candidates, same order
            uint32_t k = 0;
            if (p.kernel == CMAG_KERNEL_WENDLAND) {
                // the next pair's entries are loaded one step ahead (the force waits on
                // the chain entry -> position -> velocity and aux data)
                const uint32_t *ep = nl.entry + i;
                uint32_t e0 = 0, e1 = 0;
                if (cnt >= 2) {
                    e0 = __ldg(ep);
                    e1 = __ldg(ep + nl.stride);
                }
                for (; k + 1 < cnt; k += 2) {
                    uint32_t n0 = 0, n1 = 0;
                    if (k + 3 < cnt) {
                        n0 = __ldg(ep + (size_t)(k + 2) * nl.stride);
                        n1 = __ldg(ep + (size_t)(k + 3) * nl.stride);
                    }
                    const uint32_t j0 = e0 & kListIndexMask, j1 = e1 & kListIndexMask;
                    const uint32_t c0 = e0 >> kListIndexBits, c1 = e1 >> kListIndexBits;
                    e0 = n0;
                    e1 = n1;
                    const float4 q0 = __ldg(spos + j0), q1 = __ldg(spos + j1);
                    if (SYS == CMAG_DAMBREAK) {
                        dam_pair2(j0, q0, j1, q1);
                    } else if (SYS == CMAG_POISEUILLE) {
                        const bool unshifted = c0 == kNoShift && c1 == kNoShift;
                        const float sx0 = unshifted ? 0.0f : entry_shift(c0 << kListIndexBits).x;
                        const float sx1 = unshifted ? 0.0f : entry_shift(c1 << kListIndexBits).x;
                        poi_pair2(j0, q0, sx0, j1, q1, sx1);
                    } else {
                        float3 s0 = make_float3(0.0f, 0.0f, 0.0f), s1 = s0;
                        if (!(c0 == kNoShift && c1 == kNoShift)) {  // near a periodic boundary
                            s0 = entry_shift(c0 << kListIndexBits);
                            s1 = entry_shift(c1 << kListIndexBits);
                        }
                        if (!noslip || (q0.w == 0.0f && q1.w == 0.0f)) {
                            peri_pair2(j0, q0, s0, j1, q1, s1);
                        } else {  // wall neighbours of the no-slip extrapolation
                            pair(j0, q0, s0.x, s0.y, s0.z);
                            pair(j1, q1, s1.x, s1.y, s1.z);
                        }
                    }
                }
            }
#pragma unroll 2
            for (; k < cnt; ++k) {
                const uint32_t en = __ldg(nl.entry + (size_t)k * nl.stride + i);
                float sx = 0.0f, sy = 0.0f, sz = 0.0f;
                if (SYS != CMAG_DAMBREAK) {
                    const uint32_t cd = en >> kListIndexBits;
                    sx = (float)((int)(cd & 3u) - 1) * p.wsx;
                    if (SYS == CMAG_PERISTALSIS) {
                        sy = (float)((int)((cd >> 2) & 3u) - 1) * p.wsy;
                        sz = (float)((int)((cd >> 4) & 3u) - 1) * p.wsz;
                    }
                }
                const uint32_t j = en & kListIndexMask;
                pair(j, __ldg(spos + j), sx, sy, sz);
            }
        } else {
            for_each_candidate<SYS, PLANAR, TRIM, G>(
                p, off, lane, g, frac_cell(p, pi),
                [&](uint32_t j, float sx, float sy, float sz) { pair(j, __ldg(spos + j), sx, sy, sz); });
        }
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

struct ForceArgs {
    const float4 *spos, *svel;
    const float2 *aux;
    const uint32_t *idx, *off;
    float4 *a, *b;
    const PhaseState *ph;
    NeighborList nl;
};

template <int SYS, bool PLANAR, bool TRIM, int G, bool LIST>
void launch_f(const DevParams &p, const BatchView &bv, const ForceArgs &x, cudaStream_t st)
{
    const uint64_t threads = (uint64_t)(bv.scenes ? bv.count : p.n) * G;
    const uint32_t blocks = (uint32_t)((threads + 255) / 256);
    if (bv.scenes)
        launch_pdl(k_force<SYS, PLANAR, TRIM, G, true, LIST>, blocks, 256, 0, st, p, bv, x.spos, x.svel, x.aux, x.idx, x.off, x.a, x.b, x.ph, x.nl);
    else
        launch_pdl(k_force<SYS, PLANAR, TRIM, G, false, LIST>, blocks, 256, 0, st, p, bv, x.spos, x.svel, x.aux, x.idx, x.off, x.a, x.b, x.ph, x.nl);
}

template <int SYS, bool PLANAR, bool TRIM>
void dispatch_g(int group, const DevParams &p, const BatchView &bv, const ForceArgs &x, cudaStream_t st)
{
    if (x.nl.entry) {  // lists: one lane per particle
        launch_f<SYS, PLANAR, TRIM, 1, true>(p, bv, x, st);
        return;
    }
    switch (group) {
    case 2: launch_f<SYS, PLANAR, TRIM, 2, false>(p, bv, x, st); break;
    case 4: launch_f<SYS, PLANAR, TRIM, 4, false>(p, bv, x, st); break;
    default: launch_f<SYS, PLANAR, TRIM, 1, false>(p, bv, x, st); break;
    }
}

template <int SYS>
void dispatch(int group, const DevParams &p, const BatchView &bv, const ForceArgs &x, cudaStream_t st)
{
    if (p.planar) {
        if (p.trim) dispatch_g<SYS, true, true>(group, p, bv, x, st);
        else dispatch_g<SYS, true, false>(group, p, bv, x, st);
    } else {
        if (p.trim) dispatch_g<SYS, false, true>(group, p, bv, x, st);
        else dispatch_g<SYS, false, false>(group, p, bv, x, st);
    }
}

}  // namespace

void launch_force(const DevParams &p, const BatchView &bv, int group, const float4 *spos,
                  const float4 *svel, const float2 *aux, const uint32_t *idx, const uint32_t *off,
                  float4 *out_a, float4 *out_b, const PhaseState *ph, const NeighborList &nl,
                  cudaStream_t st)
{
    if ((bv.scenes ? bv.count : p.n) == 0) return;
    const ForceArgs x{spos, svel, aux, idx, off, out_a, out_b, ph, nl};
    if (p.system == CMAG_DAMBREAK) dispatch<CMAG_DAMBREAK>(group, p, bv, x, st);
    else if (p.system == CMAG_POISEUILLE) dispatch<CMAG_POISEUILLE>(group, p, bv, x, st);
    else dispatch<CMAG_PERISTALSIS>(group, p, bv, x, st);
}

}  // namespace cmag
