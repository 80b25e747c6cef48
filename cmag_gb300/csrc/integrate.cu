// integrate.cu -- time integration, wall motion and the dam gate.
//
//   integrate                    DamBreak.Core/fluid_kernel.cu:323-366
//   integratePoiseuilleSystemD   Poiseuille.Core/poiseuilleFlowKernel.cu:311-348
//   computeCoordinatesD          Peristalsis.Core/PeristalsisIntegrate.cu:1-66
//   configureBoundaryD           Peristalsis.Core/PeristalsisKernel.cu:144-171
//   shift/removeRightBoundaryD   DamBreak.Core/fluid_kernel.cu:294-321
//   Peristalsis phase machine    Peristalsis.Core/PeristalsisSystem.cpp:330-343
#include <cuda_runtime.h>

#include "kernels.h"

namespace cmag {

namespace {

// Advance one boundary-configuration phase exactly as the host mirror does
// (separately rounded adds and multiplies, no contraction).
__device__ __forceinline__ void advance_phase(const DevParams &p, PhaseState *ph, float k_milli)
{
    PhaseState s = *ph;
    s.configure = 0;
    if (s.is_bc) {
        s.time_shift = __fadd_rn(s.time_shift, p.dt);
        if (s.wave_height < p.amplitude) {
            s.configure = 1;
            s.configure_height = s.wave_height;
            s.wave_height = __fadd_rn(s.wave_height, __fmul_rn(p.dt, k_milli));
        } else {
            s.time_relax = __fsub_rn(s.time_relax, p.dt);
            if (s.time_relax < 0.0f) s.is_bc = 0;
        }
    }
    s.t = s.is_bc ? 0.0f : __fsub_rn(s.elapsed, s.time_shift);
    s.elapsed = __fadd_rn(s.elapsed, p.dt);
    *ph = s;
}

__global__ void k_phase(DevParams p, PhaseState *ph, float k_milli)
{
    pdl_entry();
    advance_phase(p, ph, k_milli);
}

__global__ void k_phase_batch(const DevParams *__restrict__ scenes, uint32_t nscenes,
                              PhaseState *ph, float k_milli)
{
    pdl_entry();
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nscenes && scenes[s].system == CMAG_PERISTALSIS) advance_phase(scenes[s], ph + s, k_milli);
}

// Kept neighbour lists: flag the next step's rebuild when the particle is now
// more than skin/2 from where the lists were built (a NaN position flags it too).
__device__ __forceinline__ void check_moved(const DevParams &p, float4 q, float4 b, uint32_t *moved)
{
    const float dx = q.x - b.x, dy = q.y - b.y, dz = q.z - b.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (!(d2 <= p.vl_move2)) *moved = 1u;
}

template <bool BATCH>
__global__ void __launch_bounds__(256)
    k_configure_boundary(DevParams pv, BatchView bv, float4 *__restrict__ pos,
                         const PhaseState *__restrict__ ph_all, const float4 *__restrict__ xb,
                         uint32_t *__restrict__ moved)
{
    pdl_entry();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (BATCH ? bv.n_total : pv.n)) return;
    const uint32_t sc = BATCH ? bv.scene_of[i] : 0u;
    const DevParams &p = BATCH ? bv.scenes[sc] : pv;
    if (BATCH && p.system != CMAG_PERISTALSIS) return;
    const PhaseState *ph = ph_all + sc;
    if (!ph->configure) return;
    float4 q = pos[i];
    if (!configure_wall(p, ph->configure_height, q)) return;
    pos[i] = q;
    if (xb) check_moved(p, q, xb[i], moved);
}

template <bool BATCH>
__global__ void __launch_bounds__(256)
    k_integrate(DevParams pv, BatchView bv, float4 *__restrict__ pos, float4 *__restrict__ vel,
                float4 *__restrict__ vlf, const float4 *__restrict__ acc,
                const float4 *__restrict__ vforce, const float4 *__restrict__ pforce,
                const PhaseState *__restrict__ ph_all, const float4 *__restrict__ xb,
                uint32_t *__restrict__ moved)
{
    pdl_entry();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (BATCH ? bv.n_total : pv.n)) return;
    const uint32_t sc = BATCH ? bv.scene_of[i] : 0u;
    const DevParams &p = BATCH ? bv.scenes[sc] : pv;
    const PhaseState *ph = ph_all + sc;
    float4 q = pos[i];
    float ax, ay, az;
    if (p.system == CMAG_DAMBREAK) {
        if (q.w != (float)CMAG_FLUID) return;
        float4 a = acc[i];
        ax = a.x; ay = a.y; az = a.z;
    } else if (p.system == CMAG_POISEUILLE) {
        if (q.w == 1.0f) return;  // walls stay fixed
        float4 a = acc[i];
        ax = a.x; ay = a.y; az = a.z;
    } else {
        const int is_bc = ph->is_bc;
        if (q.w != 0.0f && is_bc) return;  // walls frozen while configuring
        if (q.w != 0.0f) {                 // moving walls
            const float wave = get_wave(p, q.x, ph->t);
            if (q.w > 0.0f) q.y = -p.half_fluid_h + p.amplitude * wave - p.r * (q.w - 1.0f);
            else q.y = p.half_fluid_h - p.amplitude * wave + p.r * (-q.w - 1.0f);
            pos[i] = q;
            if (xb) check_moved(p, q, xb[i], moved);
            return;
        }
        float4 fv = vforce[i], fp = pforce[i];
        ax = fv.x + fp.x; ay = fv.y + fp.y; az = fv.z + fp.z;
    }
    float4 v = vel[i];
    const float nvx = v.x + (p.gvx + ax) * p.dt;
    const float nvy = v.y + (p.gvy + ay) * p.dt;
    const float nvz = v.z + (p.gvz + az) * p.dt;
    const float4 lf = vlf[i];
    vlf[i] = make_float4((v.x + nvx) * 0.5f, (v.y + nvy) * 0.5f, (v.z + nvz) * 0.5f, lf.w);
    v.x = nvx; v.y = nvy; v.z = nvz;
    q.x += v.x * p.dt; q.y += v.y * p.dt; q.z += v.z * p.dt;
    if (p.system == CMAG_DAMBREAK) {
        if (q.x < p.left_border) { q.x = p.left_border; v.x *= p.damping; }
        if (q.x > p.right_boundary) { q.x = p.right_boundary; v.x *= p.damping; }
        if (q.y < p.bottom_border) { q.y = p.bottom_border; v.y *= p.damping; }
        if (p.clamp_z) {
            if (q.z < p.z_min_border) { q.z = p.z_min_border; v.z *= p.damping; }
            if (q.z > p.z_max_border) { q.z = p.z_max_border; v.z *= p.damping; }
        }
    } else {
        if (q.x > p.half_world_x) q.x -= 2.0f * p.half_world_x;
        if (p.system == CMAG_PERISTALSIS && q.x < -p.half_world_x) q.x += 2.0f * p.half_world_x;
    }
    pos[i] = q;
    vel[i] = v;
    if (xb) check_moved(p, q, xb[i], moved);
}

__global__ void k_gate(DevParams p, float4 *__restrict__ pos, int remove, float dx, float fx, float fy)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float4 q = pos[i];
    if (q.w != (float)CMAG_RIGHT_FIRST_TYPE && q.w != (float)CMAG_RIGHT_SECOND_TYPE) return;
    if (remove) { q.x = fx; q.y = fy; }
    else q.x = q.x + dx;
    pos[i] = q;
}

}  // namespace

void launch_phase(const DevParams &p, PhaseState *ph, float k_milli, cudaStream_t st)
{
    launch_pdl(k_phase, 1, 1, 0, st, p, ph, k_milli);
}

void launch_phase_batch(const DevParams *scenes, uint32_t nscenes, PhaseState *ph, float k_milli,
                        cudaStream_t st)
{
    if (nscenes == 0) return;
    launch_pdl(k_phase_batch, (nscenes + 127) / 128, 128, 0, st, scenes, nscenes, ph, k_milli);
}

void launch_configure_boundary(const DevParams &p, const BatchView &bv, float4 *pos,
                               const PhaseState *ph, cudaStream_t st, const float4 *xb, uint32_t *moved)
{
    const uint32_t n = bv.scenes ? bv.n_total : p.n;
    if (n == 0) return;
    if (bv.scenes)
        launch_pdl(k_configure_boundary<true>, (n + 255) / 256, 256, 0, st, p, bv, pos, ph, xb, moved);
    else
        launch_pdl(k_configure_boundary<false>, (n + 255) / 256, 256, 0, st, p, bv, pos, ph, xb, moved);
}

void launch_integrate(const DevParams &p, const BatchView &bv, float4 *pos, float4 *vel,
                      float4 *vlf, const float4 *acc, const float4 *vforce, const float4 *pforce,
                      const PhaseState *ph, cudaStream_t st, const float4 *xb, uint32_t *moved)
{
    const uint32_t n = bv.scenes ? bv.n_total : p.n;
    if (n == 0) return;
    if (bv.scenes)
        launch_pdl(k_integrate<true>, (n + 255) / 256, 256, 0, st, p, bv, pos, vel, vlf, acc, vforce, pforce, ph,
                   xb, moved);
    else
        launch_pdl(k_integrate<false>, (n + 255) / 256, 256, 0, st, p, bv, pos, vel, vlf, acc, vforce, pforce, ph,
                   xb, moved);
}

// shiftRightBoundaryD (remove = 0: x += dx) and removeRightBoundaryD
// (remove = 1: park the gate particles at (fx, fy))
void launch_gate(const DevParams &p, float4 *pos, int remove, float dx, float fx, float fy,
                 cudaStream_t st)
{
    if (p.n == 0) return;
    k_gate<<<(p.n + 255) / 256, 256, 0, st>>>(p, pos, remove, dx, fx, fy);
}

}  // namespace cmag
