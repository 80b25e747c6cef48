// sph_common.cuh -- device parameter block and per-pair helpers shared by the
// hash, neighbour-loop and integration kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/cmag_sph.h"

namespace cmag {

constexpr uint32_t kEmptyCell = 0xffffffffu;

// Launch-time parameter block: the cmag_sph_params fields the kernels read,
// plus coefficients the host derives once (kernel normalisation, clamps).
struct DevParams {
    int32_t system, dims, kernel, eos;
    uint32_t gx, gy, gz;          // grid cells per axis
    uint32_t n;                   // particles
    uint32_t scan_base;           // first cell covered by the dense offset table
    uint32_t scan_cells;          // cells covered (one z layer for planar scenes)
    float ox, oy, oz;             // world origin
    float csx, csy, csz;          // cell size (DamBreak hash divides by it)
    float r;                      // particle radius (other families' hash)
    float h, inv_h, support2;     // smoothing length, 1/h, (2h)^2
    float mass, rho0, c0, B, gamma, dt, damping, mu;
    float gvx, gvy, gvz;          // gravity
    int32_t cell_count;
    int32_t planar;               // 1: search only the particle's own z layer
    int32_t trim;                 // 1: trim rows/columns to the support sphere
    float wsx, wsy, wsz;          // periodic image shift per axis
    float right_boundary, left_border, bottom_border;
    int32_t clamp_z;
    float z_min_border, z_max_border;
    float lj_D, lj_a;
    int32_t lj_cutoff;
    float av_alpha, av_eps2;      // artificial viscosity alpha, 0.001 h^2
    float w_norm, dw_norm;        // kernel normalisations (see kernel_w/kernel_dw)
    float dwr_norm;               // Wendland dW/dr / r = dwr_norm (1 - q/2)^3 (kernel_dw_over_r)
    float nhalf_inv_h;            // -1 / (2h): 1 - q/2 = 1 + r * nhalf_inv_h
    float wall_bottom, wall_top;  // Poiseuille extrapolation lines
    float amplitude, wave_k, wave_speed, half_fluid_h;  // Peristalsis wall law
    float half_world_x;
    float p_wall;                 // Poiseuille wall pressure (EOS at rho0)
    // derived on the host for the neighbour loops
    float inv_csx, inv_csy, inv_csz; // 1 / cell size (trimming only; not the hash)
    float support2_cells;         // (2h / cell size)^2
    uint32_t planar_layer;        // z layer of a planar scene
    uint32_t pow2_grid;           // 1: every grid dimension is a power of two
    float lj_a2;                  // a^2 of the wall force
    float av_coeff;               // 2 alpha h c0 (fluid_kernel.cu:229-230)
    float visc_coeff;             // m (mu + mu) (poiseuilleFlowKernel.cu:242-243)
    // Peristalsis no-slip extrapolation into moving walls (0: reference v_i - v_j)
    int32_t wall_noslip;
    float wall_beta_max;
    // batches: where this scene's cell table and particles start in the shared arrays
    uint32_t table_base;
    uint32_t part_base;
    // neighbour lists kept over several steps (cmag_system_set_verlet): a list
    // records every particle j != i closer than sqrt(list_r2) = 2h + skin;
    // verlet = 0: the per-step lists of the force's exact pair set
    float list_r2;
    int32_t verlet;
    float vl_move2;  // (skin / 2)^2: a larger displacement since the rebuild forces the next one
    // DamBreak: the density of a non-fluid particle with no fluid particle in its
    // searched cell box depends only on the non-fluid particles, which stay put,
    // so it is kept over steps (null: not kept).  Per particle in original order
    // (of the whole batch in a batch): wc_entry = (rho, p, epoch bits, 0) and
    // wc_snap = the position it had at the last hash; per 4x4x4 block of the
    // scene's cells: wc_mark = the stamp of the last step a fluid particle was
    // hashed into it; wc_state = {step stamp, epoch, non-fluid particles moved}
    // (one for all scenes of a batch).
    float4 *wc_entry;
    float4 *wc_snap;
    uint32_t *wc_mark;
    uint32_t *wc_state;
    const uint32_t *wc_idx;  // sorted -> original index
    uint32_t wc_nbx, wc_nby, wc_nbz;
};

// wc_state words
constexpr int kWcStamp = 0, kWcEpoch = 1, kWcMoved = 2;

// Several independent scenes advanced by the same launches: the per-scene
// parameter blocks and the scene of every particle.  Scene s owns particles
// [part_base, part_base + n) and cells [table_base, table_base + scan_cells) of
// the shared arrays; its sort keys are table_base + cell, so the sort keeps every
// scene inside its own particle range and scene_of serves the original and the
// sorted order alike.  A neighbour-loop launch covers one launch group (scenes of
// one family and search shape): particles [first, first + count).  Empty
// (scenes == nullptr) for a single scene, whose parameters travel by value.
struct BatchView {
    const DevParams *scenes;
    const uint16_t *scene_of;
    uint32_t n_total;
    uint32_t first, count;
};

// Per-step interaction lists: the density pass records, for every particle whose
// force is computed, the sorted indices of the neighbours its force loop will use
// (entry k of particle i at entry[k * stride + i], so a warp's k-th entries are
// contiguous), in the walk's order, with the periodic image shift of each
// (2 bits per axis above bit 26); the force pass reads them instead of walking the
// cells again.  A particle with more than cap neighbours keeps count > cap and its
// force loop walks the cells.  Empty (entry == nullptr): no lists.
struct NeighborList {
    uint32_t *entry;
    uint32_t *count;
    uint32_t cap;
    uint32_t stride;
    uint32_t *overflow;  // set to 1 when a list outgrew cap (may be null)
};
constexpr uint32_t kListIndexBits = 26;
constexpr uint32_t kListIndexMask = (1u << kListIndexBits) - 1u;

// Device-resident per-step scalars of the Peristalsis phase machine
// (PeristalsisSystem.cpp:330-343), advanced on the device so that a captured
// step can be replayed without host involvement.
struct PhaseState {
    float elapsed, time_shift, time_relax, wave_height;
    int32_t is_bc;            // boundary-configuration flag seen by this step
    int32_t configure;        // 1: configureBoundary runs this step
    float configure_height;   // height passed to configureBoundary
    float t;                  // time passed to the force/integrate kernels
};

// GetWave (PeristalsisKernel.cuh:59-62), wave_k = pi * waves / (fx * r)
__device__ __forceinline__ float get_wave(const DevParams &p, float x, float t)
{
    return sinf(p.wave_k * ((x - p.ox) - p.wave_speed * t));
}

// configureBoundaryD (Peristalsis.Core/PeristalsisKernel.cu:144-171): a wall
// particle (w > 0 bottom, w < 0 top; |w| its layer) placed on the wall of height
// wh; false for a fluid particle (w = 0), which stays where it is.
__device__ __forceinline__ bool configure_wall(const DevParams &p, float wh, float4 &q)
{
    if (q.w > 0.0f) {
        q.y = -p.half_fluid_h + wh * get_wave(p, q.x, 0.0f) - p.r * (q.w - 1.0f);
        return true;
    }
    if (q.w < 0.0f) {
        q.y = p.half_fluid_h - wh * get_wave(p, q.x, 0.0f) + p.r * (-q.w - 1.0f);
        return true;
    }
    return false;
}

// ---------------------------------------------------------------- hashing ---

// calcGridPos: DamBreak divides by the cell size (fluid_kernel.cu:19-25); the
// Poiseuille and Peristalsis copies multiply by 0.5f and divide by the radius
// (poiseuilleFlowKernel.cu:18-24, PeristalsisKernel.cu:18-24).  The _rn
// intrinsics keep every operation separately rounded so the result is the
// reference's bit for bit; float->int truncation saturates like cvt.rzi.
__device__ __forceinline__ int3 grid_pos(const DevParams &p, float x, float y, float z)
{
    int3 g;
    if (p.system == CMAG_DAMBREAK) {
        g.x = __float2int_rz(floorf(__fdiv_rn(__fsub_rn(x, p.ox), p.csx)));
        g.y = __float2int_rz(floorf(__fdiv_rn(__fsub_rn(y, p.oy), p.csy)));
        g.z = __float2int_rz(floorf(__fdiv_rn(__fsub_rn(z, p.oz), p.csz)));
    } else {
        g.x = __float2int_rz(floorf(__fdiv_rn(__fmul_rn(__fsub_rn(x, p.ox), 0.5f), p.r)));
        g.y = __float2int_rz(floorf(__fdiv_rn(__fmul_rn(__fsub_rn(y, p.oy), 0.5f), p.r)));
        g.z = __float2int_rz(floorf(__fdiv_rn(__fmul_rn(__fsub_rn(z, p.oz), 0.5f), p.r)));
    }
    return g;
}

// Periodic wrap of a cell coordinate onto [0, n): the reference's mask
// (fluid_kernel.cu:28-30) for power-of-two grids, the same residue for any other
// size (an extension: the mask is only defined for powers of two).
__device__ __forceinline__ uint32_t wrap_cell(int v, uint32_t n, uint32_t pow2)
{
    if (pow2) return (uint32_t)v & (n - 1u);
    if ((uint32_t)v < n) return (uint32_t)v;
    int m = v % (int)n;
    return (uint32_t)(m < 0 ? m + (int)n : m);
}

// calcGridHash (fluid_kernel.cu:27-32): z*Y*X + y*X + x of the wrapped cell.
// The host checks that every product stays below 2^24 per operand, where the
// reference's __umul24 equals a plain multiply.
__device__ __forceinline__ uint32_t grid_hash(const DevParams &p, int gx, int gy, int gz)
{
    const uint32_t x = wrap_cell(gx, p.gx, p.pow2_grid), y = wrap_cell(gy, p.gy, p.pow2_grid),
                   z = wrap_cell(gz, p.gz, p.pow2_grid);
    return (z * p.gy) * p.gx + y * p.gx + x;
}

// Wall density cache, hash side (DevParams::wc_*): a fluid particle stamps its
// 4x4x4 cell block with this step's stamp; a non-fluid particle whose position
// or type differs from its snapshot takes the new one and marks the cached
// densities stale (the next scan kernel starts a new epoch).  g: the particle's
// unwrapped cell.
__device__ __forceinline__ void wall_cache_note(const DevParams &p, uint32_t i, float4 q, int3 g)
{
    if (q.w == (float)CMAG_FLUID) {
        const uint32_t bx = wrap_cell(g.x, p.gx, p.pow2_grid) >> 2, by = wrap_cell(g.y, p.gy, p.pow2_grid) >> 2,
                       bz = wrap_cell(g.z, p.gz, p.pow2_grid) >> 2;
        p.wc_mark[(bz * p.wc_nby + by) * p.wc_nbx + bx] = p.wc_state[kWcStamp] + 1u;
    } else {
        const float4 s = p.wc_snap[i];
        if (__float_as_uint(s.x) != __float_as_uint(q.x) || __float_as_uint(s.y) != __float_as_uint(q.y) ||
            __float_as_uint(s.z) != __float_as_uint(q.z) || __float_as_uint(s.w) != __float_as_uint(q.w)) {
            p.wc_snap[i] = q;
            p.wc_state[kWcMoved] = 1u;
        }
    }
}

// EvaluateShift, PeristalsisUtil.cu:4-11
__device__ __forceinline__ int eval_shift(int pos, uint32_t size)
{
    return pos < 0 ? -1 : (pos > (int)size - 1 ? 1 : 0);
}

// ----------------------------------------------------------- kernel W, dW ---

// W(q) for q < 2.  Wendland C2: w_norm (1-q/2)^4 (2q+1) with w_norm = 7/(4 pi h^2)
// in 2-D (fluid_kernel.cu:121-124) or 21/(16 pi h^3) in 3-D.  Cubic spline (M4):
// w_norm = 10/(7 pi h^2) or 1/(pi h^3).
__device__ __forceinline__ float kernel_w(const DevParams &p, float q)
{
    if (p.kernel == CMAG_KERNEL_WENDLAND) {
        float t = __fmaf_rn(q, -0.5f, 1.0f);  // = 1 - q/2 (q/2 is exact)
        float t2 = t * t;
        return p.w_norm * (t2 * t2) * __fmaf_rn(q, 2.0f, 1.0f);
    }
    if (q < 1.0f) return p.w_norm * (1.0f - 1.5f * q * q + 0.75f * q * q * q);
    float t = 2.0f - q;
    return p.w_norm * 0.25f * t * t * t;
}

// dW/dr for q < 2.  Wendland: the reference's dw_norm (-(1-q/2)^3 (2q+1) + (1-q/2)^4)
// with dw_norm = 7/(2 pi h^3) (fluid_kernel.cu:222-224) simplifies to
// -2.5 dw_norm q (1-q/2)^3.  Cubic spline: dw_norm = w_norm / h.
__device__ __forceinline__ float kernel_dw(const DevParams &p, float q)
{
    if (p.kernel == CMAG_KERNEL_WENDLAND) {
        float t = __fmaf_rn(q, -0.5f, 1.0f);
        return -2.5f * p.dw_norm * q * (t * t * t);
    }
    if (q < 1.0f) return p.dw_norm * (-3.0f * q + 2.25f * q * q);
    float t = 2.0f - q;
    return p.dw_norm * (-0.75f * t * t);
}

// dW/dr / r at distance r (inv_r = 1 / r, 0 < r < 2h).  Wendland: since q / r =
// 1 / h, -2.5 dw_norm q (1-q/2)^3 / r = dwr_norm (1-q/2)^3 with dwr_norm =
// -2.5 dw_norm / h, and 1 - q/2 = fma(r, -1/(2h), 1).
__device__ __forceinline__ float kernel_dw_over_r(const DevParams &p, float r, float inv_r)
{
    if (p.kernel == CMAG_KERNEL_WENDLAND) {
        const float t = __fmaf_rn(r, p.nhalf_inv_h, 1.0f);
        return p.dwr_norm * (t * t * t);
    }
    return kernel_dw(p, r * p.inv_h) * inv_r;
}

// Equation of state (fluid_kernel.cu:168, poiseuilleFlowKernel.cu:181,
// PeristalsisDensity.cu:75).
__device__ __forceinline__ float eos_pressure(const DevParams &p, float rho)
{
    if (p.eos == CMAG_EOS_TAIT || p.system == CMAG_DAMBREAK) {
        float x = rho / p.rho0;
        float xg;
        if (p.gamma == 7.0f) {
            float x2 = x * x;
            xg = x2 * x2 * x2 * x;
        } else {
            xg = powf(x, p.gamma);
        }
        return p.B * (xg - 1.0f);
    }
    if (p.system == CMAG_POISEUILLE) return (p.c0 * p.c0) * rho;
    return 50.0f * p.c0 * rho;
}

// Programmatic dependent launch (kernels of the per-step chain, launched with
// launch_pdl): let the next kernel on the stream begin launching, then wait until
// the previous kernel has completed and its writes are visible.  The first
// statement of such a kernel, before any memory access, so every kernel body still
// runs after its predecessor; only launch and block scheduling overlap.  A no-op
// for a kernel launched without the attribute.
__device__ __forceinline__ void pdl_entry()
{
    asm volatile("griddepcontrol.launch_dependents;\n\tgriddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void set_error(uint32_t *err, uint32_t bits)
{
    if (err) atomicOr(err, bits);
}

}  // namespace cmag
