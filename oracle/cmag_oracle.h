/*
 * cmag_oracle.h -- CPU restatement of cmag's WCSPH time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path: the
 * tests, the smoke check and the CPU baseline leg of the benchmark call it; the
 * product never links or loads it.
 *
 * It restates, in the reference's own floating-point evaluation order, the CUDA
 * kernels of the three reference solvers, their host-side parameter derivations,
 * scene generators and update() orchestration:
 *
 *   DamBreak.Core/fluid_kernel.cu:19-366, fluidSystem.cpp:17-523
 *   Poiseuille.Core/poiseuilleFlowKernel.cu:18-348, poiseuilleFlowSystem.cpp:21-383
 *   Peristalsis.Core/Peristalsis{Kernel,Density,PressureForce,ViscousForce,
 *                    Integrate,Util}.cu, PeristalsisSystem.cpp:17-407
 *
 * plus the documented extensions (3-D normalisation, cubic spline kernel, Tait
 * EOS for every family, parameterised artificial viscosity, wall-force cut-off,
 * several wavelengths per domain, the 3-D dam-break scene).
 *
 * Arrays are float4 AoS as in the reference (4 floats per particle).
 * Neighbour loops visit the (2c+1)^3 cell box cell by cell, as the reference.
 */
#ifndef CMAG_ORACLE_H
#define CMAG_ORACLE_H

#include <stdint.h>
#include "../include/cmag_sph.h"

#ifdef __cplusplus
extern "C" {
#endif

/* reference constructors */
int orc_dambreak_params(const uint32_t fs[3], int32_t off, const uint32_t gs[3], float r,
                        cmag_sph_params *p);
int orc_poiseuille_params(const uint32_t fs[3], int32_t off, const uint32_t gs[3], float r,
                          cmag_sph_params *p);
int orc_peristalsis_params(float dt, const uint32_t fs[3], float amplitude, float wave_speed,
                           float soundspeed, const float g[3], int32_t off,
                           const uint32_t gs[3], float r, cmag_sph_params *p);
uint32_t orc_particle_count(const cmag_sph_params *p);

/* reference scene generators (reset) */
void orc_scene(const cmag_sph_params *p, float *pos, uint32_t n);
float orc_peristalsis_mass_sum(const cmag_sph_params *p, const float *pos, uint32_t n);

/* 3-D dam-break scene (extension) */
uint32_t orc_dambreak3d_count(const uint32_t fs[3], const uint32_t tank[3], uint32_t layers);
void orc_dambreak3d_scene(const cmag_sph_params *p, const uint32_t tank[3], uint32_t layers,
                          float jitter_frac, uint64_t seed, float *pos, uint32_t n);

/* stages */
void orc_calc_hash(const cmag_sph_params *p, const float *pos, uint32_t *hash, uint32_t *idx,
                   uint32_t n);
void orc_sort_pairs(uint32_t *hash, uint32_t *idx, uint32_t n);
void orc_reorder(const uint32_t *hash, const uint32_t *idx, const float *pos, const float *vel,
                 uint32_t *cell_start, uint32_t *cell_end, float *spos, float *svel, uint32_t n,
                 uint64_t ncells);
void orc_density(const cmag_sph_params *p, const float *spos, float *meas,
                 const uint32_t *cell_start, const uint32_t *cell_end, uint32_t n, int threads);
/* DamBreak/Poiseuille: out_a = acceleration.  Peristalsis: out_a = viscous force,
 * out_b = pressure force.  Outputs are scattered to original order. */
void orc_force(const cmag_sph_params *p, const float *spos, const float *svel, const float *meas,
               const uint32_t *idx, const uint32_t *cell_start, const uint32_t *cell_end,
               float *out_a, float *out_b, uint32_t n, int threads);
/* Per particle (original order), the component-wise sum of |pair term| of the
 * force: the magnitude that bounds the rounding error of any summation order. */
void orc_force_scale(const cmag_sph_params *p, const float *spos, const float *svel,
                     const float *meas, const uint32_t *idx, const uint32_t *cell_start,
                     const uint32_t *cell_end, float *scale_a, float *scale_b, uint32_t n,
                     int threads);
/* Peristalsis with wall_noslip: the wall state the force uses (interface
 * amplitude, time of the wall law, whether the walls move) */
void orc_set_wall_state(float amp, float t, int32_t moving);
/* single-particle evaluations on given sorted arrays (spot checks at full size) */
float orc_density_at(const cmag_sph_params *p, const float *spos, const uint32_t *cell_start,
                     const uint32_t *cell_end, uint32_t i);
void orc_force_at(const cmag_sph_params *p, const float *spos, const float *svel,
                  const float *meas, const uint32_t *cell_start, const uint32_t *cell_end,
                  uint32_t i, float out_a[3], float out_b[3], int32_t *written);
void orc_integrate(const cmag_sph_params *p, float *pos, float *vel, float *vlf, const float *acc,
                   const float *vforce, const float *pforce, float t, uint32_t n);
void orc_configure_boundary(const cmag_sph_params *p, float *pos, float wave_height, uint32_t n);
void orc_shift_right_boundary(const cmag_sph_params *p, float *pos, uint32_t n);
void orc_remove_right_boundary(cmag_sph_params *p, float *pos, uint32_t n);

/* Whole update() of one step.  phase[5] = {elapsed, time_shift, time_relax,
 * current_wave_height, t} (only elapsed is used outside Peristalsis; t is an
 * output: the time the integration of this step used); p may be
 * modified (Peristalsis boundary-configuration flag).  stop_after: enum
 * cmag_stage, stages after it are skipped and time is not advanced unless the
 * whole step runs. */
void orc_step(cmag_sph_params *p, uint32_t n, uint64_t ncells, float *pos, float *vel, float *vlf,
              float *meas, float *acc, float *vforce, float *pforce, float *spos, float *svel,
              uint32_t *hash, uint32_t *idx, uint32_t *cell_start, uint32_t *cell_end,
              float phase[5], int threads, int stop_after);

#ifdef __cplusplus
}
#endif
#endif
