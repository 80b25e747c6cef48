/*
 * ref_peristalsis.cpp -- runs the reference's Peristalsis kernels
 * (Peristalsis.Core/Peristalsis{Kernel,Density,PressureForce,ViscousForce,
 * Integrate}.cu, compiled for the CPU) in the order of PeristalsisSystem::Update,
 * Peristalsis.Core/PeristalsisSystem.cpp:320-407.  TEST INFRASTRUCTURE ONLY.
 *
 * PeristalsisDensity.cu:51 reads FETCH(oldVel, index) although oldVel is not a
 * parameter of that kernel (it only compiled with texture references, where it
 * named a global texture); the value is unused.  A file-scope pointer of that
 * name is declared here and aimed at a valid buffer before each density launch.
 */
#include "ref_launch_pre.h"
static float4 *oldVel = nullptr;
#include "PeristalsisKernel.cu"
#include "PeristalsisDensity.cu"
#include "PeristalsisPressureForce.cu"
#include "PeristalsisViscousForce.cu"
#include "PeristalsisIntegrate.cu"
#include "ref_launch.h"

unsigned int sharedHash[1024]; /* backs `extern __shared__ uint sharedHash[]` */

extern "C" {

/* setParameters (PeristalsisSystem.cu:21-23) */
void ref_ps_set_params(const cmag_sph_params *p)
{
    Peristalsiscfg s;
    std::memset(&s, 0, sizeof(s));
    s.gridSize = cmref_u3(p->grid_size);
    s.worldOrigin = cmref_f3(p->world_origin);
    s.cellSize = cmref_f3(p->cell_size);
    s.worldSize = cmref_f3(p->world_size);
    s.fluid_size = cmref_u3(p->fluid_size);
    s.cellcount = p->cell_count;
    s.gravity = cmref_f3(p->gravity);
    s.radius = p->particle_radius;
    s.smoothingRadius = p->smoothing_radius;
    s.particleMass = p->particle_mass;
    s.restDensity = p->rest_density;
    s.soundspeed = p->soundspeed;
    s.deltaTime = p->delta_time;
    s.boundaryDamping = p->boundary_damping;
    s.mu = p->mu;
    s.boundaryOffset = p->boundary_offset;
    s.amplitude = p->amplitude;
    s.wave_speed = p->wave_speed;
    s.IsBoundaryConfiguration = p->is_boundary_configuration != 0;
    s.B = p->B;
    s.gamma = p->gamma;
    cfg = s;
}

void ref_ps_calc_hash(float *pos, unsigned *hash, unsigned *idx, unsigned n)
{
    cmref_launch(n, 256, [&] { calculatePeristalsisHashD(hash, idx, (float4 *)pos, n); });
}

void ref_ps_sort(unsigned *hash, unsigned *idx, unsigned n) { cmref_sort(hash, idx, n); }

void ref_ps_reorder(unsigned *cs, unsigned *ce, float *spos, float *svel, unsigned *hash,
                    unsigned *idx, float *pos, float *vel, unsigned n, unsigned ncells)
{
    std::memset(cs, 0xff, sizeof(unsigned) * ncells);
    cmref_launch(n, 256, [&] {
        reorderPeristalsisDataD(cs, ce, (float4 *)spos, (float4 *)svel, hash, idx, (float4 *)pos,
                                (float4 *)vel, n);
    });
}

void ref_ps_density(float *meas, float *spos, float *svel, unsigned *idx, unsigned *cs,
                    unsigned *ce, unsigned n)
{
    oldVel = (float4 *)svel;
    cmref_launch(n, 64, [&] {
        computeDensityVariationD((float4 *)meas, (float4 *)meas, (float4 *)spos, idx, cs, ce, n);
    });
}

void ref_ps_force(float *vforce, float *pforce, float *meas, float *spos, float *svel,
                  unsigned *idx, unsigned *cs, unsigned *ce, unsigned n, float t)
{
    cmref_launch(n, 64, [&] {
        computeViscousForceD((float4 *)vforce, (float4 *)meas, (float4 *)spos, (float4 *)svel, idx,
                             cs, ce, n, t);
    });
    cmref_launch(n, 64, [&] {
        computePressureForceD((float4 *)pforce, (float4 *)meas, (float4 *)spos, idx, cs, ce, n, t);
    });
}

void ref_ps_integrate(float *pos, float *vel, float *vlf, float *vforce, float *pforce, float t,
                      unsigned n)
{
    cmref_launch(n, 256, [&] {
        computeCoordinatesD((float4 *)pos, (float4 *)vel, (float4 *)vlf, (float4 *)vforce,
                            (float4 *)pforce, t, n);
    });
}

void ref_ps_configure_boundary(float *pos, float wave_height, unsigned n)
{
    cmref_launch(n, 256, [&] { configureBoundaryD((float4 *)pos, wave_height, n); });
}

} /* extern "C" */
