/*
 * ref_poiseuille.cpp -- runs Poiseuille.Core/poiseuilleFlowKernel.cu (the
 * reference's own kernels, compiled for the CPU) in the order of
 * PoiseuilleFlowSystem::update, Poiseuille.Core/poiseuilleFlowSystem.cpp:212-270.
 * TEST INFRASTRUCTURE ONLY.
 */
#include "poiseuilleFlowKernel.cu"
#include "ref_launch.h"

unsigned int sharedHash[1024]; /* backs `extern __shared__ uint sharedHash[]` */

extern "C" {

/* setParameters (poiseuilleFlowSystem.cu:19-21) */
void ref_pf_set_params(const cmag_sph_params *p)
{
    PoiseuilleParams s;
    std::memset(&s, 0, sizeof(s));
    s.gridSize = cmref_u3(p->grid_size);
    s.worldOrigin = cmref_f3(p->world_origin);
    s.cellSize = cmref_f3(p->cell_size);
    s.fluidParticlesSize = cmref_u3(p->fluid_size);
    s.cellcount = p->cell_count;
    s.gravity = cmref_f3(p->gravity);
    s.particleRadius = p->particle_radius;
    s.smoothingRadius = p->smoothing_radius;
    s.particleMass = p->particle_mass;
    s.restDensity = p->rest_density;
    s.soundspeed = p->soundspeed;
    s.deltaTime = p->delta_time;
    s.boundaryDamping = p->boundary_damping;
    s.mu = p->mu;
    s.boundaryOffset = p->boundary_offset;
    params = s;
}

void ref_pf_calc_hash(float *pos, unsigned *hash, unsigned *idx, unsigned n)
{
    cmref_launch(n, 256, [&] { calculatePoiseuilleHashD(hash, idx, (float4 *)pos, n); });
}

void ref_pf_sort(unsigned *hash, unsigned *idx, unsigned n) { cmref_sort(hash, idx, n); }

void ref_pf_reorder(unsigned *cs, unsigned *ce, float *spos, float *svel, unsigned *hash,
                    unsigned *idx, float *pos, float *vel, unsigned n, unsigned ncells)
{
    std::memset(cs, 0xff, sizeof(unsigned) * ncells);
    cmref_launch(n, 256, [&] {
        reorderPoiseuilleDataD(cs, ce, (float4 *)spos, (float4 *)svel, hash, idx, (float4 *)pos,
                               (float4 *)vel, n);
    });
}

void ref_pf_density(float *meas, float *spos, float *svel, unsigned *idx, unsigned *cs,
                    unsigned *ce, unsigned n)
{
    cmref_launch(n, 64, [&] {
        calculatePoiseuilleDensityD((float4 *)meas, (float4 *)spos, (float4 *)svel, idx, cs, ce, n);
    });
}

void ref_pf_force(float *acc, float *meas, float *spos, float *svel, unsigned *idx, unsigned *cs,
                  unsigned *ce, unsigned n)
{
    cmref_launch(n, 64, [&] {
        calculatePoiseuilleAccelerationD((float4 *)acc, (float4 *)meas, (float4 *)spos,
                                         (float4 *)svel, idx, cs, ce, n);
    });
}

void ref_pf_integrate(float *pos, float *vel, float *vlf, float *acc, unsigned n)
{
    cmref_launch(n, 256, [&] {
        integratePoiseuilleSystemD((float4 *)pos, (float4 *)vel, (float4 *)vlf, (float4 *)acc, n);
    });
}

} /* extern "C" */
