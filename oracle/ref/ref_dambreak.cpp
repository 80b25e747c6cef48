/*
 * ref_dambreak.cpp -- runs DamBreak.Core/fluid_kernel.cu (the reference's own
 * kernels, compiled for the CPU) in the order of DamBreakSystem::update,
 * DamBreak.Core/fluidSystem.cpp:257-319.  TEST INFRASTRUCTURE ONLY.
 */
#include "fluid_kernel.cu"
#include "ref_launch.h"

unsigned int sharedHash[1024]; /* backs `extern __shared__ uint sharedHash[]` */

extern "C" {

/* setParameters (fluidSystem.cu:17-19): fill the reference's __constant__ block */
void ref_db_set_params(const cmag_sph_params *p)
{
    SimParams s;
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
    s.B = p->B;
    s.deltaTime = p->delta_time;
    s.gamma = p->gamma;
    s.boundaryDamping = p->boundary_damping;
    s.boundaryOffset = p->boundary_offset;
    s.rightBoundary = p->right_boundary;
    s.D = p->lj_D;
    s.a = p->lj_a;
    params = s;
}

void ref_db_calc_hash(float *pos, unsigned *hash, unsigned *idx, unsigned n)
{
    cmref_launch(n, 256, [&] { calcHashD(hash, idx, (float4 *)pos, n); });
}

void ref_db_sort(unsigned *hash, unsigned *idx, unsigned n) { cmref_sort(hash, idx, n); }

void ref_db_reorder(unsigned *cs, unsigned *ce, float *spos, float *svel, unsigned *hash,
                    unsigned *idx, float *pos, float *vel, unsigned n, unsigned ncells)
{
    std::memset(cs, 0xff, sizeof(unsigned) * ncells);
    cmref_launch(n, 256, [&] {
        reorderDataAndFindCellStartD(cs, ce, (float4 *)spos, (float4 *)svel, hash, idx,
                                     (float4 *)pos, (float4 *)vel, n);
    });
}

void ref_db_density(float *meas, float *spos, float *svel, unsigned *idx, unsigned *cs,
                    unsigned *ce, unsigned n)
{
    cmref_launch(n, 64, [&] {
        calculateDamBreakDensityD((float4 *)meas, (float4 *)meas, (float4 *)spos,
                                  (float4 *)svel, idx, cs, ce, n);
    });
}

void ref_db_force(float *acc, float *meas, float *spos, float *svel, unsigned *idx, unsigned *cs,
                  unsigned *ce, unsigned n)
{
    cmref_launch(n, 64, [&] {
        calcAndApplyAccelerationD((float4 *)acc, (float4 *)meas, (float4 *)spos, (float4 *)svel,
                                  idx, cs, ce, n);
    });
}

void ref_db_integrate(float *pos, float *vel, float *vlf, float *acc, unsigned n)
{
    cmref_launch(n, 256, [&] {
        integrate((float4 *)pos, (float4 *)vel, (float4 *)vlf, (float4 *)acc, n);
    });
}

void ref_db_shift_right_boundary(float *pos, unsigned n)
{
    cmref_launch(n, 256, [&] { shiftRightBoundaryD((float4 *)pos, n); });
}

void ref_db_remove_right_boundary(float *pos, unsigned n)
{
    cmref_launch(n, 256, [&] { removeRightBoundaryD((float4 *)pos, n); });
}

} /* extern "C" */
