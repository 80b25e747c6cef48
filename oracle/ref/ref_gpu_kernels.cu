/*
 * ref_gpu_kernels.cu -- the reference's own DamBreak kernels
 * (DamBreak.Core/fluid_kernel.cu) built for the GB300, to time them beside this
 * library.  TEST INFRASTRUCTURE ONLY: compiled by oracle/ref/Makefile (target
 * gpu-cubin) from the reference sources where they lie, into a cubin under
 * oracle/_ref/; never part of the product.
 *
 * -D__DEVICE_EMULATION__ turns the reference's texture fetches into plain array
 * reads (fluid_kernel.cuh:4-12: FETCH(t, i) = t[i]), which give the same values
 * and compile with CUDA 13 (its texture references do not).  The reference
 * kernels become device functions behind extern "C" kernels of the same
 * signatures, so a host launcher can name them without the reference headers.
 * Their parameter block (the reference's __constant__ SimParams, set by
 * setParameters, fluidSystem.cu:17-19) is filled on the device from a
 * cmag_sph_params and copied into the constant bank by the launcher.
 */
#include "../../include/cmag_sph.h"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include "fluid_kernel.cu"
#pragma pop_macro("__global__")

/* the SimParams the launcher copies into `params` (fluid_kernel.cu:17) */
__device__ SimParams ref_params_stage;

extern "C" {

__global__ void ref_stage_params(cmag_sph_params p)
{
    SimParams s;
    s.gridSize = make_uint3(p.grid_size[0], p.grid_size[1], p.grid_size[2]);
    s.worldOrigin = make_float3(p.world_origin[0], p.world_origin[1], p.world_origin[2]);
    s.cellSize = make_float3(p.cell_size[0], p.cell_size[1], p.cell_size[2]);
    s.fluidParticlesSize = make_uint3(p.fluid_size[0], p.fluid_size[1], p.fluid_size[2]);
    s.cellcount = p.cell_count;
    s.gravity = make_float3(p.gravity[0], p.gravity[1], p.gravity[2]);
    s.particleRadius = p.particle_radius;
    s.smoothingRadius = p.smoothing_radius;
    s.particleMass = p.particle_mass;
    s.restDensity = p.rest_density;
    s.soundspeed = p.soundspeed;
    s.B = p.B;
    s.deltaTime = p.delta_time;
    s.gamma = p.gamma;
    s.boundaryDamping = p.boundary_damping;
    s.boundaryOffset = p.boundary_offset;
    s.rightBoundary = p.right_boundary;
    s.D = p.lj_D;
    s.a = p.lj_a;
    ref_params_stage = s;
}

__global__ void ref_calcHashD(uint *hash, uint *index, float4 *pos, uint n)
{
    calcHashD(hash, index, pos, n);
}

__global__ void ref_reorderDataAndFindCellStartD(uint *cellStart, uint *cellEnd, float4 *sortedPos,
                                                 float4 *sortedVel, uint *hash, uint *index, float4 *oldPos,
                                                 float4 *oldVel, uint n)
{
    reorderDataAndFindCellStartD(cellStart, cellEnd, sortedPos, sortedVel, hash, index, oldPos, oldVel, n);
}

__global__ void ref_calculateDamBreakDensityD(float4 *measuresOut, float4 *measuresIn, float4 *sortedPos,
                                              float4 *sortedVel, uint *index, uint *cellStart, uint *cellEnd,
                                              uint n)
{
    calculateDamBreakDensityD(measuresOut, measuresIn, sortedPos, sortedVel, index, cellStart, cellEnd, n);
}

__global__ void ref_calcAndApplyAccelerationD(float4 *acc, float4 *measures, float4 *sortedPos, float4 *sortedVel,
                                              uint *index, uint *cellStart, uint *cellEnd, uint n)
{
    calcAndApplyAccelerationD(acc, measures, sortedPos, sortedVel, index, cellStart, cellEnd, n);
}

__global__ void ref_integrate(float4 *pos, float4 *vel, float4 *velLeapFrog, float4 *acc, uint n)
{
    integrate(pos, vel, velLeapFrog, acc, n);
}

__global__ void ref_removeRightBoundaryD(float4 *pos, uint n) { removeRightBoundaryD(pos, n); }

} /* extern "C" */
