/*
 * ref_gpu_launch.cu -- headless GPU launcher of the reference's own DamBreak
 * kernels (the cubin oracle/ref/Makefile builds from DamBreak.Core/fluid_kernel.cu
 * with ref_gpu_kernels.cu), to time the reference on the GB300 beside this
 * library.  TEST INFRASTRUCTURE ONLY: the reference's host classes need GL/GLUT
 * and cutil, so this replays DamBreakSystem::update (fluidSystem.cpp:257-319)
 * with the reference's launch shapes (fluidSystem.cu): calcHashD with 256
 * threads, thrust::sort_by_key on the (hash, index) pairs (fluidSystem.cu:94-99),
 * a cudaMemset of cellStart over the whole grid and reorderDataAndFindCellStartD
 * with (threads + 1) words of shared memory, the density and force kernels with
 * 64 threads, integrate with 256; all on the legacy default stream as the
 * reference.  The parameter block is copied into the kernels' __constant__ bank
 * once per step, as setParameters does (a device-to-device copy here).
 */
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/sort.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/cmag_sph.h"

namespace {

struct RefGpu {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t k_stage = nullptr, k_hash = nullptr, k_reorder = nullptr, k_density = nullptr, k_force = nullptr,
                 k_integrate = nullptr, k_remove = nullptr;
    void *d_params = nullptr, *d_stage = nullptr;
    size_t params_bytes = 0;
    uint32_t n = 0;
    uint64_t ncells = 0;
    float4 *pos = nullptr, *vel = nullptr, *vlf = nullptr, *acc = nullptr, *meas = nullptr, *spos = nullptr,
           *svel = nullptr;
    uint32_t *hash = nullptr, *idx = nullptr, *cs = nullptr, *ce = nullptr;
    cudaEvent_t ev[8] = {};
};

thread_local std::string g_err;

int fail(const char *what, cudaError_t e)
{
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    (void)cudaGetLastError();
    return 2;
}

#define RG(call)                                  \
    do {                                          \
        cudaError_t e_ = (call);                  \
        if (e_ != cudaSuccess) return fail(#call, e_); \
    } while (0)

// computeGridSize (fluidSystem.cu:25-28)
void grid_of(uint32_t n, uint32_t block, uint32_t &blocks, uint32_t &threads)
{
    threads = n < block ? n : block;
    blocks = (n + threads - 1) / threads;
}

cudaError_t launch(cudaKernel_t k, uint32_t n, uint32_t block, size_t smem, void **args, bool with_smem_halo = false)
{
    uint32_t blocks, threads;
    grid_of(n, block, blocks, threads);
    if (with_smem_halo) smem = sizeof(uint32_t) * (threads + 1);
    return cudaLaunchKernel((const void *)k, dim3(blocks), dim3(threads), args, smem, 0);
}

// one update() of the reference (fluidSystem.cpp:257-319); ev: 8 events or null
int step(RefGpu *r, bool timed)
{
    uint32_t n = r->n;
    if (timed) RG(cudaEventRecord(r->ev[0], 0));
    RG(cudaMemcpyAsync(r->d_params, r->d_stage, r->params_bytes, cudaMemcpyDeviceToDevice, 0));  // setParameters
    void *a_hash[] = {&r->hash, &r->idx, &r->pos, &n};
    RG(launch(r->k_hash, n, 256, 0, a_hash));
    if (timed) RG(cudaEventRecord(r->ev[1], 0));
    thrust::sort_by_key(thrust::device_ptr<uint32_t>(r->hash), thrust::device_ptr<uint32_t>(r->hash + n),
                        thrust::device_ptr<uint32_t>(r->idx));
    if (timed) RG(cudaEventRecord(r->ev[2], 0));
    RG(cudaMemsetAsync(r->cs, 0xff, sizeof(uint32_t) * r->ncells, 0));
    void *a_reorder[] = {&r->cs, &r->ce, &r->spos, &r->svel, &r->hash, &r->idx, &r->pos, &r->vlf, &n};
    RG(launch(r->k_reorder, n, 256, 0, a_reorder, true));
    if (timed) RG(cudaEventRecord(r->ev[3], 0));
    void *a_density[] = {&r->meas, &r->meas, &r->spos, &r->svel, &r->idx, &r->cs, &r->ce, &n};
    RG(launch(r->k_density, n, 64, 0, a_density));
    if (timed) RG(cudaEventRecord(r->ev[4], 0));
    void *a_force[] = {&r->acc, &r->meas, &r->spos, &r->svel, &r->idx, &r->cs, &r->ce, &n};
    RG(launch(r->k_force, n, 64, 0, a_force));
    if (timed) RG(cudaEventRecord(r->ev[5], 0));
    void *a_int[] = {&r->pos, &r->vel, &r->vlf, &r->acc, &n};
    RG(launch(r->k_integrate, n, 256, 0, a_int));
    if (timed) RG(cudaEventRecord(r->ev[6], 0));
    RG(cudaGetLastError());
    return 0;
}

float4 *array_of(RefGpu *r, int a)
{
    switch (a) {
    case CMAG_POSITION: return r->pos;
    case CMAG_VELOCITY: return r->vel;
    case CMAG_VELOCITYLEAPFROG: return r->vlf;
    case CMAG_ACCELERATION: return r->acc;
    case CMAG_MEASURES: return r->meas;
    case CMAG_SORTEDPOSITION: return r->spos;
    default: return nullptr;
    }
}

void release(RefGpu *r)
{
    void *ptrs[] = {r->pos, r->vel, r->vlf, r->acc, r->meas, r->spos, r->svel, r->hash, r->idx, r->cs, r->ce};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &e : r->ev)
        if (e) cudaEventDestroy(e);
    if (r->lib) cudaLibraryUnload(r->lib);
}

}  // namespace

extern "C" {

const char *ref_gpu_error(void) { return g_err.c_str(); }

/* Load the reference kernels from `cubin`, allocate an instance of n particles on
 * the current device with positions pos (n x 4 floats; velocities zero, density
 * rest density as DamBreakSystem::_initialize sets it, fluidSystem.cpp:131-132)
 * and parameters p (grid sizes powers of two: the reference masks the hash). */
int ref_gpu_create(const char *cubin, const cmag_sph_params *p, uint32_t n, const float *pos, void **out)
{
    if (!cubin || !p || !pos || !out || n == 0) {
        g_err = "null argument";
        return 1;
    }
    RefGpu *r = new RefGpu;
    auto bail = [&](int rc) {
        release(r);
        delete r;
        return rc;
    };
    cudaError_t e = cudaLibraryLoadFromFile(&r->lib, cubin, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) return bail(fail("cudaLibraryLoadFromFile", e));
    struct {
        cudaKernel_t *k;
        const char *name;
    } ks[] = {{&r->k_stage, "ref_stage_params"},
              {&r->k_hash, "ref_calcHashD"},
              {&r->k_reorder, "ref_reorderDataAndFindCellStartD"},
              {&r->k_density, "ref_calculateDamBreakDensityD"},
              {&r->k_force, "ref_calcAndApplyAccelerationD"},
              {&r->k_integrate, "ref_integrate"},
              {&r->k_remove, "ref_removeRightBoundaryD"}};
    for (auto &k : ks)
        if ((e = cudaLibraryGetKernel(k.k, r->lib, k.name)) != cudaSuccess) return bail(fail(k.name, e));
    size_t stage_bytes = 0;
    if ((e = cudaLibraryGetGlobal(&r->d_params, &r->params_bytes, r->lib, "params")) != cudaSuccess)
        return bail(fail("params", e));
    if ((e = cudaLibraryGetGlobal(&r->d_stage, &stage_bytes, r->lib, "ref_params_stage")) != cudaSuccess)
        return bail(fail("ref_params_stage", e));
    if (stage_bytes != r->params_bytes) {
        g_err = "parameter block sizes differ";
        return bail(1);
    }
    r->n = n;
    r->ncells = (uint64_t)p->grid_size[0] * p->grid_size[1] * p->grid_size[2];
    float4 **f4[] = {&r->pos, &r->vel, &r->vlf, &r->acc, &r->meas, &r->spos, &r->svel};
    for (auto a : f4) {
        if ((e = cudaMalloc((void **)a, sizeof(float4) * (size_t)n)) != cudaSuccess) return bail(fail("cudaMalloc", e));
        cudaMemset(*a, 0, sizeof(float4) * (size_t)n);
    }
    uint32_t **u[] = {&r->hash, &r->idx};
    for (auto a : u)
        if ((e = cudaMalloc((void **)a, sizeof(uint32_t) * (size_t)n)) != cudaSuccess) return bail(fail("cudaMalloc", e));
    if ((e = cudaMalloc((void **)&r->cs, sizeof(uint32_t) * r->ncells)) != cudaSuccess ||
        (e = cudaMalloc((void **)&r->ce, sizeof(uint32_t) * r->ncells)) != cudaSuccess)
        return bail(fail("cudaMalloc(cells)", e));
    for (auto &ev : r->ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return bail(fail("cudaEventCreate", e));
    if ((e = cudaMemcpy(r->pos, pos, sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(fail("cudaMemcpy(pos)", e));
    {
        // density starts at rest density (fluidSystem.cpp:131-132)
        float4 *m = new float4[n];
        for (uint32_t i = 0; i < n; ++i) m[i] = make_float4(p->rest_density, 0.0f, 0.0f, 0.0f);
        e = cudaMemcpy(r->meas, m, sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice);
        delete[] m;
        if (e != cudaSuccess) return bail(fail("cudaMemcpy(meas)", e));
    }
    cmag_sph_params pp = *p;
    void *args[] = {&pp};
    if ((e = cudaLaunchKernel((const void *)r->k_stage, dim3(1), dim3(1), args, 0, 0)) != cudaSuccess)
        return bail(fail("ref_stage_params", e));
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return bail(fail("stage", e));
    *out = r;
    return 0;
}

/* removeRightBoundary (fluidSystem.cpp:222-255): release the dam */
int ref_gpu_remove_right_boundary(void *h, const cmag_sph_params *p)
{
    RefGpu *r = static_cast<RefGpu *>(h);
    cmag_sph_params pp = *p;
    void *args[] = {&pp};
    RG(cudaLaunchKernel((const void *)r->k_stage, dim3(1), dim3(1), args, 0, 0));
    RG(cudaMemcpy(r->d_params, r->d_stage, r->params_bytes, cudaMemcpyDeviceToDevice));
    uint32_t n = r->n;
    void *a[] = {&r->pos, &n};
    RG(launch(r->k_remove, n, 256, 0, a));
    RG(cudaDeviceSynchronize());
    return 0;
}

/* `steps` updates; with ms_total, the device time between events around them and
 * per stage (ms_stage[6]: hash, sort, reorder with the cellStart clear, density,
 * force, integrate; summed over the steps) */
int ref_gpu_steps(void *h, uint32_t steps, float *ms_total, float *ms_stage)
{
    RefGpu *r = static_cast<RefGpu *>(h);
    if (ms_stage)
        for (int k = 0; k < 6; ++k) ms_stage[k] = 0.0f;
    cudaEvent_t a = r->ev[7];
    if (ms_total && !ms_stage) RG(cudaEventRecord(a, 0));
    for (uint32_t s = 0; s < steps; ++s) {
        if (int rc = step(r, ms_stage != nullptr)) return rc;
        if (ms_stage) {
            RG(cudaEventSynchronize(r->ev[6]));
            for (int k = 0; k < 6; ++k) {
                float ms = 0.0f;
                RG(cudaEventElapsedTime(&ms, r->ev[k], r->ev[k + 1]));
                ms_stage[k] += ms;
            }
        }
    }
    if (ms_total && !ms_stage) {
        RG(cudaEventRecord(r->ev[6], 0));
        RG(cudaEventSynchronize(r->ev[6]));
        RG(cudaEventElapsedTime(ms_total, a, r->ev[6]));
    }
    RG(cudaDeviceSynchronize());
    return 0;
}

/* float4 array (POSITION, VELOCITY, VELOCITYLEAPFROG, ACCELERATION, MEASURES,
 * SORTEDPOSITION) to the host, n x 4 floats */
int ref_gpu_get(void *h, int32_t array, float *host)
{
    RefGpu *r = static_cast<RefGpu *>(h);
    float4 *d = array_of(r, array);
    if (!d || !host) {
        g_err = "unknown array";
        return 1;
    }
    RG(cudaMemcpy(host, d, sizeof(float4) * (size_t)r->n, cudaMemcpyDeviceToHost));
    return 0;
}

/* set a float4 array (POSITION, VELOCITY, VELOCITYLEAPFROG, MEASURES) from the host */
int ref_gpu_set(void *h, int32_t array, const float *host)
{
    RefGpu *r = static_cast<RefGpu *>(h);
    float4 *d = array_of(r, array);
    if (!d || !host || array == CMAG_SORTEDPOSITION) {
        g_err = "unknown array";
        return 1;
    }
    RG(cudaMemcpy(d, host, sizeof(float4) * (size_t)r->n, cudaMemcpyHostToDevice));
    return 0;
}

int ref_gpu_get_index(void *h, uint32_t *host)
{
    RefGpu *r = static_cast<RefGpu *>(h);
    RG(cudaMemcpy(host, r->idx, sizeof(uint32_t) * (size_t)r->n, cudaMemcpyDeviceToHost));
    return 0;
}

int ref_gpu_destroy(void *h)
{
    RefGpu *r = static_cast<RefGpu *>(h);
    if (!r) return 0;
    cudaDeviceSynchronize();
    release(r);
    delete r;
    return 0;
}

} /* extern "C" */
