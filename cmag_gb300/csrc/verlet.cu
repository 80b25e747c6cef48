// verlet.cu -- neighbour lists kept over several steps: the per-step gather in
// the rebuild's order and the device-side choice between a rebuild step and a
// step on the kept lists.
//
// The reference sorts, reorders and walks the 7^3 neighbour cells of every
// particle on every step (fluidSystem.cpp:257-319: calcHash, sortParticles,
// reorderDataAndFindCellStart, density, force).  With kept lists the hash, sort
// and cell walk run only on rebuild steps; every other step gathers the current
// positions and leap-frog velocities in the rebuild's order and runs the
// neighbour loops from the lists, which hold every particle within 2h + skin at
// the rebuild.  Integration flags the next rebuild as soon as a particle is more
// than skin/2 from where the lists were built, so every pair within 2h is always
// in the lists.
#include <cuda_runtime.h>

#include "kernels.h"

namespace cmag {

namespace {

__global__ void __launch_bounds__(256)
    k_gather_sorted(const uint32_t *__restrict__ idx, const float4 *__restrict__ pos,
                    const float4 *__restrict__ vlf, uint32_t n, float4 *__restrict__ spos,
                    float4 *__restrict__ svel)
{
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = idx[i];
    if (o >= n) return;  // only after a failed sort (reported by the sort)
    spos[i] = pos[o];
    svel[i] = vlf[o];
}

__global__ void k_verlet_decide(VerletFlags *f, cudaGraphConditionalHandle cond, int use_cond)
{
    pdl_entry();
    if (threadIdx.x != 0) return;
    const uint32_t rebuild = (f->moved | f->overflow) ? 1u : 0u;
    f->moved = 0u;
    if (rebuild) {
        f->overflow = 0u;  // the rebuild's density pass sets it again if needed
        f->rebuilds += 1u;
    }
    f->decision = rebuild;
    if (use_cond) cudaGraphSetConditional(cond, rebuild);
}

// Positions set from the host: flag a rebuild when one of them lies more than
// skin/2 from where the lists were built.
__global__ void __launch_bounds__(256)
    k_verlet_check(const float4 *__restrict__ pos, const float4 *__restrict__ xb, uint32_t start,
                   uint32_t count, float move2, uint32_t *moved)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const float4 q = pos[start + k], b = xb[start + k];
    const float dx = q.x - b.x, dy = q.y - b.y, dz = q.z - b.z;
    if (!(dx * dx + dy * dy + dz * dz <= move2)) *moved = 1u;
}

}  // namespace

void launch_verlet_check(const float4 *pos, const float4 *xb, uint32_t start, uint32_t count, float move2,
                         uint32_t *moved, cudaStream_t st)
{
    if (count == 0) return;
    k_verlet_check<<<(count + 255) / 256, 256, 0, st>>>(pos, xb, start, count, move2, moved);
}

void launch_gather_sorted(const uint32_t *idx, const float4 *pos, const float4 *vlf, uint32_t n,
                          float4 *spos, float4 *svel, cudaStream_t st)
{
    if (n == 0) return;
    launch_pdl(k_gather_sorted, (n + 255) / 256, 256, 0, st, idx, pos, vlf, n, spos, svel);
}

void launch_verlet_decide(VerletFlags *flags, unsigned long long cond, int use_cond, cudaStream_t st)
{
    launch_pdl(k_verlet_decide, 1, 32, 0, st, flags, (cudaGraphConditionalHandle)cond, use_cond);
}

}  // namespace cmag
