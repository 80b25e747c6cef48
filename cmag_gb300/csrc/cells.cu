// cells.cu -- grid hash, per-cell counts and dense cell offsets, the per-step
// counting sort with the sorted gather.
//
// The reference finds cell ranges after the sort: it clears cellStart for the
// whole grid (cudaMemset, fluidSystem.cu:161) and writes cellStart/cellEnd where
// the sorted hash changes (reorderDataAndFindCellStartD, fluid_kernel.cu:50-97).
// Here the hash kernel also counts particles per cell (one atomic increment per
// particle, whose return value is the particle's arrival rank in its cell), and
// one chained-scan pass turns the counts into a dense offset table
//     off[c] = number of particles with hash < c,   c = 0 .. scan_cells,
// so the particles of any run of consecutive cells [a, b] are the sorted range
// [off[a], off[b+1]).  A row of neighbour cells costs two loads instead of one
// or two per cell, and no full-grid clear is needed: the scan re-zeroes exactly
// the counters it consumed.  The reference's cellStart/cellEnd arrays are
// derived from the table on request (launch_cell_view).
//
// The table also sorts the particles (sortParticles, fluidSystem.cu:94-99): each
// particle goes to off[cell] + rank, and a second pass orders every cell's few
// entries by original index, which is the order of a stable sort by hash.
#include <cuda_runtime.h>

#include "kernels.h"

namespace cmag {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

// calcHashD (fluid_kernel.cu:34-48) + per-cell counts, one particle per thread.
// The sort key is the reference hash for a single scene; in a batch it is the
// particle's cell index in the shared offset table (scene table base + cell), so
// the sort orders by scene, then by cell.  A particle whose cell lies outside
// its offset table (a planar scene's particle that left its z layer) is counted
// in the table's last cell and reported as CMAG_DEVERR_RANGE.  rank[i] (when
// given) is the count the particle's atomic increment found: its arrival order
// among the particles of its cell.
//
// ph_all (one PhaseState per scene, or null): a Peristalsis wall particle is
// first placed on its wall when the step configures the boundary (the
// configureBoundaryD pass fused into the hash: the same arithmetic, one read of
// the positions instead of two).
template <bool BATCH>
__global__ void __launch_bounds__(256)
    k_hash(DevParams pv, BatchView bv, float4 *__restrict__ pos, uint32_t *__restrict__ hash,
           uint32_t *__restrict__ cnt, uint32_t *__restrict__ rank, uint32_t *err,
           float4 *__restrict__ snap, const PhaseState *__restrict__ ph_all)
{
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (BATCH ? bv.n_total : pv.n)) return;
    const DevParams &p = BATCH ? bv.scenes[bv.scene_of[i]] : pv;
    float4 q = pos[i];
    if (ph_all && p.system == CMAG_PERISTALSIS) {
        const PhaseState *ph = ph_all + (BATCH ? bv.scene_of[i] : 0u);
        if (ph->configure && configure_wall(p, ph->configure_height, q)) pos[i] = q;
    }
    if (snap) snap[i] = q;  // positions the kept lists are built from
    const int3 g = grid_pos(p, q.x, q.y, q.z);
    const uint32_t hr = grid_hash(p, g.x, g.y, g.z);
    uint32_t rel = hr - p.scan_base;  // wraps for hr < scan_base
    if (rel >= p.scan_cells) {
        set_error(err, CMAG_DEVERR_RANGE);
        rel = p.scan_cells - 1;
    }
    const uint32_t slot = p.table_base + rel;
    hash[i] = BATCH ? slot : p.scan_base + rel;  // = hr inside the table
    const uint32_t r = atomicAdd(cnt + slot, 1u);
    if (rank) rank[i] = r;
    if (p.wc_mark) wall_cache_note(p, i, q, g);
}

// The 16 counts of cells [first, first + 16) (zeros past m).
__device__ __forceinline__ void load_counts(const uint32_t *__restrict__ cnt, uint32_t first,
                                            uint32_t m, uint32_t (&v)[kScanItems])
{
    if (first + kScanItems <= m) {
        const uint4 *src = reinterpret_cast<const uint4 *>(cnt + first);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) {
            const uint4 q = src[k];
            v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] = (first + k < m) ? cnt[first + k] : 0u;
    }
}

// Sum over the block (result in every thread).
__device__ __forceinline__ uint32_t block_sum(uint32_t x, uint32_t *s_warp)
{
    x = __reduce_add_sync(0xffffffffu, x);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = x;
    __syncthreads();
    uint32_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_warp[w];
    __syncthreads();
    return t;
}

// Scan, step 1: the particle count of each tile of kScanTile cells.
__global__ void __launch_bounds__(kScanThreads)
    k_tile_sum(const uint32_t *__restrict__ cnt, uint32_t m, uint32_t *__restrict__ tot)
{
    pdl_entry();
    __shared__ uint32_t s_warp[kScanThreads / 32];
    uint32_t v[kScanItems];
    load_counts(cnt, blockIdx.x * kScanTile + threadIdx.x * kScanItems, m, v);
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
    sum = block_sum(sum, s_warp);
    if (threadIdx.x == 0) tot[blockIdx.x] = sum;
}

// Scan, step 2: exclusive scan of the tile counts in place, by one block: each
// thread sums a contiguous chunk of tiles, the block scans the chunk sums, and
// each thread rewrites its chunk from its offset.
// wc_state (a single scene's wall density cache, or null): the step stamp
// advances, and a new epoch starts when the hash pass saw a non-fluid particle
// move (the hash pass has completed; the density pass follows).
__global__ void __launch_bounds__(1024) k_tile_prefix(uint32_t *__restrict__ tot, uint32_t tiles,
                                                      uint32_t *__restrict__ wc_state)
{
    pdl_entry();
    if (wc_state && threadIdx.x == 0) {
        wc_state[kWcStamp] += 1u;
        if (wc_state[kWcMoved]) {
            wc_state[kWcEpoch] += 1u;
            wc_state[kWcMoved] = 0u;
        }
    }
    __shared__ uint32_t s_warp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t per = (tiles + blockDim.x - 1) / blockDim.x;
    const uint32_t a = min(tiles, threadIdx.x * per), b = min(tiles, a + per);
    uint32_t sum = 0;
    for (uint32_t k = a; k < b; ++k) sum += tot[k];
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t run = x - sum;
    for (int w = 0; w < warp; ++w) run += s_warp[w];
    for (uint32_t k = a; k < b; ++k) {
        const uint32_t v = tot[k];
        tot[k] = run;
        run += v;
    }
}

// Scan, step 3: each tile's cells from its prefix: off[c] = particles in cells
// before c.  Clears the counts it read (the next hash pass adds to zeros).
__global__ void __launch_bounds__(kScanThreads)
    k_cell_offsets(uint32_t *__restrict__ cnt, uint32_t *__restrict__ off, uint32_t m,
                   const uint32_t *__restrict__ tot)
{
    pdl_entry();
    __shared__ uint32_t s_warp[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t first = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const uint32_t prefix = __ldg(tot + blockIdx.x);
    uint32_t v[kScanItems];
    load_counts(cnt, first, m, v);
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
    if (first + kScanItems <= m) {
        uint4 *c4 = reinterpret_cast<uint4 *>(cnt + first);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k)
            if (v[4 * k] | v[4 * k + 1] | v[4 * k + 2] | v[4 * k + 3]) c4[k] = make_uint4(0, 0, 0, 0);
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
            if (first + k < m && v[k]) cnt[first + k] = 0;
    }
    // block exclusive scan of the thread sums
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t wbase = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) wbase += (w < warp) ? s_warp[w] : 0u;
    uint32_t run = prefix + wbase + x - sum;
    if (first + kScanItems <= m) {
        uint4 *dst = reinterpret_cast<uint4 *>(off + first);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) {
            uint4 q;
            q.x = run; run += v[4 * k];
            q.y = run; run += v[4 * k + 1];
            q.z = run; run += v[4 * k + 2];
            q.w = run; run += v[4 * k + 3];
            dst[k] = q;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (first + k < m) off[first + k] = run;
            run += v[k];
        }
    }
}

// Counting sort, step 1: particle i goes to slot off[cell] + rank[i] of its
// cell's range (arrival order within the cell).
__global__ void __launch_bounds__(256)
    k_cell_scatter(const uint32_t *__restrict__ hash, const uint32_t *__restrict__ rank,
                   const uint32_t *__restrict__ off, uint32_t key_base, uint32_t n,
                   uint32_t *__restrict__ shash, uint32_t *__restrict__ tmp, uint32_t *err)
{
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t h = hash[i];
    const uint32_t q = __ldg(off + (h - key_base)) + rank[i];
    if (q < n) {  // always, unless the counts and offsets disagree
        shash[q] = h;
        tmp[q] = i;
    } else {
        set_error(err, CMAG_DEVERR_RANGE);
    }
}

// Counting sort, step 2: within each cell, the entry at slot q moves to the
// cell's start + the number of the cell's entries with a smaller original index,
// so each cell lists its particles by original index: the order of a stable
// sort by hash.  A cell of c particles costs c loads per entry; the neighbour
// loops read every particle of a cell for each of its particles as well.  The
// same thread gathers the particle's position and leap-frog velocity into the
// sorted copies (the copy half of reorderDataAndFindCellStartD,
// fluid_kernel.cu:91-96).
__global__ void __launch_bounds__(256)
    k_cell_order(const uint32_t *__restrict__ shash, const uint32_t *__restrict__ tmp,
                 const uint32_t *__restrict__ off, uint32_t key_base, uint32_t n,
                 uint32_t *__restrict__ idx, const float4 *__restrict__ pos,
                 const float4 *__restrict__ vlf, float4 *__restrict__ spos,
                 float4 *__restrict__ svel, uint32_t *err)
{
    pdl_entry();
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const uint32_t c = shash[q] - key_base;
    const uint32_t a = __ldg(off + c), b = __ldg(off + c + 1);
    const uint32_t own = tmp[q];
    uint32_t dst = q;
    if (!(b - a == 1u && a == q)) {
        if (!(a <= q && q < b && b <= n)) {  // counts and offsets disagree
            set_error(err, CMAG_DEVERR_RANGE);
        } else {
            uint32_t r = 0;
            for (uint32_t k = a; k < b; ++k) r += __ldg(tmp + k) < own ? 1u : 0u;
            dst = a + r;
        }
    }
    idx[dst] = own;
    const uint32_t j = own < n ? own : dst;  // own >= n only after a failed sort
    spos[dst] = __ldg(pos + j);
    svel[dst] = __ldg(vlf + j);
}

__global__ void k_cell_view(const uint32_t *__restrict__ off, uint32_t scan_base,
                            uint32_t scan_cells, uint64_t ncells, uint32_t *__restrict__ cs,
                            uint32_t *__restrict__ ce)
{
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < ncells;
         c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t a = 0, b = 0;
        if (c >= scan_base && c - scan_base < scan_cells) {
            a = off[c - scan_base];
            b = off[c - scan_base + 1];
        }
        bool occupied = b > a;
        cs[c] = occupied ? a : kEmptyCell;
        ce[c] = occupied ? b : 0u;
    }
}

}  // namespace

void launch_hash(const DevParams &p, const BatchView &bv, float4 *pos, uint32_t *hash,
                 uint32_t *cnt, uint32_t *rank, uint32_t *err, cudaStream_t st, float4 *snap,
                 const PhaseState *ph)
{
    const uint32_t n = bv.scenes ? bv.n_total : p.n;
    if (n == 0) return;
    const uint32_t blocks = (n + 255) / 256;
    if (bv.scenes) launch_pdl(k_hash<true>, blocks, 256, 0, st, p, bv, pos, hash, cnt, rank, err, snap, ph);
    else launch_pdl(k_hash<false>, blocks, 256, 0, st, p, bv, pos, hash, cnt, rank, err, snap, ph);
}

void launch_cell_sort(const uint32_t *hash, const uint32_t *rank, const uint32_t *off,
                      uint32_t key_base, uint32_t n, uint32_t *shash, uint32_t *tmp,
                      uint32_t *idx, const float4 *pos, const float4 *vlf, float4 *spos,
                      float4 *svel, uint32_t *err, cudaStream_t st)
{
    if (n == 0) return;
    const uint32_t blocks = (n + 255) / 256;
    launch_pdl(k_cell_scatter, blocks, 256, 0, st, hash, rank, off, key_base, n, shash, tmp, err);
    launch_pdl(k_cell_order, blocks, 256, 0, st, shash, tmp, off, key_base, n, idx, pos, vlf, spos, svel, err);
}

size_t cell_scan_workspace_words(uint32_t m) { return (m + kScanTile - 1) / kScanTile; }

void launch_cell_scan(uint32_t *cnt, uint32_t *off, uint32_t m, uint32_t *ws, cudaStream_t st,
                      uint32_t *wc_state)
{
    const uint32_t tiles = (m + kScanTile - 1) / kScanTile;
    if (tiles == 0) return;
    launch_pdl(k_tile_sum, tiles, kScanThreads, 0, st, cnt, m, ws);
    launch_pdl(k_tile_prefix, 1, 1024, 0, st, ws, tiles, wc_state);
    launch_pdl(k_cell_offsets, tiles, kScanThreads, 0, st, cnt, off, m, ws);
}

void launch_cell_view(const uint32_t *off, uint32_t scan_base, uint32_t scan_cells,
                      uint64_t ncells, uint32_t *cell_start, uint32_t *cell_end, cudaStream_t st)
{
    uint64_t blocks = (ncells + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (blocks == 0) return;
    k_cell_view<<<(uint32_t)blocks, 256, 0, st>>>(off, scan_base, scan_cells, ncells, cell_start,
                                                  cell_end);
}

}  // namespace cmag
