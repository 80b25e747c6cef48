// cells.cu -- grid hash, per-cell counts and dense cell offsets, the per-step
// counting sort, sorted gather.
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
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr int kSpinLimit = 1 << 22;

// calcHashD (fluid_kernel.cu:34-48) + per-cell counts, one particle per thread.
// The sort key is the reference hash for a single scene; in a batch it is the
// particle's cell index in the shared offset table (scene table base + cell), so
// the sort orders by scene, then by cell.  A particle whose cell lies outside
// its offset table (a planar scene's particle that left its z layer) is counted
// in the table's last cell and reported as CMAG_DEVERR_RANGE.  rank[i] (when
// given) is the count the particle's atomic increment found: its arrival order
// among the particles of its cell.
template <bool BATCH>
__global__ void __launch_bounds__(256)
    k_hash(DevParams pv, BatchView bv, const float4 *__restrict__ pos, uint32_t *__restrict__ hash,
           uint32_t *__restrict__ cnt, uint32_t *__restrict__ rank, uint32_t *err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (BATCH ? bv.n_total : pv.n)) return;
    const DevParams &p = BATCH ? bv.scenes[bv.scene_of[i]] : pv;
    const float4 q = pos[i];
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
}

__global__ void __launch_bounds__(kScanThreads, 4)
    k_cell_scan(uint32_t *__restrict__ cnt, uint32_t *__restrict__ off, uint32_t m,
                uint32_t *tile_ctr, uint32_t *status, uint32_t *err)
{
    __shared__ uint32_t s_warp[kScanThreads / 32];
    __shared__ uint32_t s_tile, s_prefix;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t first = tile * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t sum = 0;
    if (first + kScanItems <= m) {
        const uint4 *src = reinterpret_cast<const uint4 *>(cnt + first);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) {
            uint4 q = src[k];
            v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
            if (q.x | q.y | q.z | q.w)
                reinterpret_cast<uint4 *>(cnt + first)[k] = make_uint4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            uint32_t c = first + k;
            v[k] = (c < m) ? cnt[c] : 0u;
            if (c < m && v[k]) cnt[c] = 0;
        }
    }
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];

    // block exclusive scan of the thread sums
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t wbase = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) {
        uint32_t t = s_warp[w];
        wbase += (w < warp) ? t : 0u;
        total += t;
    }
    uint32_t texcl = wbase + x - sum;

    // decoupled look-back by warp 0: lane k reads tile t - k, so each round covers
    // 32 predecessors (the counts add up in the same way as one tile at a time)
    if (warp == 0) {
        volatile uint32_t *st = status;
        uint32_t exclusive = 0;
        if (tile == 0) {
            if (lane == 0) st[0] = kFlagPrefix | total;
        } else {
            if (lane == 0) st[tile] = kFlagAgg | total;
            int t = (int)tile - 1;
            int spins = 0;
            while (t >= 0) {
                const uint32_t v = (t - lane >= 0) ? (uint32_t)st[t - lane] : (uint32_t)kFlagPrefix;
                const uint32_t pub = __ballot_sync(0xffffffffu, (v & (kFlagAgg | kFlagPrefix)) != 0);
                const uint32_t pre = __ballot_sync(0xffffffffu, (v & kFlagPrefix) != 0);
                // lanes before the first unpublished tile, up to the first prefix
                const uint32_t unpub = ~pub;
                const int first_unpub = unpub ? __ffs(unpub) - 1 : 32;
                const int first_pre = pre ? __ffs(pre) - 1 : 32;
                const bool done = first_pre < first_unpub;
                const int used = done ? first_pre + 1 : first_unpub;
                exclusive += __reduce_add_sync(0xffffffffu, lane < used ? (v & kCountMask) : 0u);
                if (done) break;
                t -= used;
                if (used == 0) {
                    if (++spins > kSpinLimit) {
                        if (lane == 0) set_error(err, CMAG_DEVERR_LOOKBACK_TIMEOUT);
                        break;  // give up: the rest counts as zero
                    }
                    if (spins > 8) __nanosleep(64);
                }
            }
            if (lane == 0) st[tile] = kFlagPrefix | (exclusive + total);
        }
        if (lane == 0) s_prefix = exclusive;
    }
    __syncthreads();
    uint32_t run = s_prefix + texcl;
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
            uint32_t c = first + k;
            if (c < m) off[c] = run;
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
// loops read every particle of a cell for each of its particles as well.
__global__ void __launch_bounds__(256)
    k_cell_order(const uint32_t *__restrict__ shash, const uint32_t *__restrict__ tmp,
                 const uint32_t *__restrict__ off, uint32_t key_base, uint32_t n,
                 uint32_t *__restrict__ idx, uint32_t *err)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const uint32_t c = shash[q] - key_base;
    const uint32_t a = __ldg(off + c), b = __ldg(off + c + 1);
    const uint32_t own = tmp[q];
    if (b - a == 1u && a == q) {
        idx[q] = own;
        return;
    }
    if (!(a <= q && q < b && b <= n)) {  // counts and offsets disagree
        set_error(err, CMAG_DEVERR_RANGE);
        idx[q] = own;
        return;
    }
    uint32_t r = 0;
    for (uint32_t k = a; k < b; ++k) r += __ldg(tmp + k) < own ? 1u : 0u;
    idx[a + r] = own;
}

// the copy half of reorderDataAndFindCellStartD (fluid_kernel.cu:91-96)
__global__ void __launch_bounds__(256)
    k_reorder(const uint32_t *__restrict__ idx, const float4 *__restrict__ pos,
              const float4 *__restrict__ vlf, float4 *__restrict__ spos,
              float4 *__restrict__ svel, uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t j = idx[i];
    if (j >= n) j = i;  // only after a failed sort (reported by the sort itself)
    spos[i] = __ldg(pos + j);
    svel[i] = __ldg(vlf + j);
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

void launch_hash(const DevParams &p, const BatchView &bv, const float4 *pos, uint32_t *hash,
                 uint32_t *cnt, uint32_t *rank, uint32_t *err, cudaStream_t st)
{
    const uint32_t n = bv.scenes ? bv.n_total : p.n;
    if (n == 0) return;
    const uint32_t blocks = (n + 255) / 256;
    if (bv.scenes) k_hash<true><<<blocks, 256, 0, st>>>(p, bv, pos, hash, cnt, rank, err);
    else k_hash<false><<<blocks, 256, 0, st>>>(p, bv, pos, hash, cnt, rank, err);
}

void launch_cell_sort(const uint32_t *hash, const uint32_t *rank, const uint32_t *off,
                      uint32_t key_base, uint32_t n, uint32_t *shash, uint32_t *tmp,
                      uint32_t *idx, uint32_t *err, cudaStream_t st)
{
    if (n == 0) return;
    const uint32_t blocks = (n + 255) / 256;
    k_cell_scatter<<<blocks, 256, 0, st>>>(hash, rank, off, key_base, n, shash, tmp, err);
    k_cell_order<<<blocks, 256, 0, st>>>(shash, tmp, off, key_base, n, idx, err);
}

size_t cell_scan_workspace_words(uint32_t m) { return 1 + (m + kScanTile - 1) / kScanTile; }

void launch_cell_scan(uint32_t *cnt, uint32_t *off, uint32_t m, uint32_t *ws, uint32_t *err,
                      cudaStream_t st)
{
    uint32_t tiles = (m + kScanTile - 1) / kScanTile;
    k_cell_scan<<<tiles, kScanThreads, 0, st>>>(cnt, off, m, ws, ws + 1, err);
}

void launch_reorder(const uint32_t *idx, const float4 *pos, const float4 *vlf, float4 *spos,
                    float4 *svel, uint32_t n, cudaStream_t st)
{
    if (n == 0) return;
    k_reorder<<<(n + 255) / 256, 256, 0, st>>>(idx, pos, vlf, spos, svel, n);
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
