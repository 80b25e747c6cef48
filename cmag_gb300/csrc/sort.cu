// sort.cu -- stable LSD radix sort of (cell hash, particle index) pairs.
//
// Replaces thrust::sort_by_key in sortParticles (DamBreak.Core/fluidSystem.cu:94-99,
// Poiseuille.Core/poiseuilleFlowSystem.cu:103-108, PeristalsisSystem.cu:116-121).
// One kernel launch per 8-bit digit, following the single-pass "onesweep" scheme
// of Adinets & Merrill (2022):
//   * the digit histograms of every pass come from one read of the keys (fused
//     into the hash kernel, or launch_digit_hist);
//   * each CTA takes the next tile from an atomic counter, ranks its keys with a
//     warp-level multisplit (__match_any_sync), publishes its per-digit counts and
//     resolves its global offsets by decoupled look-back over earlier tiles;
//   * ranks follow input order inside a warp, warps follow each other inside a
//     tile and tiles follow tile order, so the sort is stable and equals a stable
//     sort by key -- bit-identical to the reference's thrust result.
// Every look-back wait is bounded: after g_spin_limit polls (kSpinLimit unless a
// test lowered it) the CTA records CMAG_DEVERR_LOOKBACK_TIMEOUT, treats the
// missing counts as zero and finishes; its scatter then writes only positions
// below n (underestimated offsets stay in range) and flags any other as
// CMAG_DEVERR_RANGE.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "kernels.h"

namespace cmag {

namespace {

constexpr uint32_t kFlagAgg = 1u << 30;     // tile aggregate published
constexpr uint32_t kFlagPrefix = 2u << 30;  // inclusive prefix published
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr int kSpinLimit = 1 << 22;
// polls before a look-back wait gives up (cmag_testing_set_sort_spin_limit)
__device__ int g_spin_limit = kSpinLimit;
constexpr int kWarps = kSortThreads / 32;
constexpr uint32_t kInvalidDigit = 256;
constexpr int kLookback = 16;  // predecessor tiles read per look-back round

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// exclusive scan of one value per thread over a 256-thread block
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *s_warp,
                                                         uint32_t *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t wbase = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        uint32_t t = s_warp[w];
        wbase += (w < warp) ? t : 0u;
        all += t;
    }
    __syncthreads();
    if (total) *total = all;
    return wbase + x - v;
}

__global__ void __launch_bounds__(256) k_digit_hist(const uint32_t *__restrict__ keys, uint32_t n,
                                                    int passes, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t s_hist[kMaxPasses * kRadix];
    for (int b = threadIdx.x; b < passes * kRadix; b += blockDim.x) s_hist[b] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k = keys[i];
        for (int ps = 0; ps < passes; ++ps) atomicAdd(&s_hist[ps * kRadix + ((k >> (8 * ps)) & 255u)], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < passes * kRadix; b += blockDim.x)
        if (s_hist[b]) atomicAdd(&hist[b], s_hist[b]);
}

template <bool kIdentity>
__global__ void __launch_bounds__(kSortThreads)
    k_onesweep(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
               uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, uint32_t n, int shift,
               const uint32_t *__restrict__ hist, uint32_t *tile_ctr, uint32_t *status,
               uint32_t *err)
{
    __shared__ uint32_t s_whist[kWarps][kRadix];  // per-warp digit counts -> offsets
    __shared__ uint32_t s_base[kRadix];           // global start of each digit in this tile
    __shared__ uint32_t s_scan[kWarps];
    __shared__ uint32_t s_tile;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (int b = threadIdx.x; b < kWarps * kRadix; b += kSortThreads) (&s_whist[0][0])[b] = 0;
    // digit offsets of this pass: exclusive scan of the global histogram
    uint32_t digit_start = block_exclusive_scan(hist[threadIdx.x], s_scan, nullptr);
    const uint32_t tile = s_tile;  // visible: block_exclusive_scan synchronised

    const uint32_t chunk = tile * kSortTile + (uint32_t)warp * (32u * kSortItems);
    uint32_t key[kSortItems], val[kSortItems], off[kSortItems];
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        uint32_t i = chunk + (uint32_t)it * 32u + (uint32_t)lane;
        if (i < n) {
            key[it] = kin[i];
            val[it] = kIdentity ? i : vin[i];
        } else {
            key[it] = 0xffffffffu;
            val[it] = 0;
        }
    }
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        uint32_t i = chunk + (uint32_t)it * 32u + (uint32_t)lane;
        uint32_t d = (i < n) ? ((key[it] >> shift) & 255u) : kInvalidDigit;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = 0;
        if (d != kInvalidDigit) before = s_whist[warp][d];
        __syncwarp();
        if (d != kInvalidDigit && lane == __ffs(peers) - 1) s_whist[warp][d] = before + __popc(peers);
        __syncwarp();
        off[it] = before + __popc(peers & lt);
    }
    __syncthreads();

    // thread d owns digit d: warp-exclusive offsets and the tile total
    const uint32_t d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        uint32_t c = s_whist[w][d];
        s_whist[w][d] = run;
        run += c;
    }
    // decoupled look-back over the tiles before this one, kLookback tiles per
    // round: the counts add up in the same way, in fewer dependent round trips
    volatile uint32_t *st = status;
    const int spin_limit = g_spin_limit;
    uint32_t exclusive = 0;
    if (tile == 0) {
        st[d] = kFlagPrefix | run;
    } else {
        st[(size_t)tile * kRadix + d] = kFlagAgg | run;
        int t = (int)tile - 1;
        int spins = 0;
        while (t >= 0) {
            uint32_t v[kLookback];
#pragma unroll
            for (int k = 0; k < kLookback; ++k)
                v[k] = (t - k >= 0) ? (uint32_t)st[(size_t)(t - k) * kRadix + d] : (uint32_t)kFlagPrefix;
            // consume published tiles up to the first inclusive prefix; stop at the
            // first tile that has published nothing yet
            uint32_t add = 0;
            int used = 0;
            bool stop = false, done = false;
#pragma unroll
            for (int k = 0; k < kLookback; ++k) {
                if (!stop) {
                    if (v[k] & (kFlagAgg | kFlagPrefix)) {
                        add += v[k] & kCountMask;
                        ++used;
                        if (v[k] & kFlagPrefix) stop = done = true;
                    } else {
                        stop = true;
                    }
                }
            }
            exclusive += add;
            if (done) break;
            t -= used;
            if (used == 0) {
                if (++spins > spin_limit) {
                    set_error(err, CMAG_DEVERR_LOOKBACK_TIMEOUT);
                    break;  // give up: the rest counts as zero
                }
                if (spins > 8) __nanosleep(64);
            }
        }
        st[(size_t)tile * kRadix + d] = kFlagPrefix | (exclusive + run);
    }
    s_base[d] = digit_start + exclusive;
    __syncthreads();

#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        uint32_t i = chunk + (uint32_t)it * 32u + (uint32_t)lane;
        if (i < n) {
            uint32_t dd = (key[it] >> shift) & 255u;
            uint32_t o = s_base[dd] + s_whist[warp][dd] + off[it];
            if (o < n) {  // always true unless a look-back gave up
                kout[o] = key[it];
                vout[o] = val[it];
            } else {
                set_error(err, CMAG_DEVERR_RANGE);
            }
        }
    }
}

}  // namespace

size_t sort_workspace_words(uint32_t n, int passes)
{
    return (size_t)kMaxPasses * kRadix + kMaxPasses +
           (size_t)(passes > 0 ? passes : 1) * sort_tiles(n) * kRadix;
}

SortWorkspace sort_workspace_view(uint32_t *base, uint32_t n)
{
    SortWorkspace ws;
    ws.hist = base;
    ws.tile_ctr = base + kMaxPasses * kRadix;
    ws.status = ws.tile_ctr + kMaxPasses;
    (void)n;
    return ws;
}

void launch_digit_hist(const uint32_t *keys, uint32_t n, int passes, uint32_t *hist,
                       cudaStream_t st)
{
    if (n == 0 || passes == 0) return;
    uint32_t blocks = (n + 2047) / 2048;
    const uint32_t cap = 8u * (uint32_t)device_sm_count();  // 8 blocks per SM
    if (blocks > cap) blocks = cap;
    k_digit_hist<<<blocks, 256, 0, st>>>(keys, n, passes, hist);
}

void launch_onesweep_pass(const uint32_t *kin, const uint32_t *vin, uint32_t *kout,
                          uint32_t *vout, uint32_t n, int pass, bool identity_values,
                          const SortWorkspace &ws, uint32_t *err, cudaStream_t st)
{
    if (n == 0) return;
    uint32_t tiles = sort_tiles(n);
    uint32_t *status = ws.status + (size_t)pass * tiles * kRadix;
    if (identity_values)
        k_onesweep<true><<<tiles, kSortThreads, 0, st>>>(kin, vin, kout, vout, n, 8 * pass,
                                                         ws.hist + pass * kRadix,
                                                         ws.tile_ctr + pass, status, err);
    else
        k_onesweep<false><<<tiles, kSortThreads, 0, st>>>(kin, vin, kout, vout, n, 8 * pass,
                                                          ws.hist + pass * kRadix,
                                                          ws.tile_ctr + pass, status, err);
}

}  // namespace cmag

// ---------------------------------------------------------------------------
// Sort without any allocation: fixed scratch in device memory of this library.
//
// Some callers cannot call cudaMalloc at the moment they need the sort:
// latency-critical loops where an allocation would stall the device, and hosts
// whose device memory all comes from their own pool (a framework's caching
// allocator, an embedded runtime with a fixed budget).  For them the sort's
// workspace lives in one file-scope device array, sized for at most
// kNoAllocMaxKeys keys and held by every GPU that loads this library until the
// process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;  // 1,048,576 (hash, index) pairs
constexpr uint32_t kNoAllocMaxTiles = (kNoAllocMaxKeys + cmag::kSortTile - 1) / cmag::kSortTile;
// histograms + tile counters + look-back status of up to four passes
constexpr size_t kNoAllocWsWords = (size_t)cmag::kMaxPasses * cmag::kRadix + cmag::kMaxPasses +
                                   (size_t)cmag::kMaxPasses * kNoAllocMaxTiles * cmag::kRadix;
// + error word, then the alternate key and value buffers
constexpr size_t kNoAllocWords = kNoAllocWsWords + 1 + 2 * (size_t)kNoAllocMaxKeys;

__device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

// The array's device address belongs to the CUDA context the module was loaded
// in (normally the device's primary context).  It is looked up once per context,
// with that context current, and cached under the context handle, so a host that
// makes its own context current gets that context's copy.  The driver's
// cuCtxGetCurrent is reached through the runtime (no link to the driver library).
typedef int (*CtxGetCurrentFn)(void **ctx);
CtxGetCurrentFn ctx_get_current()
{
    static CtxGetCurrentFn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (CtxGetCurrentFn) nullptr;
        return reinterpret_cast<CtxGetCurrentFn>(f);
    }();
    return fn;
}

constexpr int kMaxContexts = 64;
struct ScratchAddr {
    void *ctx;
    uint32_t *ptr;
};
std::mutex g_noalloc_mu;
ScratchAddr g_noalloc_addr[kMaxContexts] = {};
int g_noalloc_used = 0;

thread_local char g_noalloc_msg[256];

int noalloc_fail(int code, const char *msg, cudaError_t e = cudaSuccess)
{
    if (e != cudaSuccess)
        std::snprintf(g_noalloc_msg, sizeof(g_noalloc_msg), "%s: %s", msg, cudaGetErrorString(e));
    else
        std::snprintf(g_noalloc_msg, sizeof(g_noalloc_msg), "%s", msg);
    return code;
}

// Device address of the scratch array in the current context (set-up on the first
// call in each context; later calls read the cache).
int noalloc_scratch(uint32_t **out)
{
    void *ctx = nullptr;
    CtxGetCurrentFn get = ctx_get_current();
    // no context current yet (the runtime creates the primary one on the lookup
    // below): nothing to key the cache on this time
    if (get && get(&ctx) != 0) ctx = nullptr;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (ctx)
        for (int k = 0; k < g_noalloc_used; ++k)
            if (g_noalloc_addr[k].ctx == ctx) {
                *out = g_noalloc_addr[k].ptr;
                return CMAG_OK;
            }
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
        return noalloc_fail(CMAG_ERR_CUDA, "cudaGetSymbolAddress(scratch)", e);
    // without a context handle (driver entry point unavailable) nothing is cached
    if (ctx && g_noalloc_used < kMaxContexts) g_noalloc_addr[g_noalloc_used++] = {ctx, static_cast<uint32_t *>(ptr)};
    *out = static_cast<uint32_t *>(ptr);
    return CMAG_OK;
}

int device_error_fail(uint32_t bits)
{
    char msg[160];
    std::snprintf(msg, sizeof(msg), "sort: device-side check failed (bits 0x%x:%s%s)", bits,
                  (bits & CMAG_DEVERR_LOOKBACK_TIMEOUT) ? " look-back spin limit reached" : "",
                  (bits & CMAG_DEVERR_RANGE) ? " scatter index out of range" : "");
    return noalloc_fail(CMAG_ERR_DEVICE, msg);
}

}  // namespace

extern "C" {

const char *cmag_sort_particles_noalloc_error(void) { return g_noalloc_msg; }

int cmag_sort_particles_noalloc(uint32_t *d_hash, uint32_t *d_index, uint32_t n, uint32_t key_bits,
                                void *cuda_stream)
{
    using namespace cmag;
    if (n == 0) return CMAG_OK;
    if (!d_hash || !d_index) return noalloc_fail(CMAG_ERR_INVALID, "null argument");
    if (n > kNoAllocMaxKeys)
        return noalloc_fail(CMAG_ERR_INVALID,
                            "cmag_sort_particles_noalloc sorts at most 1048576 pairs; use "
                            "cmag_sort_particles for more");
    if (key_bits > 32) return noalloc_fail(CMAG_ERR_INVALID, "key_bits must be at most 32");
    uint32_t *base = nullptr;
    if (int rc = noalloc_scratch(&base)) return rc;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    int passes = sort_passes(key_bits);
    if (passes < 1) passes = 1;
    // the scratch keeps the previous call's contents: clear the counters and the
    // look-back status this call reads, and the error word
    const size_t clear_words = sort_workspace_words(n, passes);
    uint32_t *err = base + kNoAllocWsWords;
    uint32_t *alt_keys = err + 1, *alt_vals = alt_keys + kNoAllocMaxKeys;
    cudaError_t e = cudaMemsetAsync(base, 0, clear_words * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return noalloc_fail(CMAG_ERR_CUDA, "cudaMemsetAsync", e);
    SortWorkspace sw = sort_workspace_view(base, n);
    launch_digit_hist(d_hash, n, passes, sw.hist, st);
    uint32_t *kb[2] = {d_hash, alt_keys}, *vb[2] = {d_index, alt_vals};
    for (int k = 0; k < passes; ++k) {
        const int src = k & 1, dst = src ^ 1;
        launch_onesweep_pass(kb[src], vb[src], kb[dst], vb[dst], n, k, false, sw, err, st);
    }
    // a launch that failed leaves its error pending; it is reported but not
    // cleared (an error left by the caller's earlier work stays the caller's)
    e = cudaPeekAtLastError();
    if (e != cudaSuccess) return noalloc_fail(CMAG_ERR_CUDA, "sort launch (or an earlier pending error)", e);
    if (passes & 1) {
        e = cudaMemcpyAsync(d_hash, alt_keys, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_index, alt_vals, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return noalloc_fail(CMAG_ERR_CUDA, "cudaMemcpyAsync", e);
    }
    // wait for the sort and read its device-side check word
    uint32_t bits = 0;
    e = cudaMemcpyAsync(&bits, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return noalloc_fail(CMAG_ERR_CUDA, "sort", e);
    if (bits) return device_error_fail(bits);
    return CMAG_OK;
}

int cmag_testing_set_sort_spin_limit(int32_t polls)
{
    using namespace cmag;
    const int v = polls < 0 ? kSpinLimit : polls;
    cudaError_t e = cudaMemcpyToSymbol(g_spin_limit, &v, sizeof(int));
    if (e != cudaSuccess) return noalloc_fail(CMAG_ERR_CUDA, "cudaMemcpyToSymbol(spin limit)", e);
    return CMAG_OK;
}

}  // extern "C"
