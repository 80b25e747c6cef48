// kernels.h -- host-side launchers of the device kernels (internal interface
// between the C ABI in system.cu and the kernel translation units).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "sph_common.cuh"

namespace cmag {

// Launches of this thread without the programmatic-dependent-launch attribute
// (set while capturing the bodies of a conditional graph node, whose kernels
// then follow each other with full dependencies).
inline thread_local bool g_plain_launches = false;

// Launch `kernel` (which begins with pdl_entry()) with programmatic dependent
// launch allowed: it may start launching while the previous kernel on the stream
// finishes (in a captured graph too).
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args &&...args)
{
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = g_plain_launches ? 0 : 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}


// Streaming multiprocessors of the current device (grid sizing of grid-stride
// kernels; 152 on a GB300).
inline int device_sm_count()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        (void)cudaGetLastError();
        return 152;
    }
    return sms;
}

// ---- onesweep radix sort (sort.cu) ----------------------------------------
constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;  // keys per tile
constexpr int kRadixBits = 8;
constexpr int kRadix = 256;
constexpr int kMaxPasses = 4;

inline int sort_passes(uint32_t key_bits) { return (int)((key_bits + kRadixBits - 1) / kRadixBits); }
inline uint32_t sort_tiles(uint32_t n) { return (n + kSortTile - 1) / kSortTile; }

// Workspace of one sort, in 32-bit words: digit histograms [4][256], tile
// counters [4], then one look-back status array of tiles*256 words per pass.
// Must be zero when a sort starts (sort_workspace_clear or a memset).
size_t sort_workspace_words(uint32_t n, int passes);
struct SortWorkspace {
    uint32_t *hist;       // [kMaxPasses][256]
    uint32_t *tile_ctr;   // [kMaxPasses]
    uint32_t *status;     // [passes][tiles][256]
};
SortWorkspace sort_workspace_view(uint32_t *base, uint32_t n);

// Digit histograms of all passes (used when the hash kernel did not fill them).
void launch_digit_hist(const uint32_t *keys, uint32_t n, int passes, uint32_t *hist,
                       cudaStream_t st);
// One LSD pass on digit `pass`; identity_values: value = input position.
void launch_onesweep_pass(const uint32_t *kin, const uint32_t *vin, uint32_t *kout,
                          uint32_t *vout, uint32_t n, int pass, bool identity_values,
                          const SortWorkspace &ws, uint32_t *err, cudaStream_t st);

// ---- cells (cells.cu) --------------------------------------------------------
// Hash every particle and count particles per cell.  rank (may be null): per
// particle, its arrival order among the particles of its cell (0, 1, ...; not
// deterministic).  ph (Peristalsis phase blocks, may be null): first place the
// wall particles on their walls where the step configures the boundary (the
// work of launch_configure_boundary, fused).
void launch_hash(const DevParams &p, const BatchView &bv, float4 *pos, uint32_t *hash,
                 uint32_t *cnt, uint32_t *rank, uint32_t *err, cudaStream_t st,
                 float4 *snap = nullptr, const PhaseState *ph = nullptr);
// Stable counting sort of the hashed particles by cell, from the dense offsets
// (after launch_cell_scan): shash/idx = the hashes and original indices in the
// order of a stable sort by hash (the radix sort's result exactly), and
// spos/svel = pos/vlf gathered in that order.  Cell of a hash: h - key_base.
// tmp: n words of scratch; idx may alias rank.
void launch_cell_sort(const uint32_t *hash, const uint32_t *rank, const uint32_t *off,
                      uint32_t key_base, uint32_t n, uint32_t *shash, uint32_t *tmp,
                      uint32_t *idx, const float4 *pos, const float4 *vlf, float4 *spos,
                      float4 *svel, uint32_t *err, cudaStream_t st);
// Exclusive scan of cnt[0..m) into off[0..m) (tile totals, their scan, then
// every tile from its prefix), clearing cnt for the next step.  ws must hold
// cell_scan_workspace_words(m) words (no clearing needed).
size_t cell_scan_workspace_words(uint32_t m);
// wc_state: a single scene's wall density cache state (DevParams::wc_state) or
// null; its step stamp and epoch advance in the scan (after the hash pass).
void launch_cell_scan(uint32_t *cnt, uint32_t *off, uint32_t m, uint32_t *ws, cudaStream_t st,
                      uint32_t *wc_state = nullptr);
// Reference cellStart/cellEnd view of the dense offsets.
void launch_cell_view(const uint32_t *off, uint32_t scan_base, uint32_t scan_cells,
                      uint64_t ncells, uint32_t *cell_start, uint32_t *cell_end, cudaStream_t st);

// ---- neighbour loops (density.cu, force.cu) ---------------------------------
// density also writes aux[i] = (p/rho^2, rho) (DamBreak) or (p/rho^2, 1/rho).
// bv empty: one scene with parameters p; otherwise one launch group of a batch
// (p = the parameters of any of the group's scenes).
// nl (entry != nullptr): density records the interaction lists, force reads them
// (both with one lane per particle; group is then ignored)
void launch_density(const DevParams &p, const BatchView &bv, int group, const float4 *spos,
                    const uint32_t *off, float4 *meas, float2 *aux, const NeighborList &nl,
                    cudaStream_t st);
// Density of every particle from neighbour lists kept since their last rebuild
// (single scenes; nl.count <= nl.cap for every particle).
void launch_density_list(const DevParams &p, const float4 *spos, const NeighborList &nl, float4 *meas,
                         float2 *aux, cudaStream_t st);
// ph: the Peristalsis phase (one per scene in a batch; read with wall_noslip only)
void launch_force(const DevParams &p, const BatchView &bv, int group, const float4 *spos,
                  const float4 *svel, const float2 *aux, const uint32_t *idx, const uint32_t *off,
                  float4 *out_a, float4 *out_b, const PhaseState *ph, const NeighborList &nl,
                  cudaStream_t st);

// ---- integration and wall motion (integrate.cu) ------------------------------
// bv empty: one scene; otherwise every particle of the batch with its scene's
// parameters and phase (ph holds one PhaseState per scene).
void launch_phase(const DevParams &p, PhaseState *ph, float k_milli, cudaStream_t st);
void launch_configure_boundary(const DevParams &p, const BatchView &bv, float4 *pos,
                               const PhaseState *ph, cudaStream_t st, const float4 *xb = nullptr,
                               uint32_t *moved = nullptr);
// xb (may be null): positions at the last rebuild of kept neighbour lists; a
// particle now more than skin/2 from it sets *moved
void launch_integrate(const DevParams &p, const BatchView &bv, float4 *pos, float4 *vel,
                      float4 *vlf, const float4 *acc, const float4 *vforce, const float4 *pforce,
                      const PhaseState *ph, cudaStream_t st, const float4 *xb = nullptr,
                      uint32_t *moved = nullptr);
// the phase machines of the batch's Peristalsis scenes (one thread per scene)
void launch_phase_batch(const DevParams *scenes, uint32_t nscenes, PhaseState *ph, float k_milli,
                        cudaStream_t st);
void launch_gate(const DevParams &p, float4 *pos, int remove, float dx, float fx, float fy,
                 cudaStream_t st);

// ---- neighbour lists kept over several steps (verlet.cu) ------------------------
// spos[i] = pos[idx[i]], svel[i] = vlf[idx[i]]: the step's positions and leap-frog
// velocities in the order of the last rebuild.
void launch_gather_sorted(const uint32_t *idx, const float4 *pos, const float4 *vlf, uint32_t n,
                          float4 *spos, float4 *svel, cudaStream_t st);
// Whether this step rebuilds (a particle moved more than skin/2 since the last
// rebuild, a list overflowed, or the host asked): sets the graph's conditional
// (cond != 0) and/or decision[0], clears the flags for the next step and counts
// rebuilds in decision[1].
struct VerletFlags {
    uint32_t moved;     // set by integrate (or by the host to force a rebuild)
    uint32_t overflow;  // set by the rebuilding density pass
    uint32_t decision;  // this step's choice (1 = rebuild)
    uint32_t rebuilds;  // rebuilds so far
};
void launch_verlet_decide(VerletFlags *flags, unsigned long long cond, int use_cond, cudaStream_t st);
// positions [start, start + count) were set from the host: *moved = 1 when one
// lies more than sqrt(move2) from xb
void launch_verlet_check(const float4 *pos, const float4 *xb, uint32_t start, uint32_t count, float move2,
                         uint32_t *moved, cudaStream_t st);

// ---- reductions over fluid particles (reduce.cu) -------------------------------
// out6: order-preserving keys of min x,y,z then max x,y,z (init 0xffffffff, 0)
void launch_fluid_extent(int32_t system, const float4 *pos, uint32_t n, uint32_t *out6,
                         cudaStream_t st);
// per-scene extents of a batch: out[6 s ..] as out6 above (initialised the same way)
void launch_fluid_extents_batch(const BatchView &bv, const float4 *pos, uint32_t *out,
                                cudaStream_t st);
// *flag = 1 when some a[i].z (i < n) differs from z, else 0.
void launch_z_differs(const float4 *a, uint32_t n, float z, uint32_t *flag, cudaStream_t st);
// flags[slot] = 1 when a particle of a checked slot (expect[slot].y != 0) has a z
// other than expect[slot].x, else 0 (slots entries).
void launch_z_differs_slots(const float4 *a, const uint16_t *slot_of, uint32_t n, const float2 *expect,
                            uint32_t *flags, uint32_t slots, cudaStream_t st);
void launch_fluid_sum(int32_t system, const float4 *type_src, const float4 *a, uint32_t n,
                      double *sums4, unsigned long long *count, cudaStream_t st);

// ---- headless colours and point view (render.cu) -------------------------------
// the reference's colour buffer values per particle (original order)
void launch_colors(const DevParams &p, const float4 *pos, uint32_t fluid, uint32_t type_one,
                   float4 *out, cudaStream_t st);
// x-y point image (w x h RGB bytes, row 0 at the top) of n particles
void launch_render(const float4 *pos, const float4 *color, uint32_t n, float x0, float y0,
                   float inv_px, uint32_t w, uint32_t h, float scale, uint32_t *owner,
                   uint8_t *rgb, cudaStream_t st);

}  // namespace cmag
