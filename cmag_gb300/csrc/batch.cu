// batch.cu -- many independent scenes advanced by one set of launches.
//
// The reference runs one scene per process: every system object owns its device
// arrays and the kernels read one global __constant__ parameter block
// (fluidSystem.cu:17-19, poiseuilleFlowSystem.cu:19-21, PeristalsisSystem.cu:21-23).
// A cmag_batch holds S scenes of any family in shared arrays:
//   * particles: scene s owns [part_base, part_base + n) of every particle array;
//   * cells: scene s owns [table_base, table_base + table_cells) of one shared
//     offset table (its whole grid, or one z layer for a planar 2-D scene);
//   * parameters: one DevParams per scene in device memory, found through a
//     per-particle scene index (uint16).
// One hash, one cell scan, one sort (keys table_base + cell, so each scene stays
// in its particle range), one gather and one integration cover every scene; the
// neighbour loops run once per launch group: scenes of one family, search shape
// and size bucket, whose lanes-per-particle the autotuner picks.  Launch groups
// run concurrently on forked streams; the whole step (or several steps) is one
// CUDA graph.  Each scene's arithmetic is the single-scene solver's, so a scene's
// trajectory in a batch equals its trajectory alone bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "host_common.h"
#include "host_scenes.h"
#include "kernels.h"

using namespace cmag;

namespace {

struct BatchScene {
    cmag_sph_params p{};
    uint32_t n = 0;
    uint32_t user = 0;             // the caller's scene index
    uint32_t part_base = 0;
    uint32_t table_base = 0;
    uint32_t table_cells = 0;      // reserved at creation
    bool planar_slot = false;      // table sized for one z layer
    SceneLayout lay;
    bool z_uniform = true;
    float z_value = 0.0f;
    float elapsed = 0.0f;
    PhaseState host_phase{};
    uint32_t group = 0;
    uint32_t mark_base = 0;        // DamBreak: first word of its cell-block stamps
    uint32_t nb[3] = {0, 0, 0};    // 4x4x4 cell blocks per axis
};

struct LaunchGroup {
    uint32_t slot_first = 0, slot_end = 0;   // scenes [slot_first, slot_end)
    uint32_t first = 0, count = 0;           // particles
    int32_t system = 0;
    bool planar = false, trim = false;
    uint32_t bucket = 0;
    int g_density = 1, g_force = 1;
    bool lists = false;  // interaction lists (one lane per particle)
    cudaStream_t side = nullptr;
    cudaEvent_t done = nullptr;
};

constexpr int kMaxSideStreams = 8;

}  // namespace

struct cmag_batch {
    std::vector<BatchScene> sc;          // slot order (grouped)
    std::vector<uint32_t> slot_of_user;
    std::vector<LaunchGroup> groups;
    std::vector<DevParams> host_dev;     // per slot
    uint32_t n_total = 0;
    uint32_t table_total = 0;
    bool any_peristalsis = false;
    float k_milli = 0.0f;

    cudaStream_t own_stream = nullptr, stream = nullptr;
    std::vector<cudaStream_t> side;
    cudaEvent_t fork = nullptr;

    float4 *pos = nullptr, *vel = nullptr, *vlf = nullptr, *meas = nullptr, *acc = nullptr,
           *vforce = nullptr, *pforce = nullptr, *pred = nullptr, *spos = nullptr, *svel = nullptr;
    uint32_t *hash[2] = {nullptr, nullptr}, *idx[2] = {nullptr, nullptr};
    // interaction lists of the groups that use them: entry k of particle i at
    // nl_entry[k * n_total + i] (allocated when the autotuner first tries them)
    uint32_t *nl_entry = nullptr, *nl_count = nullptr;
    uint32_t nl_cap = 0;
    uint32_t *cnt = nullptr, *off = nullptr, *ws = nullptr, *err = nullptr, *red = nullptr;
    size_t ws_words = 0;
    float2 *aux = nullptr;
    PhaseState *phase = nullptr;
    DevParams *dev = nullptr;
    uint16_t *scene_of = nullptr;
    // kept densities of dam-break walls (DevParams::wc_*; one epoch for the batch)
    float4 *wc_entry = nullptr, *wc_snap = nullptr;
    uint32_t *wc_mark = nullptr, *wc_state = nullptr;
    uint64_t wc_marks = 0;
    bool wc_on = false;
    float2 *zexpect = nullptr;  // whole-batch uploads: z each planar slot must keep
    uint32_t *zflags = nullptr;
    bool dev_dirty = true;

    bool use_graphs = true;
    uint32_t graph_steps = 1;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // 1 step, graph_steps steps
    uint32_t gsteps[2] = {0, 0};
    int last_stage = CMAG_STAGE_INTEGRATE;

    bool timing = false;
    std::vector<cudaEvent_t> events;
    size_t events_used = 0;
    double stage_ms[6] = {0, 0, 0, 0, 0, 0};
    uint32_t timed_steps = 0;

    std::string last_error;
};

namespace {

int bfail(cmag_batch *b, int code, const std::string &msg)
{
    if (b) b->last_error = msg;
    set_last_error(msg);
    return code;
}

#define CB_CUDA(b, call)                                                                    \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            (void)cudaGetLastError();                                                       \
            return bfail((b), e_ == cudaErrorMemoryAllocation ? CMAG_ERR_NOMEM : CMAG_ERR_CUDA, \
                         std::string(#call) + ": " + cudaGetErrorString(e_));               \
        }                                                                                   \
    } while (0)

// factor-4 size classes: bucket k holds 2^(2k-1) < n <= 2^(2k+1)
uint32_t size_bucket(uint32_t n) { return log2u(n) / 2; }

bool planar_slot_for(const cmag_sph_params &p) { return planar_allowed(p, true, false); }

// The kept wall densities are stale: the next step's scan starts a new epoch.
void wall_cache_reset(cmag_batch *b)
{
    if (b->wc_state &&
        cudaMemsetAsync(b->wc_state + kWcMoved, 0x01, sizeof(uint32_t), b->stream) != cudaSuccess)
        (void)cudaGetLastError();
}

// lanes, lists or streams changed: the captured steps are re-recorded and the
// kept wall densities recomputed
void invalidate_graphs(cmag_batch *b)
{
    for (int k = 0; k < 2; ++k) {
        if (b->gexec[k]) cudaGraphExecDestroy(b->gexec[k]);
        b->gexec[k] = nullptr;
        b->gsteps[k] = 0;
    }
    wall_cache_reset(b);
}

DevParams scene_dev(const cmag_batch *b, const BatchScene &s)
{
    DevParams d = make_dev_params(s.p, s.n, s.lay);
    d.table_base = s.table_base;
    d.part_base = s.part_base;
    if (b->wc_on && b->wc_entry && s.p.system == CMAG_DAMBREAK) {
        d.wc_entry = b->wc_entry;  // original order of the whole batch
        d.wc_snap = b->wc_snap;
        d.wc_mark = b->wc_mark + s.mark_base;
        d.wc_state = b->wc_state;
        d.wc_idx = b->idx[0];  // the counting sort's sorted -> original index
        d.wc_nbx = s.nb[0];
        d.wc_nby = s.nb[1];
        d.wc_nbz = s.nb[2];
    }
    return d;
}

// parameters changed (in any scene): upload them, recompute kept wall densities
void refresh_dev(cmag_batch *b)
{
    for (size_t k = 0; k < b->sc.size(); ++k) b->host_dev[k] = scene_dev(b, b->sc[k]);
    b->dev_dirty = true;
    wall_cache_reset(b);
}

int upload_dev(cmag_batch *b)
{
    if (!b->dev_dirty) return CMAG_OK;
    CB_CUDA(b, cudaMemcpyAsync(b->dev, b->host_dev.data(), sizeof(DevParams) * b->host_dev.size(),
                               cudaMemcpyHostToDevice, b->stream));
    CB_CUDA(b, cudaStreamSynchronize(b->stream));
    b->dev_dirty = false;
    return CMAG_OK;
}

int upload_phase(cmag_batch *b)
{
    std::vector<PhaseState> ph(b->sc.size());
    for (size_t k = 0; k < b->sc.size(); ++k) ph[k] = b->sc[k].host_phase;
    CB_CUDA(b, cudaMemcpyAsync(b->phase, ph.data(), sizeof(PhaseState) * ph.size(),
                               cudaMemcpyHostToDevice, b->stream));
    CB_CUDA(b, cudaStreamSynchronize(b->stream));
    return CMAG_OK;
}

BatchView view_of(const cmag_batch *b)
{
    BatchView v;
    v.scenes = b->dev;
    v.scene_of = b->scene_of;
    v.n_total = b->n_total;
    v.first = 0;
    v.count = b->n_total;
    return v;
}

// the counting sort's outputs (hash[0]: keys in particle order, idx[1]: scratch)
uint32_t *sorted_idx(cmag_batch *b) { return b->idx[0]; }
uint32_t *sorted_hash(cmag_batch *b) { return b->hash[1]; }

int ensure_events(cmag_batch *b, size_t count)
{
    while (b->events.size() < count) {
        cudaEvent_t e;
        CB_CUDA(b, cudaEventCreate(&e));
        b->events.push_back(e);
    }
    return CMAG_OK;
}

NeighborList lists_of(const cmag_batch *b)
{
    NeighborList nl{};
    if (b->nl_entry) {
        nl.entry = b->nl_entry;
        nl.count = b->nl_count;
        nl.cap = b->nl_cap;
        nl.stride = b->n_total;
    }
    return nl;
}

void free_lists(cmag_batch *b)
{
    if (b->nl_entry) cudaFree(b->nl_entry);
    if (b->nl_count) cudaFree(b->nl_count);
    b->nl_entry = b->nl_count = nullptr;
    b->nl_cap = 0;
    for (LaunchGroup &g : b->groups) g.lists = false;
}

// Lists for every particle of the batch, with room for the largest per-scene
// capacity; returns false when they cannot be had (too many particles or no memory).
bool alloc_lists(cmag_batch *b)
{
    if (b->nl_entry) return true;
    if (b->n_total >= (1u << kListIndexBits)) return false;
    uint32_t cap = 0;
    for (size_t k = 0; k < b->sc.size(); ++k) cap = std::max(cap, list_cap(b->sc[k].p, b->host_dev[k].trim != 0));
    cudaError_t e = cudaMalloc((void **)&b->nl_entry, sizeof(uint32_t) * (size_t)cap * b->n_total);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->nl_count, sizeof(uint32_t) * (size_t)b->n_total);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        free_lists(b);
        return false;
    }
    b->nl_cap = cap;
    return true;
}

// Neighbour-loop launches of every group.  Consecutive groups that run the same
// kernel variant (family, search shape, lanes per particle, lists) are one launch
// over their joined particle range: every particle reads its own scene's
// parameters, so merging changes no result.  Launches after the first run on side
// streams forked from the main stream and joined before the next stage.
int launch_groups(cmag_batch *b, bool force)
{
    cudaStream_t st = b->stream;
    const BatchView base = view_of(b);
    const size_t ng = b->groups.size();
    auto same_variant = [&](const LaunchGroup &a, const LaunchGroup &c) {
        return a.system == c.system && a.planar == c.planar && a.trim == c.trim && a.lists == c.lists &&
               (force ? a.g_force == c.g_force : a.g_density == c.g_density) && a.first + a.count == c.first;
    };
    std::vector<std::pair<size_t, size_t>> runs;  // [first group, end group)
    for (size_t g = 0; g < ng;) {
        size_t e = g + 1;
        while (e < ng && same_variant(b->groups[e - 1], b->groups[e])) ++e;
        runs.emplace_back(g, e);
        g = e;
    }
    if (runs.size() > 1) CB_CUDA(b, cudaEventRecord(b->fork, st));
    for (size_t r = 0; r < runs.size(); ++r) {
        LaunchGroup &lg = b->groups[runs[r].first];
        const LaunchGroup &last = b->groups[runs[r].second - 1];
        cudaStream_t gs = (r == 0) ? st : lg.side;
        if (r > 0) CB_CUDA(b, cudaStreamWaitEvent(gs, b->fork, 0));
        BatchView v = base;
        v.first = lg.first;
        v.count = last.first + last.count - lg.first;
        const DevParams &rep = b->host_dev[lg.slot_first];
        const NeighborList nl = lg.lists ? lists_of(b) : NeighborList{};
        if (force) {
            const bool per = lg.system == CMAG_PERISTALSIS;
            launch_force(rep, v, lg.g_force, b->spos, b->svel, b->aux, sorted_idx(b), b->off,
                         per ? b->vforce : b->acc, per ? b->pforce : nullptr, b->phase, nl, gs);
        } else {
            launch_density(rep, v, lg.g_density, b->spos, b->off, b->meas, b->aux, nl, gs);
        }
        if (r > 0) {
            CB_CUDA(b, cudaEventRecord(lg.done, gs));
            CB_CUDA(b, cudaStreamWaitEvent(st, lg.done, 0));
        }
    }
    return CMAG_OK;
}

int record_step(cmag_batch *b, int last, bool timed)
{
    cudaStream_t st = b->stream;
    const BatchView v = view_of(b);
    const DevParams &rep = b->host_dev[0];
    cudaEvent_t *ev = nullptr;
    if (timed) {
        if (ensure_events(b, b->events_used + 7) != CMAG_OK) return CMAG_ERR_CUDA;
        ev = &b->events[b->events_used];
        b->events_used += 7;
    }
    auto mark = [&](int k) { if (ev) cudaEventRecord(ev[k], st); };
    // Peristalsis scenes: this step's phase blocks (walls configured in the hash pass)
    if (b->any_peristalsis) launch_phase_batch(b->dev, (uint32_t)b->sc.size(), b->phase, b->k_milli, st);
    mark(0);
    // keys = table slots: hash + counts + arrival ranks, offsets, counting sort
    launch_hash(rep, v, b->pos, b->hash[0], b->cnt, b->idx[0], b->err, st, nullptr,
                b->any_peristalsis ? b->phase : nullptr);
    launch_cell_scan(b->cnt, b->off, b->table_total + 1, b->ws, st, b->wc_on ? b->wc_state : nullptr);
    mark(1);
    if (last >= CMAG_STAGE_SORT)
        launch_cell_sort(b->hash[0], b->idx[0], b->off, 0u, b->n_total, b->hash[1], b->idx[1],
                         b->idx[0], b->pos, b->vlf, b->spos, b->svel, b->err, st);
    mark(2);
    // (the gather of sorted positions and velocities ran with the sort)
    mark(3);
    if (last >= CMAG_STAGE_DENSITY) {
        int rc = launch_groups(b, false);
        if (rc) return rc;
    }
    mark(4);
    if (last >= CMAG_STAGE_FORCE) {
        int rc = launch_groups(b, true);
        if (rc) return rc;
    }
    mark(5);
    if (last >= CMAG_STAGE_INTEGRATE)
        launch_integrate(rep, v, b->pos, b->vel, b->vlf, b->acc, b->vforce, b->pforce, b->phase, st);
    mark(6);
    CB_CUDA(b, cudaGetLastError());
    return CMAG_OK;
}

// host mirrors of the per-scene time and Peristalsis phase (k_phase)
void advance_host(cmag_batch *b)
{
    for (BatchScene &s : b->sc) {
        const float dt = s.p.delta_time;
        if (s.p.system == CMAG_PERISTALSIS) {
            PhaseState &h = s.host_phase;
            h.configure = 0;
            if (h.is_bc) {
                h.time_shift = h.time_shift + dt;
                if (h.wave_height < s.p.amplitude) {
                    h.configure = 1;
                    h.configure_height = h.wave_height;
                    h.wave_height = h.wave_height + dt * b->k_milli;
                } else {
                    h.time_relax = h.time_relax - dt;
                    if (h.time_relax < 0.0f) h.is_bc = 0;
                }
            }
            h.t = h.is_bc ? 0.0f : h.elapsed - h.time_shift;
            h.elapsed = h.elapsed + dt;
            s.p.is_boundary_configuration = h.is_bc;
            s.elapsed = h.elapsed;
        } else {
            s.elapsed = s.elapsed + dt;
        }
    }
}

int capture(cmag_batch *b, int which, uint32_t steps)
{
    if (b->gexec[which]) cudaGraphExecDestroy(b->gexec[which]);
    b->gexec[which] = nullptr;
    cudaStream_t st = b->stream;
    CB_CUDA(b, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = CMAG_OK;
    for (uint32_t k = 0; k < steps && rc == CMAG_OK; ++k) rc = record_step(b, CMAG_STAGE_INTEGRATE, false);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != CMAG_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return bfail(b, CMAG_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->gexec[which], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, CMAG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    b->gsteps[which] = steps;
    return CMAG_OK;
}

// advance `steps` steps: whole multi-step graphs first, then single-step ones
int do_steps(cmag_batch *b, uint32_t steps)
{
    int rc = upload_dev(b);
    if (rc) return rc;
    const bool graphs = b->use_graphs && !b->timing;
    while (steps > 0) {
        if (graphs) {
            const int which = (b->graph_steps > 1 && steps >= b->graph_steps) ? 1 : 0;
            const uint32_t k = which ? b->graph_steps : 1;
            if (!b->gexec[which] || b->gsteps[which] != k)
                if ((rc = capture(b, which, k))) return rc;
            CB_CUDA(b, cudaGraphLaunch(b->gexec[which], b->stream));
            for (uint32_t j = 0; j < k; ++j) advance_host(b);
            steps -= k;
        } else {
            if ((rc = record_step(b, CMAG_STAGE_INTEGRATE, b->timing))) return rc;
            if (b->timing) b->timed_steps++;
            advance_host(b);
            steps -= 1;
        }
    }
    b->last_stage = CMAG_STAGE_INTEGRATE;
    return CMAG_OK;
}

void free_all(cmag_batch *b)
{
    invalidate_graphs(b);
    for (auto e : b->events) cudaEventDestroy(e);
    b->events.clear();
    for (auto &g : b->groups)
        if (g.done) cudaEventDestroy(g.done);
    if (b->fork) cudaEventDestroy(b->fork);
    for (auto s : b->side) cudaStreamDestroy(s);
    void *ptrs[] = {b->pos, b->vel, b->vlf, b->meas, b->acc, b->vforce, b->pforce, b->pred,
                    b->spos, b->svel, b->hash[0], b->hash[1], b->idx[0], b->idx[1], b->cnt,
                    b->off, b->ws, b->err, b->red, b->aux, b->phase, b->dev, b->scene_of,
                    b->zexpect, b->zflags, b->wc_entry, b->wc_snap, b->wc_mark, b->wc_state};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    free_lists(b);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
}

template <class T>
int dalloc(cmag_batch *b, T **ptr, size_t bytes)
{
    CB_CUDA(b, cudaMalloc((void **)ptr, bytes));
    CB_CUDA(b, cudaMemset(*ptr, 0, bytes));
    return CMAG_OK;
}

float4 *float_array(cmag_batch *b, int a)
{
    switch (a) {
    case CMAG_POSITION: return b->pos;
    case CMAG_VELOCITY: return b->vel;
    case CMAG_MEASURES: return b->meas;
    case CMAG_ACCELERATION: return b->acc;
    case CMAG_VELOCITYLEAPFROG: return b->vlf;
    case CMAG_VISCOUSFORCE: return b->vforce;
    case CMAG_PRESSUREFORCE: return b->pforce;
    case CMAG_PREDICTEDPOSITION: return b->pred;
    case CMAG_SORTEDPOSITION: return b->spos;
    case CMAG_SORTEDVELOCITY: return b->svel;
    default: return nullptr;
    }
}

int scene_slot(cmag_batch *b, uint32_t scene, BatchScene **out)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (scene >= b->slot_of_user.size())
        return bfail(b, CMAG_ERR_INVALID, "scene " + std::to_string(scene) + " out of range");
    *out = &b->sc[b->slot_of_user[scene]];
    return CMAG_OK;
}

int check_range(cmag_batch *b, uint32_t start, uint32_t count, uint64_t size)
{
    if ((uint64_t)start + count > size)
        return bfail(b, CMAG_ERR_INVALID, "array range [" + std::to_string(start) + ", " +
                                              std::to_string((uint64_t)start + count) +
                                              ") exceeds " + std::to_string(size));
    return CMAG_OK;
}

int set_scene_positions_check(cmag_batch *b, BatchScene &s, const float *host, uint32_t start,
                              uint32_t count)
{
    if (!s.planar_slot || count == 0) return CMAG_OK;
    const float z0 = host[2];
    for (uint32_t i = 0; i < count; ++i)
        if (host[4 * (size_t)i + 2] != z0)
            return bfail(b, CMAG_ERR_INVALID, "a planar 2-D batch scene keeps every particle at one z");
    if (!(start == 0 && count == s.n) && z0 != s.z_value && s.z_uniform)
        return bfail(b, CMAG_ERR_INVALID, "a planar 2-D batch scene keeps every particle at one z");
    return CMAG_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================

extern "C" {

int cmag_batch_create(const cmag_sph_params *params, const uint32_t *counts, uint32_t scenes,
                      cmag_batch **out)
{
    if (!params || !counts || !out) return bfail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (scenes == 0 || scenes > 65535) return bfail(nullptr, CMAG_ERR_INVALID, "scene count must be in [1, 65535]");
    uint64_t total = 0;
    for (uint32_t k = 0; k < scenes; ++k) {
        std::string why;
        if (validate_params(params[k], counts[k], why))
            return bfail(nullptr, CMAG_ERR_INVALID, "scene " + std::to_string(k) + ": " + why);
        total += counts[k];
    }
    if (total >= (1u << 30)) return bfail(nullptr, CMAG_ERR_INVALID, "more than 2^30 particles in the batch");
    cmag_batch *b = new (std::nothrow) cmag_batch();
    if (!b) return bfail(nullptr, CMAG_ERR_NOMEM, "host allocation failed");
    b->k_milli = std::pow(10.0f, -3.0f);

    // slot order: family, search shape, size bucket, then the caller's order
    std::vector<BatchScene> tmp(scenes);
    for (uint32_t k = 0; k < scenes; ++k) {
        BatchScene &s = tmp[k];
        s.p = params[k];
        s.n = counts[k];
        s.user = k;
        s.planar_slot = planar_slot_for(s.p);
        s.lay = layout_for(s.p, s.planar_slot, 0.0f);
        s.table_cells = s.lay.scan_cells;
        s.host_phase.is_bc = s.p.is_boundary_configuration;
        s.host_phase.time_relax = 1000 * s.p.delta_time;
    }
    auto key = [&](const BatchScene &s) {
        const DevParams d = make_dev_params(s.p, s.n, s.lay);
        return std::make_tuple(s.p.system, (int)s.planar_slot, d.trim, size_bucket(s.n), s.user);
    };
    std::stable_sort(tmp.begin(), tmp.end(), [&](const BatchScene &x, const BatchScene &y) { return key(x) < key(y); });
    b->sc = tmp;
    b->slot_of_user.assign(scenes, 0);
    uint64_t part = 0, table = 0;
    for (uint32_t k = 0; k < scenes; ++k) {
        BatchScene &s = b->sc[k];
        b->slot_of_user[s.user] = k;
        s.part_base = (uint32_t)part;
        s.table_base = (uint32_t)table;
        part += s.n;
        table += s.table_cells;
        if (s.p.system == CMAG_PERISTALSIS) b->any_peristalsis = true;
        if (s.p.system == CMAG_DAMBREAK) {
            s.mark_base = (uint32_t)b->wc_marks;
            for (int a = 0; a < 3; ++a) s.nb[a] = (s.p.grid_size[a] + 3u) / 4u;
            b->wc_marks += (uint64_t)s.nb[0] * s.nb[1] * s.nb[2];
        }
    }
    if (b->wc_marks >= (1ull << 32)) {
        delete b;
        return bfail(nullptr, CMAG_ERR_INVALID, "the dam-break scenes' cell blocks exceed 2^32");
    }
    if (table >= (1ull << 32) - 1) {
        delete b;
        return bfail(nullptr, CMAG_ERR_INVALID, "the scenes' cell tables exceed 2^32 cells");
    }
    b->n_total = (uint32_t)part;
    b->table_total = (uint32_t)table;
    // launch groups: runs of scenes with equal (family, shape, trim, bucket)
    for (uint32_t k = 0; k < scenes; ++k) {
        const BatchScene &s = b->sc[k];
        const DevParams d = make_dev_params(s.p, s.n, s.lay);
        const bool same = !b->groups.empty() && b->groups.back().system == s.p.system &&
                          b->groups.back().planar == s.planar_slot && b->groups.back().trim == (d.trim != 0) &&
                          b->groups.back().bucket == size_bucket(s.n);
        if (!same) {
            LaunchGroup g;
            g.slot_first = k;
            g.first = s.part_base;
            g.system = s.p.system;
            g.planar = s.planar_slot;
            g.trim = d.trim != 0;
            g.bucket = size_bucket(s.n);
            g.g_density = g.g_force = (s.p.dims == 3) ? 2 : 1;
            b->groups.push_back(g);
        }
        LaunchGroup &g = b->groups.back();
        g.slot_end = k + 1;
        g.count = s.part_base + s.n - g.first;
        b->sc[k].group = (uint32_t)(b->groups.size() - 1);
    }
    b->host_dev.resize(scenes);
    refresh_dev(b);

    int rc = CMAG_OK;
    auto step = [&](int r) { if (rc == CMAG_OK) rc = r; };
    auto cuda = [&](cudaError_t e, const char *what) {
        if (rc == CMAG_OK && e != cudaSuccess) {
            (void)cudaGetLastError();
            rc = bfail(b, CMAG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
        }
    };
    cuda(cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    b->stream = b->own_stream;
    cuda(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate");
    const size_t ng = b->groups.size();
    for (size_t g = 1; g < ng && rc == CMAG_OK; ++g) {
        if (b->side.size() < std::min<size_t>(ng - 1, kMaxSideStreams)) {
            cudaStream_t s = nullptr;
            cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
            if (s) b->side.push_back(s);
        }
        if (!b->side.empty()) b->groups[g].side = b->side[(g - 1) % b->side.size()];
        cuda(cudaEventCreateWithFlags(&b->groups[g].done, cudaEventDisableTiming), "cudaEventCreate");
    }
    const size_t n = b->n_total;
    const size_t f4 = sizeof(float4) * n, u4 = sizeof(uint32_t) * n;
    if (rc == CMAG_OK) {
        step(dalloc(b, &b->pos, f4));
        step(dalloc(b, &b->vel, f4));
        step(dalloc(b, &b->vlf, f4));
        step(dalloc(b, &b->meas, f4));
        step(dalloc(b, &b->acc, f4));
        step(dalloc(b, &b->spos, f4));
        step(dalloc(b, &b->svel, f4));
        step(dalloc(b, &b->aux, sizeof(float2) * n));
        if (b->any_peristalsis) {
            step(dalloc(b, &b->vforce, f4));
            step(dalloc(b, &b->pforce, f4));
            step(dalloc(b, &b->pred, f4));
        }
        for (int k = 0; k < 2; ++k) {
            step(dalloc(b, &b->hash[k], u4));
            step(dalloc(b, &b->idx[k], u4));
        }
        step(dalloc(b, &b->cnt, sizeof(uint32_t) * ((size_t)b->table_total + 1)));
        step(dalloc(b, &b->off, sizeof(uint32_t) * ((size_t)b->table_total + 1)));
        b->ws_words = cell_scan_workspace_words(b->table_total + 1);
        step(dalloc(b, &b->ws, sizeof(uint32_t) * b->ws_words));
        step(dalloc(b, &b->err, sizeof(uint32_t)));
        step(dalloc(b, &b->red, sizeof(uint32_t) * 6 * (size_t)scenes));
        step(dalloc(b, &b->phase, sizeof(PhaseState) * (size_t)scenes));
        step(dalloc(b, &b->dev, sizeof(DevParams) * (size_t)scenes));
        step(dalloc(b, &b->scene_of, sizeof(uint16_t) * n));
        step(dalloc(b, &b->zexpect, sizeof(float2) * (size_t)scenes));
        step(dalloc(b, &b->zflags, sizeof(uint32_t) * (size_t)scenes));
    }
    if (rc == CMAG_OK && b->wc_marks) {
        // kept wall densities: an optimisation, so the batch is made without them
        // when their memory cannot be had
        void **bufs[4] = {(void **)&b->wc_entry, (void **)&b->wc_snap, (void **)&b->wc_mark, (void **)&b->wc_state};
        const size_t sizes[4] = {f4, f4, sizeof(uint32_t) * b->wc_marks, 4 * sizeof(uint32_t)};
        bool ok = true;
        for (int k = 0; k < 4 && ok; ++k)
            ok = cudaMalloc(bufs[k], sizes[k]) == cudaSuccess && cudaMemset(*bufs[k], 0, sizes[k]) == cudaSuccess;
        if (!ok) {
            (void)cudaGetLastError();
            for (int k = 0; k < 4; ++k) {
                if (*bufs[k]) cudaFree(*bufs[k]);
                *bufs[k] = nullptr;
            }
        }
        b->wc_on = ok;
    }
    // the clears above ran on the legacy stream, which the batch's non-blocking
    // stream does not wait for
    if (rc == CMAG_OK) cuda(cudaStreamSynchronize(cudaStreamLegacy), "cudaStreamSynchronize");
    if (rc == CMAG_OK) {
        std::vector<uint16_t> so(n);
        for (uint32_t k = 0; k < scenes; ++k)
            std::fill(so.begin() + b->sc[k].part_base, so.begin() + b->sc[k].part_base + b->sc[k].n, (uint16_t)k);
        cudaError_t e = cudaMemcpy(b->scene_of, so.data(), sizeof(uint16_t) * n, cudaMemcpyHostToDevice);
        cuda(e, "cudaMemcpy");
    }
    if (rc == CMAG_OK) {
        refresh_dev(b);  // with the kept wall densities' arrays
        step(upload_dev(b));
    }
    if (rc == CMAG_OK) step(upload_phase(b));
    if (rc != CMAG_OK) {
        std::string msg = b->last_error;
        free_all(b);
        delete b;
        set_last_error(msg);
        return rc;
    }
    *out = b;
    return CMAG_OK;
}

int cmag_batch_destroy(cmag_batch *b)
{
    if (!b) return CMAG_OK;
    cudaStreamSynchronize(b->stream);
    free_all(b);
    delete b;
    return CMAG_OK;
}

int cmag_batch_num_scenes(const cmag_batch *b, uint32_t *out)
{
    if (!b || !out) return bfail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = (uint32_t)b->sc.size();
    return CMAG_OK;
}

int cmag_batch_num_particles(const cmag_batch *b, uint32_t *out)
{
    if (!b || !out) return bfail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = b->n_total;
    return CMAG_OK;
}

int cmag_batch_scene_range(cmag_batch *b, uint32_t scene, uint32_t *first, uint32_t *count)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (first) *first = s->part_base;
    if (count) *count = s->n;
    return CMAG_OK;
}

int cmag_batch_set_array(cmag_batch *b, uint32_t scene, int32_t array, const float *host,
                         uint32_t start, uint32_t count)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (!host && count) return bfail(b, CMAG_ERR_INVALID, "null argument");
    float4 *d = float_array(b, array);
    if (!d) return bfail(b, CMAG_ERR_INVALID, "not a settable float4 array: " + std::to_string(array));
    if (check_range(b, start, count, s->n) != CMAG_OK) return CMAG_ERR_INVALID;
    if (count == 0) return CMAG_OK;
    if (array == CMAG_POSITION && (rc = set_scene_positions_check(b, *s, host, start, count))) return rc;
    if ((array == CMAG_VELOCITY || array == CMAG_VELOCITYLEAPFROG) && s->planar_slot)
        for (uint32_t i = 0; i < count; ++i)
            if (host[4 * (size_t)i + 2] != 0.0f)
                return bfail(b, CMAG_ERR_INVALID, "a planar 2-D batch scene has no z velocity");
    CB_CUDA(b, cudaMemcpyAsync(d + s->part_base + start, host, sizeof(float4) * (size_t)count,
                               cudaMemcpyHostToDevice, b->stream));
    CB_CUDA(b, cudaStreamSynchronize(b->stream));
    if (array == CMAG_POSITION && s->planar_slot) {
        s->z_value = host[2];
        s->z_uniform = true;
        const SceneLayout l = layout_for(s->p, true, s->z_value);
        if (l.scan_base != s->lay.scan_base) {
            s->lay = l;
            refresh_dev(b);
        }
    }
    return CMAG_OK;
}

int cmag_batch_get_array(cmag_batch *b, uint32_t scene, int32_t array, float *host,
                         uint32_t start, uint32_t count)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (!host && count) return bfail(b, CMAG_ERR_INVALID, "null argument");
    float4 *d = float_array(b, array);
    if (!d) return bfail(b, CMAG_ERR_INVALID, "not a float4 array: " + std::to_string(array));
    if (check_range(b, start, count, s->n) != CMAG_OK) return CMAG_ERR_INVALID;
    if (count == 0) return CMAG_OK;
    CB_CUDA(b, cudaMemcpyAsync(host, d + s->part_base + start, sizeof(float4) * (size_t)count,
                               cudaMemcpyDeviceToHost, b->stream));
    CB_CUDA(b, cudaStreamSynchronize(b->stream));
    return CMAG_OK;
}

// Every scene's array in one call: one asynchronous copy per scene, one
// synchronisation, and the planar scenes' z checks on the device.
int cmag_batch_set_array_all(cmag_batch *b, int32_t array, const float *host)
{
    if (!b || !host) return bfail(b, CMAG_ERR_INVALID, "null argument");
    float4 *d = float_array(b, array);
    if (!d) return bfail(b, CMAG_ERR_INVALID, "not a settable float4 array: " + std::to_string(array));
    cudaStream_t st = b->stream;
    const bool pos_up = array == CMAG_POSITION;
    const bool vel_up = array == CMAG_VELOCITY || array == CMAG_VELOCITYLEAPFROG;
    std::vector<float2> expect(b->sc.size(), make_float2(0.0f, 0.0f));
    bool check = false;
    size_t row = 0;
    for (size_t k = 0; k < b->slot_of_user.size(); ++k) {
        const BatchScene &s = b->sc[b->slot_of_user[k]];
        CB_CUDA(b, cudaMemcpyAsync(d + s.part_base, host + 4 * row, sizeof(float4) * (size_t)s.n,
                                   cudaMemcpyHostToDevice, st));
        if (s.planar_slot && (pos_up || vel_up)) {
            expect[b->slot_of_user[k]] = make_float2(pos_up ? host[4 * row + 2] : 0.0f, 1.0f);
            check = true;
        }
        row += s.n;
    }
    std::vector<uint32_t> flags(b->sc.size(), 0u);
    if (check) {
        CB_CUDA(b, cudaMemcpyAsync(b->zexpect, expect.data(), sizeof(float2) * expect.size(),
                                   cudaMemcpyHostToDevice, st));
        launch_z_differs_slots(d, b->scene_of, b->n_total, b->zexpect, b->zflags, (uint32_t)flags.size(), st);
        CB_CUDA(b, cudaGetLastError());
        CB_CUDA(b, cudaMemcpyAsync(flags.data(), b->zflags, sizeof(uint32_t) * flags.size(),
                                   cudaMemcpyDeviceToHost, st));
    }
    CB_CUDA(b, cudaStreamSynchronize(st));
    for (size_t k = 0; k < b->slot_of_user.size(); ++k)
        if (flags[b->slot_of_user[k]])
            return bfail(b, CMAG_ERR_INVALID,
                         std::string("scene ") + std::to_string(k) +
                             (pos_up ? ": a planar 2-D batch scene keeps every particle at one z"
                                     : ": a planar 2-D batch scene has no z velocity") +
                             " (the array holds the new data; set it again)");
    if (pos_up) {
        bool moved = false;
        for (size_t slot = 0; slot < b->sc.size(); ++slot) {
            BatchScene &s = b->sc[slot];
            if (!s.planar_slot) continue;
            s.z_value = expect[slot].x;
            s.z_uniform = true;
            const SceneLayout l = layout_for(s.p, true, s.z_value);
            if (l.scan_base != s.lay.scan_base) {
                s.lay = l;
                moved = true;
            }
        }
        if (moved) refresh_dev(b);
    }
    return CMAG_OK;
}

int cmag_batch_get_array_all(cmag_batch *b, int32_t array, float *host)
{
    if (!b || !host) return bfail(b, CMAG_ERR_INVALID, "null argument");
    float4 *d = float_array(b, array);
    if (!d) return bfail(b, CMAG_ERR_INVALID, "not a float4 array: " + std::to_string(array));
    size_t row = 0;
    for (size_t k = 0; k < b->slot_of_user.size(); ++k) {
        const BatchScene &s = b->sc[b->slot_of_user[k]];
        CB_CUDA(b, cudaMemcpyAsync(host + 4 * row, d + s.part_base, sizeof(float4) * (size_t)s.n,
                                   cudaMemcpyDeviceToHost, b->stream));
        row += s.n;
    }
    CB_CUDA(b, cudaStreamSynchronize(b->stream));
    return CMAG_OK;
}

// Scene-local views: HASH = the reference hash (cell index in the scene's grid),
// INDEX = scene-local original index, CELLOFFSET = scene-local offsets over the
// scene's table, CELLSTART/CELLEND = the reference arrays over the scene's grid.
int cmag_batch_get_uint_array(cmag_batch *b, uint32_t scene, int32_t array, uint32_t *host,
                              uint32_t start, uint32_t count)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (!host && count) return bfail(b, CMAG_ERR_INVALID, "null argument");
    cudaStream_t st = b->stream;
    const bool before_sort = b->last_stage == CMAG_STAGE_HASH;
    switch (array) {
    case CMAG_HASH:
    case CMAG_INDEX: {
        if (check_range(b, start, count, s->n) != CMAG_OK) return CMAG_ERR_INVALID;
        if (count == 0) return CMAG_OK;
        if (array == CMAG_INDEX && before_sort) {
            for (uint32_t i = 0; i < count; ++i) host[i] = start + i;
            return CMAG_OK;
        }
        const uint32_t *src = (array == CMAG_HASH) ? (before_sort ? b->hash[0] : sorted_hash(b)) : sorted_idx(b);
        CB_CUDA(b, cudaMemcpyAsync(host, src + s->part_base + start, sizeof(uint32_t) * (size_t)count,
                                   cudaMemcpyDeviceToHost, st));
        CB_CUDA(b, cudaStreamSynchronize(st));
        const uint32_t shift = (array == CMAG_HASH) ? s->table_base - s->lay.scan_base : s->part_base;
        for (uint32_t i = 0; i < count; ++i) host[i] -= shift;
        return CMAG_OK;
    }
    case CMAG_CELLOFFSET:
    case CMAG_CELLSTART:
    case CMAG_CELLEND: {
        std::vector<uint32_t> off((size_t)s->lay.scan_cells + 1);
        CB_CUDA(b, cudaMemcpyAsync(off.data(), b->off + s->table_base, sizeof(uint32_t) * off.size(),
                                   cudaMemcpyDeviceToHost, st));
        CB_CUDA(b, cudaStreamSynchronize(st));
        for (auto &o : off) o -= s->part_base;
        if (array == CMAG_CELLOFFSET) {
            if (check_range(b, start, count, off.size()) != CMAG_OK) return CMAG_ERR_INVALID;
            std::memcpy(host, off.data() + start, sizeof(uint32_t) * (size_t)count);
            return CMAG_OK;
        }
        const uint64_t ncells = (uint64_t)s->p.grid_size[0] * s->p.grid_size[1] * s->p.grid_size[2];
        if (check_range(b, start, count, ncells) != CMAG_OK) return CMAG_ERR_INVALID;
        for (uint32_t i = 0; i < count; ++i) {
            const uint64_t c = (uint64_t)start + i;
            uint32_t a = 0, e = 0;
            if (c >= s->lay.scan_base && c - s->lay.scan_base < s->lay.scan_cells) {
                a = off[c - s->lay.scan_base];
                e = off[c - s->lay.scan_base + 1];
            }
            const bool occ = e > a;
            host[i] = (array == CMAG_CELLSTART) ? (occ ? a : kEmptyCell) : (occ ? e : 0u);
        }
        return CMAG_OK;
    }
    default: return bfail(b, CMAG_ERR_INVALID, "not a uint32 array: " + std::to_string(array));
    }
}

void *cmag_batch_device_array(cmag_batch *b, int32_t array)
{
    if (!b) return nullptr;
    switch (array) {
    case CMAG_HASH: return sorted_hash(b);
    case CMAG_INDEX: return sorted_idx(b);
    case CMAG_CELLOFFSET: return b->off;
    default: return float_array(b, array);
    }
}

int cmag_batch_reset_scene(cmag_batch *b, uint32_t scene)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    const uint32_t want = reference_particle_count(s->p);
    if (want != s->n)
        return bfail(b, CMAG_ERR_STATE, "scene " + std::to_string(scene) + " holds " + std::to_string(s->n) +
                                            " particles, the reference scene has " + std::to_string(want));
    std::vector<float> pos((size_t)s->n * 4, 0.0f), zero((size_t)s->n * 4, 0.0f),
        meas((size_t)s->n * 4, 0.0f);
    reference_scene(s->p, pos.data(), s->n);
    if (s->p.system != CMAG_PERISTALSIS)  // fluidSystem.cpp:131-132
        for (uint32_t i = 0; i < s->n; ++i) meas[4 * (size_t)i] = s->p.rest_density;
    if ((rc = cmag_batch_set_array(b, scene, CMAG_POSITION, pos.data(), 0, s->n))) return rc;
    for (int a : {CMAG_VELOCITY, CMAG_ACCELERATION, CMAG_VELOCITYLEAPFROG})
        if ((rc = cmag_batch_set_array(b, scene, a, zero.data(), 0, s->n))) return rc;
    if ((rc = cmag_batch_set_array(b, scene, CMAG_MEASURES, meas.data(), 0, s->n))) return rc;
    s->elapsed = 0.0f;
    if (s->p.system == CMAG_DAMBREAK) {  // fluidSystem.cpp:378-379
        const uint32_t gate_cells = (uint32_t)(s->p.boundary_offset + (int32_t)s->p.fluid_size[0]) * 2u;
        s->p.right_boundary = s->p.world_origin[0] + gate_cells * s->p.particle_radius;
    }
    if (s->p.system == CMAG_PERISTALSIS) {  // PeristalsisSystem.cpp:213-236
        for (int a : {CMAG_VISCOUSFORCE, CMAG_PRESSUREFORCE, CMAG_PREDICTEDPOSITION})
            if ((rc = cmag_batch_set_array(b, scene, a, zero.data(), 0, s->n))) return rc;
        s->host_phase = PhaseState{};
        s->host_phase.time_relax = 1000 * s->p.delta_time;
        s->host_phase.is_bc = 1;
        s->p.is_boundary_configuration = 1;
        s->p.particle_mass = s->p.rest_density / peristalsis_mass_sum(s->p, pos.data(), s->n);
        if ((rc = upload_phase(b))) return rc;
    }
    refresh_dev(b);
    return CMAG_OK;
}

int cmag_batch_reset(cmag_batch *b)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    for (uint32_t k = 0; k < b->sc.size(); ++k) {
        int rc = cmag_batch_reset_scene(b, k);
        if (rc) return rc;
    }
    return CMAG_OK;
}

int cmag_batch_get_params(cmag_batch *b, uint32_t scene, cmag_sph_params *out)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (!out) return bfail(b, CMAG_ERR_INVALID, "null argument");
    *out = s->p;
    return CMAG_OK;
}

int cmag_batch_set_params(cmag_batch *b, uint32_t scene, const cmag_sph_params *p)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (!p) return bfail(b, CMAG_ERR_INVALID, "null argument");
    std::string why;
    if (validate_params(*p, s->n, why)) return bfail(b, CMAG_ERR_INVALID, why);
    const DevParams now = make_dev_params(s->p, s->n, s->lay), next = make_dev_params(*p, s->n, s->lay);
    if (p->system != s->p.system || std::memcmp(p->grid_size, s->p.grid_size, sizeof(p->grid_size)) ||
        planar_slot_for(*p) != s->planar_slot || now.trim != next.trim)
        return bfail(b, CMAG_ERR_INVALID, "family, grid size and search shape of a batch scene are fixed at creation");
    s->p = *p;
    if (s->p.system == CMAG_PERISTALSIS && s->host_phase.is_bc != p->is_boundary_configuration) {
        s->host_phase.is_bc = p->is_boundary_configuration;
        if ((rc = upload_phase(b))) return rc;
    }
    if (s->planar_slot) s->lay = layout_for(s->p, true, s->z_value);
    refresh_dev(b);
    return CMAG_OK;
}

int cmag_batch_update(cmag_batch *b)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    return do_steps(b, 1);
}

int cmag_batch_update_n(cmag_batch *b, uint32_t steps)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    return do_steps(b, steps);
}

int cmag_batch_timed_update(cmag_batch *b, uint32_t steps, float *ms_out)
{
    if (!b || !ms_out) return bfail(b, CMAG_ERR_INVALID, "null argument");
    int rc = upload_dev(b);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    CB_CUDA(b, cudaEventCreate(&e0));
    CB_CUDA(b, cudaEventCreate(&e1));
    cudaEventRecord(e0, b->stream);
    rc = do_steps(b, steps);
    cudaEventRecord(e1, b->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != CMAG_OK) return rc;
    if (e != cudaSuccess) return bfail(b, CMAG_ERR_CUDA, std::string("timed update: ") + cudaGetErrorString(e));
    *ms_out = ms;
    return CMAG_OK;
}

int cmag_batch_run_stages(cmag_batch *b, int32_t last_stage)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (last_stage < CMAG_STAGE_HASH || last_stage > CMAG_STAGE_INTEGRATE)
        return bfail(b, CMAG_ERR_INVALID, "unknown stage");
    int rc = upload_dev(b);
    if (rc) return rc;
    if ((rc = record_step(b, last_stage, false))) return rc;
    b->last_stage = last_stage;
    if (last_stage == CMAG_STAGE_INTEGRATE) advance_host(b);
    else if (b->any_peristalsis && (rc = upload_phase(b))) return rc;
    CB_CUDA(b, cudaStreamSynchronize(b->stream));
    return CMAG_OK;
}

int cmag_batch_elapsed_time(cmag_batch *b, uint32_t scene, float *out)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (!out) return bfail(b, CMAG_ERR_INVALID, "null argument");
    *out = s->elapsed;
    return CMAG_OK;
}

int cmag_batch_dambreak_change_right_boundary(cmag_batch *b, uint32_t scene)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (s->p.system != CMAG_DAMBREAK) return bfail(b, CMAG_ERR_STATE, "not a dam-break scene");
    const float width = s->p.fluid_size[0] * 2 * s->p.particle_radius;
    s->p.right_boundary += width;  // fluidSystem.cpp:240
    launch_gate(make_dev_params(s->p, s->n, s->lay), b->pos + s->part_base, 0, width, 0.0f, 0.0f, b->stream);
    CB_CUDA(b, cudaGetLastError());
    refresh_dev(b);
    return CMAG_OK;
}

int cmag_batch_dambreak_remove_right_boundary(cmag_batch *b, uint32_t scene)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (s->p.system != CMAG_DAMBREAK) return bfail(b, CMAG_ERR_STATE, "not a dam-break scene");
    s->p.right_boundary = (float)0xffffffffu;  // fluidSystem.cpp:223
    const float fw = s->p.fluid_size[0] * 2 * s->p.particle_radius;
    const float fh = s->p.grid_size[1] * 2 * s->p.particle_radius;
    launch_gate(make_dev_params(s->p, s->n, s->lay), b->pos + s->part_base, 1, 0.0f, fw, fh, b->stream);
    CB_CUDA(b, cudaGetLastError());
    s->elapsed = 0.0f;
    refresh_dev(b);
    return CMAG_OK;
}

int cmag_batch_poiseuille_change_gravity(cmag_batch *b, uint32_t scene)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (s->p.system != CMAG_POISEUILLE) return bfail(b, CMAG_ERR_STATE, "not a Poiseuille scene");
    s->p.gravity[1] *= -1.0f;
    refresh_dev(b);
    return CMAG_OK;
}

int cmag_batch_fluid_extents(cmag_batch *b, float *lo, float *hi)
{
    if (!b || !lo || !hi) return bfail(b, CMAG_ERR_INVALID, "null argument");
    int rc = upload_dev(b);
    if (rc) return rc;
    const size_t S = b->sc.size();
    cudaStream_t st = b->stream;
    std::vector<uint32_t> init(6 * S);
    for (size_t k = 0; k < S; ++k)
        for (int j = 0; j < 6; ++j) init[6 * k + j] = j < 3 ? 0xffffffffu : 0u;
    CB_CUDA(b, cudaMemcpyAsync(b->red, init.data(), sizeof(uint32_t) * init.size(), cudaMemcpyHostToDevice, st));
    launch_fluid_extents_batch(view_of(b), b->pos, b->red, st);
    CB_CUDA(b, cudaGetLastError());
    std::vector<uint32_t> keys(6 * S);
    CB_CUDA(b, cudaMemcpyAsync(keys.data(), b->red, sizeof(uint32_t) * keys.size(), cudaMemcpyDeviceToHost, st));
    CB_CUDA(b, cudaStreamSynchronize(st));
    auto back = [](uint32_t k) {
        uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
        float f;
        std::memcpy(&f, &u, sizeof(f));
        return f;
    };
    for (size_t u = 0; u < S; ++u) {
        const size_t k = b->slot_of_user[u];
        for (int j = 0; j < 3; ++j) {
            lo[3 * u + j] = back(keys[6 * k + j]);
            hi[3 * u + j] = back(keys[6 * k + 3 + j]);
        }
    }
    return CMAG_OK;
}

int cmag_batch_set_stream(cmag_batch *b, void *cuda_stream)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    cudaStreamSynchronize(b->stream);
    b->stream = cuda_stream ? (cudaStream_t)cuda_stream : b->own_stream;
    invalidate_graphs(b);
    return CMAG_OK;
}

void *cmag_batch_stream(const cmag_batch *b) { return b ? (void *)b->stream : nullptr; }

int cmag_batch_set_graphs(cmag_batch *b, int32_t enable, uint32_t steps_per_graph)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (steps_per_graph < 1 || steps_per_graph > 1024)
        return bfail(b, CMAG_ERR_INVALID, "steps_per_graph must be in [1, 1024]");
    b->use_graphs = enable != 0;
    b->graph_steps = steps_per_graph;
    invalidate_graphs(b);
    return CMAG_OK;
}

int cmag_batch_device_error_bits(cmag_batch *b, uint32_t *bits)
{
    if (!b || !bits) return bfail(b, CMAG_ERR_INVALID, "null argument");
    CB_CUDA(b, cudaStreamSynchronize(b->stream));
    CB_CUDA(b, cudaMemcpy(bits, b->err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return CMAG_OK;
}

int cmag_batch_synchronize(cmag_batch *b)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    uint32_t bits = 0;
    int rc = cmag_batch_device_error_bits(b, &bits);
    if (rc) return rc;
    if (bits) {
        std::string m = "device check failed:";
        if (bits & CMAG_DEVERR_LOOKBACK_TIMEOUT) m += " look-back spin limit reached;";
        if (bits & CMAG_DEVERR_RANGE) m += " particle hash outside the scanned cell range;";
        return bfail(b, CMAG_ERR_DEVICE, m);
    }
    return CMAG_OK;
}

int cmag_batch_num_groups(const cmag_batch *b, uint32_t *out)
{
    if (!b || !out) return bfail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = (uint32_t)b->groups.size();
    return CMAG_OK;
}

int cmag_batch_group_info(cmag_batch *b, uint32_t group, cmag_batch_group *out)
{
    if (!b || !out) return bfail(b, CMAG_ERR_INVALID, "null argument");
    if (group >= b->groups.size()) return bfail(b, CMAG_ERR_INVALID, "group out of range");
    const LaunchGroup &g = b->groups[group];
    out->system = g.system;
    out->planar = g.planar ? 1 : 0;
    out->trim = g.trim ? 1 : 0;
    out->size_bucket = g.bucket;
    out->scenes = g.slot_end - g.slot_first;
    out->particles = g.count;
    out->density_lanes = g.g_density;
    out->force_lanes = g.g_force;
    out->lists = g.lists ? 1 : 0;
    return CMAG_OK;
}

int cmag_batch_scene_group(cmag_batch *b, uint32_t scene, uint32_t *group)
{
    BatchScene *s;
    int rc = scene_slot(b, scene, &s);
    if (rc) return rc;
    if (!group) return bfail(b, CMAG_ERR_INVALID, "null argument");
    *group = s->group;
    return CMAG_OK;
}

int cmag_batch_set_group_lanes(cmag_batch *b, uint32_t group, int32_t density_lanes, int32_t force_lanes)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (group >= b->groups.size()) return bfail(b, CMAG_ERR_INVALID, "group out of range");
    auto ok = [](int32_t g) { return g == 1 || g == 2 || g == 4; };
    if (!ok(density_lanes) || !ok(force_lanes))
        return bfail(b, CMAG_ERR_INVALID, "lanes per particle must be 1, 2 or 4");
    b->groups[group].g_density = density_lanes;
    b->groups[group].g_force = force_lanes;
    b->groups[group].lists = false;  // lanes chosen by hand: the cell walk
    invalidate_graphs(b);
    return CMAG_OK;
}

int cmag_batch_set_group_lists(cmag_batch *b, uint32_t group, int32_t enable)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (group >= b->groups.size()) return bfail(b, CMAG_ERR_INVALID, "group out of range");
    LaunchGroup &g = b->groups[group];
    if (enable) {
        if (!alloc_lists(b))
            return bfail(b, CMAG_ERR_NOMEM, "interaction lists: no device memory, or 2^26 particles or more");
        g.lists = true;
        g.g_density = g.g_force = 1;
    } else {
        g.lists = false;
    }
    invalidate_graphs(b);
    return CMAG_OK;
}

// Per launch group, time density and force for 1, 2 and 4 lanes per particle on
// the current state (`reps` launches each) and keep the fastest, then try the
// interaction lists.
int cmag_batch_autotune(cmag_batch *b, int32_t reps)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (reps < 1) reps = 1;
    int rc = upload_dev(b);
    if (rc) return rc;
    if ((rc = record_step(b, CMAG_STAGE_REORDER, false))) return rc;
    if (b->any_peristalsis && (rc = upload_phase(b))) return rc;
    cudaStream_t st = b->stream;
    cudaEvent_t e0, e1;
    CB_CUDA(b, cudaEventCreate(&e0));
    CB_CUDA(b, cudaEventCreate(&e1));
    const int lanes[3] = {1, 2, 4};
    const BatchView base = view_of(b);
    for (LaunchGroup &g : b->groups) {
        BatchView v = base;
        v.first = g.first;
        v.count = g.count;
        const DevParams &rep = b->host_dev[g.slot_first];
        const bool per = g.system == CMAG_PERISTALSIS;
        float4 *fa = per ? b->vforce : b->acc, *fb = per ? b->pforce : nullptr;
        float walk_ms[2] = {0.0f, 0.0f};
        for (int pass = 0; pass < 2; ++pass) {
            float best = 1e30f;
            int pick = pass == 0 ? g.g_density : g.g_force;
            for (int k = 0; k < 3; ++k) {
                auto run = [&]() {
                    if (pass == 0) launch_density(rep, v, lanes[k], b->spos, b->off, b->meas, b->aux, NeighborList{}, st);
                    else launch_force(rep, v, lanes[k], b->spos, b->svel, b->aux, sorted_idx(b), b->off, fa, fb,
                                      b->phase, NeighborList{}, st);
                };
                run();
                cudaEventRecord(e0, st);
                for (int r = 0; r < reps; ++r) run();
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) { best = ms; pick = lanes[k]; }
            }
            if (pass == 0) {
                g.g_density = pick;
                launch_density(rep, v, pick, b->spos, b->off, b->meas, b->aux, NeighborList{}, st);
            } else {
                g.g_force = pick;
            }
            walk_ms[pass] = best;
        }
        // interaction lists (one lane per particle, the same bits as the one-lane
        // walk): kept unless more than 3 % slower on this state, since the walk's
        // force cost grows as the flow develops
        g.lists = false;
        if (alloc_lists(b)) {
            const NeighborList nl = lists_of(b);
            auto timed = [&](auto &&run) {
                run();
                cudaEventRecord(e0, st);
                for (int r = 0; r < reps; ++r) run();
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                return ms;
            };
            const float ld = timed([&] { launch_density(rep, v, 1, b->spos, b->off, b->meas, b->aux, nl, st); });
            const float lf = timed([&] {
                launch_force(rep, v, 1, b->spos, b->svel, b->aux, sorted_idx(b), b->off, fa, fb, b->phase, nl, st);
            });
            if (ld + lf < 1.03f * (walk_ms[0] + walk_ms[1])) {
                g.lists = true;
                g.g_density = g.g_force = 1;
            }
        }
    }
    bool any_lists = false;
    for (const LaunchGroup &g : b->groups) any_lists |= g.lists;
    if (!any_lists) free_lists(b);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CB_CUDA(b, cudaGetLastError());
    CB_CUDA(b, cudaStreamSynchronize(st));
    b->last_stage = CMAG_STAGE_FORCE;
    invalidate_graphs(b);
    return CMAG_OK;
}

int cmag_batch_set_wall_cache(cmag_batch *b, int32_t enable)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (enable && !b->wc_entry) return bfail(b, CMAG_ERR_STATE, "no kept wall densities here (no dam-break scene, or their memory could not be had)");
    if ((enable != 0) != b->wc_on) {
        b->wc_on = enable != 0;
        refresh_dev(b);
        invalidate_graphs(b);
    }
    return CMAG_OK;
}

int cmag_batch_get_wall_cache(const cmag_batch *b, int32_t *enabled)
{
    if (!b || !enabled) return bfail(nullptr, CMAG_ERR_INVALID, "null argument");
    *enabled = b->wc_on ? 1 : 0;
    return CMAG_OK;
}

int cmag_batch_set_stage_timing(cmag_batch *b, int32_t enable)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    b->timing = enable != 0;
    return CMAG_OK;
}

int cmag_batch_stage_times(cmag_batch *b, float ms_out[6], uint32_t *steps_out)
{
    if (!b) return bfail(nullptr, CMAG_ERR_INVALID, "null handle");
    CB_CUDA(b, cudaStreamSynchronize(b->stream));
    for (size_t e = 0; e + 7 <= b->events_used; e += 7)
        for (int k = 0; k < 6; ++k) {
            float ms = 0.0f;
            CB_CUDA(b, cudaEventElapsedTime(&ms, b->events[e + k], b->events[e + k + 1]));
            b->stage_ms[k] += ms;
        }
    b->events_used = 0;
    if (ms_out)
        for (int k = 0; k < 6; ++k) ms_out[k] = (float)b->stage_ms[k];
    if (steps_out) *steps_out = b->timed_steps;
    for (int k = 0; k < 6; ++k) b->stage_ms[k] = 0;
    b->timed_steps = 0;
    return CMAG_OK;
}

const char *cmag_batch_last_error(const cmag_batch *b)
{
    return b ? b->last_error.c_str() : last_error().c_str();
}

}  // extern "C"
