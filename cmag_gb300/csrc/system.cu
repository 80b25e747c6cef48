// system.cu -- solver instances and the C ABI of include/cmag_sph.h.
//
// One cmag_system replaces one reference system object (DamBreakSystem,
// PoiseuilleFlowSystem, PeristalsisSystem): it owns the device arrays the
// reference allocates in _initialize (fluidSystem.cpp:116-190), a per-instance
// parameter block (the reference keeps one global __constant__ block per library,
// fluidSystem.cu:17-19) and a CUDA stream.  A step is the reference update()
// stage sequence; it is captured once as a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "closure.h"
#include "host_common.h"
#include "host_scenes.h"
#include "kernels.h"

using namespace cmag;

// arrays moved by one cmag_system_set_arrays / get_arrays call at most
constexpr uint32_t kMaxArraysPerCall = 8;

struct cmag_system {
    cmag_sph_params p{};
    uint32_t n = 0;
    uint64_t ncells = 0;
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    bool user_stream = false;

    float4 *pos = nullptr, *vel = nullptr, *vlf = nullptr, *meas = nullptr, *acc = nullptr,
           *vforce = nullptr, *pforce = nullptr, *pred = nullptr, *spos = nullptr,
           *svel = nullptr;
    uint32_t *hash[2] = {nullptr, nullptr}, *idx[2] = {nullptr, nullptr};
    uint32_t *cnt = nullptr, *off = nullptr;
    float2 *aux = nullptr;   // per sorted particle: p/rho^2 and rho or 1/rho
    uint32_t *ws = nullptr;  // cell scan: per-tile counts and their prefixes
    size_t ws_words = 0;
    uint32_t *err = nullptr;
    uint32_t *zflag = nullptr;  // set_array(s): whether uploaded z components differ (one word per array)
    PhaseState *phase = nullptr;
    uint32_t *view_cs = nullptr, *view_ce = nullptr;
    uint32_t *red = nullptr;  // reduction results: 6 extent keys, pad, 4 doubles, 1 count

    // host mirrors of device-side scalars
    float elapsed = 0.0f;
    PhaseState host_phase{};
    float k_milli = 0.0f;  // powf(10, -3): configuration ramp rate factor

    // layout
    bool planar = false;
    uint32_t planar_layer = 0;
    uint32_t scan_base = 0, scan_cells = 0;
    bool z_uniform = false;
    float z_value = 0.0f;
    bool vz_nonzero = false;
    int last_stage = CMAG_STAGE_INTEGRATE;

    int g_density = 1, g_force = 1;  // lanes per particle (cmag_system_autotune)
    uint32_t *nl_entry = nullptr, *nl_count = nullptr;  // interaction lists (when enabled)
    uint32_t nl_cap = 0;
    // lists kept over several steps (cmag_system_set_verlet): skin in particle
    // spacings (0: lists, sort and walk every step), the device flags of the
    // rebuild choice, positions at the last rebuild (original order), and the
    // stream that records the rebuild / reuse bodies of the captured step
    float vl_skin = 0.0f;
    VerletFlags *vl_flags = nullptr;
    float4 *vl_xb = nullptr;
    cudaStream_t vl_side = nullptr;
    // DamBreak: densities of non-fluid particles far from the fluid kept over
    // steps (DevParams::wc_*); wc_on: in use (cmag_system_set_wall_cache)
    float4 *wc_entry = nullptr, *wc_snap = nullptr;
    uint32_t *wc_mark = nullptr, *wc_state = nullptr;
    uint32_t wc_nb[3] = {0, 0, 0};
    bool wc_on = false;
    cmag_closure *closure = nullptr;   // learned correction added after the force stage
    __nv_bfloat16 *closure_x = nullptr;  // its normalised input rows (n x 16)

    bool use_graphs = true;
    cudaGraphExec_t gexec = nullptr;
    bool gvalid = false;

    bool timing = false;
    std::vector<cudaEvent_t> events;  // 7 per timed step
    size_t events_used = 0;
    double stage_ms[6] = {0, 0, 0, 0, 0, 0};
    uint32_t timed_steps = 0;

    std::string last_error;
};

namespace cmag {

namespace {
thread_local std::string g_last_error;
}

void set_last_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error() { return g_last_error; }

bool is_pow2(uint32_t v) { return v && !(v & (v - 1)); }

uint32_t log2u(uint64_t v)
{
    uint32_t b = 0;
    while ((1ull << b) < v) ++b;
    return b;
}

int validate_params(const cmag_sph_params &p, uint32_t n, std::string &why)
{
    if (p.system < CMAG_DAMBREAK || p.system > CMAG_PERISTALSIS) return why = "unknown system", 1;
    for (int k = 0; k < 3; ++k)
        if (p.grid_size[k] == 0 || p.grid_size[k] > (1u << 24)) return why = "grid_size out of range", 1;
    const uint64_t cells = (uint64_t)p.grid_size[0] * p.grid_size[1] * p.grid_size[2];
    if (cells > (1ull << 31)) return why = "more than 2^31 grid cells", 1;
    // the reference hashes with __umul24: equal to a plain product below 2^24
    if ((uint64_t)p.grid_size[2] * p.grid_size[1] > (1u << 24) || p.grid_size[0] > (1u << 24))
        return why = "grid too large for the 24-bit hash products", 1;
    if (p.cell_count < 0 || p.cell_count > 64) return why = "cell_count out of range", 1;
    // a run of 2c+1 cells must wrap at most once along x, and rows at most once in y
    if (p.grid_size[0] < (uint32_t)(2 * p.cell_count + 1) || p.grid_size[1] < (uint32_t)(2 * p.cell_count + 1))
        return why = "grid_size[0] and grid_size[1] must be at least 2*cell_count+1", 1;
    // grids that are not powers of two wrap by residue; a 3-D search must then
    // wrap z at most once too
    const bool pow2 = is_pow2(p.grid_size[0]) && is_pow2(p.grid_size[1]) && is_pow2(p.grid_size[2]);
    if (!pow2 && p.grid_size[2] < (uint32_t)(2 * p.cell_count + 1) && p.dims == 3)
        return why = "grid_size[2] must be at least 2*cell_count+1", 1;
    if (!(p.smoothing_radius > 0.0f) || !(p.particle_radius > 0.0f))
        return why = "smoothing_radius and particle_radius must be positive", 1;
    if (p.kernel != CMAG_KERNEL_WENDLAND && p.kernel != CMAG_KERNEL_CUBIC_SPLINE)
        return why = "unknown kernel", 1;
    if (p.dims != 2 && p.dims != 3) return why = "dims must be 2 or 3", 1;
    if (n == 0 || n >= (1u << 30)) return why = "particle count must be in [1, 2^30)", 1;
    return 0;
}

namespace {
const double kPi = 3.14159265358979323846;
}

DevParams make_dev_params(const cmag_sph_params &p, uint32_t n, const SceneLayout &lay)
{
    DevParams d;
    std::memset(&d, 0, sizeof(d));
    d.system = p.system; d.dims = p.dims; d.kernel = p.kernel; d.eos = p.eos;
    d.gx = p.grid_size[0]; d.gy = p.grid_size[1]; d.gz = p.grid_size[2];
    d.n = n;
    d.scan_base = lay.scan_base;
    d.scan_cells = lay.scan_cells;
    d.ox = p.world_origin[0]; d.oy = p.world_origin[1]; d.oz = p.world_origin[2];
    d.csx = p.cell_size[0]; d.csy = p.cell_size[1]; d.csz = p.cell_size[2];
    d.r = p.particle_radius;
    const double h = p.smoothing_radius;
    d.h = p.smoothing_radius;
    d.inv_h = (float)(1.0 / h);
    d.support2 = (float)(4.0 * h * h);
    d.mass = p.particle_mass; d.rho0 = p.rest_density; d.c0 = p.soundspeed;
    d.B = p.B; d.gamma = p.gamma; d.dt = p.delta_time; d.damping = p.boundary_damping;
    d.mu = p.mu;
    d.gvx = p.gravity[0]; d.gvy = p.gravity[1]; d.gvz = p.gravity[2];
    d.cell_count = p.cell_count;
    d.planar = lay.planar ? 1 : 0;
    // rows can be trimmed to the support sphere unless some interaction reaches
    // past q = 2 (the reference DamBreak wall force has no cut-off)
    d.trim = (p.system != CMAG_DAMBREAK || p.lj_cutoff) ? 1 : 0;
    if (p.system == CMAG_POISEUILLE) {
        d.wsx = p.grid_size[0] * 2.0f * p.particle_radius;  // poiseuilleFlowKernel.cu:120
    } else if (p.system == CMAG_PERISTALSIS) {
        d.wsx = p.world_size[0]; d.wsy = p.world_size[1]; d.wsz = p.world_size[2];
    }
    d.right_boundary = p.right_boundary;
    d.left_border = p.world_origin[0] + p.boundary_offset * 2 * p.particle_radius;
    d.bottom_border = p.world_origin[1] + p.boundary_offset * 2 * p.particle_radius;
    d.clamp_z = p.clamp_z;
    d.z_min_border = p.z_min_border;
    d.z_max_border = p.z_max_border;
    d.lj_D = p.lj_D; d.lj_a = p.lj_a; d.lj_cutoff = p.lj_cutoff;
    d.av_alpha = p.av_alpha;
    d.av_eps2 = 0.001f * std::pow(p.smoothing_radius, 2.0f);
    double wn, dwn;
    if (p.kernel == CMAG_KERNEL_WENDLAND) {
        wn = (p.dims == 2) ? 7.0 / (4.0 * kPi * h * h) : 21.0 / (16.0 * kPi * h * h * h);
        dwn = 2.0 * wn / h;
    } else {
        wn = (p.dims == 2) ? 10.0 / (7.0 * kPi * h * h) : 1.0 / (kPi * h * h * h);
        dwn = wn / h;
    }
    d.w_norm = (float)wn;
    d.dw_norm = (float)dwn;
    d.dwr_norm = (float)(-2.5 * dwn / h);
    d.nhalf_inv_h = -0.5f * d.inv_h;
    d.wall_bottom = p.world_origin[1] + p.boundary_offset * 2.0f * p.particle_radius;
    d.wall_top = d.wall_bottom + p.fluid_size[1] * 2.0f * p.particle_radius;
    d.amplitude = p.amplitude;
    d.wave_k = 3.141592654f * p.wave_count / (p.fluid_size[0] * p.particle_radius);
    d.wave_speed = p.wave_speed;
    d.half_fluid_h = p.fluid_size[1] * p.particle_radius;
    d.half_world_x = p.grid_size[0] * p.particle_radius;
    if (p.eos == CMAG_EOS_TAIT) d.p_wall = 0.0f;
    else d.p_wall = std::pow(p.soundspeed, 2.0f) * p.rest_density;  // poiseuilleFlowKernel.cu:156
    d.inv_csx = (float)(1.0 / p.cell_size[0]);
    d.inv_csy = (float)(1.0 / p.cell_size[1]);
    d.inv_csz = (float)(1.0 / p.cell_size[2]);
    const double sc = 2.0 * h / p.cell_size[0];
    d.support2_cells = (float)(sc * sc);
    // trimming works in cell units: it needs cubic cells
    if (!(p.cell_size[0] == p.cell_size[1] && p.cell_size[1] == p.cell_size[2])) d.trim = 0;
    d.pow2_grid = (is_pow2(p.grid_size[0]) && is_pow2(p.grid_size[1]) && is_pow2(p.grid_size[2])) ? 1u : 0u;
    d.planar_layer = lay.planar_layer;
    d.lj_a2 = p.lj_a * p.lj_a;
    d.av_coeff = (float)(2.0 * p.av_alpha * h * p.soundspeed);
    d.visc_coeff = (float)((double)p.particle_mass * (2.0 * p.mu));
    d.wall_noslip = (p.system == CMAG_PERISTALSIS && p.wall_noslip) ? 1 : 0;
    d.wall_beta_max = p.wall_beta_max > 0.0f ? p.wall_beta_max : 1000.0f;
    return d;
}

int z_cell(const cmag_sph_params &p, float z)
{
    float c = (p.system == CMAG_DAMBREAK) ? std::floor((z - p.world_origin[2]) / p.cell_size[2])
                                          : std::floor((z - p.world_origin[2]) * 0.5f / p.particle_radius);
    if (!(c == c)) return 0;
    if (c >= 2147483648.0f) return 2147483647;
    if (c <= -2147483648.0f) return -2147483647 - 1;
    return (int)c;
}

bool planar_allowed(const cmag_sph_params &p, bool z_uniform, bool vz_nonzero)
{
    return p.dims == 2 && z_uniform && !vz_nonzero && p.gravity[2] == 0.0f &&
           (int)p.grid_size[2] > p.cell_count;
}

SceneLayout layout_for(const cmag_sph_params &p, bool planar, float z_value)
{
    SceneLayout l;
    l.planar = planar;
    l.scan_cells = p.grid_size[0] * p.grid_size[1] * p.grid_size[2];
    if (planar) {
        const int64_t zc = z_cell(p, z_value), nz = p.grid_size[2];
        l.planar_layer = (uint32_t)(((zc % nz) + nz) % nz);
        l.scan_cells = p.grid_size[0] * p.grid_size[1];
        l.scan_base = l.planar_layer * l.scan_cells;
    }
    return l;
}

// Room per particle in the interaction lists: 1.5 times the lattice neighbour
// count inside the support (or, with the un-cut DamBreak wall force, every
// particle of the searched cell box) plus 32.  Particles beyond it walk the cells.
uint32_t list_cap(const cmag_sph_params &p, bool trim, double skin)
{
    const double dx = 2.0 * p.particle_radius, s = 2.0 * p.smoothing_radius / dx + skin;
    const bool planar = p.dims == 2;
    double expected = planar ? kPi * s * s : 4.0 / 3.0 * kPi * s * s * s;
    if (!trim) {
        const double c = 2 * p.cell_count + 1, per = p.cell_size[0] / dx;
        expected = planar ? c * c * per * per : c * c * c * per * per * per;
    }
    return (uint32_t)std::ceil(1.5 * expected) + 32u;
}

}  // namespace cmag

namespace {

int fail(cmag_system *s, int code, const std::string &msg)
{
    if (s) s->last_error = msg;
    set_last_error(msg);
    return code;
}

// On failure: report, and clear the runtime's (non-sticky) last error so that it
// does not surface later in an unrelated caller's CUDA call.
#define CM_CUDA(s, call)                                                                    \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            (void)cudaGetLastError();                                                       \
            return fail((s), e_ == cudaErrorMemoryAllocation ? CMAG_ERR_NOMEM : CMAG_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                \
        }                                                                                   \
    } while (0)

int validate(const cmag_sph_params &p, uint32_t n, std::string &why) { return validate_params(p, n, why); }

SceneLayout layout_of(const cmag_system *s)
{
    SceneLayout l;
    l.planar = s->planar;
    l.planar_layer = s->planar_layer;
    l.scan_base = s->scan_base;
    l.scan_cells = s->scan_cells;
    return l;
}

// Kept lists are in use: enabled, with lists allocated, and no learned closure
// attached (its feature walk needs this step's cell table).
bool verlet_on(const cmag_system *s) { return s->vl_skin > 0.0f && s->nl_entry && !s->closure; }

DevParams make_dev(const cmag_system *s)
{
    DevParams d = make_dev_params(s->p, s->n, layout_of(s));
    if (verlet_on(s)) {
        const double half = 0.5 * s->vl_skin * 2.0 * s->p.particle_radius;
        d.vl_move2 = (float)(half * half);
    } else if (s->wc_on && s->wc_entry) {
        d.wc_entry = s->wc_entry;
        d.wc_snap = s->wc_snap;
        d.wc_mark = s->wc_mark;
        d.wc_state = s->wc_state;
        d.wc_idx = s->idx[0];  // the counting sort's sorted -> original index
        d.wc_nbx = s->wc_nb[0];
        d.wc_nby = s->wc_nb[1];
        d.wc_nbz = s->wc_nb[2];
    }
    return d;
}

// The kept wall densities are stale: the next step's scan starts a new epoch.
void wall_cache_reset(cmag_system *s)
{
    if (s->wc_state &&
        cudaMemsetAsync(s->wc_state + kWcMoved, 0x01, sizeof(uint32_t), s->stream) != cudaSuccess)
        (void)cudaGetLastError();
}

// Parameters of the rebuild's density walk: rows trimmed to, and lists recording,
// every particle within 2h + skin (the density itself still sums q < 2 only).
DevParams rebuild_params(const cmag_system *s, const DevParams &d)
{
    DevParams b = d;
    const double R = 2.0 * s->p.smoothing_radius + s->vl_skin * 2.0 * s->p.particle_radius;
    const double rc = R / s->p.cell_size[0];
    b.verlet = 1;
    b.list_r2 = (float)(R * R);
    b.support2_cells = (float)(rc * rc);
    b.cell_count = std::max(d.cell_count, (int32_t)std::ceil(rc - 1e-6));
    return b;
}

NeighborList nl_of(const cmag_system *s)
{
    NeighborList nl{};
    if (s->nl_entry) {
        nl.entry = s->nl_entry;
        nl.count = s->nl_count;
        nl.cap = s->nl_cap;
        nl.stride = s->n;
        if (verlet_on(s)) nl.overflow = &s->vl_flags->overflow;
    }
    return nl;
}

// The next step rebuilds the kept lists (positions, parameters or sorted arrays
// changed behind them).
void verlet_force(cmag_system *s)
{
    if (s->vl_flags && cudaMemsetAsync(&s->vl_flags->moved, 0x01, sizeof(uint32_t), s->stream) != cudaSuccess)
        (void)cudaGetLastError();
}

int free_lists(cmag_system *s)
{
    if (s->nl_entry) cudaFree(s->nl_entry);
    if (s->nl_count) cudaFree(s->nl_count);
    s->nl_entry = s->nl_count = nullptr;
    s->nl_cap = 0;
    return CMAG_OK;
}

int alloc_lists(cmag_system *s, uint32_t cap = 0)
{
    if (s->nl_entry && (cap == 0 || cap == s->nl_cap)) return CMAG_OK;
    free_lists(s);
    if (s->n >= (1u << kListIndexBits))
        return fail(s, CMAG_ERR_INVALID, "interaction lists need fewer than 2^26 particles");
    if (cap == 0) cap = list_cap(s->p, make_dev(s).trim != 0);
    cudaError_t e = cudaMalloc((void **)&s->nl_entry, sizeof(uint32_t) * (size_t)cap * s->n);
    if (e == cudaSuccess) e = cudaMalloc((void **)&s->nl_count, sizeof(uint32_t) * (size_t)s->n);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        free_lists(s);
        return fail(s, e == cudaErrorMemoryAllocation ? CMAG_ERR_NOMEM : CMAG_ERR_CUDA,
                    std::string("interaction lists: ") + cudaGetErrorString(e));
    }
    s->nl_cap = cap;
    return CMAG_OK;
}

// Every change of parameters, lanes, lists or layout comes through here: the
// captured step is re-recorded, kept lists are rebuilt and kept wall densities
// recomputed.
void invalidate_graph(cmag_system *s)
{
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
    s->gvalid = false;
    verlet_force(s);
    wall_cache_reset(s);
}

// Planar 2-D scenes search and scan only their own z layer (planar_allowed).
void refresh_layout(cmag_system *s)
{
    const SceneLayout l = layout_for(s->p, planar_allowed(s->p, s->z_uniform, s->vz_nonzero), s->z_value);
    if (l.planar != s->planar || l.scan_base != s->scan_base || l.scan_cells != s->scan_cells)
        invalidate_graph(s);
    s->planar = l.planar;
    s->planar_layer = l.planar_layer;
    s->scan_base = l.scan_base;
    s->scan_cells = l.scan_cells;
}

cudaStream_t st_of(cmag_system *s) { return s->stream; }

// the counting sort's outputs (hash[0]: hashes in particle order, idx[1]: scratch)
uint32_t *sorted_hash(cmag_system *s) { return s->hash[1]; }
uint32_t *sorted_idx(cmag_system *s) { return s->idx[0]; }

int ensure_events(cmag_system *s, size_t count)
{
    while (s->events.size() < count) {
        cudaEvent_t e;
        CM_CUDA(s, cudaEventCreate(&e));
        s->events.push_back(e);
    }
    return CMAG_OK;
}

// ---- steps on lists kept over several steps ---------------------------------
// A step either rebuilds (hash, scan, counting sort with the gather, and the
// density walk over 2h + skin, which records every particle's list and computes
// the density) or reuses the lists (gather in the rebuild's order, density from
// the lists); force and integration follow in both.  The choice is made on the
// device (launch_verlet_decide): in a captured step it selects the body of a
// conditional graph node, in plain launches the host reads it.

// Peristalsis phase and wall configuration (first in every step); with kept
// lists the configured walls' displacement is checked like integration's.
void record_prologue(cmag_system *s, const DevParams &d, cudaStream_t st, bool kept)
{
    if (s->p.system != CMAG_PERISTALSIS) return;
    launch_phase(d, s->phase, s->k_milli, st);
    launch_configure_boundary(d, BatchView{}, s->pos, s->phase, st, kept ? s->vl_xb : nullptr,
                              kept ? &s->vl_flags->moved : nullptr);
}

void record_rebuild(cmag_system *s, const DevParams &d, cudaStream_t st, cudaEvent_t *ev)
{
    auto mark = [&](int k) { if (ev) cudaEventRecord(ev[k], st); };
    launch_hash(d, BatchView{}, s->pos, s->hash[0], s->cnt, s->idx[0], s->err, st, s->vl_xb);
    launch_cell_scan(s->cnt, s->off, s->scan_cells + 1, s->ws, st);
    mark(1);
    launch_cell_sort(s->hash[0], s->idx[0], s->off, s->scan_base, s->n, s->hash[1], s->idx[1], s->idx[0],
                     s->pos, s->vlf, s->spos, s->svel, s->err, st);
    mark(2);
    mark(3);
    launch_density(rebuild_params(s, d), BatchView{}, 1, s->spos, s->off, s->meas, s->aux, nl_of(s), st);
    mark(4);
}

void record_reuse(cmag_system *s, const DevParams &d, cudaStream_t st, cudaEvent_t *ev)
{
    auto mark = [&](int k) { if (ev) cudaEventRecord(ev[k], st); };
    mark(1);
    mark(2);
    launch_gather_sorted(s->idx[0], s->pos, s->vlf, s->n, s->spos, s->svel, st);
    mark(3);
    launch_density_list(d, s->spos, nl_of(s), s->meas, s->aux, st);
    mark(4);
}

void record_kept_tail(cmag_system *s, const DevParams &d, cudaStream_t st, cudaEvent_t *ev,
                      bool plain_force = false)
{
    auto mark = [&](int k) { if (ev) cudaEventRecord(ev[k], st); };
    g_plain_launches = plain_force;
    if (s->p.system == CMAG_PERISTALSIS)
        launch_force(d, BatchView{}, 1, s->spos, s->svel, s->aux, s->idx[0], s->off, s->vforce, s->pforce,
                     s->phase, nl_of(s), st);
    else
        launch_force(d, BatchView{}, 1, s->spos, s->svel, s->aux, s->idx[0], s->off, s->acc, nullptr,
                     s->phase, nl_of(s), st);
    g_plain_launches = false;
    mark(5);
    launch_integrate(d, BatchView{}, s->pos, s->vel, s->vlf, s->acc, s->vforce, s->pforce, s->phase, st,
                     s->vl_xb, &s->vl_flags->moved);
    mark(6);
}

int ensure_events(cmag_system *s, size_t count);

// one step on kept lists in plain launches (the host waits for the choice)
int record_kept_host(cmag_system *s, bool timed)
{
    const DevParams d = make_dev(s);
    cudaStream_t st = st_of(s);
    cudaEvent_t *ev = nullptr;
    if (timed) {
        if (ensure_events(s, s->events_used + 7) != CMAG_OK) return CMAG_ERR_CUDA;
        ev = &s->events[s->events_used];
        s->events_used += 7;
    }
    record_prologue(s, d, st, true);
    if (ev) cudaEventRecord(ev[0], st);
    launch_verlet_decide(s->vl_flags, 0ull, 0, st);
    uint32_t rebuild = 1;
    CM_CUDA(s, cudaMemcpyAsync(&rebuild, &s->vl_flags->decision, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CM_CUDA(s, cudaStreamSynchronize(st));
    if (rebuild) record_rebuild(s, d, st, ev);
    else record_reuse(s, d, st, ev);
    record_kept_tail(s, d, st, ev);
    CM_CUDA(s, cudaGetLastError());
    return CMAG_OK;
}

// The step as one graph: prologue, the choice, a conditional node whose bodies
// are the rebuild and the reuse, then force and integration.  plain_bodies: the
// bodies' kernels without programmatic dependent launch.
int capture_kept_graph(cmag_system *s, bool plain_bodies)
{
    cudaStream_t st = st_of(s);
    const DevParams d = make_dev(s);
    if (!s->vl_side) CM_CUDA(s, cudaStreamCreateWithFlags(&s->vl_side, cudaStreamNonBlocking));
    CM_CUDA(s, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    cudaGraph_t g = nullptr;
    cudaGraphNode_t cnode = nullptr;
    const char *what = "capture";
    do {
        record_prologue(s, d, st, true);
        cudaStreamCaptureStatus cs;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t *deps = nullptr;
        const cudaGraphEdgeData *edges = nullptr;  // queried (a programmatic edge is not lost)
        size_t nd = 0;
        what = "cudaStreamGetCaptureInfo";
        if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, &edges, &nd)) != cudaSuccess) break;
        cudaGraphConditionalHandle h;
        what = "cudaGraphConditionalHandleCreate";
        if ((e = cudaGraphConditionalHandleCreate(&h, cg, 0, 0)) != cudaSuccess) break;
        launch_verlet_decide(s->vl_flags, (unsigned long long)h, 1, st);
        what = "cudaStreamGetCaptureInfo";
        if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, &edges, &nd)) != cudaSuccess) break;
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 2;  // body 0: rebuild (condition 1); body 1: reuse
        what = "cudaGraphAddNode(conditional)";
        if ((e = cudaGraphAddNode(&cnode, cg, deps, nullptr, nd, &cp)) != cudaSuccess) break;
        g_plain_launches = plain_bodies;
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
            what = "cudaStreamBeginCaptureToGraph";
            e = cudaStreamBeginCaptureToGraph(s->vl_side, cp.conditional.phGraph_out[b], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) break;
            if (b == 0) record_rebuild(s, d, s->vl_side, nullptr);
            else record_reuse(s, d, s->vl_side, nullptr);
            cudaGraph_t body = nullptr;
            what = "body capture";
            e = cudaStreamEndCapture(s->vl_side, &body);
        }
        g_plain_launches = false;
        if (e != cudaSuccess) break;
        what = "cudaStreamUpdateCaptureDependencies";
        if ((e = cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies)) !=
            cudaSuccess)
            break;
        // the force kernel follows the conditional node with a full dependency
        record_kept_tail(s, d, st, nullptr, true);
        what = "launch";
        e = cudaGetLastError();
    } while (false);
    cudaError_t e2 = cudaStreamEndCapture(st, &g);
    if (e == cudaSuccess) {
        e = e2;
        what = "stream capture";
    }
    if (e == cudaSuccess) {
        what = "graph instantiate";
        e = cudaGraphInstantiate(&s->gexec, g, 0);
    }
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        s->gexec = nullptr;
        return fail(s, CMAG_ERR_CUDA, std::string("kept-list step graph: ") + what + ": " + cudaGetErrorString(e));
    }
    s->gvalid = true;
    return CMAG_OK;
}

// Enqueue the stages of one step up to and including `last` on the stream.
int record_step(cmag_system *s, int last, bool timed)
{
    if (verlet_on(s) && last >= CMAG_STAGE_INTEGRATE) return record_kept_host(s, timed);
    const DevParams d = make_dev(s);
    cudaStream_t st = st_of(s);
    const cmag_sph_params &p = s->p;
    cudaEvent_t *ev = nullptr;
    if (timed) {
        if (ensure_events(s, s->events_used + 7) != CMAG_OK) return CMAG_ERR_CUDA;
        ev = &s->events[s->events_used];
        s->events_used += 7;
    }
    auto mark = [&](int k) { if (ev) cudaEventRecord(ev[k], st); };

    // Peristalsis: the phase block of this step (the walls are configured in the hash pass)
    if (p.system == CMAG_PERISTALSIS) launch_phase(d, s->phase, s->k_milli, st);
    mark(0);
    // hash + per-cell counts (and each particle's arrival rank in its cell), dense
    // offsets, then the stable counting sort by cell
    launch_hash(d, BatchView{}, s->pos, s->hash[0], s->cnt, s->idx[0], s->err, st, nullptr,
                p.system == CMAG_PERISTALSIS ? s->phase : nullptr);
    launch_cell_scan(s->cnt, s->off, s->scan_cells + 1, s->ws, st, d.wc_state);
    mark(1);
    if (last >= CMAG_STAGE_SORT)
        launch_cell_sort(s->hash[0], s->idx[0], s->off, s->scan_base, s->n, s->hash[1], s->idx[1],
                         s->idx[0], s->pos, s->vlf, s->spos, s->svel, s->err, st);
    mark(2);
    // (the gather of sorted positions and velocities ran with the sort)
    mark(3);
    if (last >= CMAG_STAGE_DENSITY)
        launch_density(d, BatchView{}, s->g_density, s->spos, s->off, s->meas, s->aux, nl_of(s), st);
    mark(4);
    if (last >= CMAG_STAGE_FORCE) {
        if (p.system == CMAG_PERISTALSIS)
            launch_force(d, BatchView{}, s->g_force, s->spos, s->svel, s->aux, sorted_idx(s), s->off,
                         s->vforce, s->pforce, s->phase, nl_of(s), st);
        else
            launch_force(d, BatchView{}, s->g_force, s->spos, s->svel, s->aux, sorted_idx(s), s->off, s->acc,
                         nullptr, s->phase, nl_of(s), st);
        if (s->closure)
            launch_closure_apply(d, s->closure->view(), s->spos, s->svel, s->aux, s->meas,
                                 sorted_idx(s), s->off, s->acc, s->closure_x, st);
    }
    mark(5);
    if (last >= CMAG_STAGE_INTEGRATE)
        launch_integrate(d, BatchView{}, s->pos, s->vel, s->vlf, s->acc, s->vforce, s->pforce, s->phase, st);
    mark(6);
    CM_CUDA(s, cudaGetLastError());
    // the sorted order (and the lists) of this step replace the kept ones
    if (s->vl_flags) verlet_force(s);
    return CMAG_OK;
}

// host mirror of k_phase (PeristalsisSystem.cpp:330-343, 407)
void advance_host_mirror(cmag_system *s)
{
    const float dt = s->p.delta_time;
    if (s->p.system == CMAG_PERISTALSIS) {
        PhaseState &h = s->host_phase;
        h.configure = 0;
        if (h.is_bc) {
            h.time_shift = h.time_shift + dt;
            if (h.wave_height < s->p.amplitude) {
                h.configure = 1;
                h.configure_height = h.wave_height;
                h.wave_height = h.wave_height + dt * s->k_milli;
            } else {
                h.time_relax = h.time_relax - dt;
                if (h.time_relax < 0.0f) h.is_bc = 0;
            }
        }
        h.t = h.is_bc ? 0.0f : h.elapsed - h.time_shift;
        h.elapsed = h.elapsed + dt;
        s->p.is_boundary_configuration = h.is_bc;
        s->elapsed = h.elapsed;
    } else {
        s->elapsed = s->elapsed + dt;
    }
}

int upload_phase(cmag_system *s)
{
    CM_CUDA(s, cudaMemcpyAsync(s->phase, &s->host_phase, sizeof(PhaseState),
                               cudaMemcpyHostToDevice, st_of(s)));
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    return CMAG_OK;
}

int capture_graph(cmag_system *s)
{
    invalidate_graph(s);
    if (verlet_on(s)) {
        // conditional bodies with programmatic dependent launch, else without
        if (capture_kept_graph(s, false) == CMAG_OK) return CMAG_OK;
        return capture_kept_graph(s, true);
    }
    cudaStream_t st = st_of(s);
    CM_CUDA(s, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = record_step(s, CMAG_STAGE_INTEGRATE, false);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != CMAG_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(s, CMAG_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(s, CMAG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    s->gvalid = true;
    return CMAG_OK;
}

int do_step(cmag_system *s)
{
    if (s->use_graphs && !s->timing && s->stream != nullptr) {
        if (!s->gvalid) {
            int rc = capture_graph(s);
            if (rc != CMAG_OK) return rc;
        }
        CM_CUDA(s, cudaGraphLaunch(s->gexec, st_of(s)));
    } else {
        int rc = record_step(s, CMAG_STAGE_INTEGRATE, s->timing);
        if (rc != CMAG_OK) return rc;
        if (s->timing) s->timed_steps++;
    }
    s->last_stage = CMAG_STAGE_INTEGRATE;
    advance_host_mirror(s);
    return CMAG_OK;
}

float4 *float_array(cmag_system *s, int a)
{
    switch (a) {
    case CMAG_POSITION: return s->pos;
    case CMAG_VELOCITY: return s->vel;
    case CMAG_MEASURES: return s->meas;
    case CMAG_ACCELERATION: return s->acc;
    case CMAG_VELOCITYLEAPFROG: return s->vlf;
    case CMAG_VISCOUSFORCE: return s->vforce;
    case CMAG_PRESSUREFORCE: return s->pforce;
    case CMAG_PREDICTEDPOSITION: return s->pred;
    case CMAG_SORTEDPOSITION: return s->spos;
    case CMAG_SORTEDVELOCITY: return s->svel;
    default: return nullptr;
    }
}

void free_all(cmag_system *s)
{
    invalidate_graph(s);
    for (auto e : s->events) cudaEventDestroy(e);
    s->events.clear();
    void *ptrs[] = {s->pos, s->vel, s->vlf, s->meas, s->acc, s->vforce, s->pforce, s->pred,
                    s->spos, s->svel, s->hash[0], s->hash[1], s->idx[0], s->idx[1], s->cnt,
                    s->off, s->aux, s->ws, s->err, s->phase, s->view_cs, s->view_ce, s->red,
                    s->zflag, s->closure_x, s->vl_flags, s->vl_xb, s->wc_entry, s->wc_snap,
                    s->wc_mark, s->wc_state};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    free_lists(s);
    if (s->vl_side) cudaStreamDestroy(s->vl_side);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
}

template <class T>
int dalloc(cmag_system *s, T **ptr, size_t bytes)
{
    CM_CUDA(s, cudaMalloc((void **)ptr, bytes));
    CM_CUDA(s, cudaMemset(*ptr, 0, bytes));
    return CMAG_OK;
}

int check_range(cmag_system *s, uint32_t start, uint32_t count, uint64_t size)
{
    if ((uint64_t)start + count > size)
        return fail(s, CMAG_ERR_INVALID, "array range [" + std::to_string(start) + ", " +
                                             std::to_string((uint64_t)start + count) +
                                             ") exceeds " + std::to_string(size));
    return CMAG_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================

extern "C" {

const char *cmag_version(void) { return "cmag_gb300 0.1 (sm_103a)"; }

size_t cmag_sph_params_size(void) { return sizeof(cmag_sph_params); }

const char *cmag_last_error(void) { return last_error().c_str(); }

const char *cmag_system_last_error(const cmag_system *s)
{
    return s ? s->last_error.c_str() : last_error().c_str();
}

int cmag_dambreak_default_params(const uint32_t fluid_size[3], int32_t boundary_offset,
                                 const uint32_t grid_size[3], float particle_radius,
                                 cmag_sph_params *out)
{
    if (!out || !fluid_size || !grid_size) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    dambreak_params(fluid_size, boundary_offset, grid_size, particle_radius, *out);
    return CMAG_OK;
}

int cmag_poiseuille_default_params(const uint32_t fluid_size[3], int32_t boundary_offset,
                                   const uint32_t grid_size[3], float particle_radius,
                                   cmag_sph_params *out)
{
    if (!out || !fluid_size || !grid_size) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    poiseuille_params(fluid_size, boundary_offset, grid_size, particle_radius, *out);
    return CMAG_OK;
}

int cmag_peristalsis_default_params(float delta_time, const uint32_t fluid_size[3],
                                    float amplitude, float wave_speed, float soundspeed,
                                    const float gravity[3], int32_t boundary_offset,
                                    const uint32_t grid_size[3], float radius,
                                    cmag_sph_params *out)
{
    if (!out || !fluid_size || !grid_size || !gravity)
        return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    peristalsis_params(delta_time, fluid_size, amplitude, wave_speed, soundspeed, gravity,
                       boundary_offset, grid_size, radius, *out);
    return CMAG_OK;
}

int cmag_reference_particle_count(const cmag_sph_params *p, uint32_t *out)
{
    if (!p || !out) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = reference_particle_count(*p);
    return CMAG_OK;
}

int cmag_reference_scene(const cmag_sph_params *p, float *pos, uint32_t n)
{
    if (!p || (!pos && n)) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    reference_scene(*p, pos, n);
    return CMAG_OK;
}

int cmag_peristalsis_mass_sum(const cmag_sph_params *p, const float *pos, uint32_t n, float *out)
{
    if (!p || !out || (!pos && n)) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    if (n <= p->grid_size[0] / 2) return fail(nullptr, CMAG_ERR_INVALID, "probe particle out of range");
    *out = peristalsis_mass_sum(*p, pos, n);
    return CMAG_OK;
}

int cmag_dambreak3d_scene_host(const cmag_sph_params *p, const uint32_t tank_cells[3],
                               uint32_t layers, float jitter_frac, uint64_t seed, float *pos,
                               uint32_t n)
{
    if (!p || !tank_cells || (!pos && n)) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    std::memset(pos, 0, sizeof(float) * 4 * (size_t)n);
    dambreak3d_scene(*p, tank_cells, layers, jitter_frac, seed, pos, n);
    return CMAG_OK;
}

int cmag_dambreak3d_particle_count(const uint32_t fluid_size[3], const uint32_t tank_cells[3],
                                   uint32_t layers, uint32_t *out)
{
    if (!fluid_size || !tank_cells || !out) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = dambreak3d_count(fluid_size, tank_cells, layers);
    return CMAG_OK;
}

int cmag_system_create(const cmag_sph_params *params, uint32_t n, cmag_system **out)
{
    if (!params || !out) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = nullptr;
    std::string why;
    if (validate(*params, n, why)) return fail(nullptr, CMAG_ERR_INVALID, why);
    cmag_system *s = new (std::nothrow) cmag_system();
    if (!s) return fail(nullptr, CMAG_ERR_NOMEM, "host allocation failed");
    s->p = *params;
    s->n = n;
    s->ncells = (uint64_t)params->grid_size[0] * params->grid_size[1] * params->grid_size[2];
    s->k_milli = std::pow(10.0f, -3.0f);
    s->scan_base = 0;
    s->scan_cells = (uint32_t)s->ncells;
    // 3-D searches need every axis wide enough for one wrap per run
    if (params->dims == 3) {  // 49 rows per particle: split them over 2 lanes
        s->g_density = 2;
        s->g_force = 2;
    }
    int rc = CMAG_OK;
    auto step = [&](int r) { if (rc == CMAG_OK) rc = r; };
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) {
        fail(nullptr, CMAG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        delete s;
        return CMAG_ERR_CUDA;
    }
    e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        fail(nullptr, CMAG_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
        delete s;
        return CMAG_ERR_CUDA;
    }
    s->stream = s->own_stream;
    const size_t f4 = sizeof(float4) * (size_t)n, u4 = sizeof(uint32_t) * (size_t)n;
    step(dalloc(s, &s->pos, f4));
    step(dalloc(s, &s->vel, f4));
    step(dalloc(s, &s->vlf, f4));
    step(dalloc(s, &s->meas, f4));
    step(dalloc(s, &s->acc, f4));
    step(dalloc(s, &s->spos, f4));
    step(dalloc(s, &s->svel, f4));
    step(dalloc(s, &s->aux, sizeof(float2) * (size_t)n));
    if (params->system == CMAG_PERISTALSIS) {
        step(dalloc(s, &s->vforce, f4));
        step(dalloc(s, &s->pforce, f4));
        step(dalloc(s, &s->pred, f4));
    }
    for (int k = 0; k < 2; ++k) {
        step(dalloc(s, &s->hash[k], u4));
        step(dalloc(s, &s->idx[k], u4));
    }
    // per-cell counters and offsets for the whole grid (+1 sentinel entry)
    step(dalloc(s, &s->cnt, sizeof(uint32_t) * (s->ncells + 1)));
    step(dalloc(s, &s->off, sizeof(uint32_t) * (s->ncells + 1)));
    s->ws_words = cell_scan_workspace_words((uint32_t)(s->ncells + 1));
    step(dalloc(s, &s->ws, sizeof(uint32_t) * s->ws_words));
    step(dalloc(s, &s->err, sizeof(uint32_t)));
    step(dalloc(s, &s->phase, sizeof(PhaseState)));
    // 6 extent keys + pad (32 B), 4 doubles (32 B), 1 count (8 B)
    step(dalloc(s, &s->red, 128));
    step(dalloc(s, &s->zflag, kMaxArraysPerCall * sizeof(uint32_t)));
    if (rc == CMAG_OK && params->system == CMAG_DAMBREAK) {
        // kept wall densities: an optimisation, so the instance is made without
        // them when their memory cannot be had
        for (int a = 0; a < 3; ++a) s->wc_nb[a] = (params->grid_size[a] + 3u) / 4u;
        const size_t marks = sizeof(uint32_t) * (size_t)s->wc_nb[0] * s->wc_nb[1] * s->wc_nb[2];
        void **bufs[4] = {(void **)&s->wc_entry, (void **)&s->wc_snap, (void **)&s->wc_mark, (void **)&s->wc_state};
        const size_t sizes[4] = {f4, f4, marks, 4 * sizeof(uint32_t)};
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
        s->wc_on = ok;
    }
    if (rc != CMAG_OK) {
        std::string msg = s->last_error;
        free_all(s);
        delete s;
        set_last_error(msg);
        return rc;
    }
    // the clears above ran on the legacy stream, which the instance's
    // non-blocking stream does not wait for
    e = cudaStreamSynchronize(cudaStreamLegacy);
    if (e != cudaSuccess) {
        fail(nullptr, CMAG_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
        free_all(s);
        delete s;
        return CMAG_ERR_CUDA;
    }
    s->host_phase.is_bc = params->is_boundary_configuration;
    s->host_phase.time_relax = 1000 * params->delta_time;
    upload_phase(s);
    wall_cache_reset(s);
    refresh_layout(s);
    *out = s;
    return CMAG_OK;
}

int cmag_system_destroy(cmag_system *s)
{
    if (!s) return CMAG_OK;
    cudaStreamSynchronize(s->stream);
    free_all(s);
    delete s;
    return CMAG_OK;
}

int cmag_system_set_array(cmag_system *s, int32_t array, const float *host, uint32_t start,
                          uint32_t count)
{
    if (!s || (!host && count)) return fail(s, CMAG_ERR_INVALID, "null argument");
    float4 *d = float_array(s, array);
    if (!d) return fail(s, CMAG_ERR_INVALID, "not a settable float4 array: " + std::to_string(array));
    if (check_range(s, start, count, s->n) != CMAG_OK) return CMAG_ERR_INVALID;
    if (count == 0) return CMAG_OK;
    CM_CUDA(s, cudaMemcpyAsync(d + start, host, sizeof(float4) * (size_t)count,
                               cudaMemcpyHostToDevice, st_of(s)));
    // a 2-D scene searches one z layer while its particles share one z and have no
    // z velocity: check the uploaded z components on the device (3-D scenes never
    // search one layer)
    const bool pos_up = array == CMAG_POSITION;
    const bool vel_up = array == CMAG_VELOCITY || array == CMAG_VELOCITYLEAPFROG;
    uint32_t differs = 0;
    const float z0 = pos_up ? host[2] : 0.0f;
    if (s->p.dims == 2 && (pos_up || vel_up)) {
        launch_z_differs(d + start, count, z0, s->zflag, st_of(s));
        CM_CUDA(s, cudaGetLastError());
        CM_CUDA(s, cudaMemcpyAsync(&differs, s->zflag, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                   st_of(s)));
    }
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    if (s->p.dims != 2) {
        s->z_uniform = false;
    } else if (pos_up) {
        if (start == 0 && count == s->n) {
            s->z_uniform = !differs;
            s->z_value = z0;
        } else if (differs || z0 != s->z_value) {
            s->z_uniform = false;
        }
    } else if (vel_up) {
        if (differs) s->vz_nonzero = true;
        else if (start == 0 && count == s->n && array == CMAG_VELOCITY) s->vz_nonzero = false;
    }
    refresh_layout(s);
    // kept lists depend on positions only: a rebuild when an uploaded position
    // lies more than skin/2 from where the lists were built
    if (pos_up && verlet_on(s)) {
        launch_verlet_check(s->pos, s->vl_xb, start, count, make_dev(s).vl_move2, &s->vl_flags->moved,
                            st_of(s));
        CM_CUDA(s, cudaGetLastError());
    }
    return CMAG_OK;
}

int cmag_system_set_arrays(cmag_system *s, uint32_t count, const int32_t *arrays, const float *const *host)
{
    if (!s || (count && (!arrays || !host))) return fail(s, CMAG_ERR_INVALID, "null argument");
    if (count > kMaxArraysPerCall) return fail(s, CMAG_ERR_INVALID, "at most 8 arrays per call");
    float4 *d[kMaxArraysPerCall];
    for (uint32_t k = 0; k < count; ++k) {
        d[k] = float_array(s, arrays[k]);
        if (!d[k] || !host[k]) return fail(s, CMAG_ERR_INVALID, "not a settable float4 array: " + std::to_string(arrays[k]));
    }
    if (s->n == 0) return CMAG_OK;
    for (uint32_t k = 0; k < count; ++k)
        CM_CUDA(s, cudaMemcpyAsync(d[k], host[k], sizeof(float4) * (size_t)s->n, cudaMemcpyHostToDevice, st_of(s)));
    // the z checks of set_array, one flag word per array, read back together
    uint32_t differs[kMaxArraysPerCall] = {};
    bool checked = false;
    for (uint32_t k = 0; k < count; ++k) {
        const bool pos_up = arrays[k] == CMAG_POSITION;
        const bool vel_up = arrays[k] == CMAG_VELOCITY || arrays[k] == CMAG_VELOCITYLEAPFROG;
        if (s->p.dims == 2 && (pos_up || vel_up)) {
            launch_z_differs(d[k], s->n, pos_up ? host[k][2] : 0.0f, s->zflag + k, st_of(s));
            checked = true;
        }
    }
    if (checked) {
        CM_CUDA(s, cudaGetLastError());
        CM_CUDA(s, cudaMemcpyAsync(differs, s->zflag, sizeof(uint32_t) * count, cudaMemcpyDeviceToHost, st_of(s)));
    }
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    bool pos_any = false;
    for (uint32_t k = 0; k < count; ++k) {
        const int32_t a = arrays[k];
        if (s->p.dims != 2) {
            s->z_uniform = false;
        } else if (a == CMAG_POSITION) {
            s->z_uniform = !differs[k];
            s->z_value = host[k][2];
        } else if (a == CMAG_VELOCITY || a == CMAG_VELOCITYLEAPFROG) {
            if (differs[k]) s->vz_nonzero = true;
            else if (a == CMAG_VELOCITY) s->vz_nonzero = false;
        }
        pos_any = pos_any || a == CMAG_POSITION;
    }
    refresh_layout(s);
    if (pos_any && verlet_on(s)) {
        launch_verlet_check(s->pos, s->vl_xb, 0, s->n, make_dev(s).vl_move2, &s->vl_flags->moved, st_of(s));
        CM_CUDA(s, cudaGetLastError());
    }
    return CMAG_OK;
}

int cmag_system_get_arrays(cmag_system *s, uint32_t count, const int32_t *arrays, float *const *host)
{
    if (!s || (count && (!arrays || !host))) return fail(s, CMAG_ERR_INVALID, "null argument");
    if (count > kMaxArraysPerCall) return fail(s, CMAG_ERR_INVALID, "at most 8 arrays per call");
    for (uint32_t k = 0; k < count; ++k) {
        float4 *d = float_array(s, arrays[k]);
        if (!d || !host[k]) return fail(s, CMAG_ERR_INVALID, "not a float4 array: " + std::to_string(arrays[k]));
        CM_CUDA(s, cudaMemcpyAsync(host[k], d, sizeof(float4) * (size_t)s->n, cudaMemcpyDeviceToHost, st_of(s)));
    }
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    return CMAG_OK;
}

int cmag_system_get_array(cmag_system *s, int32_t array, float *host, uint32_t start,
                          uint32_t count)
{
    if (!s || (!host && count)) return fail(s, CMAG_ERR_INVALID, "null argument");
    float4 *d = float_array(s, array);
    if (!d) return fail(s, CMAG_ERR_INVALID, "not a float4 array: " + std::to_string(array));
    if (check_range(s, start, count, s->n) != CMAG_OK) return CMAG_ERR_INVALID;
    if (count == 0) return CMAG_OK;
    CM_CUDA(s, cudaMemcpyAsync(host, d + start, sizeof(float4) * (size_t)count,
                               cudaMemcpyDeviceToHost, st_of(s)));
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    return CMAG_OK;
}

int cmag_system_get_uint_array(cmag_system *s, int32_t array, uint32_t *host, uint32_t start,
                               uint32_t count)
{
    if (!s || (!host && count)) return fail(s, CMAG_ERR_INVALID, "null argument");
    const uint32_t *src = nullptr;
    uint64_t size = s->n;
    switch (array) {
    case CMAG_HASH: src = (s->last_stage == CMAG_STAGE_HASH) ? s->hash[0] : sorted_hash(s); break;
    case CMAG_INDEX:
        if (s->last_stage == CMAG_STAGE_HASH) {  // before the sort: identity
            if (check_range(s, start, count, s->n) != CMAG_OK) return CMAG_ERR_INVALID;
            for (uint32_t i = 0; i < count; ++i) host[i] = start + i;
            return CMAG_OK;
        }
        src = sorted_idx(s);
        break;
    case CMAG_CELLOFFSET: src = s->off; size = (uint64_t)s->scan_cells + 1; break;
    case CMAG_CELLSTART:
    case CMAG_CELLEND: {
        size = s->ncells;
        if (!s->view_cs) {
            if (dalloc(s, &s->view_cs, sizeof(uint32_t) * s->ncells) != CMAG_OK) return CMAG_ERR_NOMEM;
            if (dalloc(s, &s->view_ce, sizeof(uint32_t) * s->ncells) != CMAG_OK) return CMAG_ERR_NOMEM;
        }
        launch_cell_view(s->off, s->scan_base, s->scan_cells, s->ncells, s->view_cs, s->view_ce,
                         st_of(s));
        CM_CUDA(s, cudaGetLastError());
        src = (array == CMAG_CELLSTART) ? s->view_cs : s->view_ce;
        break;
    }
    default: return fail(s, CMAG_ERR_INVALID, "not a uint32 array: " + std::to_string(array));
    }
    if (check_range(s, start, count, size) != CMAG_OK) return CMAG_ERR_INVALID;
    if (count == 0) return CMAG_OK;
    CM_CUDA(s, cudaMemcpyAsync(host, src + start, sizeof(uint32_t) * (size_t)count,
                               cudaMemcpyDeviceToHost, st_of(s)));
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    return CMAG_OK;
}

void *cmag_system_device_array(cmag_system *s, int32_t array)
{
    if (!s) return nullptr;
    switch (array) {
    case CMAG_HASH: return sorted_hash(s);
    case CMAG_INDEX: return sorted_idx(s);
    case CMAG_CELLOFFSET: return s->off;
    default: return float_array(s, array);
    }
}

int cmag_system_reset(cmag_system *s)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    const uint32_t want = reference_particle_count(s->p);
    if (want != s->n)
        return fail(s, CMAG_ERR_STATE, "instance holds " + std::to_string(s->n) +
                                           " particles, the reference scene has " +
                                           std::to_string(want));
    std::vector<float> pos((size_t)s->n * 4, 0.0f), zero((size_t)s->n * 4, 0.0f),
        meas((size_t)s->n * 4, 0.0f);
    reference_scene(s->p, pos.data(), s->n);
    if (s->p.system != CMAG_PERISTALSIS)  // fluidSystem.cpp:131-132
        for (uint32_t i = 0; i < s->n; ++i) meas[4 * (size_t)i] = s->p.rest_density;
    int rc;
    if ((rc = cmag_system_set_array(s, CMAG_POSITION, pos.data(), 0, s->n))) return rc;
    const int zero_arrays[] = {CMAG_VELOCITY, CMAG_ACCELERATION, CMAG_VELOCITYLEAPFROG};
    for (int a : zero_arrays)
        if ((rc = cmag_system_set_array(s, a, zero.data(), 0, s->n))) return rc;
    if ((rc = cmag_system_set_array(s, CMAG_MEASURES, meas.data(), 0, s->n))) return rc;
    s->elapsed = 0.0f;
    if (s->p.system == CMAG_DAMBREAK) {  // fluidSystem.cpp:378-379
        const uint32_t gate_cells = (uint32_t)(s->p.boundary_offset + (int32_t)s->p.fluid_size[0]) * 2u;
        s->p.right_boundary = s->p.world_origin[0] + gate_cells * s->p.particle_radius;
    }
    if (s->p.system == CMAG_PERISTALSIS) {  // PeristalsisSystem.cpp:213-236
        for (int a : {CMAG_VISCOUSFORCE, CMAG_PRESSUREFORCE, CMAG_PREDICTEDPOSITION})
            if ((rc = cmag_system_set_array(s, a, zero.data(), 0, s->n))) return rc;
        s->host_phase = PhaseState{};
        s->host_phase.time_relax = 1000 * s->p.delta_time;
        s->host_phase.is_bc = 1;
        s->p.is_boundary_configuration = 1;
        s->p.particle_mass = s->p.rest_density / peristalsis_mass_sum(s->p, pos.data(), s->n);
        if ((rc = upload_phase(s))) return rc;
    }
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_dambreak3d_scene(cmag_system *s, const uint32_t tank_cells[3], uint32_t layers,
                          float jitter_frac, uint64_t seed)
{
    if (!s || !tank_cells) return fail(s, CMAG_ERR_INVALID, "null argument");
    if (s->p.system != CMAG_DAMBREAK) return fail(s, CMAG_ERR_STATE, "not a dam-break system");
    const uint32_t want = dambreak3d_count(s->p.fluid_size, tank_cells, layers);
    if (want != s->n)
        return fail(s, CMAG_ERR_STATE, "instance holds " + std::to_string(s->n) +
                                           " particles, the 3-D scene has " + std::to_string(want));
    std::vector<float> pos((size_t)s->n * 4, 0.0f), zero((size_t)s->n * 4, 0.0f),
        meas((size_t)s->n * 4, 0.0f);
    dambreak3d_scene(s->p, tank_cells, layers, jitter_frac, seed, pos.data(), s->n);
    for (uint32_t i = 0; i < s->n; ++i) meas[4 * (size_t)i] = s->p.rest_density;
    int rc;
    if ((rc = cmag_system_set_array(s, CMAG_POSITION, pos.data(), 0, s->n))) return rc;
    for (int a : {CMAG_VELOCITY, CMAG_ACCELERATION, CMAG_VELOCITYLEAPFROG})
        if ((rc = cmag_system_set_array(s, a, zero.data(), 0, s->n))) return rc;
    if ((rc = cmag_system_set_array(s, CMAG_MEASURES, meas.data(), 0, s->n))) return rc;
    s->elapsed = 0.0f;
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_system_update(cmag_system *s)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    return do_step(s);
}

int cmag_system_update_dt(cmag_system *s, float dt)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(s, CMAG_ERR_INVALID, "dt must be positive and finite");
    if (dt != s->p.delta_time) {
        // dt travels in the step's parameter block: the captured graph is redone
        s->p.delta_time = dt;
        invalidate_graph(s);
    }
    return do_step(s);
}

int cmag_system_update_n(cmag_system *s, uint32_t steps)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    for (uint32_t k = 0; k < steps; ++k) {
        int rc = do_step(s);
        if (rc != CMAG_OK) return rc;
    }
    return CMAG_OK;
}

int cmag_system_timed_update(cmag_system *s, uint32_t steps, float *ms_out)
{
    if (!s || !ms_out) return fail(s, CMAG_ERR_INVALID, "null argument");
    cudaEvent_t a, b;
    CM_CUDA(s, cudaEventCreate(&a));
    CM_CUDA(s, cudaEventCreate(&b));
    cudaEventRecord(a, st_of(s));
    int rc = CMAG_OK;
    for (uint32_t k = 0; k < steps && rc == CMAG_OK; ++k) rc = do_step(s);
    cudaEventRecord(b, st_of(s));
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc != CMAG_OK) return rc;
    if (e != cudaSuccess) return fail(s, CMAG_ERR_CUDA, std::string("timed update: ") + cudaGetErrorString(e));
    *ms_out = ms;
    return CMAG_OK;
}

int cmag_system_run_stages(cmag_system *s, int32_t last_stage)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (last_stage < CMAG_STAGE_HASH || last_stage > CMAG_STAGE_INTEGRATE)
        return fail(s, CMAG_ERR_INVALID, "unknown stage");
    int rc = record_step(s, last_stage, false);
    if (rc != CMAG_OK) return rc;
    s->last_stage = last_stage;
    if (last_stage == CMAG_STAGE_INTEGRATE) {
        advance_host_mirror(s);
    } else if (s->p.system == CMAG_PERISTALSIS) {
        // the stages ran with this step's phase; time does not advance
        if ((rc = upload_phase(s))) return rc;
    }
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    return CMAG_OK;
}

int cmag_system_num_particles(const cmag_system *s, uint32_t *out)
{
    if (!s || !out) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = s->n;
    return CMAG_OK;
}

int cmag_system_num_grid_cells(const cmag_system *s, uint64_t *out)
{
    if (!s || !out) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = s->ncells;
    return CMAG_OK;
}

int cmag_system_elapsed_time(const cmag_system *s, float *out)
{
    if (!s || !out) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = s->elapsed;
    return CMAG_OK;
}

int cmag_system_get_params(const cmag_system *s, cmag_sph_params *out)
{
    if (!s || !out) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = s->p;
    return CMAG_OK;
}

int cmag_system_set_params(cmag_system *s, const cmag_sph_params *p)
{
    if (!s || !p) return fail(s, CMAG_ERR_INVALID, "null argument");
    if (p->system != s->p.system || std::memcmp(p->grid_size, s->p.grid_size, sizeof(p->grid_size)))
        return fail(s, CMAG_ERR_INVALID, "system kind and grid size are fixed at creation");
    std::string why;
    if (validate(*p, s->n, why)) return fail(s, CMAG_ERR_INVALID, why);
    s->p = *p;
    if (s->p.system == CMAG_PERISTALSIS && s->host_phase.is_bc != p->is_boundary_configuration) {
        s->host_phase.is_bc = p->is_boundary_configuration;
        int rc = upload_phase(s);
        if (rc) return rc;
    }
    refresh_layout(s);
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_dambreak_change_right_boundary(cmag_system *s)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (s->p.system != CMAG_DAMBREAK) return fail(s, CMAG_ERR_STATE, "not a dam-break system");
    const float width = s->p.fluid_size[0] * 2 * s->p.particle_radius;
    s->p.right_boundary += width;  // fluidSystem.cpp:240
    launch_gate(make_dev(s), s->pos, 0, width, 0.0f, 0.0f, st_of(s));
    CM_CUDA(s, cudaGetLastError());
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_dambreak_remove_right_boundary(cmag_system *s)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (s->p.system != CMAG_DAMBREAK) return fail(s, CMAG_ERR_STATE, "not a dam-break system");
    s->p.right_boundary = (float)0xffffffffu;  // fluidSystem.cpp:223
    const float fw = s->p.fluid_size[0] * 2 * s->p.particle_radius;
    const float fh = s->p.grid_size[1] * 2 * s->p.particle_radius;
    launch_gate(make_dev(s), s->pos, 1, 0.0f, fw, fh, st_of(s));
    CM_CUDA(s, cudaGetLastError());
    s->elapsed = 0.0f;
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_poiseuille_change_gravity(cmag_system *s)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (s->p.system != CMAG_POISEUILLE) return fail(s, CMAG_ERR_STATE, "not a Poiseuille system");
    s->p.gravity[1] *= -1.0f;
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_peristalsis_phase(const cmag_system *s, float *wave_height, float *time_relax,
                           float *time_shift, int32_t *is_bc)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (wave_height) *wave_height = s->host_phase.wave_height;
    if (time_relax) *time_relax = s->host_phase.time_relax;
    if (time_shift) *time_shift = s->host_phase.time_shift;
    if (is_bc) *is_bc = s->host_phase.is_bc;
    return CMAG_OK;
}

int cmag_system_fluid_extent(cmag_system *s, float lo[3], float hi[3])
{
    if (!s || !lo || !hi) return fail(s, CMAG_ERR_INVALID, "null argument");
    cudaStream_t st = st_of(s);
    CM_CUDA(s, cudaMemsetAsync(s->red, 0xff, 3 * sizeof(uint32_t), st));
    CM_CUDA(s, cudaMemsetAsync(s->red + 3, 0, 3 * sizeof(uint32_t), st));
    launch_fluid_extent(s->p.system, s->pos, s->n, s->red, st);
    uint32_t keys[6];
    CM_CUDA(s, cudaMemcpyAsync(keys, s->red, sizeof(keys), cudaMemcpyDeviceToHost, st));
    CM_CUDA(s, cudaStreamSynchronize(st));
    auto back = [](uint32_t k) {
        uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
        float f;
        std::memcpy(&f, &u, sizeof(f));
        return f;
    };
    for (int k = 0; k < 3; ++k) {
        lo[k] = back(keys[k]);
        hi[k] = back(keys[3 + k]);
    }
    return CMAG_OK;
}

int cmag_system_fluid_sum(cmag_system *s, int32_t array, double sum[4], uint32_t *count)
{
    if (!s || !sum) return fail(s, CMAG_ERR_INVALID, "null argument");
    float4 *a = float_array(s, array);
    if (!a) return fail(s, CMAG_ERR_INVALID, "not a float4 array: " + std::to_string(array));
    const bool sorted = array == CMAG_MEASURES || array == CMAG_SORTEDPOSITION ||
                        array == CMAG_SORTEDVELOCITY;
    cudaStream_t st = st_of(s);
    double *sums = reinterpret_cast<double *>(s->red + 8);
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(s->red + 8 + 8);
    CM_CUDA(s, cudaMemsetAsync(sums, 0, 4 * sizeof(double) + sizeof(unsigned long long), st));
    launch_fluid_sum(s->p.system, sorted ? s->spos : s->pos, a, s->n, sums, cnt, st);
    double h[4];
    unsigned long long c = 0;
    CM_CUDA(s, cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, st));
    CM_CUDA(s, cudaMemcpyAsync(&c, cnt, sizeof(c), cudaMemcpyDeviceToHost, st));
    CM_CUDA(s, cudaStreamSynchronize(st));
    for (int k = 0; k < 4; ++k) sum[k] = h[k];
    if (count) *count = (uint32_t)c;
    return CMAG_OK;
}

int cmag_system_set_elapsed_time(cmag_system *s, float elapsed)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    s->elapsed = elapsed;
    if (s->p.system == CMAG_PERISTALSIS) {
        s->host_phase.elapsed = elapsed;
        return upload_phase(s);
    }
    return CMAG_OK;
}

int cmag_peristalsis_set_phase(cmag_system *s, float wave_height, float time_relax,
                               float time_shift, int32_t is_bc)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (s->p.system != CMAG_PERISTALSIS) return fail(s, CMAG_ERR_STATE, "not a Peristalsis system");
    s->host_phase.wave_height = wave_height;
    s->host_phase.time_relax = time_relax;
    s->host_phase.time_shift = time_shift;
    s->host_phase.is_bc = is_bc;
    s->p.is_boundary_configuration = is_bc;
    return upload_phase(s);
}

int cmag_system_set_stream(cmag_system *s, void *cuda_stream)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    cudaStreamSynchronize(s->stream);
    s->stream = cuda_stream ? (cudaStream_t)cuda_stream : s->own_stream;
    s->user_stream = cuda_stream != nullptr;
    invalidate_graph(s);
    return CMAG_OK;
}

void *cmag_system_stream(const cmag_system *s) { return s ? (void *)s->stream : nullptr; }

int cmag_system_set_graphs(cmag_system *s, int32_t enable)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    s->use_graphs = enable != 0;
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_system_device_error_bits(cmag_system *s, uint32_t *bits)
{
    if (!s || !bits) return fail(s, CMAG_ERR_INVALID, "null argument");
    CM_CUDA(s, cudaStreamSynchronize(s->stream));
    CM_CUDA(s, cudaMemcpy(bits, s->err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return CMAG_OK;
}

int cmag_system_synchronize(cmag_system *s)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    uint32_t bits = 0;
    int rc = cmag_system_device_error_bits(s, &bits);
    if (rc) return rc;
    if (bits) {
        std::string m = "device check failed:";
        if (bits & CMAG_DEVERR_LOOKBACK_TIMEOUT) m += " look-back spin limit reached;";
        if (bits & CMAG_DEVERR_RANGE) m += " particle hash outside the scanned cell range;";
        return fail(s, CMAG_ERR_DEVICE, m);
    }
    return CMAG_OK;
}

int cmag_system_set_groups(cmag_system *s, int32_t gd, int32_t gf)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    auto ok = [](int32_t g) { return g == 1 || g == 2 || g == 4; };
    if (!ok(gd) || !ok(gf)) return fail(s, CMAG_ERR_INVALID, "lanes per particle must be 1, 2 or 4");
    s->g_density = gd;
    s->g_force = gf;
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_system_get_groups(const cmag_system *s, int32_t *gd, int32_t *gf)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (gd) *gd = s->g_density;
    if (gf) *gf = s->g_force;
    return CMAG_OK;
}

int cmag_system_autotune(cmag_system *s, int32_t reps)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (reps < 1) reps = 1;
    if (s->vl_skin > 0.0f) return CMAG_OK;  // kept lists: one lane per particle, nothing to choose
    // hash, sort and gather of the current state, then time each variant
    PhaseState saved = s->host_phase;
    int rc = record_step(s, CMAG_STAGE_REORDER, false);
    if (rc != CMAG_OK) return rc;
    if (s->p.system == CMAG_PERISTALSIS) {
        s->host_phase = saved;
        if ((rc = upload_phase(s))) return rc;
    }
    DevParams d = make_dev(s);
    // trials walk every particle (kept wall densities belong to one lane count)
    d.wc_entry = nullptr;
    cudaStream_t st = st_of(s);
    cudaEvent_t a, b;
    CM_CUDA(s, cudaEventCreate(&a));
    CM_CUDA(s, cudaEventCreate(&b));
    auto timed = [&](auto &&launch) {
        launch();  // warm
        cudaEventRecord(a, st);
        for (int r = 0; r < reps; ++r) launch();
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        return ms;
    };
    const bool had_lists = s->nl_entry != nullptr;
    free_lists(s);
    const NeighborList none{};
    const int groups[3] = {1, 2, 4};
    float best_d = 1e30f, best_f = 1e30f;
    int gd = s->g_density, gf = s->g_force;
    float4 *fa = s->p.system == CMAG_PERISTALSIS ? s->vforce : s->acc;
    float4 *fb = s->p.system == CMAG_PERISTALSIS ? s->pforce : nullptr;
    for (int k = 0; k < 3; ++k) {
        const float ms = timed([&] { launch_density(d, BatchView{}, groups[k], s->spos, s->off, s->meas, s->aux, none, st); });
        if (ms < best_d) { best_d = ms; gd = groups[k]; }
    }
    launch_density(d, BatchView{}, gd, s->spos, s->off, s->meas, s->aux, none, st);
    for (int k = 0; k < 3; ++k) {
        const float ms = timed([&] {
            launch_force(d, BatchView{}, groups[k], s->spos, s->svel, s->aux, sorted_idx(s), s->off, fa, fb,
                         s->phase, none, st);
        });
        if (ms < best_f) { best_f = ms; gf = groups[k]; }
    }
    // interaction lists: the density pass records them, the force pass reads them
    bool lists = false;
    if (alloc_lists(s) == CMAG_OK) {
        const NeighborList nl = nl_of(s);
        const float ld = timed([&] { launch_density(d, BatchView{}, 1, s->spos, s->off, s->meas, s->aux, nl, st); });
        const float lf = timed([&] {
            launch_force(d, BatchView{}, 1, s->spos, s->svel, s->aux, sorted_idx(s), s->off, fa, fb, s->phase, nl, st);
        });
        // the walk's force cost grows as the flow develops (viscosity terms switch on,
        // branches diverge over candidates outside the support) while the lists'
        // does not: keep the lists unless they are clearly slower now
        lists = ld + lf < 1.03f * (best_d + best_f);
        if (!lists) free_lists(s);
    } else if (had_lists) {
        (void)cudaGetLastError();
    }
    s->last_error.clear();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    CM_CUDA(s, cudaGetLastError());
    s->g_density = gd;
    s->g_force = gf;
    s->last_stage = CMAG_STAGE_FORCE;
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_system_set_neighbor_lists(cmag_system *s, int32_t enable)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (enable < 0) return fail(s, CMAG_ERR_INVALID, "enable must be 0, 1 or an entry count");
    s->vl_skin = 0.0f;  // per-step lists (or none): lists are no longer kept
    int rc = enable ? alloc_lists(s, enable > 1 ? (uint32_t)enable : 0u) : free_lists(s);
    invalidate_graph(s);
    return rc;
}

int cmag_system_set_verlet(cmag_system *s, float skin)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (!(skin >= 0.0f) || skin > 4.0f) return fail(s, CMAG_ERR_INVALID, "skin must be in [0, 4] particle spacings");
    if (skin == 0.0f) {
        s->vl_skin = 0.0f;
        invalidate_graph(s);
        return CMAG_OK;
    }
    const DevParams d = make_dev_params(s->p, s->n, layout_of(s));
    if (!d.trim)
        return fail(s, CMAG_ERR_INVALID,
                    "kept lists need a cut-off on every interaction (DamBreak: lj_cutoff = 1) and cubic cells");
    const double rc = (2.0 * s->p.smoothing_radius + skin * 2.0 * s->p.particle_radius) / s->p.cell_size[0];
    const uint32_t cb = (uint32_t)std::ceil(rc - 1e-6);
    for (int k = 0; k < (s->planar ? 2 : 3); ++k)
        if (s->p.grid_size[k] < 2 * cb + 1)
            return fail(s, CMAG_ERR_INVALID, "grid too small for the list radius 2h + skin");
    if (!s->vl_flags) {
        CM_CUDA(s, cudaMalloc((void **)&s->vl_flags, sizeof(VerletFlags)));
        CM_CUDA(s, cudaMemset(s->vl_flags, 0, sizeof(VerletFlags)));
    }
    if (!s->vl_xb) CM_CUDA(s, cudaMalloc((void **)&s->vl_xb, sizeof(float4) * (size_t)s->n));
    const uint32_t cap = list_cap(s->p, true, skin);
    if (int rc2 = alloc_lists(s, cap)) return rc2;
    s->vl_skin = skin;
    invalidate_graph(s);  // and the next step rebuilds
    return CMAG_OK;
}

int cmag_system_get_verlet(cmag_system *s, float *skin, uint32_t *rebuilds)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (skin) *skin = s->vl_skin;
    if (rebuilds) {
        VerletFlags f{};
        if (s->vl_flags) {
            CM_CUDA(s, cudaMemcpyAsync(&f, s->vl_flags, sizeof(f), cudaMemcpyDeviceToHost, st_of(s)));
            CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
        }
        *rebuilds = f.rebuilds;
    }
    return CMAG_OK;
}

int cmag_system_set_wall_cache(cmag_system *s, int32_t enable)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (enable && !s->wc_entry) return fail(s, CMAG_ERR_STATE, "no kept wall densities here (dam-break systems only; none when their memory could not be had)");
    if ((enable != 0) != s->wc_on) {
        s->wc_on = enable != 0;
        invalidate_graph(s);
    }
    return CMAG_OK;
}

int cmag_system_get_wall_cache(const cmag_system *s, int32_t *enabled)
{
    if (!s || !enabled) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    *enabled = s->wc_on ? 1 : 0;
    return CMAG_OK;
}

int cmag_system_get_neighbor_lists(const cmag_system *s, int32_t *enabled, uint32_t *cap)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (enabled) *enabled = s->nl_entry != nullptr;
    if (cap) *cap = s->nl_cap;
    return CMAG_OK;
}


int cmag_system_set_closure(cmag_system *s, cmag_closure *c)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (c && s->p.system != CMAG_DAMBREAK)
        return fail(s, CMAG_ERR_STATE, "the learned closure corrects DamBreak scenes only");
    if (c && !s->closure_x)
        CM_CUDA(s, cudaMalloc((void **)&s->closure_x, sizeof(__nv_bfloat16) * 16 * (size_t)s->n));
    s->closure = c;
    invalidate_graph(s);
    return CMAG_OK;
}

int cmag_system_closure_features(cmag_system *s, float *d_features)
{
    if (!s || !d_features) return fail(s, CMAG_ERR_INVALID, "null argument");
    if (s->p.system != CMAG_DAMBREAK) return fail(s, CMAG_ERR_STATE, "not a dam-break system");
    if (s->last_stage < CMAG_STAGE_FORCE)
        return fail(s, CMAG_ERR_STATE, "features need this step's density and forces (run_stages FORCE)");
    launch_closure_features(make_dev(s), s->spos, s->svel, s->aux, s->meas, sorted_idx(s), s->off,
                            s->acc, d_features, st_of(s));
    CM_CUDA(s, cudaGetLastError());
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    return CMAG_OK;
}

int cmag_system_interpolate(cmag_system *s, int32_t array, const float *d_points, uint32_t n,
                            float *d_out)
{
    if (!s || (n && (!d_points || !d_out))) return fail(s, CMAG_ERR_INVALID, "null argument");
    if (s->p.system != CMAG_DAMBREAK) return fail(s, CMAG_ERR_STATE, "not a dam-break system");
    if (s->last_stage < CMAG_STAGE_DENSITY)
        return fail(s, CMAG_ERR_STATE, "interpolation needs this step's densities (run_stages DENSITY)");
    const float4 *a = nullptr;
    switch (array) {
    case CMAG_POSITION: a = s->pos; break;
    case CMAG_VELOCITY: a = s->vel; break;
    case CMAG_ACCELERATION: a = s->acc; break;
    case CMAG_VELOCITYLEAPFROG: a = s->vlf; break;
    default: return fail(s, CMAG_ERR_INVALID, "not an original-order float4 array: " + std::to_string(array));
    }
    launch_interpolate(make_dev(s), s->spos, s->aux, sorted_idx(s), s->off, a,
                       reinterpret_cast<const float4 *>(d_points), n, reinterpret_cast<float4 *>(d_out),
                       st_of(s));
    CM_CUDA(s, cudaGetLastError());
    CM_CUDA(s, cudaStreamSynchronize(st_of(s)));
    return CMAG_OK;
}

namespace {
int color_buffer(cmag_system *s, float4 *d_out)
{
    const cmag_sph_params &p = s->p;
    const uint32_t fluid = p.fluid_size[0] * p.fluid_size[1] * p.fluid_size[2];
    // fluidSystem.cpp:169-170
    const uint32_t type_one = fluid + (p.grid_size[0] - p.boundary_offset + 1) + 2 * (p.grid_size[1] - p.boundary_offset);
    launch_colors(make_dev(s), s->pos, fluid, type_one, d_out, st_of(s));
    CM_CUDA(s, cudaGetLastError());
    return CMAG_OK;
}
}  // namespace

int cmag_system_colors(cmag_system *s, float *rgba)
{
    if (!s || !rgba) return fail(s, CMAG_ERR_INVALID, "null argument");
    float4 *d = nullptr;
    CM_CUDA(s, cudaMalloc((void **)&d, sizeof(float4) * (size_t)s->n));
    int rc = color_buffer(s, d);
    cudaError_t e = cudaSuccess;
    if (rc == CMAG_OK) e = cudaMemcpyAsync(rgba, d, sizeof(float4) * (size_t)s->n, cudaMemcpyDeviceToHost, st_of(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_of(s));
    cudaFree(d);
    if (rc != CMAG_OK) return rc;
    CM_CUDA(s, e);
    return CMAG_OK;
}

int cmag_system_render_ppm(cmag_system *s, const char *path, uint32_t width, uint32_t height)
{
    if (!s || !path) return fail(s, CMAG_ERR_INVALID, "null argument");
    const cmag_sph_params &p = s->p;
    const float wx = p.grid_size[0] * p.cell_size[0], wy = p.grid_size[1] * p.cell_size[1];
    if (width == 0 || width > 16384) return fail(s, CMAG_ERR_INVALID, "width must be in [1, 16384]");
    if (height == 0) height = (uint32_t)std::lround(width * (double)wy / wx);
    if (height == 0 || height > 16384) return fail(s, CMAG_ERR_INVALID, "height must be in [1, 16384]");
    const size_t npix = (size_t)width * height;
    float4 *color = nullptr;
    uint32_t *owner = nullptr;
    uint8_t *rgb = nullptr;
    std::vector<uint8_t> host(3 * npix);
    cudaError_t e = cudaMalloc((void **)&color, sizeof(float4) * (size_t)s->n);
    if (e == cudaSuccess) e = cudaMalloc((void **)&owner, sizeof(uint32_t) * npix);
    if (e == cudaSuccess) e = cudaMalloc((void **)&rgb, 3 * npix);
    int rc = CMAG_OK;
    if (e == cudaSuccess) rc = color_buffer(s, color);
    if (e == cudaSuccess && rc == CMAG_OK) {
        const float scale = p.system == CMAG_PERISTALSIS ? 1.0f : 255.0f;
        launch_render(s->pos, color, s->n, p.world_origin[0], p.world_origin[1], width / wx, width,
                      height, scale, owner, rgb, st_of(s));
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(host.data(), rgb, 3 * npix, cudaMemcpyDeviceToHost, st_of(s));
        if (e == cudaSuccess) e = cudaStreamSynchronize(st_of(s));
    }
    cudaFree(color);
    cudaFree(owner);
    cudaFree(rgb);
    if (rc != CMAG_OK) return rc;
    CM_CUDA(s, e);
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(s, CMAG_ERR_INVALID, std::string("cannot open ") + path);
    std::fprintf(f, "P6\n%u %u\n255\n", width, height);
    const size_t wrote = std::fwrite(host.data(), 1, host.size(), f);
    std::fclose(f);
    if (wrote != host.size()) return fail(s, CMAG_ERR_INVALID, std::string("short write to ") + path);
    return CMAG_OK;
}

int cmag_system_set_stage_timing(cmag_system *s, int32_t enable)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    s->timing = enable != 0;
    return CMAG_OK;
}

int cmag_system_stage_times(cmag_system *s, float ms_out[6], uint32_t *steps_out)
{
    if (!s) return fail(nullptr, CMAG_ERR_INVALID, "null handle");
    CM_CUDA(s, cudaStreamSynchronize(s->stream));
    for (size_t b = 0; b + 7 <= s->events_used; b += 7)
        for (int k = 0; k < 6; ++k) {
            float ms = 0.0f;
            CM_CUDA(s, cudaEventElapsedTime(&ms, s->events[b + k], s->events[b + k + 1]));
            s->stage_ms[k] += ms;
        }
    s->events_used = 0;
    if (ms_out)
        for (int k = 0; k < 6; ++k) ms_out[k] = (float)s->stage_ms[k];
    if (steps_out) *steps_out = s->timed_steps;
    for (int k = 0; k < 6; ++k) s->stage_ms[k] = 0;
    s->timed_steps = 0;
    return CMAG_OK;
}

// ---------------------------------------------------------------- sorting --

namespace {
struct SortCache {
    uint32_t *ws = nullptr, *keys = nullptr, *vals = nullptr;
    size_t ws_words = 0, cap = 0;
};
std::mutex g_sort_mu;
std::map<int, SortCache> g_sort_cache;
}  // namespace

int cmag_sort_particles(uint32_t *d_hash, uint32_t *d_index, uint32_t n, uint32_t key_bits,
                        void *cuda_stream)
{
    if (n == 0) return CMAG_OK;
    if (!d_hash || !d_index) return fail(nullptr, CMAG_ERR_INVALID, "null argument");
    if (key_bits > 32 || n >= (1u << 30)) return fail(nullptr, CMAG_ERR_INVALID, "key_bits or n out of range");
    cudaStream_t st = (cudaStream_t)cuda_stream;
    int passes = sort_passes(key_bits);
    if (passes < 1) passes = 1;
    int dev = 0;
    CM_CUDA(nullptr, cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_sort_mu);
    SortCache &c = g_sort_cache[dev];
    const size_t words = sort_workspace_words(n, kMaxPasses) + 1;
    if (c.cap < n || c.ws_words < words) {
        if (c.ws) cudaFree(c.ws);
        if (c.keys) cudaFree(c.keys);
        if (c.vals) cudaFree(c.vals);
        c = SortCache{};
        CM_CUDA(nullptr, cudaMalloc((void **)&c.ws, words * sizeof(uint32_t)));
        CM_CUDA(nullptr, cudaMalloc((void **)&c.keys, sizeof(uint32_t) * (size_t)n));
        CM_CUDA(nullptr, cudaMalloc((void **)&c.vals, sizeof(uint32_t) * (size_t)n));
        c.ws_words = words;
        c.cap = n;
    }
    uint32_t *err = c.ws + (words - 1);
    CM_CUDA(nullptr, cudaMemsetAsync(c.ws, 0, words * sizeof(uint32_t), st));
    SortWorkspace sw = sort_workspace_view(c.ws, n);
    launch_digit_hist(d_hash, n, passes, sw.hist, st);
    uint32_t *kb[2] = {d_hash, c.keys}, *vb[2] = {d_index, c.vals};
    for (int k = 0; k < passes; ++k) {
        const int src = k & 1, dst = src ^ 1;
        launch_onesweep_pass(kb[src], vb[src], kb[dst], vb[dst], n, k, false, sw, err, st);
    }
    if (passes & 1) {
        CM_CUDA(nullptr, cudaMemcpyAsync(d_hash, c.keys, sizeof(uint32_t) * (size_t)n,
                                         cudaMemcpyDeviceToDevice, st));
        CM_CUDA(nullptr, cudaMemcpyAsync(d_index, c.vals, sizeof(uint32_t) * (size_t)n,
                                         cudaMemcpyDeviceToDevice, st));
    }
    uint32_t bits = 0;
    CM_CUDA(nullptr, cudaMemcpyAsync(&bits, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CM_CUDA(nullptr, cudaStreamSynchronize(st));
    if (bits)
        return fail(nullptr, CMAG_ERR_DEVICE,
                    std::string("sort: device-side check failed (bits ") + std::to_string(bits) + ":" +
                        ((bits & CMAG_DEVERR_LOOKBACK_TIMEOUT) ? " look-back spin limit reached" : "") +
                        ((bits & CMAG_DEVERR_RANGE) ? " scatter index out of range" : "") + ")");
    return CMAG_OK;
}

}  // extern "C"
