// walk_check.cpp -- the neighbour walk of the density/force passes
// (cmag_gb300/csrc/neighbor_walk.cuh), compiled for the host, checked against
// brute force.  Test infrastructure: the few device intrinsics the header uses
// are restated below with host arithmetic; the walk code itself is the product's
// header, included unchanged.
//
// walk_check() hashes and stably sorts a scene's particles like the hash/sort
// stages, builds the dense cell offset table, runs for_each_candidate for every
// particle and every lane of a lane group, and compares the candidates inside the
// support (through the image shift the walk reports) with a brute-force scan over
// all particles and their periodic images: every in-support pair must be visited
// exactly once.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include <cuda_runtime.h>

// ---- host restatements of the device intrinsics used by the walk headers ----
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline int sat_int(float v)
{
    if (v != v) return 0;
    if (v >= 2147483648.0f) return 2147483647;
    if (v <= -2147483648.0f) return (-2147483647 - 1);
    return (int)v;
}
static inline int __float2int_rz(float x) { return sat_int(std::trunc(x)); }
static inline int __float2int_rd(float x) { return sat_int(std::floor(x)); }
static inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
static inline uint32_t __float_as_uint(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, sizeof u);
    return u;
}
template <class T>
static inline T __ldg(const T *p) { return *p; }
static inline float __shfl_down_sync(unsigned, float v, int, int) { return v; }
static inline uint32_t atomicOr(uint32_t *a, uint32_t v)
{
    const uint32_t old = *a;
    *a |= v;
    return old;
}
static inline int max(int a, int b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }

#include "neighbor_walk.cuh"

using namespace cmag;

namespace {

struct Scene {
    DevParams p;
    std::vector<float4> spos;   // sorted positions
    std::vector<uint32_t> off;  // dense offset table (scan_cells + 1)
};

// 0: ok; -1: a particle of a planar scene outside its layer
int build(Scene &sc, int system, int planar, int trim, const uint32_t grid[3], const float origin[3],
          float cell, float h, int cell_count, const float *pos, uint32_t n)
{
    DevParams &p = sc.p;
    std::memset(&p, 0, sizeof p);
    p.system = system;
    p.dims = planar ? 2 : 3;
    p.gx = grid[0];
    p.gy = grid[1];
    p.gz = grid[2];
    p.n = n;
    p.ox = origin[0];
    p.oy = origin[1];
    p.oz = origin[2];
    p.csx = p.csy = p.csz = cell;
    p.r = 0.5f * cell;  // Poiseuille and Peristalsis hash with 2 r = one cell
    p.h = h;
    p.inv_h = (float)(1.0 / h);
    p.support2 = (float)(4.0 * (double)h * h);
    p.cell_count = cell_count;
    p.planar = planar;
    p.trim = trim;
    p.wsx = grid[0] * cell;
    p.wsy = grid[1] * cell;
    p.wsz = grid[2] * cell;
    p.inv_csx = p.inv_csy = p.inv_csz = (float)(1.0 / cell);
    const double sc2 = 2.0 * h / cell;
    p.support2_cells = (float)(sc2 * sc2);
    auto pow2 = [](uint32_t v) { return v && !(v & (v - 1)); };
    p.pow2_grid = (pow2(grid[0]) && pow2(grid[1]) && pow2(grid[2])) ? 1u : 0u;
    std::vector<uint32_t> hash(n);
    for (uint32_t i = 0; i < n; ++i) {
        const int3 g = grid_pos(p, pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]);
        hash[i] = grid_hash(p, g.x, g.y, g.z);
    }
    const uint32_t layer_cells = grid[0] * grid[1];
    if (planar) {
        p.planar_layer = n ? hash[0] / layer_cells : 0;
        p.scan_base = p.planar_layer * layer_cells;
        p.scan_cells = layer_cells;
    } else {
        p.scan_base = 0;
        p.scan_cells = grid[0] * grid[1] * grid[2];
    }
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return hash[a] < hash[b]; });
    sc.spos.resize(n);
    sc.off.assign((size_t)p.scan_cells + 1, 0u);
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t i = order[k];
        sc.spos[k] = make_float4(pos[4 * i], pos[4 * i + 1], pos[4 * i + 2], pos[4 * i + 3]);
        const uint32_t c = hash[i] - p.scan_base;
        if (c >= p.scan_cells) return -1;
        ++sc.off[c + 1];
    }
    for (uint32_t c = 0; c < p.scan_cells; ++c) sc.off[c + 1] += sc.off[c];
    return 0;
}

// squared distance of i to j seen through image shift (sx, sy, sz), as the
// neighbour loops form it (walk::rel)
template <int SYS>
float dist2(float4 pi, float4 pj, float sx, float sy, float sz)
{
    const float3 r = walk::rel<SYS>(pi, pj, sx, sy, sz);
    return r.x * r.x + r.y * r.y + r.z * r.z;
}

template <int SYS, bool PLANAR, bool TRIM, int G>
uint64_t check(const Scene &sc, uint64_t *visited)
{
    const DevParams &p = sc.p;
    const uint32_t n = p.n;
    uint64_t bad = 0;
    // image shifts a brute-force scan considers: none for DamBreak (its wrapped
    // cells hold particles at their own positions), x for Poiseuille, every axis
    // (z only in 3-D) for Peristalsis
    const int kx = SYS == CMAG_DAMBREAK ? 0 : 1;
    const int ky = SYS == CMAG_PERISTALSIS ? 1 : 0;
    const int kz = (SYS == CMAG_PERISTALSIS && !PLANAR) ? 1 : 0;
    std::map<uint32_t, int> walk, brute;
    for (uint32_t i = 0; i < n; ++i) {
        const float4 pi = sc.spos[i];
        const int3 g = grid_pos(p, pi.x, pi.y, pi.z);
        const float3 f = walk::frac_cell(p, pi);
        walk.clear();
        brute.clear();
        for (int lane = 0; lane < G; ++lane) {
            walk::for_each_candidate<SYS, PLANAR, TRIM, G>(
                p, sc.off.data(), lane, g, f, [&](uint32_t j, float sx, float sy, float sz) {
                    ++*visited;
                    if (j >= n) {
                        ++bad;
                        return;
                    }
                    if (dist2<SYS>(pi, sc.spos[j], sx, sy, sz) < p.support2) ++walk[j];
                });
        }
        for (uint32_t j = 0; j < n; ++j)
            for (int a = -kx; a <= kx; ++a)
                for (int b = -ky; b <= ky; ++b)
                    for (int c = -kz; c <= kz; ++c) {
                        const float sx = (float)a * p.wsx, sy = (float)b * p.wsy, sz = (float)c * p.wsz;
                        if (dist2<SYS>(pi, sc.spos[j], sx, sy, sz) < p.support2) ++brute[j];
                    }
        if (walk != brute) ++bad;
    }
    return bad;
}

template <int SYS, bool PLANAR, bool TRIM>
int64_t by_lanes(const Scene &sc, int lanes, uint64_t *visited)
{
    switch (lanes) {
    case 1: return (int64_t)check<SYS, PLANAR, TRIM, 1>(sc, visited);
    case 2: return (int64_t)check<SYS, PLANAR, TRIM, 2>(sc, visited);
    case 4: return (int64_t)check<SYS, PLANAR, TRIM, 4>(sc, visited);
    default: return -2;
    }
}

template <int SYS>
int64_t by_shape(const Scene &sc, int lanes, uint64_t *visited)
{
    if (sc.p.planar) {
        return sc.p.trim ? by_lanes<SYS, true, true>(sc, lanes, visited)
                         : by_lanes<SYS, true, false>(sc, lanes, visited);
    }
    return sc.p.trim ? by_lanes<SYS, false, true>(sc, lanes, visited)
                     : by_lanes<SYS, false, false>(sc, lanes, visited);
}

}  // namespace

// Number of particles whose in-support candidate set differs from brute force
// (or that saw an out-of-range index); -1: a planar scene's particle outside its
// layer; -2: unsupported lane count.  *visited: candidates the walk visited.
extern "C" int64_t walk_check(int system, int planar, int trim, int lanes, const uint32_t grid[3],
                              const float origin[3], float cell, float h, int cell_count,
                              const float *pos, uint32_t n, uint64_t *visited)
{
    Scene sc;
    if (build(sc, system, planar, trim, grid, origin, cell, h, cell_count, pos, n) != 0) return -1;
    *visited = 0;
    if (system == CMAG_DAMBREAK) return by_shape<CMAG_DAMBREAK>(sc, lanes, visited);
    if (system == CMAG_POISEUILLE) return by_shape<CMAG_POISEUILLE>(sc, lanes, visited);
    return by_shape<CMAG_PERISTALSIS>(sc, lanes, visited);
}

// The kept wall densities' fluid test (walk::fluid_near, the density side;
// wall_cache_note stamps a fluid particle's block of its wrapped cell) against
// brute force: for random cell-block stamps and random cells (inside the grid and
// up to two grid periods outside), fluid_near must report exactly whether some
// cell of the box g - c .. g + c, wrapped per axis, lies in a block stamped with
// the current step's stamp.  Returns the number of disagreements.
extern "C" int64_t wall_near_check(const uint32_t grid[3], int cell_count, uint32_t trials, uint64_t seed)
{
    DevParams p;
    std::memset(&p, 0, sizeof p);
    p.gx = grid[0];
    p.gy = grid[1];
    p.gz = grid[2];
    p.cell_count = cell_count;
    p.wc_nbx = (p.gx + 3u) / 4u;
    p.wc_nby = (p.gy + 3u) / 4u;
    p.wc_nbz = (p.gz + 3u) / 4u;
    std::vector<uint32_t> marks((size_t)p.wc_nbx * p.wc_nby * p.wc_nbz), state(4, 0u);
    const uint32_t stamp = 7u;
    state[kWcStamp] = stamp;
    p.wc_mark = marks.data();
    p.wc_state = state.data();
    uint64_t x = seed;
    auto next = [&]() {  // splitmix64
        x += 0x9e3779b97f4a7c15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    };
    auto residue = [](int v, uint32_t n) { const int m = v % (int)n; return (uint32_t)(m < 0 ? m + (int)n : m); };
    int64_t bad = 0;
    for (uint32_t t = 0; t < trials; ++t) {
        if (t % 64 == 0)  // a few stamped blocks among stale ones
            for (auto &m : marks) m = (next() % 97 == 0) ? stamp : (uint32_t)(next() % 7);
        const int g[3] = {(int)(next() % (5 * p.gx)) - 2 * (int)p.gx, (int)(next() % (5 * p.gy)) - 2 * (int)p.gy,
                          (int)(next() % (5 * p.gz)) - 2 * (int)p.gz};
        bool want = false;
        for (int dz = -cell_count; dz <= cell_count && !want; ++dz)
            for (int dy = -cell_count; dy <= cell_count && !want; ++dy)
                for (int dx = -cell_count; dx <= cell_count && !want; ++dx) {
                    const uint32_t bx = residue(g[0] + dx, p.gx) >> 2, by = residue(g[1] + dy, p.gy) >> 2,
                                   bz = residue(g[2] + dz, p.gz) >> 2;
                    want = marks[((size_t)bz * p.wc_nby + by) * p.wc_nbx + bx] == stamp;
                }
        if (walk::fluid_near(p, make_int3(g[0], g[1], g[2])) != want) ++bad;
    }
    return bad;
}
