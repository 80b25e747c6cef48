// neighbor_walk.cuh -- the walk over a particle's neighbour cells as runs of
// consecutive sorted particles, shared by the density/force loops
// (density.cu, force.cu) and the learned closure's feature loop (closure.cu).
//
// The (2c+1)^2 rows of the cell box (only the particle's own z layer for planar
// 2-D scenes) are walked as runs of consecutive cells: a run's particles are one
// contiguous sorted range [off[a], off[b+1]) of the dense offset table.  A group
// of G lanes shares a particle and splits its rows between them (row r goes to
// lane r mod G).  Runs wrap at most once per row; a wrapped run carries the
// periodic image shift of its unmasked cell coordinates, as the reference's
// per-cell shift (poiseuilleFlowKernel.cu:121-127, PeristalsisUtil.cu:4-11).
// With TRIM each row's run is trimmed to the support circle, in cell units from
// the particle's fractional cell coordinates.
#pragma once

#include "sph_common.cuh"

namespace cmag {
namespace walk {

constexpr float kMargin = 1e-3f;  // cells: covers rounding of the cell assignment

template <bool PLANAR>
__device__ __forceinline__ int rows_of(int c)
{
    return PLANAR ? (2 * c + 1) : (2 * c + 1) * (2 * c + 1);
}

__device__ __forceinline__ uint32_t wrap_axis(int v, uint32_t n)
{
    // one period away at most for particles inside the grid; any value for
    // particles that left it
    if ((uint32_t)v < n) return (uint32_t)v;
    if (v < 0 && v >= -(int)n) return (uint32_t)(v + (int)n);
    if (v >= (int)n && v < 2 * (int)n) return (uint32_t)(v - (int)n);
    int m = v % (int)n;
    return (uint32_t)(m < 0 ? m + (int)n : m);
}

// Wall density cache, density side: whether a fluid particle was hashed this
// step into any 4x4x4 block that holds a cell of the box of cells g - c .. g + c
// (wrapped per axis like the walk's rows).  Per axis the box's cells are one
// wrapped range, i.e. at most two ranges of blocks.
struct BlockSpan {
    uint32_t a0, a1, b0, b1;  // blocks [a0, a1] and [b0, b1] (b0 > b1: none)
};

__device__ __forceinline__ BlockSpan box_blocks(int v, int c, uint32_t n)
{
    BlockSpan r;
    r.b0 = 1;
    r.b1 = 0;
    const uint32_t len = 2u * (uint32_t)c + 1u;
    if (len >= n) {
        r.a0 = 0;
        r.a1 = (n - 1u) >> 2;
        return r;
    }
    const uint32_t s = wrap_axis(v - c, n);
    r.a0 = s >> 2;
    if (s + len <= n) {
        r.a1 = (s + len - 1u) >> 2;
    } else {
        r.a1 = (n - 1u) >> 2;
        r.b0 = 0;
        r.b1 = (s + len - 1u - n) >> 2;
    }
    return r;
}

__device__ __forceinline__ bool fluid_near(const DevParams &p, int3 g)
{
    const int c = p.cell_count;
    const BlockSpan X = box_blocks(g.x, c, p.gx), Y = box_blocks(g.y, c, p.gy), Z = box_blocks(g.z, c, p.gz);
    const uint32_t stamp = p.wc_state[kWcStamp];
    for (int zs = 0; zs < 2; ++zs) {
        const uint32_t z0 = zs ? Z.b0 : Z.a0, z1 = zs ? Z.b1 : Z.a1;
        for (uint32_t z = z0; z <= z1; ++z)
            for (int ys = 0; ys < 2; ++ys) {
                const uint32_t y0 = ys ? Y.b0 : Y.a0, y1 = ys ? Y.b1 : Y.a1;
                for (uint32_t y = y0; y <= y1; ++y) {
                    const uint32_t *row = p.wc_mark + (z * p.wc_nby + y) * p.wc_nbx;
                    for (int xs = 0; xs < 2; ++xs) {
                        const uint32_t x0 = xs ? X.b0 : X.a0, x1 = xs ? X.b1 : X.a1;
                        for (uint32_t x = x0; x <= x1; ++x)
                            if (row[x] == stamp) return true;
                    }
                }
            }
    }
    return false;
}

// The runs of one row of the cell box: [b0, e0) with x image shift sx0 and,
// when the row wraps in x, [b1, e1) with sx1 (empty otherwise); sy, sz: the
// row's image shifts.
struct RowRuns {
    uint32_t b0, e0, b1, e1;
    float sx0, sx1, sy, sz;
};

// What a row walk keeps per z slab of the cell box: the support radius squared
// (cells) left after the slab's z distance, the slab's table row base and its
// periodic image shift.
struct Slab {
    float r2z;      // support^2 - dz_min^2, in cells^2 (trimming only)
    uint32_t base;  // wrapped z cell * gy
    float sz;
};

// The trim's distance term along one axis: the distance in cells from the
// particle at f to the band of cells [u, u + 1), less the margin, is
// max(t, -1 - 2 margin - t, 0) with t = u - f - margin (u above f: the band's
// near edge; below: its far edge; the particle's own band: 0).
__device__ __forceinline__ float band_gap(float t)
{
    return fmaxf(fmaxf(t, (-1.0f - 2.0f * kMargin) - t), 0.0f);
}

template <int SYS, bool PLANAR, bool TRIM>
__device__ __forceinline__ Slab slab_at(const DevParams &p, int dz, int gz, float fz)
{
    Slab sl;
    const int zu = gz + dz;
    sl.base = (PLANAR ? p.planar_layer : wrap_axis(zu, p.gz)) * p.gy;
    sl.sz = (SYS == CMAG_PERISTALSIS && !PLANAR) ? (float)eval_shift(zu, p.gz) * p.wsz : 0.0f;
    if (TRIM) {
        const float dzm = PLANAR ? 0.0f : band_gap(((float)zu - fz) - kMargin);
        sl.r2z = __fmaf_rn(-dzm, dzm, p.support2_cells);
    } else {
        sl.r2z = 0.0f;
    }
    return sl;
}

// Row (dy, dz) of particle (fx,fy,fz) (fractional cell coordinates) in cell g,
// with the row's slab terms in sl.  Returns false when the row holds no
// candidates.
template <int SYS, bool PLANAR, bool TRIM>
__device__ __forceinline__ bool row_runs(const DevParams &p, const uint32_t *__restrict__ off,
                                         int dy, const Slab &sl, int3 g, float fx, float fy,
                                         RowRuns &rr)
{
    const int c = p.cell_count;
    const int yu = g.y + dy;
    int xa = g.x - c, xb = g.x + c;
    if (TRIM) {
        const float dym = band_gap(((float)yu - fy) - kMargin);
        // planar scenes: one slab, its terms straight from the parameters
        const float r2 = __fmaf_rn(-dym, dym, PLANAR ? p.support2_cells : sl.r2z);
        if (r2 <= 0.0f) return false;
        // conservative half width: the approximate square root errs by far less
        // than the margin
        const float R = __fmaf_rn(r2, rsqrtf(r2), kMargin);
        xa = max(xa, __float2int_rd(fx - R));
        xb = min(xb, __float2int_rd(fx + R));
        if (xa > xb) return false;
    }
    const uint32_t zbase = PLANAR ? p.planar_layer * p.gy : sl.base;
    const uint32_t row = (zbase + wrap_axis(yu, p.gy)) * p.gx - p.scan_base;
    if (row >= p.scan_cells) return false;  // outside the offset table: no particles
    rr.sy = (SYS == CMAG_PERISTALSIS) ? (float)eval_shift(yu, p.gy) * p.wsy : 0.0f;
    rr.sz = PLANAR ? 0.0f : sl.sz;
    const uint32_t xma = wrap_axis(xa, p.gx);
    const uint32_t len = (uint32_t)(xb - xa);
    rr.sx0 = (SYS == CMAG_DAMBREAK) ? 0.0f : (float)eval_shift(xa, p.gx) * p.wsx;
    rr.b0 = __ldg(off + row + xma);
    if (xma + len < p.gx) {
        rr.e0 = __ldg(off + row + xma + len + 1);
        rr.b1 = rr.e1 = 0;
        rr.sx1 = 0.0f;
    } else {
        rr.e0 = __ldg(off + row + p.gx);
        rr.b1 = __ldg(off + row);
        rr.e1 = __ldg(off + row + (xma + len - p.gx) + 1);
        rr.sx1 = (SYS == CMAG_DAMBREAK) ? 0.0f : (float)eval_shift(xb, p.gx) * p.wsx;
    }
    return true;
}

// Calls visit_run(b, e, sx, sy, sz) for every run of the rows this lane owns
// (rows r = lane, lane + G, ... of the (2c+1)^2 box, dy fastest).  The slab
// terms are recomputed when a lane's row moves to the next z slab.
template <int SYS, bool PLANAR, bool TRIM, int G, class VisitRun>
__device__ __forceinline__ void for_each_run(const DevParams &p, const uint32_t *__restrict__ off,
                                             int lane, int3 g, float3 f, VisitRun &&visit_run)
{
    const int c = p.cell_count;
    const int w = 2 * c + 1;
    int dy = (G == 1) ? -c : (lane % w) - c;
    int dz = PLANAR ? 0 : ((G == 1) ? -c : (lane / w) - c);
    const int nrows = rows_of<PLANAR>(c);
    Slab sl;
    if (!PLANAR) sl = slab_at<SYS, PLANAR, TRIM>(p, dz, g.z, f.z);
    for (int r = lane; r < nrows; r += G) {
        RowRuns rr;
        if (row_runs<SYS, PLANAR, TRIM>(p, off, dy, sl, g, f.x, f.y, rr)) {
            visit_run(rr.b0, rr.e0, rr.sx0, rr.sy, rr.sz);
            if (rr.e1 > rr.b1) visit_run(rr.b1, rr.e1, rr.sx1, rr.sy, rr.sz);
        }
        dy += G;
        if (dy > c) {
            do {
                dy -= w;
                ++dz;
            } while (dy > c);
            if (!PLANAR) sl = slab_at<SYS, PLANAR, TRIM>(p, dz, g.z, f.z);
        }
    }
}

// Calls visit(j, sx, sy, sz) for every candidate of the rows this lane owns.
template <int SYS, bool PLANAR, bool TRIM, int G, class Visit>
__device__ __forceinline__ void for_each_candidate(const DevParams &p,
                                                   const uint32_t *__restrict__ off, int lane,
                                                   int3 g, float3 f, Visit &&visit)
{
    for_each_run<SYS, PLANAR, TRIM, G>(p, off, lane, g, f,
                                       [&](uint32_t b, uint32_t e, float sx, float sy, float sz) {
#pragma unroll 2
                                           for (uint32_t j = b; j < e; ++j) visit(j, sx, sy, sz);
                                       });
}

// Relative position of candidate j seen through its image shift.  Only the
// families with periodic images add the shift (DamBreak none, Poiseuille x only);
// the compiler cannot drop an added 0.0f by itself (signed zeros).
template <int SYS>
__device__ __forceinline__ float3 rel(float4 pi, float4 pj, float sx, float sy, float sz)
{
    if (SYS == CMAG_DAMBREAK) return make_float3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z);
    if (SYS == CMAG_POISEUILLE) return make_float3(pi.x - (pj.x + sx), pi.y - pj.y, pi.z - pj.z);
    return make_float3(pi.x - (pj.x + sx), pi.y - (pj.y + sy), pi.z - (pj.z + sz));
}

__device__ __forceinline__ float3 frac_cell(const DevParams &p, float4 q)
{
    return make_float3((q.x - p.ox) * p.inv_csx, (q.y - p.oy) * p.inv_csy, (q.z - p.oz) * p.inv_csz);
}


// ---- pieces shared by the density and force loops --------------------------

// Whether the force loop of a particle uses a candidate at squared distance d2
// (type w): inside the support, 0 < d2 < (2h)^2 (d2 = 0 is the particle itself or
// a coincident one, which the force skips), or a DamBreak wall without the q < 2
// cut-off.  d2 is a sum of squares (+0 or positive, or NaN), so the range test is
// one unsigned compare of the bit patterns.
template <int SYS, bool TRIM>
__device__ __forceinline__ bool interacts(const DevParams &p, float d2, float w)
{
    const bool inside = __float_as_uint(d2) - 1u < __float_as_uint(p.support2) - 1u;
    if (SYS == CMAG_DAMBREAK && !TRIM) return inside || (w != (float)CMAG_FLUID && d2 > 0.0f);
    return inside;
}

// list entry code of a run's image shift: 2 bits per axis, 0/1/2 for -1/0/+1
__device__ __forceinline__ uint32_t shift_code(float sx, float sy, float sz)
{
    const uint32_t cx = sx > 0.0f ? 2u : (sx < 0.0f ? 0u : 1u);
    const uint32_t cy = sy > 0.0f ? 2u : (sy < 0.0f ? 0u : 1u);
    const uint32_t cz = sz > 0.0f ? 2u : (sz < 0.0f ? 0u : 1u);
    return (cx | (cy << 2) | (cz << 4)) << kListIndexBits;
}

__device__ __forceinline__ void list_append(const NeighborList &nl, uint32_t i, uint32_t &cnt,
                                            uint32_t value)
{
    if (cnt < nl.cap) nl.entry[(size_t)cnt * nl.stride + i] = value;
    ++cnt;
}

// Whether a list records candidate j (squared distance d2, type w) of particle i:
// the force's exact pair set (interacts) for per-step lists; for lists kept over
// several steps every other particle closer than 2h + skin, coincident ones
// included (the density sums them).
template <int SYS, bool TRIM, bool KEEP>
__device__ __forceinline__ bool records(const DevParams &p, uint32_t i, uint32_t j, float d2, float w)
{
    if (KEEP) return j != i && d2 < p.list_r2;
    return interacts<SYS, TRIM>(p, d2, w);
}

template <int G>
__device__ __forceinline__ float group_sum(float v)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o, G);
    return v;
}

}  // namespace walk
}  // namespace cmag
