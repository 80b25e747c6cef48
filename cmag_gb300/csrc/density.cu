// density.cu -- the density pass over cell-ordered particles (with the equation
// of state, and optionally the per-step interaction lists).
//
// Reference kernels (one thread per particle, 7^3 cell lookups each):
//   calculateDamBreakDensityD fluid_kernel.cu:130-169 (+ sumDensity :99-128)
//   calculatePoiseuilleDensityD poiseuilleFlowKernel.cu:141-182
//   computeDensityVariationD PeristalsisDensity.cu:39-79
//
// The particles of each neighbour row are visited as runs of consecutive sorted
// particles (neighbor_walk.cuh).  The pass also stores, per particle, p/rho^2 and
// rho (DamBreak) or 1/rho (the others), so the force loop needs no division per
// pair, and with interaction lists the neighbours the force loop will use.
//
// Every fused multiply-add is written out (__fmaf_rn and the paired forms); the
// library is compiled with -fmad=false, so no other multiply and add are fused.
// Results therefore do not depend on how the compiler schedules a particular
// template variant: a scene gives the same bits alone and inside a batch.
#include <cuda_runtime.h>

#include "kernels.h"
#include "neighbor_walk.cuh"

namespace cmag {

namespace {

using walk::for_each_candidate;
using walk::for_each_run;
using walk::frac_cell;
using walk::group_sum;
using walk::list_append;
using walk::records;
using walk::rel;
using walk::shift_code;

// Interaction lists the density pass records (template LIST): 0 none, 1 the
// force's exact pair set of this step, 2 lists kept over several steps (every
// particle within 2h + skin, for density and force).
constexpr int kNoList = 0, kStepList = 1, kKeptList = 2;

// Un-normalised Wendland sum over candidates [b, e) of one run, two candidates
// per step in paired FP32 (FFMA2/FMUL2/FADD2: two FP32 operations per issued
// instruction on sm_100+), scalar tail.  Adds max(1 - q/2, 0)^4 (2q + 1): zero
// outside the support without a compare and select (the loop is bound by the
// integer/compare pipe, not by FP32).
template <int SYS, bool PLANAR, bool TRIM, int LIST>
__device__ __forceinline__ void wendland_run(const DevParams &p, const float4 *__restrict__ spos,
                                             uint32_t b, uint32_t e, float4 pi, float sx, float sy,
                                             float sz, float2 &acc, bool record, uint32_t i,
                                             const NeighborList &nl, uint32_t &cnt)
{
    const uint32_t code = LIST ? shift_code(sx, sy, sz) : 0u;
    const float2 px = make_float2(pi.x, pi.x), py = make_float2(pi.y, pi.y),
                 pz = make_float2(pi.z, pi.z);
    const float2 m1 = make_float2(-1.0f, -1.0f), one = make_float2(1.0f, 1.0f),
                 nh2 = make_float2(-0.5f * p.inv_h, -0.5f * p.inv_h),
                 h2 = make_float2(2.0f * p.inv_h, 2.0f * p.inv_h), tiny = make_float2(1e-30f, 1e-30f);
    uint32_t j = b;
    for (; j + 1 < e; j += 2) {
        const float4 a = __ldg(spos + j), c = __ldg(spos + j + 1);
        float2 ax = make_float2(a.x, c.x), ay = make_float2(a.y, c.y), az = make_float2(a.z, c.z);
        if (SYS != CMAG_DAMBREAK) ax = __fadd2_rn(ax, make_float2(sx, sx));
        if (SYS == CMAG_PERISTALSIS) {
            ay = __fadd2_rn(ay, make_float2(sy, sy));
            az = __fadd2_rn(az, make_float2(sz, sz));
        }
        const float2 rx = __ffma2_rn(ax, m1, px), ry = __ffma2_rn(ay, m1, py);
        // planar scenes: all z equal, rz = 0 exactly, left out (same bits)
        const float2 dxy = __ffma2_rn(ry, ry, __fmul2_rn(rx, rx));
        const float2 rz = __ffma2_rn(az, m1, pz);
        const float2 d2 = PLANAR ? dxy : __ffma2_rn(rz, rz, dxy);
        const float2 dt = __fadd2_rn(d2, tiny);  // d2 = 0 (the particle itself) gives q = 0
        const float2 rs = make_float2(rsqrtf(dt.x), rsqrtf(dt.y));
        const float2 d = __fmul2_rn(d2, rs);  // |r|; q = |r| / h enters through nh2, h2
        float2 t = __ffma2_rn(d, nh2, one);   // 1 - q/2
        t = make_float2(fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f));  // 0 outside the support (q >= 2)
        const float2 t2 = __fmul2_rn(t, t);
        const float2 w = __fmul2_rn(__fmul2_rn(t2, t2), __ffma2_rn(d, h2, one));  // ... (2q + 1)
        acc = __fadd2_rn(acc, w);
        if (LIST && record) {
            const uint32_t v = j | code;  // j + 1 < 2^26: the next entry is v + 1
            if (records<SYS, TRIM, LIST == kKeptList>(p, i, j, d2.x, a.w)) list_append(nl, i, cnt, v);
            if (records<SYS, TRIM, LIST == kKeptList>(p, i, j + 1, d2.y, c.w)) list_append(nl, i, cnt, v + 1u);
        }
    }
    if (j < e) {  // the same operations as one half of a pair step
        const float4 pj = __ldg(spos + j);
        const float3 r = rel<SYS>(pi, pj, sx, sy, sz);
        const float dxy = __fmaf_rn(r.y, r.y, __fmul_rn(r.x, r.x));
        const float d2 = PLANAR ? dxy : __fmaf_rn(r.z, r.z, dxy);
        const float d = __fmul_rn(d2, rsqrtf(__fadd_rn(d2, 1e-30f)));
        const float t = fmaxf(__fmaf_rn(d, -0.5f * p.inv_h, 1.0f), 0.0f), t2 = __fmul_rn(t, t);
        const float w = __fmul_rn(__fmul_rn(t2, t2), __fmaf_rn(d, 2.0f * p.inv_h, 1.0f));
        acc.x = __fadd_rn(acc.x, w);
        if (LIST && record && records<SYS, TRIM, LIST == kKeptList>(p, i, j, d2, pj.w))
            list_append(nl, i, cnt, j | code);
    }
}

// ---------------------------------------------------------------- density --
// 256 threads; planar scenes (single or batched) and single 3-D DamBreak scenes
// 8 blocks per SM (32 registers: the batch and 3-D variants spill a few words to
// L1 and still run faster than at 6 blocks), the rest 6
template <int SYS, bool PLANAR, bool TRIM, int G, bool BATCH, int LIST>
__global__ void __launch_bounds__(256, (PLANAR || (!BATCH && SYS == CMAG_DAMBREAK)) ? 8 : 6)
    k_density(DevParams pv, BatchView bv, const float4 *__restrict__ spos,
              const uint32_t *__restrict__ off_all, float4 *__restrict__ meas,
              float2 *__restrict__ aux, NeighborList nl)
{
    pdl_entry();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = (BATCH ? bv.first : 0u) + t / G;
    const int lane = (int)(t % G);
    const bool active = t / G < (BATCH ? bv.count : pv.n);
    // a batch reads its scene's parameters; the scene's cells start at table_base
    const DevParams &p = BATCH ? bv.scenes[active ? bv.scene_of[i] : bv.scene_of[bv.first]] : pv;
    const uint32_t *off = off_all + p.table_base;
    const float4 pi = active ? spos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    // Poiseuille walls keep rest density (poiseuilleFlowKernel.cu:154-158)
    const bool pinned = SYS == CMAG_POISEUILLE && pi.w == 1.0f;
    // lists for every particle whose force is computed (DamBreak: fluid only);
    // lists kept over several steps serve the density too: every particle
    const bool record = LIST && active && (LIST == kKeptList || SYS != CMAG_DAMBREAK || pi.w == (float)CMAG_FLUID);
    // A DamBreak scene's non-fluid particle with no fluid particle in its cell
    // box: its walk would visit non-fluid particles only, which have not moved
    // since the epoch began, in the same runs and order, so its sum has the bits
    // of the walk of any step of the epoch.  wc: 0 walk as usual, 1 walk and keep
    // the result, 2 take the kept result.
    constexpr bool WC = SYS == CMAG_DAMBREAK && LIST != kKeptList;
    uint32_t wc = 0;
    if (WC && p.wc_entry && active && pi.w != (float)CMAG_FLUID &&
        !walk::fluid_near(p, grid_pos(p, pi.x, pi.y, pi.z))) {
        const float4 e = p.wc_entry[p.wc_idx[i]];
        wc = __float_as_uint(e.z) == p.wc_state[kWcEpoch] ? 2u : 1u;
        if (G == 1 && wc == 2u) {  // (lanes of a group leave together only at G = 1)
            meas[i] = make_float4(e.x, e.y, 0.0f, 0.0f);
            const float inv_rho = 1.0f / e.x;
            aux[i] = make_float2(e.y * inv_rho * inv_rho, e.x);
            if (LIST) nl.count[i] = 0;
            return;
        }
    }
    uint32_t cnt = 0;
    float sum = 0.0f;
    if (active && (!pinned || record) && wc != 2u) {  // a pinned wall walks only to record its list
        const int3 g = grid_pos(p, pi.x, pi.y, pi.z);
        if (p.kernel == CMAG_KERNEL_WENDLAND) {
            float2 acc = make_float2(0.0f, 0.0f);
            for_each_run<SYS, PLANAR, TRIM, G>(
                p, off, lane, g, frac_cell(p, pi),
                [&](uint32_t b, uint32_t e, float sx, float sy, float sz) {
                    wendland_run<SYS, PLANAR, TRIM, LIST>(p, spos, b, e, pi, sx, sy, sz, acc, record, i, nl, cnt);
                });
            sum = p.w_norm * (acc.x + acc.y);
        } else {
            for_each_candidate<SYS, PLANAR, TRIM, G>(
                p, off, lane, g, frac_cell(p, pi), [&](uint32_t j, float sx, float sy, float sz) {
                    const float4 pj = __ldg(spos + j);
                    const float3 r = rel<SYS>(pi, pj, sx, sy, sz);
                    const float dxy = __fmaf_rn(r.y, r.y, __fmul_rn(r.x, r.x));
                    const float d2 = PLANAR ? dxy : __fmaf_rn(r.z, r.z, dxy);
                    // evaluated for every candidate and selected: no divergent branch
                    const float w = kernel_w(p, fminf(d2 * rsqrtf(fmaxf(d2, 1e-30f)) * p.inv_h, 2.0f));
                    sum += (d2 < p.support2) ? w : 0.0f;
                    if (LIST && record && records<SYS, TRIM, LIST == kKeptList>(p, i, j, d2, pj.w))
                        list_append(nl, i, cnt, j | shift_code(sx, sy, sz));
                });
        }
    }
    if (LIST && active) {
        nl.count[i] = cnt;
        if (cnt > nl.cap && nl.overflow) *nl.overflow = 1u;
    }
    sum = group_sum<G>(sum);
    if (active && lane == 0) {
        float rho, pr;
        if (pinned) {
            rho = p.rho0;
            pr = p.p_wall;
        } else if (WC && wc == 2u) {
            const float4 e = p.wc_entry[p.wc_idx[i]];
            rho = e.x;
            pr = e.y;
        } else {
            rho = sum * p.mass;
            pr = eos_pressure(p, rho);
        }
        meas[i] = make_float4(rho, pr, 0.0f, SYS == CMAG_PERISTALSIS ? pi.w : 0.0f);
        const float inv_rho = 1.0f / rho;
        aux[i] = make_float2(pr * inv_rho * inv_rho, SYS == CMAG_DAMBREAK ? rho : inv_rho);
        if (WC && wc == 1u)
            p.wc_entry[p.wc_idx[i]] = make_float4(rho, pr, __uint_as_float(p.wc_state[kWcEpoch]), 0.0f);
    }
}

template <int SYS, bool PLANAR, bool TRIM, int G, int LIST>
void launch_d(const DevParams &p, const BatchView &bv, const float4 *spos, const uint32_t *off,
              float4 *meas, float2 *aux, const NeighborList &nl, cudaStream_t st)
{
    const uint64_t threads = (uint64_t)(bv.scenes ? bv.count : p.n) * G;
    const uint32_t blocks = (uint32_t)((threads + 255) / 256);
    if (bv.scenes)
        launch_pdl(k_density<SYS, PLANAR, TRIM, G, true, LIST>, blocks, 256, 0, st, p, bv, spos, off, meas, aux, nl);
    else
        launch_pdl(k_density<SYS, PLANAR, TRIM, G, false, LIST>, blocks, 256, 0, st, p, bv, spos, off, meas, aux, nl);
}

template <int SYS, bool PLANAR, bool TRIM>
void dispatch_g(int group, const DevParams &p, const BatchView &bv, const float4 *spos,
                const uint32_t *off, float4 *meas, float2 *aux, const NeighborList &nl, cudaStream_t st)
{
    if (nl.entry) {  // lists: one lane per particle
        if (p.verlet) launch_d<SYS, PLANAR, TRIM, 1, kKeptList>(p, bv, spos, off, meas, aux, nl, st);
        else launch_d<SYS, PLANAR, TRIM, 1, kStepList>(p, bv, spos, off, meas, aux, nl, st);
        return;
    }
    switch (group) {
    case 2: launch_d<SYS, PLANAR, TRIM, 2, kNoList>(p, bv, spos, off, meas, aux, nl, st); break;
    case 4: launch_d<SYS, PLANAR, TRIM, 4, kNoList>(p, bv, spos, off, meas, aux, nl, st); break;
    default: launch_d<SYS, PLANAR, TRIM, 1, kNoList>(p, bv, spos, off, meas, aux, nl, st); break;
    }
}

template <int SYS>
void dispatch(int group, const DevParams &p, const BatchView &bv, const float4 *spos,
              const uint32_t *off, float4 *meas, float2 *aux, const NeighborList &nl, cudaStream_t st)
{
    if (p.planar) {
        if (p.trim) dispatch_g<SYS, true, true>(group, p, bv, spos, off, meas, aux, nl, st);
        else dispatch_g<SYS, true, false>(group, p, bv, spos, off, meas, aux, nl, st);
    } else {
        if (p.trim) dispatch_g<SYS, false, true>(group, p, bv, spos, off, meas, aux, nl, st);
        else dispatch_g<SYS, false, false>(group, p, bv, spos, off, meas, aux, nl, st);
    }
}

// ------------------------------------------------- density from kept lists --
// Steps between list rebuilds (cmag_system_set_verlet): the density of every
// particle from its list (all other particles within 2h + skin at the rebuild,
// sorted indices of the rebuild's order), summed with the walk's arithmetic: the
// particle itself first (W(0)), then its entries in list order, two per step in
// paired FP32, zero beyond the support by the clamp of 1 - q/2.  The same pairs
// as the walk (every particle within 2h has moved less than skin/2 since the
// rebuild), in another summation order.  One thread per particle, entries of
// the next step loaded one step ahead.
template <int SYS, bool PLANAR>
__global__ void __launch_bounds__(256, 8)
    k_density_list(DevParams p, const float4 *__restrict__ spos, NeighborList nl,
                   float4 *__restrict__ meas, float2 *__restrict__ aux)
{
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 pi = spos[i];
    const bool pinned = SYS == CMAG_POISEUILLE && pi.w == 1.0f;
    float sum = 0.0f;
    if (!pinned) {
        const uint32_t cnt = min(__ldg(nl.count + i), nl.cap);
        const uint32_t *ep = nl.entry + i;
        auto shift_of = [&](uint32_t en, float &sx, float &sy, float &sz) {
            const uint32_t cd = en >> kListIndexBits;
            sx = (float)((int)(cd & 3u) - 1) * p.wsx;
            sy = (float)((int)((cd >> 2) & 3u) - 1) * p.wsy;
            sz = PLANAR ? 0.0f : (float)((int)((cd >> 4) & 3u) - 1) * p.wsz;
        };
        if (p.kernel == CMAG_KERNEL_WENDLAND) {
            const float2 px = make_float2(pi.x, pi.x), py = make_float2(pi.y, pi.y),
                         pz = make_float2(pi.z, pi.z);
            const float2 m1 = make_float2(-1.0f, -1.0f), one = make_float2(1.0f, 1.0f),
                         nh2 = make_float2(-0.5f * p.inv_h, -0.5f * p.inv_h),
                         h2 = make_float2(2.0f * p.inv_h, 2.0f * p.inv_h),
                         tiny = make_float2(1e-30f, 1e-30f);
            float2 acc = make_float2(1.0f, 0.0f);  // the particle itself: W(0) / w_norm = 1
            uint32_t k = 0;
            uint32_t e0 = 0, e1 = 0;
            if (cnt >= 2) {
                e0 = __ldg(ep);
                e1 = __ldg(ep + nl.stride);
            }
            for (; k + 1 < cnt; k += 2) {
                uint32_t n0 = 0, n1 = 0;
                if (k + 3 < cnt) {
                    n0 = __ldg(ep + (size_t)(k + 2) * nl.stride);
                    n1 = __ldg(ep + (size_t)(k + 3) * nl.stride);
                }
                const float4 a = __ldg(spos + (e0 & kListIndexMask)), c = __ldg(spos + (e1 & kListIndexMask));
                float2 ax = make_float2(a.x, c.x), ay = make_float2(a.y, c.y), az = make_float2(a.z, c.z);
                if (SYS != CMAG_DAMBREAK) {
                    float sx0, sy0, sz0, sx1, sy1, sz1;
                    shift_of(e0, sx0, sy0, sz0);
                    shift_of(e1, sx1, sy1, sz1);
                    ax = __fadd2_rn(ax, make_float2(sx0, sx1));
                    if (SYS == CMAG_PERISTALSIS) {
                        ay = __fadd2_rn(ay, make_float2(sy0, sy1));
                        az = __fadd2_rn(az, make_float2(sz0, sz1));
                    }
                }
                e0 = n0;
                e1 = n1;
                const float2 rx = __ffma2_rn(ax, m1, px), ry = __ffma2_rn(ay, m1, py);
                const float2 dxy = __ffma2_rn(ry, ry, __fmul2_rn(rx, rx));
                const float2 rz = __ffma2_rn(az, m1, pz);
                const float2 d2 = PLANAR ? dxy : __ffma2_rn(rz, rz, dxy);
                const float2 dt = __fadd2_rn(d2, tiny);
                const float2 rs = make_float2(rsqrtf(dt.x), rsqrtf(dt.y));
                const float2 d = __fmul2_rn(d2, rs);
                float2 t = __ffma2_rn(d, nh2, one);
                t = make_float2(fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f));
                const float2 t2 = __fmul2_rn(t, t);
                const float2 w = __fmul2_rn(__fmul2_rn(t2, t2), __ffma2_rn(d, h2, one));
                acc = __fadd2_rn(acc, w);
            }
            if (k < cnt) {
                const uint32_t en = __ldg(ep + (size_t)k * nl.stride);
                float sx = 0.0f, sy = 0.0f, sz = 0.0f;
                if (SYS != CMAG_DAMBREAK) shift_of(en, sx, sy, sz);
                const float4 pj = __ldg(spos + (en & kListIndexMask));
                const float3 r = rel<SYS>(pi, pj, sx, sy, sz);
                const float dxy = __fmaf_rn(r.y, r.y, __fmul_rn(r.x, r.x));
                const float d2 = PLANAR ? dxy : __fmaf_rn(r.z, r.z, dxy);
                const float d = __fmul_rn(d2, rsqrtf(__fadd_rn(d2, 1e-30f)));
                const float t = fmaxf(__fmaf_rn(d, -0.5f * p.inv_h, 1.0f), 0.0f), t2 = __fmul_rn(t, t);
                acc.x = __fadd_rn(acc.x, __fmul_rn(__fmul_rn(t2, t2), __fmaf_rn(d, 2.0f * p.inv_h, 1.0f)));
            }
            sum = p.w_norm * (acc.x + acc.y);
        } else {
            sum = kernel_w(p, 0.0f);  // the particle itself
            for (uint32_t k = 0; k < cnt; ++k) {
                const uint32_t en = __ldg(ep + (size_t)k * nl.stride);
                float sx = 0.0f, sy = 0.0f, sz = 0.0f;
                if (SYS != CMAG_DAMBREAK) shift_of(en, sx, sy, sz);
                const float4 pj = __ldg(spos + (en & kListIndexMask));
                const float3 r = rel<SYS>(pi, pj, sx, sy, sz);
                const float dxy = __fmaf_rn(r.y, r.y, __fmul_rn(r.x, r.x));
                const float d2 = PLANAR ? dxy : __fmaf_rn(r.z, r.z, dxy);
                const float w = kernel_w(p, fminf(d2 * rsqrtf(fmaxf(d2, 1e-30f)) * p.inv_h, 2.0f));
                sum += (d2 < p.support2) ? w : 0.0f;
            }
        }
    }
    float rho, pr;
    if (pinned) {
        rho = p.rho0;
        pr = p.p_wall;
    } else {
        rho = sum * p.mass;
        pr = eos_pressure(p, rho);
    }
    meas[i] = make_float4(rho, pr, 0.0f, SYS == CMAG_PERISTALSIS ? pi.w : 0.0f);
    const float inv_rho = 1.0f / rho;
    aux[i] = make_float2(pr * inv_rho * inv_rho, SYS == CMAG_DAMBREAK ? rho : inv_rho);
}

template <int SYS>
void launch_dl(const DevParams &p, const float4 *spos, const NeighborList &nl, float4 *meas, float2 *aux,
               cudaStream_t st)
{
    const uint32_t blocks = (p.n + 255) / 256;
    if (p.planar) launch_pdl(k_density_list<SYS, true>, blocks, 256, 0, st, p, spos, nl, meas, aux);
    else launch_pdl(k_density_list<SYS, false>, blocks, 256, 0, st, p, spos, nl, meas, aux);
}

}  // namespace

// p: the scene's parameters, or for a batch launch group the parameters of any
// scene of the group (family, planar and trim select the kernel variant)
void launch_density(const DevParams &p, const BatchView &bv, int group, const float4 *spos,
                    const uint32_t *off, float4 *meas, float2 *aux, const NeighborList &nl,
                    cudaStream_t st)
{
    if ((bv.scenes ? bv.count : p.n) == 0) return;
    if (p.system == CMAG_DAMBREAK) dispatch<CMAG_DAMBREAK>(group, p, bv, spos, off, meas, aux, nl, st);
    else if (p.system == CMAG_POISEUILLE) dispatch<CMAG_POISEUILLE>(group, p, bv, spos, off, meas, aux, nl, st);
    else dispatch<CMAG_PERISTALSIS>(group, p, bv, spos, off, meas, aux, nl, st);
}

// Density from the lists kept since the last rebuild (single scenes).
void launch_density_list(const DevParams &p, const float4 *spos, const NeighborList &nl, float4 *meas,
                         float2 *aux, cudaStream_t st)
{
    if (p.n == 0) return;
    if (p.system == CMAG_DAMBREAK) launch_dl<CMAG_DAMBREAK>(p, spos, nl, meas, aux, st);
    else if (p.system == CMAG_POISEUILLE) launch_dl<CMAG_POISEUILLE>(p, spos, nl, meas, aux, st);
    else launch_dl<CMAG_PERISTALSIS>(p, spos, nl, meas, aux, st);
}

}  // namespace cmag
