// closure.cu -- the learned closure's kernels (the C ABI is in closure_api.cu).
//
// A coarse DamBreak run misses the sub-grid part of the pressure, viscous and
// wall accelerations that a run at half its spacing resolves.  The closure
// predicts that part per fluid particle from 16 features of the particle and its
// neighbours and adds it to the acceleration before integration.  No reference
// counterpart; the features reuse the neighbour walk of the density and force
// loops.
//
// Features of fluid particle i (V_j = m / rho_j, W_ij = W(|x_i - x_j| / h), the
// sums over every particle j, i included, inside the support):
//   0      rho_i / rho0 - 1            1      p_i / B
//   2..4   sum V_j W_ij (x_j - x_i) / h
//   5..7   sum V_j W_ij (v_j - v_i) / c0
//   8      sum V_j W_ij                 9      sum V_j W_ij |x_j - x_i|^2 / h^2
//   10     sum over wall particles of V_j W_ij
//   11..13 the uncorrected acceleration a_i / |g|
//   14     sum V_j (v_j - v_i) . grad_i W_ij * h / c0
//   15     |v_i| / c0
// (v: the leap-frog velocity the force loop uses; rho, p: this step's density.)
//
// Network: x = bf16((f - mean) * inv_std); h1 = bf16(silu(W1 x + b1));
// h2 = bf16(silu(W2 h1 + b2)); h3 = bf16(silu(W3 h2 + b3)); y = W4 h3 + b4;
// correction = out_scale * clamp(y, +-out_limit) (the limit guards a coarse run
// against outputs far outside the training data; none by default).  BF16
// parameters and activations, FP32 dot products
// on the FP32 pipes (the products of two BF16 values are exact in FP32).
// Training: the loss 0.5/n sum |y - t|^2, gradients through the same forward
// (rounding treated as identity), Adam on an FP32 master copy.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "closure.h"
#include "host_common.h"
#include "neighbor_walk.cuh"

namespace cmag {

namespace {

constexpr int kTile = 128;       // samples (particles) per block
constexpr int kRow = 68;         // floats per per-sample row (conflict-free float4 rows)
constexpr int kXRow = 20;        // floats per input row
constexpr int kWPad = (kClosureParams + 3) & ~3;

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }

__device__ __forceinline__ float act(float z) { return bf16r(z * sigmoid(z)); }

__device__ __forceinline__ float dact(float z)
{
    const float s = sigmoid(z);
    return s * (1.0f + z * (1.0f - s));
}

// BF16 parameters -> FP32 shared copy
__device__ __forceinline__ void load_weights(float *sw, const __nv_bfloat16 *w)
{
    for (int k = threadIdx.x; k < kWPad; k += blockDim.x)
        sw[k] = k < kClosureParams ? __bfloat162float(w[k]) : 0.0f;
}

// One dense layer for the calling thread's sample: out[o] = act(b[o] + W[o] . in)
// for o < NO, input in registers, outputs to the thread's row of `dst`
// (pre-activation values when STORE_Z).
template <int NI, int NO, bool STORE_Z>
__device__ __forceinline__ void dense_row(const float *__restrict__ sw, int offw, int offb,
                                          const float (&in)[NI], float *dst)
{
#pragma unroll 1
    for (int o = 0; o < NO; ++o) {
        const float4 *wr = reinterpret_cast<const float4 *>(sw + offw + o * NI);
        float z = sw[offb + o];
#pragma unroll
        for (int q = 0; q < NI / 4; ++q) {
            const float4 w = wr[q];
            z = __fmaf_rn(w.x, in[4 * q], z);
            z = __fmaf_rn(w.y, in[4 * q + 1], z);
            z = __fmaf_rn(w.z, in[4 * q + 2], z);
            z = __fmaf_rn(w.w, in[4 * q + 3], z);
        }
        dst[o] = STORE_Z ? z : act(z);
    }
}

template <int N>
__device__ __forceinline__ void load_row(const float *src, float (&v)[N])
{
    const float4 *s = reinterpret_cast<const float4 *>(src);
#pragma unroll
    for (int q = 0; q < N / 4; ++q) {
        const float4 t = s[q];
        v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
    }
}

__device__ __forceinline__ void normalise(const float *mean, const float *inv_std,
                                          const float (&f)[kFeat], float (&x)[kFeat])
{
#pragma unroll
    for (int k = 0; k < kFeat; ++k) x[k] = bf16r((f[k] - mean[k]) * inv_std[k]);
}

// The 16 features of sorted fluid particle i (acc_i: its uncorrected acceleration).
template <bool PLANAR, bool TRIM>
__device__ __forceinline__ void features(const DevParams &p, const float4 *__restrict__ spos,
                                         const float4 *__restrict__ svel,
                                         const float2 *__restrict__ aux, float4 mi,
                                         const uint32_t *__restrict__ off, uint32_t i, float4 pi,
                                         float4 acc_i, float (&f)[kFeat])
{
    const float4 vi = __ldg(svel + i);
    const float ih = p.inv_h, ic = 1.0f / p.c0;
    float s1x = 0.f, s1y = 0.f, s1z = 0.f, svx = 0.f, svy = 0.f, svz = 0.f;
    float shep = 0.f, s2 = 0.f, wall = 0.f, div = 0.f;
    const int3 g = grid_pos(p, pi.x, pi.y, pi.z);
    walk::for_each_candidate<CMAG_DAMBREAK, PLANAR, TRIM, 1>(
        p, off, 0, g, walk::frac_cell(p, pi), [&](uint32_t j, float, float, float) {
            const float4 pj = __ldg(spos + j);
            const float rx = pj.x - pi.x, ry = pj.y - pi.y, rz = pj.z - pi.z;  // x_j - x_i
            const float d2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, rx * rx));
            if (!(d2 < p.support2)) return;
            const float inv_d = d2 > 0.0f ? rsqrtf(d2) : 0.0f;
            const float q = d2 * inv_d * ih;
            const float vol = p.mass / __ldg(aux + j).y;
            const float vw = vol * kernel_w(p, q);
            const float4 vj = __ldg(svel + j);
            const float dvx = vj.x - vi.x, dvy = vj.y - vi.y, dvz = vj.z - vi.z;
            s1x = __fmaf_rn(vw, rx, s1x); s1y = __fmaf_rn(vw, ry, s1y); s1z = __fmaf_rn(vw, rz, s1z);
            svx = __fmaf_rn(vw, dvx, svx); svy = __fmaf_rn(vw, dvy, svy); svz = __fmaf_rn(vw, dvz, svz);
            shep += vw;
            s2 = __fmaf_rn(vw, d2, s2);
            if (pj.w != (float)CMAG_FLUID) wall += vw;
            if (d2 > 0.0f) {
                // grad_i W_ij = dW/dr (x_i - x_j) / |x_i - x_j|
                const float gw = kernel_dw(p, q) * inv_d;
                const float dot = __fmaf_rn(dvz, rz, __fmaf_rn(dvy, ry, dvx * rx));
                div = __fmaf_rn(-vol * gw, dot, div);
            }
        });
    const float ig = rsqrtf(p.gvx * p.gvx + p.gvy * p.gvy + p.gvz * p.gvz);
    f[0] = mi.x / p.rho0 - 1.0f;
    f[1] = mi.y / p.B;
    f[2] = s1x * ih; f[3] = s1y * ih; f[4] = s1z * ih;
    f[5] = svx * ic; f[6] = svy * ic; f[7] = svz * ic;
    f[8] = shep;
    f[9] = s2 * ih * ih;
    f[10] = wall;
    f[11] = acc_i.x * ig; f[12] = acc_i.y * ig; f[13] = acc_i.z * ig;
    f[14] = div * p.h * ic;
    f[15] = sqrtf(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z) * ic;
}

// NORM false: the raw features of every fluid particle to feat[o * 16] (original
// order o); NORM true: the normalised BF16 network input of every sorted particle
// to xb[i * 16] (zeros for walls).
template <bool PLANAR, bool TRIM, bool NORM>
__global__ void __launch_bounds__(256)
    k_closure_features(DevParams p, ClosureView c, const float4 *__restrict__ spos,
                       const float4 *__restrict__ svel, const float2 *__restrict__ aux,
                       const float4 *__restrict__ meas, const uint32_t *__restrict__ idx,
                       const uint32_t *__restrict__ off, const float4 *__restrict__ acc,
                       float *feat, __nv_bfloat16 *xb)
{
    pdl_entry();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 pi = spos[i];
    const uint32_t o = idx[i];
    const bool fluid = pi.w == (float)CMAG_FLUID && o < p.n;  // o < n unless the sort failed
    if (NORM && !fluid) {
        uint4 *dst = reinterpret_cast<uint4 *>(xb + (size_t)i * kFeat);
        dst[0] = dst[1] = make_uint4(0, 0, 0, 0);
    }
    if (!fluid) return;
    float f[kFeat];
    features<PLANAR, TRIM>(p, spos, svel, aux, meas[i], off, i, pi, acc[o], f);
    if (!NORM) {
        float4 *dst = reinterpret_cast<float4 *>(feat + (size_t)o * kFeat);
#pragma unroll
        for (int q = 0; q < kFeat / 4; ++q) dst[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
        return;
    }
    float x[kFeat];
    normalise(c.mean, c.inv_std, f, x);
    uint32_t w[kFeat / 2];
#pragma unroll
    for (int k = 0; k < kFeat / 2; ++k) {
        const __nv_bfloat162 v = __floats2bfloat162_rn(x[2 * k], x[2 * k + 1]);
        w[k] = *reinterpret_cast<const uint32_t *>(&v);
    }
    uint4 *dst = reinterpret_cast<uint4 *>(xb + (size_t)i * kFeat);
    dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
    dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

// raw FP32 feature rows -> normalised BF16 network input rows
__global__ void k_normalise(ClosureView c, const float *__restrict__ feat, uint32_t n,
                            __nv_bfloat16 *__restrict__ xb)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float f[kFeat], x[kFeat];
    load_row(feat + (size_t)s * kFeat, f);
    normalise(c.mean, c.inv_std, f, x);
#pragma unroll
    for (int k = 0; k < kFeat / 2; ++k)
        reinterpret_cast<__nv_bfloat162 *>(xb + (size_t)s * kFeat)[k] = __floats2bfloat162_rn(x[2 * k], x[2 * k + 1]);
}

// ---- the network on the tensor cores: mma.sync m16n8k16, BF16 in, FP32 accumulate.
// A warp evaluates 16 rows at a time; a layer's FP32 accumulator fragments become
// the next layer's BF16 A fragments in registers (the C layout of n-tiles 2j and
// 2j+1 is the A layout of k-tile j), so activations never leave the registers.

constexpr int kW1Stride = 24;   // BF16 per shared row of W1 (16 + 8: conflict-free fragment loads)
constexpr int kWStride = 72;    // BF16 per shared row of W2, W3, W4 (64 + 8)
constexpr int kSW1 = 0, kSW2 = kSW1 + kHidden * kW1Stride, kSW3 = kSW2 + kHidden * kWStride,
              kSW4 = kSW3 + kHidden * kWStride, kSWEnd = kSW4 + 8 * kWStride;
constexpr int kSB1 = 0, kSB2 = kSB1 + kHidden, kSB3 = kSB2 + kHidden, kSB4 = kSB3 + kHidden,
              kSBEnd = kSB4 + 8;

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_silu(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo * sigmoid(lo), hi * sigmoid(hi));
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16 *p)
{
    return *reinterpret_cast<const uint32_t *>(p);
}

// one hidden layer: c[nt] = bias + A x W^T over KT k-tiles; W rows of `stride` BF16
template <int KT>
__device__ __forceinline__ void hidden_layer(const __nv_bfloat16 *W, int stride, const float *b,
                                             const uint32_t (&a)[KT][4], float (&c)[8][4], int g, int t)
{
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        c[nt][0] = c[nt][2] = b[nt * 8 + 2 * t];
        c[nt][1] = c[nt][3] = b[nt * 8 + 2 * t + 1];
    }
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const __nv_bfloat16 *row = W + (nt * 8 + g) * stride + kt * 16 + 2 * t;
            mma16816(c[nt], a[kt], lds32(row), lds32(row + 8));
        }
}

__device__ __forceinline__ void to_a(const float (&c)[8][4], uint32_t (&a)[4][4])
{
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = pack_silu(c[2 * kt][0], c[2 * kt][1]);
        a[kt][1] = pack_silu(c[2 * kt][2], c[2 * kt][3]);
        a[kt][2] = pack_silu(c[2 * kt + 1][0], c[2 * kt + 1][1]);
        a[kt][3] = pack_silu(c[2 * kt + 1][2], c[2 * kt + 1][3]);
    }
}

// APPLY false: out[r * 3 ..] = network(xb row r) for r < n.
// APPLY true: rows are sorted particles; acc[idx[r]] += out_scale * clamp(y) for
// fluid rows.
// Byte layout of the staged weights: padded BF16 rows of W1..W4, then FP32 biases.
constexpr int kImageBytes = kSWEnd * 2 + kSBEnd * 4;
constexpr int kImageWords = kImageBytes / 16;
static_assert(kSWEnd * 2 % 16 == 0 && kImageBytes % 16 == 0, "image rows must stay 16-byte aligned");

// Builds the image once per parameter change (one thread per 32-bit image word),
// so each network block stages it with plain 16-byte copies.
__global__ void k_pack(const __nv_bfloat16 *__restrict__ w, uint32_t *__restrict__ image)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < kSWEnd / 2) {  // two BF16 weights per word
        __nv_bfloat16 h[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int q = 2 * k + e;
            __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
            if (q < kSW2) {
                const int o = q / kW1Stride, i = q % kW1Stride;
                if (i < kFeat) v = w[kOffW1 + o * kFeat + i];
            } else {
                const int base = q < kSW3 ? kSW2 : (q < kSW4 ? kSW3 : kSW4);
                const int off = q < kSW3 ? kOffW2 : (q < kSW4 ? kOffW3 : kOffW4);
                const int o = (q - base) / kWStride, i = (q - base) % kWStride;
                if (i < kHidden && (base != kSW4 || o < kOut)) v = w[off + o * kHidden + i];
            }
            h[e] = v;
        }
        const __nv_bfloat162 v2 = __halves2bfloat162(h[0], h[1]);
        image[k] = *reinterpret_cast<const uint32_t *>(&v2);
    } else if (k < kImageBytes / 4) {
        const int b = k - kSWEnd / 2;
        float v = 0.0f;
        if (b < kSB2) v = __bfloat162float(w[kOffB1 + b]);
        else if (b < kSB3) v = __bfloat162float(w[kOffB2 + b - kSB2]);
        else if (b < kSB4) v = __bfloat162float(w[kOffB3 + b - kSB3]);
        else if (b - kSB4 < kOut) v = __bfloat162float(w[kOffB4 + b - kSB4]);
        image[k] = __float_as_uint(v);
    }
}

// APPLY false: out[r * 3 ..] = network(xb row r) for r < n.
// APPLY true: rows are sorted particles; acc[idx[r]] += out_scale * clamp(y) for
// fluid rows.
template <bool APPLY>
__global__ void __launch_bounds__(128)
    k_mlp(ClosureView c, const __nv_bfloat16 *__restrict__ xb, uint32_t n,
          const float4 *__restrict__ spos, const uint32_t *__restrict__ idx, float4 *acc,
          float *__restrict__ out)
{
    pdl_entry();
    __shared__ uint4 simage[kImageWords];
    for (int k = threadIdx.x; k < kImageWords; k += blockDim.x) simage[k] = __ldg(c.image + k);
    const __nv_bfloat16 *sw = reinterpret_cast<const __nv_bfloat16 *>(simage);
    const float *sb = reinterpret_cast<const float *>(simage) + kSWEnd / 2;
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    const uint32_t tiles = (n + 15) / 16;
    const float scale = APPLY ? *c.out_scale : 0.0f, lim = APPLY ? *c.out_limit : 0.0f;
    for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile < tiles; tile += warps) {
        const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
        if (APPLY) {  // sorted order keeps wall cells together: skip tiles without fluid
            const bool f = (r0 < n && spos[r0].w == (float)CMAG_FLUID) ||
                           (r1 < n && spos[r1].w == (float)CMAG_FLUID);
            if (!__any_sync(0xffffffffu, f)) continue;
        }
        uint32_t a1[1][4];
        {
            const uint32_t *x0 = reinterpret_cast<const uint32_t *>(xb + (size_t)r0 * kFeat);
            const uint32_t *x1 = reinterpret_cast<const uint32_t *>(xb + (size_t)r1 * kFeat);
            a1[0][0] = r0 < n ? x0[t] : 0u;
            a1[0][1] = r1 < n ? x1[t] : 0u;
            a1[0][2] = r0 < n ? x0[t + 4] : 0u;
            a1[0][3] = r1 < n ? x1[t + 4] : 0u;
        }
        float cc[8][4];
        uint32_t a[4][4];
        hidden_layer<1>(sw + kSW1, kW1Stride, sb + kSB1, a1, cc, g, t);
        to_a(cc, a);
        hidden_layer<4>(sw + kSW2, kWStride, sb + kSB2, a, cc, g, t);
        to_a(cc, a);
        hidden_layer<4>(sw + kSW3, kWStride, sb + kSB3, a, cc, g, t);
        to_a(cc, a);
        // output layer (3 of 8 columns used)
        float y[4] = {sb[kSB4 + 2 * t], sb[kSB4 + 2 * t + 1], sb[kSB4 + 2 * t], sb[kSB4 + 2 * t + 1]};
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const __nv_bfloat16 *row = sw + kSW4 + g * kWStride + kt * 16 + 2 * t;
            mma16816(y, a[kt], lds32(row), lds32(row + 8));
        }
        // lane (g, 0) holds columns 0, 1 of rows r0 (y[0..1]) and r1 (y[2..3]);
        // column 2 sits in lane (g, 1)
        const float y2r0 = __shfl_down_sync(0xffffffffu, y[0], 1);
        const float y2r1 = __shfl_down_sync(0xffffffffu, y[2], 1);
        if (t == 0) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t r = h ? r1 : r0;
                const float o0 = h ? y[2] : y[0], o1 = h ? y[3] : y[1], o2 = h ? y2r1 : y2r0;
                if (r < n && !APPLY) {
                    out[(size_t)r * kOut + 0] = o0;
                    out[(size_t)r * kOut + 1] = o1;
                    out[(size_t)r * kOut + 2] = o2;
                }
                if (r < n && APPLY && spos[r].w == (float)CMAG_FLUID) {
                    const uint32_t o = idx[r];
                    if (o < n) {  // o >= n only after a failed sort
                        float4 av = acc[o];
                        av.x += scale * fminf(fmaxf(o0, -lim), lim);
                        av.y += scale * fminf(fmaxf(o1, -lim), lim);
                        av.z += scale * fminf(fmaxf(o2, -lim), lim);
                        acc[o] = av;
                    }
                }
            }
        }
        __syncwarp();
    }
}

// dW[o][k] += sum_s D[s][o] A[s][k], db[o] += sum_s D[s][o] over the block's
// samples; each of the (NO/TO)*(NK/TK) <= blockDim.x threads owns a TO x TK tile.
template <int NO, int NK, int TO, int TK>
__device__ __forceinline__ void weight_grad(const float *D, int ldd, const float *A, int lda,
                                            float *gw, float *gb)
{
    constexpr int CK = NK / TK, THREADS = (NO / TO) * CK;
    const int t = threadIdx.x;
    if (t >= THREADS) return;
    const int o0 = (t / CK) * TO, k0 = (t % CK) * TK;
    float acc[TO][TK];
    float bs[TO];
#pragma unroll
    for (int a = 0; a < TO; ++a) {
        bs[a] = 0.0f;
#pragma unroll
        for (int b = 0; b < TK; ++b) acc[a][b] = 0.0f;
    }
#pragma unroll 2
    for (int s = 0; s < kTile; ++s) {
        float d[TO], x[TK];
#pragma unroll
        for (int a = 0; a < TO; ++a) d[a] = D[s * ldd + o0 + a];
#pragma unroll
        for (int b = 0; b < TK; ++b) x[b] = A[s * lda + k0 + b];
#pragma unroll
        for (int a = 0; a < TO; ++a) {
            bs[a] += d[a];
#pragma unroll
            for (int b = 0; b < TK; ++b) acc[a][b] = __fmaf_rn(d[a], x[b], acc[a][b]);
        }
    }
#pragma unroll
    for (int a = 0; a < TO; ++a) {
#pragma unroll
        for (int b = 0; b < TK; ++b) atomicAdd(gw + (o0 + a) * NK + k0 + b, acc[a][b]);
        if (k0 == 0) atomicAdd(gb + o0 + a, bs[a]);
    }
}

// delta_in[k] = dact(z[k]) * sum_o W[o][k] delta_out[o] for the thread's sample,
// written over z (its own row)
template <int NO>
__device__ __forceinline__ void back_row(const float *sw, int offw, const float *dout, float *zrow)
{
    float d[NO];
#pragma unroll
    for (int o = 0; o < NO; ++o) d[o] = dout[o];
#pragma unroll 1
    for (int k = 0; k < kHidden; ++k) {
        float g = 0.0f;
#pragma unroll
        for (int o = 0; o < NO; ++o) g = __fmaf_rn(sw[offw + o * kHidden + k], d[o], g);
        zrow[k] = g * dact(zrow[k]);
    }
}

// Forward and backward over one tile of 128 samples per block; gradients and the
// loss are added to global FP32 accumulators.
__global__ void __launch_bounds__(kTile)
    k_backward(ClosureView c, const float *__restrict__ feat, const float *__restrict__ target,
               uint32_t n, float *__restrict__ grad, float *__restrict__ loss)
{
    extern __shared__ float4 smem4[];
    float *sw = reinterpret_cast<float *>(smem4);
    float *X = sw + kWPad;                 // [128][kXRow] normalised inputs
    float *Z1 = X + kTile * kXRow;         // [128][kRow] pre-activations, then deltas
    float *Z2 = Z1 + kTile * kRow;
    float *Z3 = Z2 + kTile * kRow;
    float *A = Z3 + kTile * kRow;          // [128][kRow] activations of one layer
    float *DY = A + kTile * kRow;          // [128][4] output deltas
    __shared__ float s_loss[kTile / 32];
    load_weights(sw, c.w);
    __syncthreads();

    const int t = threadIdx.x;
    const uint32_t s = blockIdx.x * kTile + t;
    const bool valid = s < n;
    float *zr1 = Z1 + t * kRow, *zr2 = Z2 + t * kRow, *zr3 = Z3 + t * kRow, *ar = A + t * kRow;
    // forward, keeping pre-activations
    float x[kFeat];
    {
        float f[kFeat];
        if (valid) load_row(feat + (size_t)s * kFeat, f);
        else
#pragma unroll
            for (int k = 0; k < kFeat; ++k) f[k] = 0.0f;
        normalise(c.mean, c.inv_std, f, x);
#pragma unroll
        for (int k = 0; k < kFeat; ++k) X[t * kXRow + k] = x[k];
    }
    dense_row<kFeat, kHidden, true>(sw, kOffW1, kOffB1, x, zr1);
    float h[kHidden];
    load_row(zr1, h);
#pragma unroll
    for (int k = 0; k < kHidden; ++k) h[k] = act(h[k]);
    dense_row<kHidden, kHidden, true>(sw, kOffW2, kOffB2, h, zr2);
    load_row(zr2, h);
#pragma unroll
    for (int k = 0; k < kHidden; ++k) h[k] = act(h[k]);
    dense_row<kHidden, kHidden, true>(sw, kOffW3, kOffB3, h, zr3);
    load_row(zr3, h);
#pragma unroll
    for (int k = 0; k < kHidden; ++k) {
        h[k] = act(h[k]);
        ar[k] = h[k];  // A = act(Z3)
    }
    float l = 0.0f;
    const float inv_n = 1.0f / (float)n;
#pragma unroll
    for (int o = 0; o < kOut; ++o) {
        float y = sw[kOffB4 + o];
#pragma unroll
        for (int k = 0; k < kHidden; ++k) y = __fmaf_rn(sw[kOffW4 + o * kHidden + k], h[k], y);
        const float e = valid ? y - target[(size_t)s * kOut + o] : 0.0f;
        l = __fmaf_rn(e, e, l);
        DY[t * 4 + o] = e * inv_n;
    }
    DY[t * 4 + 3] = 0.0f;
    for (int w = 16; w > 0; w >>= 1) l += __shfl_xor_sync(0xffffffffu, l, w);
    if ((t & 31) == 0) s_loss[t >> 5] = l;
    __syncthreads();
    if (t == 0) {
        float b = 0.0f;
        for (int w = 0; w < kTile / 32; ++w) b += s_loss[w];
        atomicAdd(loss, 0.5f * b * inv_n);
    }
    // layer 4
    weight_grad<kOut, kHidden, 3, 1>(DY, 4, A, kRow, grad + kOffW4, grad + kOffB4);
    back_row<kOut>(sw, kOffW4, DY + t * 4, zr3);  // delta3 over Z3
    __syncthreads();
    // layer 3
#pragma unroll 4
    for (int k = 0; k < kHidden; ++k) ar[k] = act(zr2[k]);
    __syncthreads();
    weight_grad<kHidden, kHidden, 4, 8>(Z3, kRow, A, kRow, grad + kOffW3, grad + kOffB3);
    back_row<kHidden>(sw, kOffW3, zr3, zr2);       // delta2 over Z2
    __syncthreads();
    // layer 2
#pragma unroll 4
    for (int k = 0; k < kHidden; ++k) ar[k] = act(zr1[k]);
    __syncthreads();
    weight_grad<kHidden, kHidden, 4, 8>(Z2, kRow, A, kRow, grad + kOffW2, grad + kOffB2);
    back_row<kHidden>(sw, kOffW2, zr2, zr1);       // delta1 over Z1
    __syncthreads();
    // layer 1
    weight_grad<kHidden, kFeat, 4, 2>(Z1, kRow, X, kXRow, grad + kOffW1, grad + kOffB1);
}

__global__ void k_adam(float *master, float *m, float *v, float *grad, __nv_bfloat16 *w, float lr,
                       float beta1, float beta2, float eps, float bias1, float bias2)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kClosureParams) return;
    const float g = grad[k];
    const float mk = beta1 * m[k] + (1.0f - beta1) * g;
    const float vk = beta2 * v[k] + (1.0f - beta2) * g * g;
    m[k] = mk;
    v[k] = vk;
    const float step = lr * (mk / bias1) / (sqrtf(vk / bias2) + eps);
    const float nw = master[k] - step;
    master[k] = nw;
    w[k] = __float2bfloat16_rn(nw);
    grad[k] = 0.0f;
}

__global__ void k_round(const float *master, __nv_bfloat16 *w)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < kClosureParams) w[k] = __float2bfloat16_rn(master[k]);
}

// Shepard-normalised SPH interpolation of a float4 array (original order) of
// the system's fluid particles at arbitrary points: out.xyz = sum_j V_j W a_j /
// sum_j V_j W, out.w = sum_j V_j W (0 where no fluid particle is in reach).
template <bool PLANAR, bool TRIM>
__global__ void __launch_bounds__(128)
    k_interp(DevParams p, const float4 *__restrict__ spos, const float2 *__restrict__ aux,
             const uint32_t *__restrict__ idx, const uint32_t *__restrict__ off,
             const float4 *__restrict__ arr, const float4 *__restrict__ pts, uint32_t n,
             float4 *__restrict__ out)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float4 q = pts[t];
    float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
    const int3 g = grid_pos(p, q.x, q.y, q.z);
    walk::for_each_candidate<CMAG_DAMBREAK, PLANAR, TRIM, 1>(
        p, off, 0, g, walk::frac_cell(p, q), [&](uint32_t j, float, float, float) {
            const float4 pj = __ldg(spos + j);
            if (pj.w != (float)CMAG_FLUID) return;
            const float rx = pj.x - q.x, ry = pj.y - q.y, rz = pj.z - q.z;
            const float d2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, rx * rx));
            if (!(d2 < p.support2)) return;
            const uint32_t o = __ldg(idx + j);
            if (o >= p.n) return;  // only after a failed sort
            const float qq = d2 > 0.0f ? d2 * rsqrtf(d2) * p.inv_h : 0.0f;
            const float vw = p.mass / __ldg(aux + j).y * kernel_w(p, qq);
            const float4 a = __ldg(arr + o);
            sx = __fmaf_rn(vw, a.x, sx); sy = __fmaf_rn(vw, a.y, sy); sz = __fmaf_rn(vw, a.z, sz);
            sw += vw;
        });
    const float inv = sw > 0.0f ? 1.0f / sw : 0.0f;
    out[t] = make_float4(sx * inv, sy * inv, sz * inv, sw);
}

constexpr size_t kSmemBackward =
    sizeof(float) * (kWPad + kTile * kXRow + 4 * kTile * kRow + kTile * 4);

template <class K>
void allow_smem(K kernel, size_t bytes)
{
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <bool NORM>
void dispatch_features(const DevParams &p, const ClosureView &c, const float4 *spos,
                       const float4 *svel, const float2 *aux, const float4 *meas,
                       const uint32_t *idx, const uint32_t *off, const float4 *acc, float *feat,
                       __nv_bfloat16 *xb, cudaStream_t st)
{
    if (p.n == 0) return;
    const uint32_t blocks = (p.n + 255) / 256;
#define CMAG_FEAT(PL, TR) \
    launch_pdl(k_closure_features<PL, TR, NORM>, blocks, 256, 0, st, p, c, spos, svel, aux, meas, idx, off, acc, feat, xb)
    if (p.planar) {
        if (p.trim) CMAG_FEAT(true, true);
        else CMAG_FEAT(true, false);
    } else {
        if (p.trim) CMAG_FEAT(false, true);
        else CMAG_FEAT(false, false);
    }
#undef CMAG_FEAT
}

// Each block stages the weight image once (23 KB) and its 4 warps loop over
// 16-row tiles, so the grid stays at a few blocks per SM (8 per SM at most)
// however many rows there are.
uint32_t mlp_blocks(uint32_t n)
{
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t cap = 8u * (uint32_t)device_sm_count();
    uint32_t b = (tiles + 3) / 4;
    return b < 1 ? 1 : (b > cap ? cap : b);
}

}  // namespace

void launch_closure_features(const DevParams &p, const float4 *spos, const float4 *svel,
                             const float2 *aux, const float4 *meas, const uint32_t *idx,
                             const uint32_t *off, const float4 *acc, float *feat, cudaStream_t st)
{
    dispatch_features<false>(p, ClosureView{}, spos, svel, aux, meas, idx, off, acc, feat, nullptr, st);
}

void launch_closure_apply(const DevParams &p, const ClosureView &c, const float4 *spos,
                          const float4 *svel, const float2 *aux, const float4 *meas,
                          const uint32_t *idx, const uint32_t *off, float4 *acc,
                          __nv_bfloat16 *xb, cudaStream_t st)
{
    if (p.n == 0) return;
    dispatch_features<true>(p, c, spos, svel, aux, meas, idx, off, acc, nullptr, xb, st);
    launch_pdl(k_mlp<true>, mlp_blocks(p.n), 128, 0, st, c, xb, p.n, spos, idx, acc, (float *)nullptr);
}

void launch_closure_forward(const ClosureView &c, const float *feat, uint32_t n,
                            __nv_bfloat16 *xb, float *out, cudaStream_t st)
{
    if (n == 0) return;
    k_normalise<<<(n + 255) / 256, 256, 0, st>>>(c, feat, n, xb);
    k_mlp<false><<<mlp_blocks(n), 128, 0, st>>>(c, xb, n, nullptr, nullptr, nullptr, out);
}

void launch_interpolate(const DevParams &p, const float4 *spos, const float2 *aux,
                        const uint32_t *idx, const uint32_t *off, const float4 *arr,
                        const float4 *pts, uint32_t n, float4 *out, cudaStream_t st)
{
    if (n == 0) return;
    const uint32_t blocks = (n + 127) / 128;
    if (p.planar) {
        if (p.trim) k_interp<true, true><<<blocks, 128, 0, st>>>(p, spos, aux, idx, off, arr, pts, n, out);
        else k_interp<true, false><<<blocks, 128, 0, st>>>(p, spos, aux, idx, off, arr, pts, n, out);
    } else {
        if (p.trim) k_interp<false, true><<<blocks, 128, 0, st>>>(p, spos, aux, idx, off, arr, pts, n, out);
        else k_interp<false, false><<<blocks, 128, 0, st>>>(p, spos, aux, idx, off, arr, pts, n, out);
    }
}

void launch_closure_backward(const ClosureView &c, const float *feat, const float *target,
                             uint32_t n, float *grad, float *loss, cudaStream_t st)
{
    if (n == 0) return;
    allow_smem(k_backward, kSmemBackward);
    k_backward<<<(n + kTile - 1) / kTile, kTile, kSmemBackward, st>>>(c, feat, target, n, grad, loss);
}

uint32_t closure_image_words() { return (uint32_t)kImageWords; }

void launch_closure_adam(float *master, float *m, float *v, float *grad, __nv_bfloat16 *w,
                         uint4 *image, float lr, float beta1, float beta2, float eps, float bias1,
                         float bias2, cudaStream_t st)
{
    k_adam<<<(kClosureParams + 255) / 256, 256, 0, st>>>(master, m, v, grad, w, lr, beta1, beta2,
                                                        eps, bias1, bias2);
    k_pack<<<(kImageBytes / 4 + 255) / 256, 256, 0, st>>>(w, reinterpret_cast<uint32_t *>(image));
}

void launch_closure_round(const float *master, __nv_bfloat16 *w, uint4 *image, cudaStream_t st)
{
    k_round<<<(kClosureParams + 255) / 256, 256, 0, st>>>(master, w);
    k_pack<<<(kImageBytes / 4 + 255) / 256, 256, 0, st>>>(w, reinterpret_cast<uint32_t *>(image));
}

}  // namespace cmag
