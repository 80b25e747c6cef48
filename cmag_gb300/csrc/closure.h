// closure.h -- the learned closure: a 16-64-64-64-3 SiLU network that corrects
// the pressure + viscous (+ wall) acceleration of a coarse DamBreak run.
//
// No reference counterpart.  Parameters are BF16 (the training master copy is
// FP32); activations are rounded to BF16 between layers; every dot product
// accumulates in FP32.  Parameter vector order (kClosureParams floats):
//   W1[64][16] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[3][64] b4[3]
// (W[o][k]: output o, input k).
#pragma once

#include <cstdint>
#include <string>

#include <cuda_bf16.h>

#include "kernels.h"

namespace cmag {

constexpr int kFeat = 16, kHidden = 64, kOut = 3;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kHidden * kFeat, kOffW2 = kOffB1 + kHidden,
              kOffB2 = kOffW2 + kHidden * kHidden, kOffW3 = kOffB2 + kHidden,
              kOffB3 = kOffW3 + kHidden * kHidden, kOffW4 = kOffB3 + kHidden,
              kOffB4 = kOffW4 + kOut * kHidden, kClosureParams = kOffB4 + kOut;

// What the device kernels read (all in device memory, so a captured graph sees
// every later update).
struct ClosureView {
    const __nv_bfloat16 *w;   // kClosureParams BF16 parameters
    const float *mean;        // kFeat feature offsets
    const float *inv_std;     // kFeat feature scales
    const float *out_scale;   // correction = *out_scale * clamp(network output, +-*out_limit)
    const float *out_limit;
    const uint4 *image;       // closure_image_words() words: the weights as the network
                              // kernel stages them in shared memory (padded BF16 rows,
                              // then FP32 biases), rebuilt whenever w changes
};

// Size of ClosureView::image in 16-byte words.
uint32_t closure_image_words();

// Per sorted fluid particle of a DamBreak scene: the 16 raw features, written
// to feat[idx[i] * 16 ..] (original order).  Rows of wall particles are left
// untouched.
void launch_closure_features(const DevParams &p, const float4 *spos, const float4 *svel,
                             const float2 *aux, const float4 *meas, const uint32_t *idx,
                             const uint32_t *off, const float4 *acc, float *feat,
                             cudaStream_t st);
// Features (normalised BF16 rows in xb, n x 16, sorted order), network on the
// tensor cores and acc[idx[i]] += correction for every fluid particle.
void launch_closure_apply(const DevParams &p, const ClosureView &c, const float4 *spos,
                          const float4 *svel, const float2 *aux, const float4 *meas,
                          const uint32_t *idx, const uint32_t *off, float4 *acc,
                          __nv_bfloat16 *xb, cudaStream_t st);
// Shepard-normalised SPH interpolation of arr (original order) over the fluid
// particles of a DamBreak scene at n points: out = (value, sum of V_j W).
void launch_interpolate(const DevParams &p, const float4 *spos, const float2 *aux,
                        const uint32_t *idx, const uint32_t *off, const float4 *arr,
                        const float4 *pts, uint32_t n, float4 *out, cudaStream_t st);
// Network outputs (unscaled) for n raw feature rows (xb: n x 16 BF16 scratch).
void launch_closure_forward(const ClosureView &c, const float *feat, uint32_t n,
                            __nv_bfloat16 *xb, float *out, cudaStream_t st);
// Loss 0.5/n sum |y - t|^2 over n rows (t: targets, n x 3) added to *loss and its
// gradient with respect to the BF16 parameters added to grad (FP32).
void launch_closure_backward(const ClosureView &c, const float *feat, const float *target,
                             uint32_t n, float *grad, float *loss, cudaStream_t st);
// Adam on the FP32 master copy; refreshes the BF16 copy and its shared-memory
// image and clears grad.
void launch_closure_adam(float *master, float *m, float *v, float *grad, __nv_bfloat16 *w,
                         uint4 *image, float lr, float beta1, float beta2, float eps,
                         float bias1, float bias2, cudaStream_t st);
// BF16 copy of the master parameters and its shared-memory image.
void launch_closure_round(const float *master, __nv_bfloat16 *w, uint4 *image, cudaStream_t st);

}  // namespace cmag

// A trainable network instance (C ABI handle).
struct cmag_closure {
    float *master = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;  // FP32, kClosureParams
    __nv_bfloat16 *w = nullptr;                                            // BF16 copy used by kernels
    uint4 *image = nullptr;                                                // w as the network kernel stages it
    float *norm = nullptr;   // mean[16], inv_std[16], out_scale, loss, out_limit
    uint32_t adam_steps = 0;
    __nv_bfloat16 *xb = nullptr;   // forward() scratch: normalised input rows
    size_t xb_rows = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    cmag::ClosureView view() const
    {
        return cmag::ClosureView{w, norm, norm + cmag::kFeat, norm + 2 * cmag::kFeat,
                                 norm + 2 * cmag::kFeat + 2, image};
    }
    float *loss() const { return norm + 2 * cmag::kFeat + 1; }
};
