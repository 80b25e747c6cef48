// closure_api.cu -- C ABI of the learned closure (cmag_closure_*): parameters,
// normalisation, inference and training on device-resident feature arrays.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "closure.h"
#include "host_common.h"

using namespace cmag;

namespace {

int cfail(cmag_closure *c, int code, const std::string &msg)
{
    if (c) c->last_error = msg;
    set_last_error(msg);
    return code;
}

#define CC_CUDA(c, call)                                                                    \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            (void)cudaGetLastError();                                                       \
            return cfail((c), e_ == cudaErrorMemoryAllocation ? CMAG_ERR_NOMEM : CMAG_ERR_CUDA, \
                         std::string(#call) + ": " + cudaGetErrorString(e_));               \
        }                                                                                   \
    } while (0)

cudaStream_t stream_of(cmag_closure *c, void *stream)
{
    return stream ? (cudaStream_t)stream : c->stream;
}

void free_all(cmag_closure *c)
{
    void *ptrs[] = {c->master, c->m, c->v, c->grad, c->w, c->image, c->norm, c->xb};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (c->stream) cudaStreamDestroy(c->stream);
}

constexpr size_t kNormFloats = 2 * kFeat + 3;  // mean, inv_std, out_scale, loss, out_limit

}  // namespace

extern "C" {

size_t cmag_closure_param_count(void) { return (size_t)kClosureParams; }

int cmag_closure_create(const float *params, cmag_closure **out)
{
    if (!out) return cfail(nullptr, CMAG_ERR_INVALID, "null argument");
    *out = nullptr;
    cmag_closure *c = new (std::nothrow) cmag_closure();
    if (!c) return cfail(nullptr, CMAG_ERR_NOMEM, "host allocation failed");
    const size_t pb = sizeof(float) * kClosureParams;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->master, pb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->m, pb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->v, pb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->grad, pb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->w, sizeof(__nv_bfloat16) * kClosureParams);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->norm, sizeof(float) * kNormFloats);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->image, sizeof(uint4) * closure_image_words());
    if (e == cudaSuccess) e = cudaMemset(c->m, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(c->v, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(c->grad, 0, pb);
    if (e == cudaSuccess) {
        std::vector<float> init(kClosureParams, 0.0f), norm(kNormFloats, 0.0f);
        if (params) std::memcpy(init.data(), params, pb);
        for (int k = 0; k < kFeat; ++k) norm[kFeat + k] = 1.0f;  // identity normalisation
        norm[2 * kFeat] = 1.0f;
        norm[2 * kFeat + 2] = 3.0e38f;  // no output limit
        e = cudaMemcpy(c->master, init.data(), pb, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(c->norm, norm.data(), sizeof(float) * kNormFloats, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            launch_closure_round(c->master, c->w, c->image, c->stream);
            e = cudaStreamSynchronize(c->stream);
        }
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        const int code = e == cudaErrorMemoryAllocation ? CMAG_ERR_NOMEM : CMAG_ERR_CUDA;
        std::string msg = std::string("closure create: ") + cudaGetErrorString(e);
        free_all(c);
        delete c;
        return cfail(nullptr, code, msg);
    }
    *out = c;
    return CMAG_OK;
}

int cmag_closure_destroy(cmag_closure *c)
{
    if (!c) return CMAG_OK;
    cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
    return CMAG_OK;
}

int cmag_closure_set_params(cmag_closure *c, const float *params)
{
    if (!c || !params) return cfail(c, CMAG_ERR_INVALID, "null argument");
    CC_CUDA(c, cudaMemcpyAsync(c->master, params, sizeof(float) * kClosureParams,
                               cudaMemcpyHostToDevice, c->stream));
    launch_closure_round(c->master, c->w, c->image, c->stream);
    CC_CUDA(c, cudaGetLastError());
    CC_CUDA(c, cudaStreamSynchronize(c->stream));
    return CMAG_OK;
}

int cmag_closure_get_params(cmag_closure *c, float *params)
{
    if (!c || !params) return cfail(c, CMAG_ERR_INVALID, "null argument");
    CC_CUDA(c, cudaMemcpyAsync(params, c->master, sizeof(float) * kClosureParams,
                               cudaMemcpyDeviceToHost, c->stream));
    CC_CUDA(c, cudaStreamSynchronize(c->stream));
    return CMAG_OK;
}

int cmag_closure_get_bf16_params(cmag_closure *c, float *params)
{
    if (!c || !params) return cfail(c, CMAG_ERR_INVALID, "null argument");
    std::vector<__nv_bfloat16> w(kClosureParams);
    CC_CUDA(c, cudaMemcpyAsync(w.data(), c->w, sizeof(__nv_bfloat16) * kClosureParams,
                               cudaMemcpyDeviceToHost, c->stream));
    CC_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int k = 0; k < kClosureParams; ++k) {
        uint16_t bits;
        std::memcpy(&bits, &w[k], sizeof(bits));
        const uint32_t u = (uint32_t)bits << 16;
        std::memcpy(params + k, &u, sizeof(float));
    }
    return CMAG_OK;
}

int cmag_closure_set_normalization(cmag_closure *c, const float mean[16], const float inv_std[16],
                                   float out_scale)
{
    if (!c || !mean || !inv_std) return cfail(c, CMAG_ERR_INVALID, "null argument");
    float h[2 * kFeat + 1];
    std::memcpy(h, mean, sizeof(float) * kFeat);
    std::memcpy(h + kFeat, inv_std, sizeof(float) * kFeat);
    h[2 * kFeat] = out_scale;
    CC_CUDA(c, cudaMemcpyAsync(c->norm, h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    CC_CUDA(c, cudaStreamSynchronize(c->stream));
    return CMAG_OK;
}

int cmag_closure_get_normalization(cmag_closure *c, float mean[16], float inv_std[16],
                                   float *out_scale)
{
    if (!c) return cfail(nullptr, CMAG_ERR_INVALID, "null handle");
    float h[2 * kFeat + 1];
    CC_CUDA(c, cudaMemcpyAsync(h, c->norm, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CC_CUDA(c, cudaStreamSynchronize(c->stream));
    if (mean) std::memcpy(mean, h, sizeof(float) * kFeat);
    if (inv_std) std::memcpy(inv_std, h + kFeat, sizeof(float) * kFeat);
    if (out_scale) *out_scale = h[2 * kFeat];
    return CMAG_OK;
}

int cmag_closure_set_output_limit(cmag_closure *c, float limit)
{
    if (!c) return cfail(nullptr, CMAG_ERR_INVALID, "null handle");
    if (!(limit > 0.0f)) return cfail(c, CMAG_ERR_INVALID, "the output limit must be positive");
    CC_CUDA(c, cudaMemcpyAsync(c->norm + 2 * kFeat + 2, &limit, sizeof(float), cudaMemcpyHostToDevice,
                               c->stream));
    CC_CUDA(c, cudaStreamSynchronize(c->stream));
    return CMAG_OK;
}

int cmag_closure_forward(cmag_closure *c, const float *d_features, uint32_t n, float *d_out,
                         void *stream)
{
    if (!c || (n && (!d_features || !d_out))) return cfail(c, CMAG_ERR_INVALID, "null argument");
    cudaStream_t st = stream_of(c, stream);
    if (c->xb_rows < n) {
        CC_CUDA(c, cudaStreamSynchronize(st));
        if (c->xb) cudaFree(c->xb);
        c->xb = nullptr;
        c->xb_rows = 0;
        CC_CUDA(c, cudaMalloc((void **)&c->xb, sizeof(__nv_bfloat16) * kFeat * (size_t)n));
        c->xb_rows = n;
    }
    launch_closure_forward(c->view(), d_features, n, c->xb, d_out, st);
    CC_CUDA(c, cudaGetLastError());
    CC_CUDA(c, cudaStreamSynchronize(st));
    return CMAG_OK;
}

int cmag_closure_gradient(cmag_closure *c, const float *d_features, const float *d_targets,
                          uint32_t n, float *grad_out, float *loss_out, void *stream)
{
    if (!c || !grad_out || (n && (!d_features || !d_targets)))
        return cfail(c, CMAG_ERR_INVALID, "null argument");
    cudaStream_t st = stream_of(c, stream);
    CC_CUDA(c, cudaMemsetAsync(c->grad, 0, sizeof(float) * kClosureParams, st));
    CC_CUDA(c, cudaMemsetAsync(c->loss(), 0, sizeof(float), st));
    launch_closure_backward(c->view(), d_features, d_targets, n, c->grad, c->loss(), st);
    CC_CUDA(c, cudaGetLastError());
    CC_CUDA(c, cudaMemcpyAsync(grad_out, c->grad, sizeof(float) * kClosureParams,
                               cudaMemcpyDeviceToHost, st));
    float l = 0.0f;
    CC_CUDA(c, cudaMemcpyAsync(&l, c->loss(), sizeof(float), cudaMemcpyDeviceToHost, st));
    CC_CUDA(c, cudaMemsetAsync(c->grad, 0, sizeof(float) * kClosureParams, st));
    CC_CUDA(c, cudaStreamSynchronize(st));
    if (loss_out) *loss_out = l;
    return CMAG_OK;
}

int cmag_closure_train_step(cmag_closure *c, const float *d_features, const float *d_targets,
                            uint32_t n, float lr, float *loss_out, void *stream)
{
    if (!c || (n && (!d_features || !d_targets))) return cfail(c, CMAG_ERR_INVALID, "null argument");
    if (!(lr > 0.0f)) return cfail(c, CMAG_ERR_INVALID, "learning rate must be positive");
    cudaStream_t st = stream_of(c, stream);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    c->adam_steps++;
    const float bias1 = (float)(1.0 - std::pow((double)b1, (double)c->adam_steps));
    const float bias2 = (float)(1.0 - std::pow((double)b2, (double)c->adam_steps));
    if (loss_out) CC_CUDA(c, cudaMemsetAsync(c->loss(), 0, sizeof(float), st));
    launch_closure_backward(c->view(), d_features, d_targets, n, c->grad, c->loss(), st);
    launch_closure_adam(c->master, c->m, c->v, c->grad, c->w, c->image, lr, b1, b2, eps, bias1, bias2, st);
    CC_CUDA(c, cudaGetLastError());
    if (loss_out) {
        CC_CUDA(c, cudaMemcpyAsync(loss_out, c->loss(), sizeof(float), cudaMemcpyDeviceToHost, st));
        CC_CUDA(c, cudaStreamSynchronize(st));
    }
    return CMAG_OK;
}

int cmag_closure_reset_optimizer(cmag_closure *c)
{
    if (!c) return cfail(nullptr, CMAG_ERR_INVALID, "null handle");
    c->adam_steps = 0;
    CC_CUDA(c, cudaMemsetAsync(c->m, 0, sizeof(float) * kClosureParams, c->stream));
    CC_CUDA(c, cudaMemsetAsync(c->v, 0, sizeof(float) * kClosureParams, c->stream));
    CC_CUDA(c, cudaMemsetAsync(c->grad, 0, sizeof(float) * kClosureParams, c->stream));
    CC_CUDA(c, cudaStreamSynchronize(c->stream));
    return CMAG_OK;
}

int cmag_closure_synchronize(cmag_closure *c)
{
    if (!c) return cfail(nullptr, CMAG_ERR_INVALID, "null handle");
    CC_CUDA(c, cudaStreamSynchronize(c->stream));
    return CMAG_OK;
}

const char *cmag_closure_last_error(const cmag_closure *c)
{
    return c ? c->last_error.c_str() : last_error().c_str();
}

}  // extern "C"
