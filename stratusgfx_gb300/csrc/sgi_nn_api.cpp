// sgi_nn_api.cpp - host side of the learned denoiser (include/sgi_nn.h).
//
// U-Net (NHWC, BF16 activations):
//   e1a 16->32, e1b 32->32      full resolution; e1b writes channels 64..95 of D1IN
//   pool                        -> 1/2
//   e2a 32->64, e2b 64->64      e2b writes channels 128..191 of D2IN
//   pool                        -> 1/4
//   b1 64->128, b2 128->128
//   up (nearest) -> D2IN 0..127; d2a 192->64, d2b 64->64
//   up -> D1IN 0..63;            d1a 96->32, d1b 32->32
//   head 32->32 (no ReLU): 25 kernel logits + 1 temporal blend logit (+6 unused)
// then the kernel apply / loss of sgi_nn.cu. Every conv is 3x3 with ReLU except
// the head. Backward runs the same schedule in reverse: ReLU masks, weight
// gradients (FP32), bias gradients, and input gradients through the forward
// kernel with flipped weights.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "../../include/sgi_nn.h"
#include "sgi_nn_internal.h"
#include "sgi_nn_net.h"

namespace sgi {
namespace nn {

using bf16 = __nv_bfloat16;

enum { E1A, E1B, E2A, E2B, B1, B2, D2A, D2B, D1A, D1B, HEAD, NUM_LAYERS };
static const int kCin[NUM_LAYERS] = {16, 32, 32, 64, 64, 128, 192, 64, 96, 32, 32};
static const int kCout[NUM_LAYERS] = {32, 32, 64, 64, 128, 128, 64, 64, 32, 32, 32};

Net::~Net() { release(); }

void Net::release() {
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
}

template <class T> cudaError_t Net::alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess) allocs.push_back(*p);
    return e;
}

cudaError_t Net::init(const sgi_nn_config& c) {
    cfg = c;
    size_t off = 0;
    for (int l = 0; l < NUM_LAYERS; ++l) {
        w_off[l] = off;
        off += (size_t)kCout[l] * 9 * kCin[l];
        b_off[l] = off;
        off += (size_t)kCout[l];
    }
    nparams = off;
    const size_t P = (size_t)c.max_batch * c.max_height * c.max_width;
    const size_t P2 = P / 4, P4 = P / 16;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
    chk(alloc(&w32, nparams));
    chk(alloc(&g32, nparams));
    chk(alloc(&m32, nparams));
    chk(alloc(&v32, nparams));
    chk(alloc(&wbf, nparams));
    chk(alloc(&wflip, nparams));
    chk(alloc(&loss_dev, 1));
    chk(alloc(&E1A_, P * 32));
    chk(alloc(&D1IN, P * 96));
    chk(alloc(&P1, P2 * 32));
    chk(alloc(&E2A_, P2 * 64));
    chk(alloc(&D2IN, P2 * 192));
    chk(alloc(&P2_, P4 * 64));
    chk(alloc(&B1_, P4 * 128));
    chk(alloc(&B2_, P4 * 128));
    chk(alloc(&D2A_, P2 * 64));
    chk(alloc(&D2B_, P2 * 64));
    chk(alloc(&D1A_, P * 32));
    chk(alloc(&D1B_, P * 32));
    chk(alloc(&LOG, P * 32));
    chk(alloc(&GA, P * 32));
    chk(alloc(&GB, P * 32));
    chk(alloc(&GC, P * 32));
    chk(alloc(&GD, P * 96));
    chk(alloc(&GH1, P2 * 64));
    chk(alloc(&GH2, P2 * 64));
    chk(alloc(&GH3, P2 * 192));
    chk(alloc(&GQ1, P4 * 128));
    chk(alloc(&GQ2, P4 * 128));
    chk(alloc(&GQ3, P4 * 64));
    chk(alloc(&fwd_out, P));
    if (e != cudaSuccess) return e;
    // He-normal weights, zero biases; the head starts near a box filter + half blend.
    std::vector<float> h(nparams, 0.0f);
    std::mt19937 rng(c.seed);
    for (int l = 0; l < NUM_LAYERS; ++l) {
        const float sd = std::sqrt(2.0f / (9.0f * kCin[l])) * (l == HEAD ? 0.1f : 1.0f);
        std::normal_distribution<float> nd(0.0f, sd);
        for (size_t i = 0; i < (size_t)kCout[l] * 9 * kCin[l]; ++i) h[w_off[l] + i] = nd(rng);
    }
    e = set_params(h.data(), nparams);
    if (e != cudaSuccess) return e;
    e = cudaMemset(m32, 0, nparams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(v32, 0, nparams * sizeof(float));
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e;
}

cudaError_t Net::set_params(const float* host, size_t n) {
    cudaError_t e = cudaMemcpy(w32, host, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    e = to_bf16(w32, wbf, nparams, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e;
}

cudaError_t Net::conv(int l, const bf16* x, int xs, bf16* y, int ys, int B, int H, int W, cudaStream_t s) {
    ConvArgs a{x, xs, wbf + w_off[l], w32 + b_off[l], y, ys, B, H, W};
    return conv3x3(kCin[l], kCout[l], l == HEAD ? 1 : 0, a, s);
}

cudaError_t Net::forward(const bf16* feat, int B, int H, int W, cudaStream_t s) {
    const int H2 = H / 2, W2 = W / 2, H4 = H / 4, W4 = W / 4;
    cudaError_t e;
#define NN_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
    NN_TRY(conv(E1A, feat, 16, E1A_, 32, B, H, W, s));
    NN_TRY(conv(E1B, E1A_, 32, D1IN + 64, 96, B, H, W, s));
    NN_TRY(pool_fwd(D1IN + 64, 96, P1, 32, B, H, W, 32, s));
    NN_TRY(conv(E2A, P1, 32, E2A_, 64, B, H2, W2, s));
    NN_TRY(conv(E2B, E2A_, 64, D2IN + 128, 192, B, H2, W2, s));
    NN_TRY(pool_fwd(D2IN + 128, 192, P2_, 64, B, H2, W2, 64, s));
    NN_TRY(conv(B1, P2_, 64, B1_, 128, B, H4, W4, s));
    NN_TRY(conv(B2, B1_, 128, B2_, 128, B, H4, W4, s));
    NN_TRY(up_fwd(B2_, 128, D2IN, 192, B, H2, W2, 128, s));
    NN_TRY(conv(D2A, D2IN, 192, D2A_, 64, B, H2, W2, s));
    NN_TRY(conv(D2B, D2A_, 64, D2B_, 64, B, H2, W2, s));
    NN_TRY(up_fwd(D2B_, 64, D1IN, 96, B, H, W, 64, s));
    NN_TRY(conv(D1A, D1IN, 96, D1A_, 32, B, H, W, s));
    NN_TRY(conv(D1B, D1A_, 32, D1B_, 32, B, H, W, s));
    NN_TRY(conv(HEAD, D1B_, 32, LOG, 32, B, H, W, s));
    launches += 15;
    return cudaSuccess;
}

// Backward of layer l: dz = relu'(dy) (or dy for the head), weight / bias
// gradients from its input x, and (if dx) the input gradient.
cudaError_t Net::layer_backward(int l, const bf16* x, int xs, const bf16* y, int ys, const bf16* dy, int dys, bf16* dz,
                                bf16* dx, int dxs, int B, int H, int W, cudaStream_t s) {
    cudaError_t e;
    const size_t pix = (size_t)B * H * W;
    const bf16* g = dy;
    int gs = dys;
    if (l != HEAD) {
        NN_TRY(relu_bwd(dy, dys, y, ys, dz, kCout[l], pix, s));
        g = dz;
        gs = kCout[l];
        launches += 1;
    }
    WgradArgs wa{x, xs, g, gs, g32 + w_off[l], kCin[l], kCout[l], B, H, W};
    NN_TRY(wgrad(wa, s));
    NN_TRY(bias_grad(g, gs, kCout[l], pix, g32 + b_off[l], s));
    launches += 2;
    if (dx) {
        NN_TRY(flip_weights(wbf + w_off[l], wflip + w_off[l], kCin[l], kCout[l], s));
        ConvArgs a{g, gs, wflip + w_off[l], nullptr, dx, dxs, B, H, W};
        NN_TRY(conv3x3(kCout[l], kCin[l], 2, a, s));
        launches += 2;
    }
    return cudaSuccess;
}

cudaError_t Net::backward(const bf16* feat, int B, int H, int W, cudaStream_t s) {
    const int H2 = H / 2, W2 = W / 2, H4 = H / 4, W4 = W / 4;
    cudaError_t e;
    NN_TRY(cudaMemsetAsync(g32, 0, nparams * sizeof(float), s));
    // full resolution decoder: dLOGITS in GA
    NN_TRY(layer_backward(HEAD, D1B_, 32, LOG, 32, GA, 32, nullptr, GB, 32, B, H, W, s));      // dD1B -> GB
    NN_TRY(layer_backward(D1B, D1A_, 32, D1B_, 32, GB, 32, GC, GA, 32, B, H, W, s));          // dD1A -> GA
    NN_TRY(layer_backward(D1A, D1IN, 96, D1A_, 32, GA, 32, GB, GD, 96, B, H, W, s));          // dD1IN -> GD
    NN_TRY(up_bwd(GD, 96, GH1, 64, B, H2, W2, 64, s));                                          // dD2B -> GH1
    NN_TRY(layer_backward(D2B, D2A_, 64, D2B_, 64, GH1, 64, GH2, GH1, 64, B, H2, W2, s));        // dD2A -> GH1
    NN_TRY(layer_backward(D2A, D2IN, 192, D2A_, 64, GH1, 64, GH2, GH3, 192, B, H2, W2, s));      // dD2IN -> GH3
    NN_TRY(up_bwd(GH3, 192, GQ1, 128, B, H4, W4, 128, s));                                       // dB2 -> GQ1
    NN_TRY(layer_backward(B2, B1_, 128, B2_, 128, GQ1, 128, GQ2, GQ1, 128, B, H4, W4, s));       // dB1 -> GQ1
    NN_TRY(layer_backward(B1, P2_, 64, B1_, 128, GQ1, 128, GQ2, GQ3, 64, B, H4, W4, s));         // dP2 -> GQ3
    NN_TRY(pool_bwd(GQ3, 64, GH3 + 128, 192, B, H2, W2, 64, 1, s));                              // skip 2
    NN_TRY(layer_backward(E2B, E2A_, 64, D2IN + 128, 192, GH3 + 128, 192, GH2, GH1, 64, B, H2, W2, s));  // dE2A -> GH1
    NN_TRY(layer_backward(E2A, P1, 32, E2A_, 64, GH1, 64, GH2, GH1, 32, B, H2, W2, s));          // dP1 -> GH1 (32 ch)
    NN_TRY(pool_bwd(GH1, 32, GD + 64, 96, B, H, W, 32, 1, s));                                  // skip 1
    NN_TRY(layer_backward(E1B, E1A_, 32, D1IN + 64, 96, GD + 64, 96, GC, GA, 32, B, H, W, s));  // dE1A -> GA
    NN_TRY(layer_backward(E1A, feat, 16, E1A_, 32, GA, 32, GB, nullptr, 0, B, H, W, s));
    launches += 5;
    return cudaSuccess;
}
#undef NN_TRY

}  // namespace nn
}  // namespace sgi

using sgi::nn::Net;

static sgi_status nn_fail(sgi_nn* n, sgi_status s, const std::string& m) {
    if (n) n->err = m;
    return s;
}
static sgi_status nn_cuda(sgi_nn* n, cudaError_t e, const char* what) {
    return nn_fail(n, e == cudaErrorMemoryAllocation ? SGI_ERR_OOM : SGI_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

static bool shape_ok(const sgi_nn* n, int B, int H, int W) {
    return B >= 1 && H >= 4 && W >= 4 && H % 4 == 0 && W % 4 == 0 && B <= n->net.cfg.max_batch &&
           (size_t)B * H * W <= (size_t)n->net.cfg.max_batch * n->net.cfg.max_height * n->net.cfg.max_width;
}

extern "C" {

sgi_status sgi_nn_create(const sgi_nn_config* cfg, sgi_nn** out) {
    if (!cfg || !out) return SGI_ERR_ARG;
    *out = nullptr;
    if (cfg->max_batch < 1 || cfg->max_height < 4 || cfg->max_width < 4 || cfg->max_height % 4 || cfg->max_width % 4)
        return SGI_ERR_ARG;
    sgi_nn* n = new (std::nothrow) sgi_nn();
    if (!n) return SGI_ERR_OOM;
    cudaError_t e = n->net.init(*cfg);
    if (e != cudaSuccess) {
        delete n;
        return e == cudaErrorMemoryAllocation ? SGI_ERR_OOM : SGI_ERR_CUDA;
    }
    *out = n;
    return SGI_OK;
}

sgi_status sgi_nn_destroy(sgi_nn* n) {
    if (!n) return SGI_ERR_ARG;
    cudaDeviceSynchronize();
    delete n;
    return SGI_OK;
}

const char* sgi_nn_last_error(const sgi_nn* n) { return n ? n->err.c_str() : "null network"; }

int64_t sgi_nn_num_params(const sgi_nn* n) { return n ? (int64_t)n->net.nparams : 0; }

sgi_status sgi_nn_get_params(sgi_nn* n, float* host, int64_t count) {
    if (!n || !host || count < (int64_t)n->net.nparams) return SGI_ERR_ARG;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(host, n->net.w32, n->net.nparams * sizeof(float), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? SGI_OK : nn_cuda(n, e, "get params");
}

sgi_status sgi_nn_set_params(sgi_nn* n, const float* host, int64_t count) {
    if (!n || !host || count < (int64_t)n->net.nparams) return SGI_ERR_ARG;
    cudaError_t e = n->net.set_params(host, n->net.nparams);
    return e == cudaSuccess ? SGI_OK : nn_cuda(n, e, "set params");
}

sgi_status sgi_nn_get_grads(sgi_nn* n, float* host, int64_t count) {
    if (!n || !host || count < (int64_t)n->net.nparams) return SGI_ERR_ARG;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(host, n->net.g32, n->net.nparams * sizeof(float), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? SGI_OK : nn_cuda(n, e, "get grads");
}

sgi_status sgi_nn_forward(sgi_nn* n, const void* features, const float* noisy, const float* prev, int32_t B,
                          int32_t H, int32_t W, float* out, void* stream) {
    if (!n || !features || !noisy || !prev || !out) return nn_fail(n, SGI_ERR_ARG, "NULL tensor");
    if (!shape_ok(n, B, H, W)) return nn_fail(n, SGI_ERR_CAP, "batch/size exceed the network's capacity or H, W % 4");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = n->net.forward((const __nv_bfloat16*)features, B, H, W, s);
    if (e != cudaSuccess) return nn_cuda(n, e, "forward");
    sgi::nn::ApplyArgs a{n->net.LOG, (const float4*)noisy, (const float4*)prev, nullptr, (float4*)out, nullptr, nullptr,
                         0.0f, B, H, W};
    e = sgi::nn::kpcn_apply(a, s);
    n->net.launches += 1;
    return e == cudaSuccess ? SGI_OK : nn_cuda(n, e, "apply");
}

sgi_status sgi_nn_train_step(sgi_nn* n, const void* features, const float* noisy, const float* prev,
                             const float* target, int32_t B, int32_t H, int32_t W, float lr, int32_t apply_update,
                             float* loss_host, void* stream) {
    if (!n || !features || !noisy || !prev || !target) return nn_fail(n, SGI_ERR_ARG, "NULL tensor");
    if (!shape_ok(n, B, H, W)) return nn_fail(n, SGI_ERR_CAP, "batch/size exceed the network's capacity or H, W % 4");
    cudaStream_t s = (cudaStream_t)stream;
    Net& net = n->net;
    cudaError_t e = net.forward((const __nv_bfloat16*)features, B, H, W, s);
    if (e != cudaSuccess) return nn_cuda(n, e, "forward");
    e = cudaMemsetAsync(net.loss_dev, 0, sizeof(float), s);
    if (e != cudaSuccess) return nn_cuda(n, e, "loss reset");
    const size_t P = (size_t)B * H * W;
    sgi::nn::ApplyArgs a{net.LOG, (const float4*)noisy, (const float4*)prev, (const float4*)target, nullptr, net.GA,
                         net.loss_dev, 1.0f / (3.0f * (float)P), B, H, W};
    e = sgi::nn::kpcn_apply(a, s);
    if (e != cudaSuccess) return nn_cuda(n, e, "apply/loss");
    e = net.backward((const __nv_bfloat16*)features, B, H, W, s);
    if (e != cudaSuccess) return nn_cuda(n, e, "backward");
    if (apply_update) {
        n->step += 1;
        e = sgi::nn::adam(net.w32, net.g32, net.m32, net.v32, net.wbf, net.nparams, lr, 0.9f, 0.999f, 1e-8f, n->step, s);
        if (e != cudaSuccess) return nn_cuda(n, e, "adam");
    }
    net.launches += 3;
    if (loss_host) {
        float l = 0.0f;
        e = cudaMemcpyAsync(&l, net.loss_dev, sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return nn_cuda(n, e, "loss readback");
        *loss_host = l / (3.0f * (float)P);
    }
    return SGI_OK;
}

}  // extern "C"
