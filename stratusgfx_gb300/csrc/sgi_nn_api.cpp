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
#include <algorithm>
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
    for (int l = 0; l < NUM_LAYERS; ++l)
        wgrad_part_n = std::max(wgrad_part_n, wgrad_part_floats(kCin[l], kCout[l]));
    chk(alloc(&wgrad_part, wgrad_part_n));
    chk(alloc(&loss_part, apply_loss_blocks(c.max_batch, c.max_height, c.max_width)));
    chk(alloc(&dev_err, 1));
    size_t sc = 0, in = 0;
    for (int l = 0; l < NUM_LAYERS; ++l) {
        sc_off[l] = sc;
        sc += kCout[l];
        in_off[l] = in;
        in += kCin[l];
    }
    chk(alloc(&wq, nparams));
    chk(alloc(&f8_wscale, sc));
    chk(alloc(&f8_oinv, sc));
    chk(alloc(&f8_sin, in));
    chk(alloc(&f8_finv, 16));
    chk(alloc(&f8_absmax, 11 * 128));
    if (e != cudaSuccess) return e;
    e = cudaMemset(dev_err, 0, sizeof(int));
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
    fp8_ready = false;   // new weights need a new FP8 calibration
    cudaError_t e = cudaMemcpy(w32, host, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    e = to_bf16(w32, wbf, nparams, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e;
}

cudaError_t Net::conv_any(int cin, int cout, int mode, const ConvArgs& a, cudaStream_t s) {
    if (conv_path != SGI_NN_CONV_TCGEN05) return conv3x3(cin, cout, mode, a, s);
    ConvArgs b = a;
    b.wait_ns = wait_ns;
    b.skip_producer = skip_producer;
    return conv3x3_tc(cin, cout, mode, b, dev_err, s);
}

cudaError_t Net::conv(int l, const View& x, const View& y, int B, int H, int W, cudaStream_t s, const View* pool) {
    ConvArgs a{x, wbf + w_off[l], w32 + b_off[l], y, B, H, W};
    if (pool) a.pool = *pool;
    if (l == HEAD && head_fuse && conv_path == SGI_NN_CONV_TCGEN05) {
        if (head_wait) {
            const cudaError_t e = cudaStreamWaitEvent(s, head_wait, 0);
            if (e != cudaSuccess) return e;
        }
        a.fuse = *head_fuse;
        a.wait_ns = wait_ns;
        a.skip_producer = skip_producer;
        return conv3x3_head_apply(a, dev_err, s);
    }
    return conv_any(kCin[l], kCout[l], l == HEAD ? 1 : 0, a, s);
}

// Activations, gradients and the input features are NHWC; the decoder inputs
// D1IN (96 channels) and D2IN (192) take the skip connections as channel slices.
#define NN_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)

cudaError_t Net::conv8(int l, const View& x, const View& y, int B, int H, int W, cudaStream_t s, bool in8, bool out8,
                       const View* pool) {
    ConvArgs a{x, in8 ? reinterpret_cast<const bf16*>(wq + w_off[l]) : wbf + w_off[l], w32 + b_off[l], y, B, H, W};
    if (pool) a.pool = *pool;
    a.wscale = in8 ? f8_wscale + sc_off[l] : nullptr;
    a.oinv = out8 ? f8_oinv + sc_off[l] : nullptr;
    a.wait_ns = wait_ns;
    a.skip_producer = skip_producer;
    return conv3x3_tc_fp8(kCin[l], kCout[l], l == HEAD ? 1 : 0, in8, out8, a, dev_err, s);
}

// FP8 E4M3 forward. The first and the last two layers keep BF16 where precision
// matters most: e1a reads the BF16 features with BF16 weights and writes E4M3,
// d1b reads E4M3 and writes BF16, and the head runs in BF16. The layers between
// read and write E4M3 with per-channel scales (each output's scales are folded
// into the next layer's weights); pooling and upsampling move E4M3 bytes
// unchanged. FP8 tensors are BF16-unit views with half the channel count.
cudaError_t Net::forward_fp8(const bf16* feat, int B, int H, int W, cudaStream_t s) {
    const int H2 = H / 2, W2 = W / 2, H4 = H / 4, W4 = W / 4;
    cudaError_t e;
    const View fb = nhwc_view(feat, 16, H, W);
    const View e1a = nhwc_view(E1A_, 16, H, W), d1in = nhwc_view(D1IN, 48, H, W);
    const View p1 = nhwc_view(P1, 16, H2, W2), e2a = nhwc_view(E2A_, 32, H2, W2);
    const View d2in = nhwc_view(D2IN, 96, H2, W2), p2 = nhwc_view(P2_, 32, H4, W4);
    const View b1 = nhwc_view(B1_, 64, H4, W4), b2 = nhwc_view(B2_, 64, H4, W4);
    const View d2a = nhwc_view(D2A_, 32, H2, W2), d2b = nhwc_view(D2B_, 32, H2, W2);
    const View d1a = nhwc_view(D1A_, 16, H, W), d1b = nhwc_view(D1B_, 32, H, W);   // d1b: BF16 output
    const View lg = planar_view(LOG, 4, H, W);
    NN_TRY(conv8(E1A, fb, e1a, B, H, W, s, false, true));
    NN_TRY(conv8(E1B, e1a, channel_slice(d1in, 32), B, H, W, s, true, true, &p1));
    NN_TRY(conv8(E2A, p1, e2a, B, H2, W2, s, true, true));
    NN_TRY(conv8(E2B, e2a, channel_slice(d2in, 64), B, H2, W2, s, true, true, &p2));
    NN_TRY(conv8(B1, p2, b1, B, H4, W4, s, true, true));
    NN_TRY(conv8(B2, b1, b2, B, H4, W4, s, true, true));
    NN_TRY(up_fwd(b2, d2in, B, H2, W2, 64, s));
    NN_TRY(conv8(D2A, d2in, d2a, B, H2, W2, s, true, true));
    NN_TRY(conv8(D2B, d2a, d2b, B, H2, W2, s, true, true));
    NN_TRY(up_fwd(d2b, d1in, B, H, W, 32, s));
    NN_TRY(conv8(D1A, d1in, d1a, B, H, W, s, true, true));
    NN_TRY(conv8(D1B, d1a, d1b, B, H, W, s, true, false));
    NN_TRY(conv(HEAD, d1b, lg, B, H, W, s));
    launches += 13;
    return cudaSuccess;
}

// Calibration: the BF16 forward on `feat`, per-channel |x| maxima of every tensor a
// convolution reads, scales = max / 448 (the largest finite E4M3), then the weights
// quantized with the input scales folded in.
cudaError_t Net::calibrate_fp8(const bf16* feat, int B, int H, int W, cudaStream_t s) {
    const int H2 = H / 2, W2 = W / 2, H4 = H / 4, W4 = W / 4;
    cudaError_t e;
    const int saved = conv_path;
    conv_path = SGI_NN_CONV_TCGEN05;
    e = forward(feat, B, H, W, s, false);
    conv_path = saved;
    if (e != cudaSuccess) return e;
    NN_TRY(cudaMemsetAsync(f8_absmax, 0, 11 * 128 * sizeof(float), s));
    struct T { View v; int c, h, w; };
    const T ts[11] = {{nhwc_view(feat, 16, H, W), 16, H, W},
                      {nhwc_view(E1A_, 32, H, W), 32, H, W},
                      {channel_slice(nhwc_view(D1IN, 96, H, W), 64), 32, H, W},
                      {nhwc_view(E2A_, 64, H2, W2), 64, H2, W2},
                      {channel_slice(nhwc_view(D2IN, 192, H2, W2), 128), 64, H2, W2},
                      {nhwc_view(B1_, 128, H4, W4), 128, H4, W4},
                      {nhwc_view(B2_, 128, H4, W4), 128, H4, W4},
                      {nhwc_view(D2A_, 64, H2, W2), 64, H2, W2},
                      {nhwc_view(D2B_, 64, H2, W2), 64, H2, W2},
                      {nhwc_view(D1A_, 32, H, W), 32, H, W},
                      {nhwc_view(D1B_, 32, H, W), 32, H, W}};
    for (int t = 0; t < 11; ++t) NN_TRY(channel_absmax(ts[t].v, ts[t].c, B, ts[t].h, ts[t].w, f8_absmax + 128 * t, s));
    std::vector<float> mx(11 * 128);
    NN_TRY(cudaMemcpyAsync(mx.data(), f8_absmax, mx.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
    NN_TRY(cudaStreamSynchronize(s));
    auto scale = [&](int t, int c) { const float m = mx[128 * t + c]; return m > 0.0f ? m / 448.0f : 1.0f; };
    // tensors feeding each layer (index, channels); decoder inputs concatenate two tensors
    const int in_t[NUM_LAYERS][2] = {{0, -1}, {1, -1}, {2, -1}, {3, -1}, {4, -1}, {5, -1},
                                     {6, 4}, {7, -1}, {8, 2}, {9, -1}, {10, -1}};
    const int out_t[NUM_LAYERS] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, -1};
    std::vector<float> sin_h(in_off[NUM_LAYERS - 1] + kCin[NUM_LAYERS - 1]);
    std::vector<float> oinv_h(sc_off[NUM_LAYERS - 1] + kCout[NUM_LAYERS - 1], 1.0f);
    for (int l = 0; l < NUM_LAYERS; ++l) {
        int k = 0;
        for (int part = 0; part < 2 && in_t[l][part] >= 0; ++part) {
            const int t = in_t[l][part];
            for (int c = 0; c < ts[t].c; ++c) sin_h[in_off[l] + k++] = scale(t, c);
        }
        if (k != kCin[l]) return cudaErrorInvalidValue;
        if (out_t[l] >= 0)
            for (int c = 0; c < kCout[l]; ++c) oinv_h[sc_off[l] + c] = 1.0f / scale(out_t[l], c);
    }
    float finv_h[16];
    for (int c = 0; c < 16; ++c) finv_h[c] = 1.0f / scale(0, c);
    NN_TRY(cudaMemcpyAsync(f8_sin, sin_h.data(), sin_h.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    NN_TRY(cudaMemcpyAsync(f8_oinv, oinv_h.data(), oinv_h.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    NN_TRY(cudaMemcpyAsync(f8_finv, finv_h, sizeof(finv_h), cudaMemcpyHostToDevice, s));
    for (int l = 0; l < NUM_LAYERS; ++l)
        NN_TRY(quantize_weights(w32 + w_off[l], f8_sin + in_off[l], kCin[l], kCout[l], wq + w_off[l],
                                f8_wscale + sc_off[l], s));
    NN_TRY(cudaStreamSynchronize(s));
    fp8_ready = true;
    return cudaSuccess;
}

cudaError_t Net::forward(const bf16* feat, int B, int H, int W, cudaStream_t s, bool allow_fp8) {
    if (allow_fp8 && precision == SGI_NN_FP8) {
        if (!fp8_ready || conv_path != SGI_NN_CONV_TCGEN05) return cudaErrorNotReady;
        return forward_fp8(feat, B, H, W, s);
    }
    const int H2 = H / 2, W2 = W / 2, H4 = H / 4, W4 = W / 4;
    cudaError_t e;
    const View f = nhwc_view(feat, 16, H, W);
    const View e1a = nhwc_view(E1A_, 32, H, W), d1in = nhwc_view(D1IN, 96, H, W);
    const View p1 = nhwc_view(P1, 32, H2, W2), e2a = nhwc_view(E2A_, 64, H2, W2);
    const View d2in = nhwc_view(D2IN, 192, H2, W2), p2 = nhwc_view(P2_, 64, H4, W4);
    const View b1 = nhwc_view(B1_, 128, H4, W4), b2 = nhwc_view(B2_, 128, H4, W4);
    const View d2a = nhwc_view(D2A_, 64, H2, W2), d2b = nhwc_view(D2B_, 64, H2, W2);
    const View d1a = nhwc_view(D1A_, 32, H, W), d1b = nhwc_view(D1B_, 32, H, W);
    const View lg = planar_view(LOG, 4, H, W);   // logits: planar, read per channel group by the kernel apply
    if (conv_path == SGI_NN_CONV_TCGEN05) {
        // the tensor-core epilogues of e1b and e2b also write the pooled copies
        NN_TRY(conv(E1A, f, e1a, B, H, W, s));
        NN_TRY(conv(E1B, e1a, channel_slice(d1in, 64), B, H, W, s, &p1));
        NN_TRY(conv(E2A, p1, e2a, B, H2, W2, s));
        NN_TRY(conv(E2B, e2a, channel_slice(d2in, 128), B, H2, W2, s, &p2));
        NN_TRY(conv(B1, p2, b1, B, H4, W4, s));
        NN_TRY(conv(B2, b1, b2, B, H4, W4, s));
        NN_TRY(up_fwd(b2, d2in, B, H2, W2, 128, s));
        NN_TRY(conv(D2A, d2in, d2a, B, H2, W2, s));
        NN_TRY(conv(D2B, d2a, d2b, B, H2, W2, s));
        NN_TRY(up_fwd(d2b, d1in, B, H, W, 64, s));
        NN_TRY(conv(D1A, d1in, d1a, B, H, W, s));
        NN_TRY(conv(D1B, d1a, d1b, B, H, W, s));
        NN_TRY(conv(HEAD, d1b, lg, B, H, W, s));
        launches += 13;
        return cudaSuccess;
    }
    NN_TRY(conv(E1A, f, e1a, B, H, W, s));
    NN_TRY(conv(E1B, e1a, channel_slice(d1in, 64), B, H, W, s));
    NN_TRY(pool_fwd(channel_slice(d1in, 64), p1, B, H, W, 32, s));
    NN_TRY(conv(E2A, p1, e2a, B, H2, W2, s));
    NN_TRY(conv(E2B, e2a, channel_slice(d2in, 128), B, H2, W2, s));
    NN_TRY(pool_fwd(channel_slice(d2in, 128), p2, B, H2, W2, 64, s));
    NN_TRY(conv(B1, p2, b1, B, H4, W4, s));
    NN_TRY(conv(B2, b1, b2, B, H4, W4, s));
    NN_TRY(up_fwd(b2, d2in, B, H2, W2, 128, s));
    NN_TRY(conv(D2A, d2in, d2a, B, H2, W2, s));
    NN_TRY(conv(D2B, d2a, d2b, B, H2, W2, s));
    NN_TRY(up_fwd(d2b, d1in, B, H, W, 64, s));
    NN_TRY(conv(D1A, d1in, d1a, B, H, W, s));
    NN_TRY(conv(D1B, d1a, d1b, B, H, W, s));
    NN_TRY(conv(HEAD, d1b, lg, B, H, W, s));
    launches += 15;
    return cudaSuccess;
}

// Backward of layer l: dz = relu'(dy) (or dy for the head) into the buffer
// dz_buf, weight / bias gradients from its input x, and (if dx.p) the input
// gradient.
cudaError_t Net::layer_backward(int l, const View& x, const View& y, const View& dy, bf16* dz_buf, const View& dx,
                                int B, int H, int W, cudaStream_t s) {
    cudaError_t e;
    View g = dy;
    if (l != HEAD) {
        const View dz = nhwc_view(dz_buf, kCout[l], H, W);
        NN_TRY(relu_bwd(dy, y, dz, kCout[l], B, H, W, s));
        g = dz;
        launches += 1;
    }
    WgradArgs wa{x, g, g32 + w_off[l], kCin[l], kCout[l], B, H, W, wgrad_part, wgrad_part_n, dev_err, wait_ns,
                 skip_producer};
    NN_TRY(wgrad(wa, s));   // weights and bias (b_off[l] follows the layer's weights)
    launches += 2;
    if (dx.p) {
        NN_TRY(flip_weights(wbf + w_off[l], wflip + w_off[l], kCin[l], kCout[l], s));
        ConvArgs a{g, wflip + w_off[l], nullptr, dx, B, H, W};
        NN_TRY(conv_any(kCout[l], kCin[l], 2, a, s));
        launches += 2;
    }
    return cudaSuccess;
}

cudaError_t Net::backward(const bf16* feat, int B, int H, int W, cudaStream_t s) {
    const int H2 = H / 2, W2 = W / 2, H4 = H / 4, W4 = W / 4;
    cudaError_t e;
    auto full = [&](bf16* p, int c) { return nhwc_view(p, c, H, W); };
    auto half = [&](bf16* p, int c) { return nhwc_view(p, c, H2, W2); };
    auto quarter = [&](bf16* p, int c) { return nhwc_view(p, c, H4, W4); };
    const View none{nullptr, 8, 8, 8};
    NN_TRY(cudaMemsetAsync(g32, 0, nparams * sizeof(float), s));
    // full resolution decoder: dLOGITS in GA
    NN_TRY(layer_backward(HEAD, full(D1B_, 32), planar_view(LOG, 4, H, W), full(GA, 32), nullptr, full(GB, 32), B, H,
                          W, s));
    NN_TRY(layer_backward(D1B, full(D1A_, 32), full(D1B_, 32), full(GB, 32), GC, full(GA, 32), B, H, W, s));
    NN_TRY(layer_backward(D1A, full(D1IN, 96), full(D1A_, 32), full(GA, 32), GB, full(GD, 96), B, H, W, s));
    NN_TRY(up_bwd(full(GD, 96), half(GH1, 64), B, H2, W2, 64, s));                          // dD2B
    NN_TRY(layer_backward(D2B, half(D2A_, 64), half(D2B_, 64), half(GH1, 64), GH2, half(GH1, 64), B, H2, W2, s));
    NN_TRY(layer_backward(D2A, half(D2IN, 192), half(D2A_, 64), half(GH1, 64), GH2, half(GH3, 192), B, H2, W2, s));
    NN_TRY(up_bwd(half(GH3, 192), quarter(GQ1, 128), B, H4, W4, 128, s));                  // dB2
    NN_TRY(layer_backward(B2, quarter(B1_, 128), quarter(B2_, 128), quarter(GQ1, 128), GQ2, quarter(GQ1, 128), B, H4,
                          W4, s));
    NN_TRY(layer_backward(B1, quarter(P2_, 64), quarter(B1_, 128), quarter(GQ1, 128), GQ2, quarter(GQ3, 64), B, H4,
                          W4, s));                                                                // dP2
    NN_TRY(pool_bwd(quarter(GQ3, 64), channel_slice(half(GH3, 192), 128), B, H2, W2, 64, 1, s));   // skip 2
    NN_TRY(layer_backward(E2B, half(E2A_, 64), channel_slice(half(D2IN, 192), 128), channel_slice(half(GH3, 192), 128),
                          GH2, half(GH1, 64), B, H2, W2, s));                                     // dE2A
    NN_TRY(layer_backward(E2A, half(P1, 32), half(E2A_, 64), half(GH1, 64), GH2, half(GH1, 32), B, H2, W2, s));  // dP1
    NN_TRY(pool_bwd(half(GH1, 32), channel_slice(full(GD, 96), 64), B, H, W, 32, 1, s));         // skip 1
    NN_TRY(layer_backward(E1B, full(E1A_, 32), channel_slice(full(D1IN, 96), 64), channel_slice(full(GD, 96), 64), GC,
                          full(GA, 32), B, H, W, s));                                             // dE1A
    NN_TRY(layer_backward(E1A, nhwc_view(feat, 16, H, W), full(E1A_, 32), full(GA, 32), GB, none, B, H, W, s));
    launches += 5;
    return cudaSuccess;
}
#undef NN_TRY

}  // namespace nn
}  // namespace sgi

using sgi::nn::Net;

static sgi_status nn_fail(sgi_nn* n, sgi_status s, const std::string& m) {
    if (n) n->err = m;
    sgi_log_message(SGI_LOG_ERROR, m.c_str());
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

sgi_status sgi_nn_get_optimizer_state(sgi_nn* n, float* m, float* v, int64_t count, int64_t* step) {
    if (!n || !m || !v || !step || count < (int64_t)n->net.nparams) return SGI_ERR_ARG;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(m, n->net.m32, n->net.nparams * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(v, n->net.v32, n->net.nparams * sizeof(float), cudaMemcpyDeviceToHost);
    *step = n->step;
    return e == cudaSuccess ? SGI_OK : nn_cuda(n, e, "get optimizer state");
}

sgi_status sgi_nn_set_optimizer_state(sgi_nn* n, const float* m, const float* v, int64_t count, int64_t step) {
    if (!n || !m || !v || count < (int64_t)n->net.nparams || step < 0 || step > 0x7fffffff) return SGI_ERR_ARG;
    cudaError_t e = cudaMemcpy(n->net.m32, m, n->net.nparams * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(n->net.v32, v, n->net.nparams * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return nn_cuda(n, e, "set optimizer state");
    n->step = (int)step;
    return SGI_OK;
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

}  // extern "C"

sgi_status nn_forward_net(sgi_nn* n, const void* features, int H, int W, cudaStream_t s) {
    if (!n || !features) return nn_fail(n, SGI_ERR_ARG, "NULL tensor");
    if (!shape_ok(n, 1, H, W)) return nn_fail(n, SGI_ERR_CAP, "batch/size exceed the network's capacity or H, W % 4");
    cudaError_t e = n->net.forward((const __nv_bfloat16*)features, 1, H, W, s);
    if (e == cudaErrorNotReady) return nn_fail(n, SGI_ERR_STATE, "FP8 precision needs sgi_nn_calibrate_fp8 after the last weight change");
    return e == cudaSuccess ? SGI_OK : nn_cuda(n, e, "forward");
}

sgi_status nn_forward_composite(sgi_nn* n, const void* features, int H, int W, const uint2* noisy, const float* prev,
                                const uint2* screen, const uint32_t* albedo, uint2* hdr, uint2* gi_out,
                                uint16_t* hist_out, cudaEvent_t before_head, cudaStream_t s) {
    if (!n || !features || !noisy || !prev || !screen || !albedo || !hdr || !gi_out || !hist_out)
        return nn_fail(n, SGI_ERR_ARG, "NULL tensor");
    if (n->net.conv_path != SGI_NN_CONV_TCGEN05 || !n->net.head_fusion) {
        sgi_status st = nn_forward_net(n, features, H, W, s);
        if (st != SGI_OK) return st;
        if (before_head && cudaStreamWaitEvent(s, before_head, 0) != cudaSuccess)
            return nn_fail(n, SGI_ERR_CUDA, "wait for the direct lighting");
        return nn_apply_composite(n, noisy, prev, H, W, screen, albedo, hdr, gi_out, hist_out, s);
    }
    const sgi::nn::ConvArgs::ApplyFuse fuse{noisy, (const float4*)prev, screen, albedo, hdr, gi_out, hist_out};
    n->net.head_fuse = &fuse;
    n->net.head_wait = before_head;
    const sgi_status st = nn_forward_net(n, features, H, W, s);
    n->net.head_fuse = nullptr;
    n->net.head_wait = nullptr;
    return st;
}

sgi_status nn_apply_composite(sgi_nn* n, const uint2* noisy, const float* prev, int H, int W, const uint2* screen,
                              const uint32_t* albedo, uint2* hdr, uint2* gi_out, uint16_t* hist_out, cudaStream_t s) {
    if (!n || !noisy || !prev || !screen || !albedo || !hdr || !gi_out || !hist_out)
        return nn_fail(n, SGI_ERR_ARG, "NULL tensor");
    if (!shape_ok(n, 1, H, W)) return nn_fail(n, SGI_ERR_CAP, "batch/size exceed the network's capacity or H, W % 4");
    const sgi::nn::View none{nullptr, 8, 8, 8};
    sgi::nn::ApplyArgs a{sgi::nn::planar_view(n->net.LOG, 4, H, W), nullptr, (const float4*)prev, nullptr,
                         nullptr, none, nullptr, nullptr, 0.0f, 1, H, W};
    a.noisy_h = noisy;
    a.screen = screen; a.albedo = albedo; a.hdr = hdr; a.gi_out = gi_out; a.hist_out = hist_out;
    const cudaError_t e = sgi::nn::kpcn_apply(a, s);
    n->net.launches += 1;
    return e == cudaSuccess ? SGI_OK : nn_cuda(n, e, "apply");
}

extern "C" {

sgi_status sgi_nn_forward(sgi_nn* n, const void* features, const float* noisy, const float* prev, int32_t B,
                          int32_t H, int32_t W, float* out, void* stream) {
    if (!n || !features || !noisy || !prev || !out) return nn_fail(n, SGI_ERR_ARG, "NULL tensor");
    if (!shape_ok(n, B, H, W)) return nn_fail(n, SGI_ERR_CAP, "batch/size exceed the network's capacity or H, W % 4");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = n->net.forward((const __nv_bfloat16*)features, B, H, W, s);
    if (e == cudaErrorNotReady) return nn_fail(n, SGI_ERR_STATE, "FP8 precision needs sgi_nn_calibrate_fp8 after the last weight change");
    if (e != cudaSuccess) return nn_cuda(n, e, "forward");
    const sgi::nn::View none{nullptr, 8, 8, 8};
    sgi::nn::ApplyArgs a{sgi::nn::planar_view(n->net.LOG, 4, H, W), (const float4*)noisy, (const float4*)prev, nullptr,
                         (float4*)out, none, nullptr, nullptr, 0.0f, B, H, W};
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
    cudaError_t e = net.forward((const __nv_bfloat16*)features, B, H, W, s, false);
    if (e != cudaSuccess) return nn_cuda(n, e, "forward");
    const size_t P = (size_t)B * H * W;
    sgi::nn::ApplyArgs a{sgi::nn::planar_view(net.LOG, 4, H, W), (const float4*)noisy, (const float4*)prev,
                         (const float4*)target, nullptr, sgi::nn::nhwc_view(net.GA, 32, H, W), net.loss_dev,
                         net.loss_part, 1.0f / (3.0f * (float)P), B, H, W};
    e = sgi::nn::kpcn_apply(a, s);
    if (e != cudaSuccess) return nn_cuda(n, e, "apply/loss");
    e = net.backward((const __nv_bfloat16*)features, B, H, W, s);
    if (e != cudaSuccess) return nn_cuda(n, e, "backward");
    if (apply_update) {
        n->step += 1;
        net.fp8_ready = false;
        e = sgi::nn::adam(net.w32, net.g32, net.m32, net.v32, net.wbf, net.nparams, lr, 0.9f, 0.999f, 1e-8f, n->step, s);
        if (e != cudaSuccess) return nn_cuda(n, e, "adam");
    }
    net.launches += 3;
    if (loss_host) {
        float l = 0.0f;
        int flag = 0;
        e = cudaMemcpyAsync(&l, net.loss_dev, sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, net.dev_err, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return nn_cuda(n, e, "loss readback");
        if (flag) return nn_fail(n, SGI_ERR_TIMEOUT, "a tensor-core convolution wait ran out");
        *loss_host = l / (3.0f * (float)P);
    }
    return SGI_OK;
}

sgi_status sgi_nn_calibrate_fp8(sgi_nn* n, const void* features, int32_t B, int32_t H, int32_t W, void* stream) {
    if (!n || !features) return nn_fail(n, SGI_ERR_ARG, "NULL tensor");
    if (!shape_ok(n, B, H, W)) return nn_fail(n, SGI_ERR_CAP, "batch/size exceed the network's capacity or H, W % 4");
    cudaError_t e = n->net.calibrate_fp8((const __nv_bfloat16*)features, B, H, W, (cudaStream_t)stream);
    return e == cudaSuccess ? SGI_OK : nn_cuda(n, e, "fp8 calibration");
}

sgi_status sgi_nn_set_precision(sgi_nn* n, int32_t precision) {
    if (!n || (precision != SGI_NN_BF16 && precision != SGI_NN_FP8)) return SGI_ERR_ARG;
    n->net.precision = precision;
    return SGI_OK;
}

sgi_status sgi_nn_set_conv_path(sgi_nn* n, int32_t path) {
    if (!n || (path != SGI_NN_CONV_WARP_MMA && path != SGI_NN_CONV_TCGEN05)) return SGI_ERR_ARG;
    n->net.conv_path = path;
    return SGI_OK;
}

sgi_status sgi_nn_set_head_fusion(sgi_nn* n, int32_t enabled) {
    if (!n) return SGI_ERR_ARG;
    n->net.head_fusion = enabled != 0;
    return SGI_OK;
}

sgi_status sgi_nn_set_wait_test(sgi_nn* n, int64_t wait_ns, int32_t skip_producer) {
    if (!n || wait_ns < 0 || wait_ns > 60000000000ll) return SGI_ERR_ARG;
    n->net.wait_ns = (unsigned long long)wait_ns;
    n->net.skip_producer = skip_producer ? 1 : 0;
    return SGI_OK;
}

sgi_status sgi_nn_device_status(sgi_nn* n) {
    if (!n) return SGI_ERR_ARG;
    int flag = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&flag, n->net.dev_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && flag) e = cudaMemset(n->net.dev_err, 0, sizeof(int));
    if (e != cudaSuccess) return nn_cuda(n, e, "device status");
    return flag ? nn_fail(n, SGI_ERR_TIMEOUT, "a tensor-core convolution wait ran out") : SGI_OK;
}

sgi_status sgi_nn_conv3x3(int32_t path, int32_t cin, int32_t cout, int32_t mode, const void* x, int32_t x_stride,
                          const void* w, const float* bias, void* y, int32_t y_stride, int32_t batch, int32_t height,
                          int32_t width, int32_t* err_flag, void* stream) {
    if (!x || !w || !y || (mode != 2 && !bias) || mode < 0 || mode > 2) return SGI_ERR_ARG;
    if (batch < 1 || height < 1 || width < 1 || x_stride < cin || y_stride < cout) return SGI_ERR_ARG;
    if ((x_stride % 8) || (y_stride % 8) || ((uintptr_t)x & 15) || ((uintptr_t)y & 15) || ((uintptr_t)w & 15))
        return SGI_ERR_ARG;
    sgi::nn::ConvArgs a{sgi::nn::nhwc_view(x, x_stride, height, width), (const __nv_bfloat16*)w, bias,
                        sgi::nn::nhwc_view(y, y_stride, height, width), batch, height, width};
    cudaError_t e;
    if (path == SGI_NN_CONV_TCGEN05) {
        if (!err_flag) return SGI_ERR_ARG;
        e = sgi::nn::conv3x3_tc(cin, cout, mode, a, err_flag, (cudaStream_t)stream);
    } else if (path == SGI_NN_CONV_WARP_MMA) {
        e = sgi::nn::conv3x3(cin, cout, mode, a, (cudaStream_t)stream);
    } else {
        return SGI_ERR_ARG;
    }
    if (e == cudaErrorInvalidValue) return SGI_ERR_ARG;
    return e == cudaSuccess ? SGI_OK : SGI_ERR_CUDA;
}

}  // extern "C"
