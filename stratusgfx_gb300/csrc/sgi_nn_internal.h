// sgi_nn_internal.h - launch wrappers of the learned denoiser kernels (sgi_nn.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace sgi {
namespace nn {

// NHWC tensor views: pointer at channel 0 of pixel 0, `*s` = channel stride per pixel.
struct ConvArgs {
    const __nv_bfloat16* x;
    int xs;
    const __nv_bfloat16* w;   // [cout][9][cin] (dgrad: flipped [cin][9][cout])
    const float* bias;        // [cout], unused in mode 2
    __nv_bfloat16* y;
    int ys;
    int B, H, W;
};

struct WgradArgs {
    const __nv_bfloat16* x;
    int xs;
    const __nv_bfloat16* dz;
    int dzs;
    float* dw;                // [cout][9][cin], accumulated
    int cin, cout;
    int B, H, W;
};

struct ApplyArgs {
    const __nv_bfloat16* logits;  // [P][32]
    const float4* noisy;          // [P]
    const float4* prev;           // [P]
    const float4* target;         // [P] or null (inference)
    float4* out;                  // [P] or null
    __nv_bfloat16* dlogits;       // [P][32] when target
    float* loss;                  // sum of |log1p(out) - log1p(target)| (device scalar) or null
    float grad_scale;             // 1 / (3 * pixels)
    int B, H, W;
};

struct FeatureArgs {
    int W, H;
    const uint2* merged;          // denoise pass-0 output (RGBA16F)
    const float4* guide;          // normal xyz, depth
    const uint32_t* albedo;
    const uint32_t* rma;
    const uint32_t* velocity;
    const uint2* gi_prev;         // GI history (RGBA16F)
    int have_history;
    float inv_pv[16];
    float cam_pos[3];
    __nv_bfloat16* features;      // [P][16]
    float4* noisy;
    float4* prev;
};

cudaError_t features(const FeatureArgs& a, cudaStream_t s);
cudaError_t composite(const float4* den, const uint2* screen, const uint32_t* albedo, uint2* hdr, uint2* gi_out,
                      uint16_t* hist_out, size_t P, cudaStream_t s);
cudaError_t conv3x3(int cin, int cout, int mode, const ConvArgs& a, cudaStream_t s);
cudaError_t flip_weights(const __nv_bfloat16* w, __nv_bfloat16* wt, int cin, int cout, cudaStream_t s);
cudaError_t wgrad(const WgradArgs& a, cudaStream_t s);
cudaError_t bias_grad(const __nv_bfloat16* dz, int dzs, int c, size_t pixels, float* db, cudaStream_t s);
cudaError_t relu_bwd(const __nv_bfloat16* dy, int dys, const __nv_bfloat16* y, int ys, __nv_bfloat16* dz, int c,
                     size_t pixels, cudaStream_t s);
cudaError_t pool_fwd(const __nv_bfloat16* in, int is, __nv_bfloat16* out, int os, int B, int H, int W, int c,
                     cudaStream_t s);
cudaError_t pool_bwd(const __nv_bfloat16* dout, int os, __nv_bfloat16* din, int is, int B, int H, int W, int c,
                     int accumulate, cudaStream_t s);
cudaError_t up_fwd(const __nv_bfloat16* in, int is, __nv_bfloat16* out, int os, int B, int H, int W, int c,
                   cudaStream_t s);
cudaError_t up_bwd(const __nv_bfloat16* dout, int os, __nv_bfloat16* din, int is, int B, int Hi, int Wi, int c,
                   cudaStream_t s);
cudaError_t kpcn_apply(const ApplyArgs& a, cudaStream_t s);
cudaError_t adam(float* w, const float* g, float* m, float* v, __nv_bfloat16* wb, size_t n, float lr, float b1,
                 float b2, float eps, int step, cudaStream_t s);
cudaError_t to_bf16(const float* w, __nv_bfloat16* wb, size_t n, cudaStream_t s);

}  // namespace nn
}  // namespace sgi
