/*
 * sgi_nn.h - learned kernel-predicting denoiser (KPCNN) for the GI stage.
 *
 * No counterpart in StratusGFX: it replaces the a-trous passes of
 * vpl_pbr_gi_denoise.fs (ComputeVirtualPointLightGlobalIllumination_,
 * StratusRendererBackend.cpp:1912-1940) with a U-Net (3 levels, 32/64/128
 * channels, 3x3 convolutions) that predicts a 5x5 filter kernel and a temporal
 * blend weight per pixel. Convolutions run on the tensor cores in BF16 with
 * FP32 accumulation; the network is trained on the GPU by the library's own
 * forward and backward kernels (Adam, FP32 master weights).
 *
 * Tensors are device pointers, NHWC, batch-major:
 *   features  BF16 [B][H][W][16]  (kpcn_features: log1p noisy GI rgb, albedo rgb,
 *                                  normal xyz, view distance / 10, roughness,
 *                                  log1p 3x3 luminance variance, log1p warped
 *                                  previous output rgb, metallic)
 *   noisy     float4 [B][H][W]    per-pixel GI estimate (denoise pass-0 output)
 *   prev      float4 [B][H][W]    previous denoised GI warped by the velocity
 *   target    float4 [B][H][W]    converged GI (sgi_gi_target)
 *   out       float4 [B][H][W]    denoised GI
 * H and W must be multiples of 4.
 */
#ifndef SGI_NN_H_
#define SGI_NN_H_

#include "sgi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgi_nn sgi_nn;

typedef struct sgi_nn_config {
    int32_t max_batch;
    int32_t max_height;
    int32_t max_width;
    uint32_t seed;         /* He-normal initialisation seed */
} sgi_nn_config;

sgi_status sgi_nn_create(const sgi_nn_config* cfg, sgi_nn** out);
sgi_status sgi_nn_destroy(sgi_nn* net);
const char* sgi_nn_last_error(const sgi_nn* net);

/* Parameters: FP32 master copy, layer by layer ([cout][3][3][cin] weights, then [cout] bias). */
int64_t sgi_nn_num_params(const sgi_nn* net);
sgi_status sgi_nn_get_params(sgi_nn* net, float* host, int64_t n);
sgi_status sgi_nn_set_params(sgi_nn* net, const float* host, int64_t n);
/* The Adam state (first and second moments, same layout as the parameters, and
 * the number of updates taken) for training checkpoints; restoring it with the
 * parameters resumes training where it stopped. */
sgi_status sgi_nn_get_optimizer_state(sgi_nn* net, float* m, float* v, int64_t n, int64_t* step);
sgi_status sgi_nn_set_optimizer_state(sgi_nn* net, const float* m, const float* v, int64_t n, int64_t step);
/* Gradients of the last sgi_nn_train_step (same layout as the parameters). */
sgi_status sgi_nn_get_grads(sgi_nn* net, float* host, int64_t n);

/* Inference: out = denoised GI. */
sgi_status sgi_nn_forward(sgi_nn* net, const void* features, const float* noisy, const float* prev, int32_t batch,
                          int32_t height, int32_t width, float* out, void* stream);

/* One training step: forward, loss = mean |log1p(out) - log1p(target)|, backward,
 * and (if apply_update) one Adam update with learning rate lr. *loss_host receives
 * the loss (this call synchronises the stream when loss_host is not NULL). */
sgi_status sgi_nn_train_step(sgi_nn* net, const void* features, const float* noisy, const float* prev,
                             const float* target, int32_t batch, int32_t height, int32_t width, float lr,
                             int32_t apply_update, float* loss_host, void* stream);

/* Builds the network inputs of the frame last gathered by `ctx` (after
 * sgi_global_illumination or sgi_render_frame with this frame's G-buffer):
 * features, noisy and prev (as above, batch 1), each 16-byte aligned (else
 * SGI_ERR_ARG). `prev` warps the context's GI history with the velocity buffer
 * (bilinear), like the temporal pass. */
sgi_status sgi_nn_features(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_camera* cam, void* features,
                           float* noisy, float* prev, void* stream);

/* Convolution engine of the 3x3 layers: tcgen05.mma with TMEM accumulators
 * (default) or warp-level mma.sync. Both accumulate BF16 products in FP32. */
enum { SGI_NN_CONV_WARP_MMA = 0, SGI_NN_CONV_TCGEN05 = 1 };
sgi_status sgi_nn_set_conv_path(sgi_nn* net, int32_t path);

/* The neural frame (sgi_render_frame_neural) on the tcgen05 path applies the
 * predicted kernels and writes the composite in the head convolution's
 * epilogue (default, enabled != 0), or writes the logits and runs the separate
 * kernel-apply pass (0); both give the same frame. */
sgi_status sgi_nn_set_head_fusion(sgi_nn* net, int32_t enabled);

/* Inference precision of the convolutions: BF16 (default) or FP8 E4M3 with
 * per-channel scales and FP32 accumulation (tcgen05 path only). FP8 needs a
 * calibration after the last change of the weights (set_params, training). */
enum { SGI_NN_BF16 = 0, SGI_NN_FP8 = 1 };
sgi_status sgi_nn_set_precision(sgi_nn* net, int32_t precision);
/* Runs the BF16 network on `features` (as for sgi_nn_forward), takes per-channel
 * maxima of every tensor a convolution reads (scale = max / 448, the largest
 * finite E4M3) and quantizes the weights per output channel with the input
 * scales folded in. Synchronises the stream. */
sgi_status sgi_nn_calibrate_fp8(sgi_nn* net, const void* features, int32_t batch, int32_t height, int32_t width,
                                void* stream);

/* Synchronises the device and reads (and clears) the network's error flag:
 * SGI_ERR_TIMEOUT when a tensor-core convolution gave up a bounded wait. */
sgi_status sgi_nn_device_status(sgi_nn* net);

/* The bounded waits of the tensor-core convolutions (no counterpart in
 * StratusGFX): every wait of a role (TMA producer, MMA issuer, epilogue) on
 * another gives up after wait_ns nanoseconds (0: the default 200 ms), raises
 * the CTA's abort flag, lets MMAs already issued finish, frees its tensor
 * memory and returns; sgi_nn_device_status then reports SGI_ERR_TIMEOUT.
 * skip_producer != 0 is a test switch: the TMA producers issue no copy, so the
 * first wait of the MMA role runs out with no copy or MMA in flight. */
sgi_status sgi_nn_set_wait_test(sgi_nn* net, int64_t wait_ns, int32_t skip_producer);

/* One 3x3 convolution layer (zero padding) as the network runs it:
 * y[b][h][w][o] = act(bias[o] + sum_{ky,kx,c} w[o][ky*3+kx][c] * x[b][h+ky-1][w+kx-1][c])
 * with act = ReLU (mode 0), identity (mode 1) or no bias and identity (mode 2).
 * x, y: BF16 NHWC with channel strides x_stride / y_stride (elements, multiples
 * of 8; pointers 16-byte aligned); w: BF16 [cout][9][cin]; bias: float [cout].
 * (cin, cout) must be one of the network's layer shapes or their transposes.
 * err_flag: device int set to 1 if a tcgen05 wait ran out (required for that path). */
sgi_status sgi_nn_conv3x3(int32_t path, int32_t cin, int32_t cout, int32_t mode, const void* x, int32_t x_stride,
                          const void* w, const float* bias, void* y, int32_t y_stride, int32_t batch, int32_t height,
                          int32_t width, int32_t* err_flag, void* stream);

/* The GI stage with the learned denoiser in place of the a-trous passes:
 * VPL cull, direct lighting, tile cull, GI gather, features, U-Net, kernel
 * apply + temporal blend, composite hdr_out = screen + gi * denoised. The
 * denoised GI becomes the context's history. */
sgi_status sgi_render_frame_neural(sgi_ctx* ctx, sgi_nn* net, const sgi_gbuffer* cur, const sgi_gbuffer* prev,
                                   const sgi_camera* cam, const sgi_frame_params* params, void* hdr_out,
                                   void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SGI_NN_H_ */
