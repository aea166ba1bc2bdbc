// sgi_nn_net.h - the U-Net object behind sgi_nn (host side, internal).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/sgi_nn.h"
#include "sgi_nn_internal.h"

namespace sgi {
namespace nn {

struct Net {
    sgi_nn_config cfg{};
    size_t nparams = 0;
    size_t w_off[11] = {}, b_off[11] = {};
    int64_t launches = 0;
    std::vector<void*> allocs;
    // parameters
    float *w32 = nullptr, *g32 = nullptr, *m32 = nullptr, *v32 = nullptr, *loss_dev = nullptr;
    __nv_bfloat16 *wbf = nullptr, *wflip = nullptr;
    // activations
    __nv_bfloat16 *E1A_ = nullptr, *D1IN = nullptr, *P1 = nullptr, *E2A_ = nullptr, *D2IN = nullptr, *P2_ = nullptr,
                  *B1_ = nullptr, *B2_ = nullptr, *D2A_ = nullptr, *D2B_ = nullptr, *D1A_ = nullptr, *D1B_ = nullptr,
                  *LOG = nullptr;
    // gradients (full, half and quarter resolution scratch)
    __nv_bfloat16 *GA = nullptr, *GB = nullptr, *GC = nullptr, *GD = nullptr, *GH1 = nullptr, *GH2 = nullptr,
                  *GH3 = nullptr, *GQ1 = nullptr, *GQ2 = nullptr, *GQ3 = nullptr;
    float4* fwd_out = nullptr;
    float* wgrad_part = nullptr;   // split-K partial sums of the weight and bias gradients
    size_t wgrad_part_n = 0;
    float* loss_part = nullptr;    // per-block loss sums of kpcn_apply
    int* dev_err = nullptr;   // set by a tcgen05 kernel whose wait ran out
    unsigned long long wait_ns = 0;   // limit of the tcgen05 waits (0: the kernels' default)
    int skip_producer = 0;            // test switch: the convolutions' TMA producers issue nothing
    int conv_path = SGI_NN_CONV_TCGEN05;
    // set while a neural frame runs: the head applies the kernels and writes the composite itself
    const ConvArgs::ApplyFuse* head_fuse = nullptr;
    bool head_fusion = true;           // sgi_nn_set_head_fusion
    cudaEvent_t head_wait = nullptr;   // waited for before the head (the direct lighting it composites)
    // FP8 E4M3 inference (after calibrate_fp8): quantized weights (offsets w_off),
    // per-output-channel weight scales and inverse output scales (offsets sc_off),
    // per-input-channel scales folded into the weights (offsets in_off)
    int precision = SGI_NN_BF16;
    bool fp8_ready = false;
    uint8_t* wq = nullptr;
    float *f8_wscale = nullptr, *f8_oinv = nullptr, *f8_sin = nullptr, *f8_finv = nullptr, *f8_absmax = nullptr;
    size_t sc_off[11] = {}, in_off[11] = {};

    ~Net();
    void release();
    template <class T> cudaError_t alloc(T** p, size_t n);
    cudaError_t init(const sgi_nn_config& c);
    cudaError_t set_params(const float* host, size_t n);
    cudaError_t conv_any(int cin, int cout, int mode, const ConvArgs& a, cudaStream_t s);
    cudaError_t conv(int l, const View& x, const View& y, int B, int H, int W, cudaStream_t s,
                     const View* pool = nullptr);
    cudaError_t forward(const __nv_bfloat16* feat, int B, int H, int W, cudaStream_t s, bool allow_fp8 = true);
    cudaError_t forward_fp8(const __nv_bfloat16* feat, int B, int H, int W, cudaStream_t s);
    cudaError_t conv8(int l, const View& x, const View& y, int B, int H, int W, cudaStream_t s, bool in8, bool out8,
                      const View* pool = nullptr);
    cudaError_t calibrate_fp8(const __nv_bfloat16* feat, int B, int H, int W, cudaStream_t s);
    cudaError_t layer_backward(int l, const View& x, const View& y, const View& dy, __nv_bfloat16* dz_buf,
                               const View& dx, int B, int H, int W, cudaStream_t s);
    cudaError_t backward(const __nv_bfloat16* feat, int B, int H, int W, cudaStream_t s);
};

}  // namespace nn
}  // namespace sgi

struct sgi_nn {
    sgi::nn::Net net;
    std::string err;
    int step = 0;
};

// The two halves of sgi_nn_forward for one image (B = 1), for the frame path:
// the U-Net, then the kernel apply with the frame's composite fused into it
// (the HDR frame, the GI history and the history length are written instead
// of the denoised GI; see composite_px in sgi_nn.cu). The noisy GI is read from the
// RGBA16F pass-0 output the features were built from.
sgi_status nn_forward_net(sgi_nn* n, const void* features, int H, int W, cudaStream_t s);
// The network's forward with the kernel apply and composite fused into the head (tcgen05 path), or the
// forward followed by the apply kernel (other paths); `before_head` (nullable) is waited for before the
// first kernel that reads `screen`.
sgi_status nn_forward_composite(sgi_nn* n, const void* features, int H, int W, const uint2* noisy, const float* prev,
                                const uint2* screen, const uint32_t* albedo, uint2* hdr, uint2* gi_out,
                                uint16_t* hist_out, cudaEvent_t before_head, cudaStream_t s);
sgi_status nn_apply_composite(sgi_nn* n, const uint2* noisy, const float* prev, int H, int W, const uint2* screen,
                              const uint32_t* albedo, uint2* hdr, uint2* gi_out, uint16_t* hist_out, cudaStream_t s);
