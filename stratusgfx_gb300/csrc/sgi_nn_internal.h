// sgi_nn_internal.h - launch wrappers of the learned denoiser kernels (sgi_nn.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace sgi {
namespace nn {

// A BF16 activation tensor [B][H][W][C] seen through element strides: element
// (image b, pixel q = y * W + x, channel c) is at
//   p[b * img + q * pix + (c / 8) * grp + c % 8].
// Kernels move 8 channels (16 bytes) at a time, so p is 16-byte aligned and the
// strides are multiples of 8. Two layouts are used:
//   NHWC with channel stride cs: pix = cs, grp = 8, img = H * W * cs;
//   channel-group planar [B][G][H][W][8]: pix = 8, grp = H * W * 8, img = G * H * W * 8,
// where each 8-channel group of an image row is one contiguous run of W * 16
// bytes (the layout the tensor-core convolution's TMA loads fetch best).
// A channel slice (skip connections write into the decoder inputs) is the same
// view with p advanced by c0 / 8 groups.
struct View {
    __nv_bfloat16* p;
    long long pix, grp, img;
    __host__ __device__ size_t at(int b, size_t q, int g) const {
        return (size_t)b * (size_t)img + q * (size_t)pix + (size_t)g * (size_t)grp;
    }
};

inline View nhwc_view(const void* p, int cs, int H, int W) {
    return View{(__nv_bfloat16*)p, cs, 8, (long long)H * W * cs};
}
inline View planar_view(const void* p, int groups, int H, int W) {
    return View{(__nv_bfloat16*)p, 8, (long long)H * W * 8, (long long)groups * H * W * 8};
}
inline View channel_slice(View v, int c0) { v.p += (size_t)(c0 / 8) * (size_t)v.grp; return v; }
inline bool view_ok(const View& v) {
    return v.p && ((uintptr_t)v.p & 15) == 0 && v.pix % 8 == 0 && v.grp % 8 == 0 && v.img % 8 == 0 && v.pix > 0 &&
           v.grp > 0 && v.img > 0;
}

struct ConvArgs {
    View x;
    const __nv_bfloat16* w;   // [cout][9][cin] (dgrad: flipped [cin][9][cout])
    const float* bias;        // [cout], unused in mode 2
    View y;
    int B, H, W;
    // Optional extra output of the tensor-core path (p == nullptr: none): the 2x2
    // mean of y, an H/2 x W/2 view (COUT <= 64).
    View pool;
    // FP8 path (conv3x3_tc_fp8): per-output-channel weight scales (the accumulator
    // is multiplied by them) and, for FP8 outputs, the inverse per-channel scales
    // of the output tensor.
    const float* wscale;
    const float* oinv;
    // Bounded waits of the tensor-core path: the limit of every wait (0 = the
    // default 200 ms) and a test switch that keeps the TMA producer from issuing
    // any copy, so the MMA role's first wait runs out with nothing in flight.
    unsigned long long wait_ns;
    int skip_producer;
    // The head (conv3x3_head_apply): the kernel apply and the composite in the
    // epilogue instead of writing the logits (see ApplyArgs for the buffers).
    struct ApplyFuse {
        const uint2* noisy;       // RGBA16F
        const float4* prev;
        const uint2* screen;      // RGBA16F
        const uint32_t* albedo;   // RGBA8
        uint2* hdr;               // RGBA16F
        uint2* gi_out;            // RGBA16F
        uint16_t* hist_out;       // R16F
    } fuse;
};

struct WgradArgs {
    View x;
    View dz;
    float* dw;                // [cout][9][cin] followed by the bias [cout], accumulated
    int cin, cout;
    int B, H, W;
    float* part;              // split-K partial sums, part_floats floats
    size_t part_floats;
    int* err;                 // set when a bounded wait ran out
    unsigned long long wait_ns;
    int skip_producer;        // test switch: the producers stage nothing
};
// floats of the partial-sum buffer wgrad needs for cin x cout
size_t wgrad_part_floats(int cin, int cout);

struct ApplyArgs {
    View logits;                  // 32 channels
    const float4* noisy;          // [P]
    const float4* prev;           // [P]
    const float4* target;         // [P] or null (inference)
    float4* out;                  // [P] or null
    View dlogits;                 // 32 channels, when target
    float* loss;                  // sum of |log1p(out) - log1p(target)| (device scalar) or null
    float* loss_part;             // per-block sums of the loss, summed into *loss in block order
    float grad_scale;             // 1 / (3 * pixels)
    int B, H, W;
    // inference only: with hdr set, the composite of the GI frame is written
    // instead of `out` (hdr = screen + albedo' * gi, gi_out = gi, hist_out = 1;
    // see composite) - B must be 1
    const uint2* noisy_h = nullptr;   // if set, noisy is read from this RGBA16F image instead
    const uint2* screen = nullptr;
    const uint32_t* albedo = nullptr;
    uint2* hdr = nullptr;
    uint2* gi_out = nullptr;
    uint16_t* hist_out = nullptr;
};

struct FeatureArgs {
    int W, H;
    float inv_w, inv_h;           // 1 / W, 1 / H
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
    float4* noisy;                // or null (not written)
    float4* prev;
};

cudaError_t features(const FeatureArgs& a, cudaStream_t s);
cudaError_t conv3x3(int cin, int cout, int mode, const ConvArgs& a, cudaStream_t s);
// The same convolution on the 5th-generation tensor cores (sgi_nn_tc.cu); *err is
// set to 1 when a bounded wait of a block ran out.
cudaError_t conv3x3_tc(int cin, int cout, int mode, const ConvArgs& a, int* err, cudaStream_t s);
// the 32 -> 32 head in BF16 with the kernel apply and composite of a.fuse in its epilogue (B = 1): the HDR
// frame, GI and history length are written, the logits are not
cudaError_t conv3x3_head_apply(const ConvArgs& a, int* err, cudaStream_t s);
// FP8 E4M3 operands (in8; x, w: one byte per channel, described by BF16-unit views
// with two channels per unit) or BF16 operands (16 -> 32 only), the output E4M3
// (out8) or BF16.
cudaError_t conv3x3_tc_fp8(int cin, int cout, int mode, bool in8, bool out8, const ConvArgs& a, int* err,
                           cudaStream_t s);
cudaError_t flip_weights(const __nv_bfloat16* w, __nv_bfloat16* wt, int cin, int cout, cudaStream_t s);
cudaError_t wgrad(const WgradArgs& a, cudaStream_t s);
// floats of kpcn_apply's loss_part for B x H x W
size_t apply_loss_blocks(int B, int H, int W);
// dz = dy * (y > 0)
cudaError_t relu_bwd(const View& dy, const View& y, const View& dz, int c, int B, int H, int W, cudaStream_t s);
// 2x2 mean pooling of an H x W input
cudaError_t pool_fwd(const View& in, const View& out, int B, int H, int W, int c, cudaStream_t s);
// din (H x W) (+)= 0.25 * dout upsampled
cudaError_t pool_bwd(const View& dout, const View& din, int B, int H, int W, int c, int accumulate, cudaStream_t s);
// nearest 2x upsampling to H x W
cudaError_t up_fwd(const View& in, const View& out, int B, int H, int W, int c, cudaStream_t s);
// din (Hi x Wi) = sum of dout over each 2x2 block
cudaError_t up_bwd(const View& dout, const View& din, int B, int Hi, int Wi, int c, cudaStream_t s);
cudaError_t kpcn_apply(const ApplyArgs& a, cudaStream_t s);
cudaError_t adam(float* w, const float* g, float* m, float* v, __nv_bfloat16* wb, size_t n, float lr, float b1,
                 float b2, float eps, int step, cudaStream_t s);
cudaError_t to_bf16(const float* w, __nv_bfloat16* wb, size_t n, cudaStream_t s);
// FP8 E4M3 support: calibration maxima, weight and activation quantization.
cudaError_t channel_absmax(const View& v, int C, int B, int H, int W, float* out, cudaStream_t s);
cudaError_t quantize_weights(const float* w, const float* s_in, int cin, int cout, uint8_t* q, float* scale,
                             cudaStream_t s);
cudaError_t quantize_act(const View& in, const View& out, int C, int B, int H, int W, const float* inv,
                         cudaStream_t s);

#ifdef __CUDACC__
// Programmatic dependent launch: the kernel may be scheduled while the previous
// kernel of the stream is still finishing. Every kernel launched this way calls
// pdl_wait() before its first global-memory access (which returns once the
// previous kernel has completed and its writes are visible) and pdl_trigger() to
// let the next kernel be scheduled early in turn.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
#endif

}  // namespace nn
}  // namespace sgi
