// sgi_nn_apply.cuh - the kernel apply of the learned denoiser for one pixel,
// shared by the stand-alone apply kernel (sgi_nn.cu, training and inference)
// and the head convolution whose epilogue applies the kernels directly
// (sgi_nn_tc.cu), so both evaluate the same expressions.
//
// logits 0..24: a 5x5 kernel (softmax), 25: the temporal blend alpha =
// sigmoid(l25); out = alpha * sum_k softmax(l)_k noisy(p + o_k) + (1 - alpha) * prev.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sgi {
namespace nn {

// noisy_at(k): the noisy estimate at offset (k % 5 - 2, k / 5 - 2), clamped to
// the image; pr: prev rgb. Writes the normalised kernel l[25], the filtered sum
// sp[3], alpha and the output o[3].
template <class NoisyAt>
__device__ __forceinline__ void kpcn_apply_px(const float* lf, NoisyAt noisy_at, const float* pr, float* l, float* sp,
                                              float& alpha, float* o) {
    float mx = -3.0e38f;
#pragma unroll
    for (int k = 0; k < 25; ++k) { l[k] = lf[k]; mx = fmaxf(mx, l[k]); }
    float den = 0.0f;
#pragma unroll
    for (int k = 0; k < 25; ++k) { l[k] = __expf(l[k] - mx); den += l[k]; }
    const float inv = 1.0f / den;
    sp[0] = sp[1] = sp[2] = 0.0f;
#pragma unroll
    for (int k = 0; k < 25; ++k) {
        l[k] *= inv;
        const float4 nv = noisy_at(k);
        sp[0] = fmaf(l[k], nv.x, sp[0]); sp[1] = fmaf(l[k], nv.y, sp[1]); sp[2] = fmaf(l[k], nv.z, sp[2]);
    }
    alpha = 1.0f / (1.0f + __expf(-lf[25]));
#pragma unroll
    for (int c = 0; c < 3; ++c) o[c] = alpha * sp[c] + (1.0f - alpha) * pr[c];
}

__device__ __forceinline__ float4 rgba16_to_f4(uint2 h) {
    return make_float4(__half2float(__ushort_as_half((uint16_t)(h.x & 0xffffu))),
                       __half2float(__ushort_as_half((uint16_t)(h.x >> 16))),
                       __half2float(__ushort_as_half((uint16_t)(h.y & 0xffffu))), 1.0f);
}

// The composite of one pixel's denoised GI (d0, d1, d2): the direct lighting
// plus the GI times the gather's colour output (albedo + 1e-5 stored as FP16),
// the GI history and a history length of 1.
__device__ __forceinline__ void composite_px(float d0, float d1, float d2, const uint2* __restrict__ screen,
                                             const uint32_t* __restrict__ albedo, uint2* __restrict__ hdr,
                                             uint2* __restrict__ gi_out, uint16_t* __restrict__ hist_out, size_t i) {
    const uint2 st = screen[i];
    const float sc0 = __half2float(__ushort_as_half((uint16_t)(st.x & 0xffffu)));
    const float sc1 = __half2float(__ushort_as_half((uint16_t)(st.x >> 16)));
    const float sc2 = __half2float(__ushort_as_half((uint16_t)(st.y & 0xffffu)));
    const uint32_t alb = albedo[i];
    const float g0 = __half2float(__float2half_rn(fmaxf((alb & 0xffu) / 255.0f, 0.01f) + 0.00001f));
    const float g1 = __half2float(__float2half_rn(fmaxf(((alb >> 8) & 0xffu) / 255.0f, 0.01f) + 0.00001f));
    const float g2 = __half2float(__float2half_rn(fmaxf(((alb >> 16) & 0xffu) / 255.0f, 0.01f) + 0.00001f));
    auto pack = [](float a0, float a1, float a2, float a3) {
        return make_uint2((uint32_t)__half_as_ushort(__float2half_rn(a0)) |
                              ((uint32_t)__half_as_ushort(__float2half_rn(a1)) << 16),
                          (uint32_t)__half_as_ushort(__float2half_rn(a2)) |
                              ((uint32_t)__half_as_ushort(__float2half_rn(a3)) << 16));
    };
    hdr[i] = pack(sc0 + g0 * d0, sc1 + g1 * d1, sc2 + g2 * d2, 1.0f);
    gi_out[i] = pack(d0, d1, d2, 1.0f);
    hist_out[i] = __half_as_ushort(__float2half_rn(1.0f));
}

}  // namespace nn
}  // namespace sgi
