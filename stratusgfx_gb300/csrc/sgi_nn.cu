// sgi_nn.cu - kernels of the learned kernel-predicting denoiser (KPCNN).
//
// No counterpart in StratusGFX: it stands in for the a-trous filter of
// vpl_pbr_gi_denoise.fs. Activations and gradients BF16, accumulation FP32,
// master weights FP32. Tensors are strided views (View in sgi_nn_internal.h:
// NHWC or channel-group planar), so skip connections are written straight into
// channel slices of the decoder inputs and no concatenation is copied.
//
// 3x3 convolutions are implicit GEMMs on the tensor cores: a block computes an
// 8 x 16 pixel tile for all output channels; the (8+2) x (16+2) input halo and
// the weights of one input-channel chunk are staged in shared memory, and each
// warp issues mma.m16n8k16 (BF16 in, FP32 accumulate) over its 16-pixel row
// with A/B fragments loaded by ldmatrix.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sgi_nn_apply.cuh"
#include "sgi_nn_internal.h"

namespace sgi {
namespace nn {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldmatrix_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

constexpr int kTileH = 8, kTileW = 16;
constexpr int kHaloH = kTileH + 2, kHaloW = kTileW + 2;

// ------------------------------------------------------------ conv 3x3 --
// y[b, p, co] = act(bias[co] + sum_{tap, ci} w[co][tap][ci] * x[b, p + off(tap), ci]), zero padding.
// MODE 0: bias + ReLU, 1: bias only, 2: neither (dgrad).
template <int CIN, int COUT, int CK, int MODE>
__global__ void __launch_bounds__(256) conv3x3_kernel(ConvArgs a) {
    static_assert(CIN % CK == 0 && (CK == 16 || CK == 32) && COUT % 16 == 0, "shape");
    constexpr int HP = CK + 8;            // padded channel pitch of the halo (bank-conflict free ldmatrix)
    constexpr int WP = 9 * HP;            // padded pitch of one output channel's weights
    constexpr int NT = COUT / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16* halo = reinterpret_cast<bf16*>(smem_raw);
    bf16* wsm = halo + kHaloH * kHaloW * HP;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int x0 = blockIdx.x * kTileW, y0 = blockIdx.y * kTileH, b = blockIdx.z;
    const int H = a.H, W = a.W;

    float acc[NT][4];
#pragma unroll
    for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;

    for (int c0 = 0; c0 < CIN; c0 += CK) {
        __syncthreads();
        // input halo: (kHaloH x kHaloW) pixels x CK channels, 16-byte vectors
        constexpr int VPP = CK / 8;
        for (int v = tid; v < kHaloH * kHaloW * VPP; v += 256) {
            const int pix = v / VPP, q = v % VPP;
            const int hy = pix / kHaloW, hx = pix % kHaloW;
            const int gy = y0 + hy - 1, gx = x0 + hx - 1;
            uint4 val = make_uint4(0u, 0u, 0u, 0u);
            if (gy >= 0 && gy < H && gx >= 0 && gx < W)
                val = *reinterpret_cast<const uint4*>(a.x.p + a.x.at(b, (size_t)gy * W + gx, c0 / 8 + q));
            *reinterpret_cast<uint4*>(halo + pix * HP + q * 8) = val;
        }
        // weights of this channel chunk: [COUT][9][CK]
        for (int v = tid; v < COUT * 9 * VPP; v += 256) {
            const int co = v / (9 * VPP), r = v % (9 * VPP);
            const int tap = r / VPP, q = r % VPP;
            *reinterpret_cast<uint4*>(wsm + co * WP + tap * HP + q * 8) =
                *reinterpret_cast<const uint4*>(a.w + ((size_t)co * 9 + tap) * CIN + c0 + q * 8);
        }
        __syncthreads();
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int ky = tap / 3, kx = tap % 3;
#pragma unroll
            for (int kk = 0; kk < CK; kk += 16) {
                uint32_t a0, a1, a2, a3;
                const int prow = lane & 15, kcol = (lane >> 4) * 8;
                ldmatrix_x4(smem_addr(halo + ((warp + ky) * kHaloW + prow + kx) * HP + kk + kcol), a0, a1, a2, a3);
#pragma unroll
                for (int n = 0; n < NT; n += 2) {
                    const int m = lane >> 3;
                    const int co = (n + (m >> 1)) * 8 + (lane & 7);
                    uint32_t b0, b1, b2, b3;
                    ldmatrix_x4(smem_addr(wsm + co * WP + tap * HP + kk + (m & 1) * 8), b0, b1, b2, b3);
                    mma_bf16(acc[n], a0, a1, a2, a3, b0, b1);
                    mma_bf16(acc[n + 1], a0, a1, a2, a3, b2, b3);
                }
            }
        }
    }
    // epilogue: rows = pixels (lane >> 2, +8), columns = channels ((lane & 3) * 2, +1)
    const int gy = y0 + warp;
    if (gy >= H) return;
#pragma unroll
    for (int n = 0; n < NT; ++n) {
        const int co = n * 8 + (lane & 3) * 2;
        float bias0 = 0.0f, bias1 = 0.0f;
        if (MODE != 2) { bias0 = a.bias[co]; bias1 = a.bias[co + 1]; }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int gx = x0 + (lane >> 2) + h * 8;
            if (gx >= W) continue;
            float v0 = acc[n][2 * h] + bias0, v1 = acc[n][2 * h + 1] + bias1;
            if (MODE == 0) { v0 = fmaxf(v0, 0.0f); v1 = fmaxf(v1, 0.0f); }
            *reinterpret_cast<__nv_bfloat162*>(a.y.p + a.y.at(b, (size_t)gy * W + gx, co / 8) + co % 8) =
                __floats2bfloat162_rn(v0, v1);
        }
    }
}

template <int CIN, int COUT, int CK, int MODE>
static cudaError_t run_conv(const ConvArgs& a, cudaStream_t s) {
    constexpr int HP = CK + 8;
    const size_t smem = (size_t)(kHaloH * kHaloW * HP + COUT * 9 * HP) * sizeof(bf16);
    auto kern = conv3x3_kernel<CIN, COUT, CK, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((a.W + kTileW - 1) / kTileW, (a.H + kTileH - 1) / kTileH, a.B);
    kern<<<grid, 256, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t conv3x3(int cin, int cout, int mode, const ConvArgs& a, cudaStream_t s) {
    if (!view_ok(a.x) || !view_ok(a.y) || ((uintptr_t)a.w & 15)) return cudaErrorInvalidValue;
#define SGI_CONV_CASE(CI, CO, CKK)                                           \
    if (cin == CI && cout == CO) {                                           \
        if (mode == 0) return run_conv<CI, CO, CKK, 0>(a, s);                \
        if (mode == 1) return run_conv<CI, CO, CKK, 1>(a, s);                \
        return run_conv<CI, CO, CKK, 2>(a, s);                               \
    }
    SGI_CONV_CASE(16, 32, 16)
    SGI_CONV_CASE(32, 32, 32)
    SGI_CONV_CASE(32, 64, 32)
    SGI_CONV_CASE(64, 64, 32)
    SGI_CONV_CASE(64, 128, 32)
    SGI_CONV_CASE(128, 128, 32)
    SGI_CONV_CASE(192, 64, 32)
    SGI_CONV_CASE(96, 32, 32)
    SGI_CONV_CASE(64, 32, 32)
    SGI_CONV_CASE(128, 64, 32)
    SGI_CONV_CASE(64, 192, 32)
    SGI_CONV_CASE(32, 96, 32)
#undef SGI_CONV_CASE
    return cudaErrorInvalidValue;
}

// dgrad weights: wt[ci][tap][co] = w[co][8 - tap][ci]
__global__ void flip_weights_kernel(const bf16* __restrict__ w, bf16* __restrict__ wt, int cin, int cout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cin * 9 * cout) return;
    const int ci = i / (9 * cout), r = i % (9 * cout), tap = r / cout, co = r % cout;
    wt[i] = w[((size_t)co * 9 + (8 - tap)) * cin + ci];
}

cudaError_t flip_weights(const bf16* w, bf16* wt, int cin, int cout, cudaStream_t s) {
    const int n = cin * 9 * cout;
    flip_weights_kernel<<<(n + 255) / 256, 256, 0, s>>>(w, wt, cin, cout);
    return cudaGetLastError();
}

// ---------------------------------------------------- elementwise / resampling --
// These kernels move 8 channels (one 16-byte vector) per thread. The thread
// index runs over (image, pixel, channel group) with the group fastest for NHWC
// views (a warp covers whole pixels) and over (image, channel group, pixel)
// with the pixel fastest for planar views (a warp covers one group's run).
__device__ __forceinline__ void bf8_to_f(const uint4& v, float* f) {
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
    for (int j = 0; j < 4; ++j) { float2 t = __bfloat1622float2(h[j]); f[2 * j] = t.x; f[2 * j + 1] = t.y; }
}
__device__ __forceinline__ uint4 f_to_bf8(const float* f) {
    uint4 v;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&v);
#pragma unroll
    for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
    return v;
}
__device__ __forceinline__ uint4& vec8(const View& v, int b, size_t q, int g) {
    return *reinterpret_cast<uint4*>(v.p + v.at(b, q, g));
}

// thread index i -> (pixel q of npix, group g of g8, image b)
template <bool PIXFAST>
__device__ __forceinline__ void split_index(unsigned i, unsigned npix, int g8, unsigned& q, int& g, int& b) {
    if (PIXFAST) {
        q = i % npix;
        const unsigned bg = i / npix;
        g = (int)(bg % g8);
        b = (int)(bg / g8);
    } else {
        g = (int)(i % g8);
        const unsigned qb = i / g8;
        q = qb % npix;
        b = (int)(qb / npix);
    }
}

// dz = dy * (y > 0)
template <bool PIXFAST>
__global__ void relu_bwd_kernel(View dy, View y, View dz, int B, int HW, int g8) {
    const unsigned n = (unsigned)B * HW * g8;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned pix;
    int g, b;
    split_index<PIXFAST>(i, (unsigned)HW, g8, pix, g, b);
    const uint4 yv = vec8(y, b, pix, g), dv = vec8(dy, b, pix, g);
    const __nv_bfloat162* yh = reinterpret_cast<const __nv_bfloat162*>(&yv);
    const __nv_bfloat162* dh = reinterpret_cast<const __nv_bfloat162*>(&dv);
    uint4 o;
    __nv_bfloat162* oh = reinterpret_cast<__nv_bfloat162*>(&o);
    const __nv_bfloat162 zero = __floats2bfloat162_rn(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float2 yf = __bfloat1622float2(yh[j]);
        oh[j] = __halves2bfloat162(yf.x > 0.0f ? dh[j].x : zero.x, yf.y > 0.0f ? dh[j].y : zero.y);
    }
    vec8(dz, b, pix, g) = o;
}

// 2x2 average pooling (H, W even): out[b, y, x] = mean of in[b, 2y.., 2x..]
template <bool PIXFAST>
__global__ void pool_fwd_kernel(View in, View out, int B, int H, int W, int g8) {
    const int Ho = H / 2, Wo = W / 2;
    const unsigned n = (unsigned)B * Ho * Wo * g8;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned q;
    int g, b;
    split_index<PIXFAST>(i, (unsigned)Ho * Wo, g8, q, g, b);
    const int xo = (int)(q % Wo), yo = (int)(q / Wo);
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0}, f[8];
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            bf8_to_f(vec8(in, b, (size_t)(2 * yo + dy) * W + 2 * xo + dx, g), f);
#pragma unroll
            for (int j = 0; j < 8; ++j) s[j] += f[j];
        }
#pragma unroll
    for (int j = 0; j < 8; ++j) s[j] *= 0.25f;
    vec8(out, b, (size_t)yo * Wo + xo, g) = f_to_bf8(s);
}

// din[b, y, x] (+)= 0.25 * dout[b, y/2, x/2]
template <bool PIXFAST>
__global__ void pool_bwd_kernel(View dout, View din, int B, int H, int W, int g8, int accumulate) {
    const unsigned n = (unsigned)B * H * W * g8;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned q;
    int g, b;
    split_index<PIXFAST>(i, (unsigned)H * W, g8, q, g, b);
    const int x = (int)(q % W), y = (int)(q / W);
    const int Wo = W / 2;
    float v[8], d[8];
    bf8_to_f(vec8(dout, b, (size_t)(y / 2) * Wo + x / 2, g), v);
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] *= 0.25f;
    uint4& dp = vec8(din, b, (size_t)y * W + x, g);
    if (accumulate) {
        bf8_to_f(dp, d);
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] += d[j];
    }
    dp = f_to_bf8(v);
}

// nearest 2x upsampling: out[b, y, x] = in[b, y/2, x/2]
template <bool PIXFAST>
__global__ void up_fwd_kernel(View in, View out, int B, int H, int W, int g8) {
    pdl_wait();
    pdl_trigger();
    const unsigned n = (unsigned)B * H * W * g8;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned q;
    int g, b;
    split_index<PIXFAST>(i, (unsigned)H * W, g8, q, g, b);
    const int x = (int)(q % W), y = (int)(q / W);
    vec8(out, b, (size_t)y * W + x, g) = vec8(in, b, (size_t)(y / 2) * (W / 2) + x / 2, g);
}

// The same for even H and W, one thread per input pixel and channel group:
// one 16-byte load, four 16-byte stores (the 2x2 block it is copied to).
template <bool PIXFAST>
__global__ void up2x2_fwd_kernel(View in, View out, int B, int Hi, int Wi, int g8) {
    pdl_wait();
    pdl_trigger();
    const unsigned n = (unsigned)B * Hi * Wi * g8;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned q;
    int g, b;
    split_index<PIXFAST>(i, (unsigned)Hi * Wi, g8, q, g, b);
    const int x = (int)(q % Wi), y = (int)(q / Wi);
    const uint4 v = vec8(in, b, q, g);
    const size_t W = 2 * (size_t)Wi, o = (size_t)(2 * y) * W + 2 * x;
    vec8(out, b, o, g) = v;
    vec8(out, b, o + 1, g) = v;
    vec8(out, b, o + W, g) = v;
    vec8(out, b, o + W + 1, g) = v;
}

// din[b, y, x] = sum of dout over the 2x2 block it was copied to
template <bool PIXFAST>
__global__ void up_bwd_kernel(View dout, View din, int B, int Hi, int Wi, int g8) {
    const unsigned n = (unsigned)B * Hi * Wi * g8;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned q;
    int g, b;
    split_index<PIXFAST>(i, (unsigned)Hi * Wi, g8, q, g, b);
    const int x = (int)(q % Wi), y = (int)(q / Wi);
    const int W = Wi * 2;
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0}, f[8];
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            bf8_to_f(vec8(dout, b, (size_t)(2 * y + dy) * W + 2 * x + dx, g), f);
#pragma unroll
            for (int j = 0; j < 8; ++j) s[j] += f[j];
        }
    vec8(din, b, (size_t)y * Wi + x, g) = f_to_bf8(s);
}

static unsigned blocks_for(size_t n) { return (unsigned)((n + 255) / 256); }
static bool launch_ok(size_t n, int c) { return c % 8 == 0 && n <= 0xffffff00u; }   // 32-bit thread indices

cudaError_t relu_bwd(const View& dy, const View& y, const View& dz, int c, int B, int H, int W, cudaStream_t s) {
    const size_t n = (size_t)B * H * W * (c / 8);
    if (!view_ok(dy) || !view_ok(y) || !view_ok(dz) || !launch_ok(n, c)) return cudaErrorInvalidValue;
    if (n == 0) return cudaSuccess;
    if (dz.grp == 8) relu_bwd_kernel<false><<<blocks_for(n), 256, 0, s>>>(dy, y, dz, B, H * W, c / 8);
    else relu_bwd_kernel<true><<<blocks_for(n), 256, 0, s>>>(dy, y, dz, B, H * W, c / 8);
    return cudaGetLastError();
}
cudaError_t pool_fwd(const View& in, const View& out, int B, int H, int W, int c, cudaStream_t s) {
    const size_t n = (size_t)B * (H / 2) * (W / 2) * (c / 8);
    if (!view_ok(in) || !view_ok(out) || !launch_ok(n, c)) return cudaErrorInvalidValue;
    if (n == 0) return cudaSuccess;
    if (out.grp == 8) pool_fwd_kernel<false><<<blocks_for(n), 256, 0, s>>>(in, out, B, H, W, c / 8);
    else pool_fwd_kernel<true><<<blocks_for(n), 256, 0, s>>>(in, out, B, H, W, c / 8);
    return cudaGetLastError();
}
cudaError_t pool_bwd(const View& dout, const View& din, int B, int H, int W, int c, int acc, cudaStream_t s) {
    const size_t n = (size_t)B * H * W * (c / 8);
    if (!view_ok(dout) || !view_ok(din) || !launch_ok(n, c)) return cudaErrorInvalidValue;
    if (n == 0) return cudaSuccess;
    if (din.grp == 8) pool_bwd_kernel<false><<<blocks_for(n), 256, 0, s>>>(dout, din, B, H, W, c / 8, acc);
    else pool_bwd_kernel<true><<<blocks_for(n), 256, 0, s>>>(dout, din, B, H, W, c / 8, acc);
    return cudaGetLastError();
}
cudaError_t up_fwd(const View& in, const View& out, int B, int H, int W, int c, cudaStream_t s) {
    const size_t n = (size_t)B * H * W * (c / 8);
    if (!view_ok(in) || !view_ok(out) || !launch_ok(n, c)) return cudaErrorInvalidValue;
    if (n == 0) return cudaSuccess;
    if (H % 2 == 0 && W % 2 == 0) {
        const size_t ni = n / 4;
        if (out.grp == 8)
            return launch_pdl(up2x2_fwd_kernel<false>, dim3(blocks_for(ni)), dim3(256), 0, s, in, out, B, H / 2, W / 2, c / 8);
        return launch_pdl(up2x2_fwd_kernel<true>, dim3(blocks_for(ni)), dim3(256), 0, s, in, out, B, H / 2, W / 2, c / 8);
    }
    if (out.grp == 8) return launch_pdl(up_fwd_kernel<false>, dim3(blocks_for(n)), dim3(256), 0, s, in, out, B, H, W, c / 8);
    return launch_pdl(up_fwd_kernel<true>, dim3(blocks_for(n)), dim3(256), 0, s, in, out, B, H, W, c / 8);
}
cudaError_t up_bwd(const View& dout, const View& din, int B, int Hi, int Wi, int c, cudaStream_t s) {
    const size_t n = (size_t)B * Hi * Wi * (c / 8);
    if (!view_ok(dout) || !view_ok(din) || !launch_ok(n, c)) return cudaErrorInvalidValue;
    if (n == 0) return cudaSuccess;
    if (din.grp == 8) up_bwd_kernel<false><<<blocks_for(n), 256, 0, s>>>(dout, din, B, Hi, Wi, c / 8);
    else up_bwd_kernel<true><<<blocks_for(n), 256, 0, s>>>(dout, din, B, Hi, Wi, c / 8);
    return cudaGetLastError();
}

// --------------------------------------------------------- kernel apply --
// logits [B, H, W, 32] (0..24: 5x5 kernel, 25: temporal blend), noisy / prev
// [B, H, W, 4] float (rgb used). out = a * sum_k softmax(l)_k noisy(p + o_k) + (1 - a) * prev,
// a = sigmoid(l25); neighbours clamped to the image. With a target, also the
// loss sum of |log1p(out) - log1p(target)| and dlogits = d(mean loss)/dlogits.
constexpr int kApplyTX = 32, kApplyTY = 8;
template <bool TRAIN>
__global__ void __launch_bounds__(256) kpcn_apply_kernel(ApplyArgs a) {
    // the block's 32 x 8 pixels of `noisy` with a 2-pixel edge-clamped border
    __shared__ float4 tile[kApplyTY + 4][kApplyTX + 4];
    __shared__ float red[8];
    pdl_wait();
    pdl_trigger();
    const int tx = threadIdx.x % kApplyTX, ty = threadIdx.x / kApplyTX;
    const int x0 = blockIdx.x * kApplyTX, y0 = blockIdx.y * kApplyTY, b = blockIdx.z;
    const int H = a.H, W = a.W;
    const float4* nz = a.noisy + (size_t)b * H * W;
    for (int v = threadIdx.x; v < (kApplyTY + 4) * (kApplyTX + 4); v += 256) {
        const int hy = v / (kApplyTX + 4), hx = v % (kApplyTX + 4);
        const int yy = min(max(y0 + hy - 2, 0), H - 1), xx = min(max(x0 + hx - 2, 0), W - 1);
        const size_t t = (size_t)yy * W + xx;
        if (a.noisy_h) {   // the same values as the float4 copy the feature pass can write
            tile[hy][hx] = rgba16_to_f4(a.noisy_h[(size_t)b * H * W + t]);
        } else {
            tile[hy][hx] = nz[t];
        }
    }
    __syncthreads();
    const int x = x0 + tx, y = y0 + ty;
    float loss = 0.0f;
    if (x < W && y < H) {
        const size_t q = (size_t)y * W + x, i = (size_t)b * H * W + q;
        float lf[32];
#pragma unroll
        for (int g = 0; g < 4; ++g) bf8_to_f(vec8(a.logits, b, q, g), lf + 8 * g);
        float l[25], sp[3], alpha, o[3];
        const float4 pv = a.prev[i];
        const float pr[3] = {pv.x, pv.y, pv.z};
        kpcn_apply_px(lf, [&](int k) { return tile[ty + k / 5][tx + k % 5]; }, pr, l, sp, alpha, o);
        if (!TRAIN) {
            if (a.hdr) composite_px(o[0], o[1], o[2], a.screen, a.albedo, a.hdr, a.gi_out, a.hist_out, i);
            else a.out[i] = make_float4(o[0], o[1], o[2], 1.0f);
        }
        if (TRAIN) {
            const float4 tv = a.target[i];
            const float t[3] = {tv.x, tv.y, tv.z};
            float dout[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float oc = fmaxf(o[c], 0.0f);
                const float d = log1pf(oc) - log1pf(fmaxf(t[c], 0.0f));
                loss += fabsf(d);
                const float g = (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f)) / (1.0f + oc) * a.grad_scale;
                dout[c] = o[c] > 0.0f ? g : 0.0f;
            }
            float dalpha = 0.0f;
#pragma unroll
            for (int c = 0; c < 3; ++c) dalpha += dout[c] * (sp[c] - pr[c]);
            float dw[25];
            float dot_wdw = 0.0f;
#pragma unroll
            for (int k = 0; k < 25; ++k) {
                const float4 nv = tile[ty + k / 5][tx + k % 5];
                dw[k] = alpha * (dout[0] * nv.x + dout[1] * nv.y + dout[2] * nv.z);
                dot_wdw += l[k] * dw[k];
            }
            float dl[32];
#pragma unroll
            for (int k = 0; k < 25; ++k) dl[k] = l[k] * (dw[k] - dot_wdw);
            dl[25] = dalpha * alpha * (1.0f - alpha);
#pragma unroll
            for (int k = 26; k < 32; ++k) dl[k] = 0.0f;
#pragma unroll
            for (int g = 0; g < 4; ++g) vec8(a.dlogits, b, q, g) = f_to_bf8(dl + 8 * g);
        }
    }
    if (TRAIN) {
        // block reduction of the loss: warp butterfly, then the 8 warp sums
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loss;
        __syncthreads();
        if (threadIdx.x == 0) {
            float t = 0.0f;
            for (int w = 0; w < 8; ++w) t += red[w];
            a.loss_part[blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z)] = t;
        }
    }
}

// *out = the n values of part summed in a fixed order (one block: strided
// partial sums per thread, then a tree over the 256 threads)
__global__ void sum_ordered_kernel(const float* __restrict__ part, size_t n, float* __restrict__ out) {
    __shared__ float red[256];
    float s = 0.0f;
    for (size_t i = threadIdx.x; i < n; i += 256) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

size_t apply_loss_blocks(int B, int H, int W) {
    return (size_t)((W + kApplyTX - 1) / kApplyTX) * ((H + kApplyTY - 1) / kApplyTY) * B;
}

cudaError_t kpcn_apply(const ApplyArgs& a, cudaStream_t s) {
    if (!view_ok(a.logits) || (a.target && !view_ok(a.dlogits))) return cudaErrorInvalidValue;
    if (a.B < 1 || a.H < 1 || a.W < 1 || a.B > 65535) return cudaErrorInvalidValue;
    if ((!a.noisy && !a.noisy_h) || !a.prev || (a.target && a.noisy_h)) return cudaErrorInvalidValue;
    dim3 grid((a.W + kApplyTX - 1) / kApplyTX, (a.H + kApplyTY - 1) / kApplyTY, a.B);
    if (a.target) {
        if (!a.loss || !a.loss_part || !a.target) return cudaErrorInvalidValue;
        cudaError_t e = launch_pdl(kpcn_apply_kernel<true>, grid, dim3(256), 0, s, a);
        if (e != cudaSuccess) return e;
        sum_ordered_kernel<<<1, 256, 0, s>>>(a.loss_part, apply_loss_blocks(a.B, a.H, a.W), a.loss);
        return cudaGetLastError();
    }
    const bool composite = a.hdr && a.screen && a.albedo && a.gi_out && a.hist_out && a.B == 1;
    if (!a.out && !composite) return cudaErrorInvalidValue;
    return launch_pdl(kpcn_apply_kernel<false>, grid, dim3(256), 0, s, a);
}

// ------------------------------------------------------------------ Adam --
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, bf16* __restrict__ wb, size_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

cudaError_t adam(float* w, const float* g, float* m, float* v, bf16* wb, size_t n, float lr, float b1, float b2,
                 float eps, int step, cudaStream_t s) {
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w, g, m, v, wb, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

__global__ void to_bf16_kernel(const float* __restrict__ w, bf16* __restrict__ wb, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16(w[i]);
}

// ------------------------------------------------------------- FP8 E4M3 --
// Per-channel |x| maxima of a BF16 view (calibration): out[c] = max over images
// and pixels (out must start at zero; non-negative floats order as their bits).
__global__ void channel_absmax_kernel(View v, int C, int B, int HW, float* __restrict__ out) {
    const int c = blockIdx.y * 32 + (threadIdx.x & 31);
    float m = 0.0f;
    if (c < C) {
        const size_t pixels = (size_t)B * HW;
        for (size_t p = (size_t)blockIdx.x * 8 + (threadIdx.x >> 5); p < pixels; p += (size_t)gridDim.x * 8) {
            const int b = (int)(p / HW);
            m = fmaxf(m, fabsf(__bfloat162float(v.p[v.at(b, p - (size_t)b * HW, c / 8) + c % 8])));
        }
        atomicMax(reinterpret_cast<unsigned int*>(out + c), __float_as_uint(m));
    }
}

cudaError_t channel_absmax(const View& v, int C, int B, int H, int W, float* out, cudaStream_t s) {
    if (!view_ok(v)) return cudaErrorInvalidValue;
    dim3 grid(128, (C + 31) / 32);
    channel_absmax_kernel<<<grid, 256, 0, s>>>(v, C, B, H * W, out);
    return cudaGetLastError();
}

// Weight quantization of one layer, one block per output channel n:
// w'[t][k] = w[n][t][k] * s_in[k]; scale[n] = max |w'| / 448; q = E4M3(w' / scale[n]).
__global__ void quantize_weights_kernel(const float* __restrict__ w, const float* __restrict__ s_in, int cin,
                                        uint8_t* __restrict__ q, float* __restrict__ scale) {
    __shared__ float red[256];
    const int n = blockIdx.x, K = 9 * cin;
    const float* wn = w + (size_t)n * K;
    float m = 0.0f;
    for (int i = threadIdx.x; i < K; i += blockDim.x) m = fmaxf(m, fabsf(wn[i] * s_in[i % cin]));
    red[threadIdx.x] = m;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + st]);
        __syncthreads();
    }
    const float sc = red[0] > 0.0f ? red[0] / 448.0f : 1.0f;
    if (threadIdx.x == 0) scale[n] = sc;
    const float inv = 1.0f / sc;
    for (int i = threadIdx.x; i < K; i += blockDim.x)
        q[(size_t)n * K + i] =
            (uint8_t)__nv_cvt_float_to_fp8(wn[i] * s_in[i % cin] * inv, __NV_SATFINITE, __NV_E4M3);
}

cudaError_t quantize_weights(const float* w, const float* s_in, int cin, int cout, uint8_t* q, float* scale,
                             cudaStream_t s) {
    quantize_weights_kernel<<<cout, 256, 0, s>>>(w, s_in, cin, q, scale);
    return cudaGetLastError();
}

// BF16 NHWC tensor (C channels, C % 16 == 0) -> E4M3 with per-channel inverse scales;
// the output is described by a BF16-unit view (two channels per unit).
__global__ void quantize_act_kernel(View in, View out, int C, int B, int HW, const float* __restrict__ inv) {
    const unsigned n = (unsigned)B * HW * (C / 16);
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int g = (int)(i % (C / 16));
    const unsigned q = i / (C / 16);
    const int b = (int)(q / HW);
    const size_t pix = q - (size_t)b * HW;
    float f[16];
    bf8_to_f(*reinterpret_cast<const uint4*>(in.p + in.at(b, pix, 2 * g)), f);
    bf8_to_f(*reinterpret_cast<const uint4*>(in.p + in.at(b, pix, 2 * g + 1)), f + 8);
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = 16 * g + 4 * j;
        const __nv_fp8x2_storage_t lo =
            __nv_cvt_float2_to_fp8x2(make_float2(f[4 * j] * inv[c], f[4 * j + 1] * inv[c + 1]), __NV_SATFINITE, __NV_E4M3);
        const __nv_fp8x2_storage_t hi = __nv_cvt_float2_to_fp8x2(
            make_float2(f[4 * j + 2] * inv[c + 2], f[4 * j + 3] * inv[c + 3]), __NV_SATFINITE, __NV_E4M3);
        w[j] = (uint32_t)lo | ((uint32_t)hi << 16);
    }
    *reinterpret_cast<uint4*>(out.p + out.at(b, pix, g)) = make_uint4(w[0], w[1], w[2], w[3]);
}

cudaError_t quantize_act(const View& in, const View& out, int C, int B, int H, int W, const float* inv,
                         cudaStream_t s) {
    const size_t n = (size_t)B * H * W * (C / 16);
    if (!view_ok(in) || !view_ok(out) || C % 16 || n > 0xffffff00u) return cudaErrorInvalidValue;
    if (n == 0) return cudaSuccess;
    quantize_act_kernel<<<blocks_for(n), 256, 0, s>>>(in, out, C, B, H * W, inv);
    return cudaGetLastError();
}

cudaError_t to_bf16(const float* w, bf16* wb, size_t n, cudaStream_t s) {
    to_bf16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w, wb, n);
    return cudaGetLastError();
}

// ------------------------------------------------------- frame features --
__device__ __forceinline__ float h2f_nn(uint32_t bits16) { return __half2float(__ushort_as_half((unsigned short)bits16)); }
__device__ __forceinline__ float4 unpack4(uint2 t) {
    return make_float4(h2f_nn(t.x & 0xffffu), h2f_nn(t.x >> 16), h2f_nn(t.y & 0xffffu), h2f_nn(t.y >> 16));
}
__device__ __forceinline__ float lum(float4 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// log(1 + max(x, 0)) to the precision of a BF16 feature: the fast natural
// logarithm of 1 + x (the features are stored in BF16, 8 significant bits).
__device__ __forceinline__ float log1p_bf(float x) { return __logf(1.0f + fmaxf(x, 0.0f)); }
constexpr float k255 = 1.0f / 255.0f;

__global__ void __launch_bounds__(256) features_kernel(FeatureArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = a.W, H = a.H;
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    const float4 nz = unpack4(a.merged[i]);
    // 3x3 luminance variance of the noisy estimate
    float s1 = 0.0f, s2 = 0.0f;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            const int xx = min(max(x + dx, 0), W - 1), yy = min(max(y + dy, 0), H - 1);
            const float l = lum(unpack4(a.merged[(size_t)yy * W + xx]));
            s1 += l; s2 += l * l;
        }
    const float mean = s1 * (1.0f / 9.0f);
    const float var = fmaxf(s2 * (1.0f / 9.0f) - mean * mean, 0.0f);
    const float4 g = a.guide[i];
    const uint32_t alb = a.albedo[i], rma = a.rma[i];
    // view distance from the unprojected depth
    const float u = (x + 0.5f) * a.inv_w, v = (y + 0.5f) * a.inv_h;
    const float* m = a.inv_pv;
    const float nx = u * 2.0f - 1.0f, ny = v * 2.0f - 1.0f, nzc = g.w * 2.0f - 1.0f;
    const float wx = m[0] * nx + m[4] * ny + m[8] * nzc + m[12];
    const float wy = m[1] * nx + m[5] * ny + m[9] * nzc + m[13];
    const float wz = m[2] * nx + m[6] * ny + m[10] * nzc + m[14];
    const float ww = m[3] * nx + m[7] * ny + m[11] * nzc + m[15];
    const float rw = __frcp_rn(ww);
    const float px = wx * rw - a.cam_pos[0], py = wy * rw - a.cam_pos[1], pz = wz * rw - a.cam_pos[2];
    const float dist = sqrtf(px * px + py * py + pz * pz);
    // previous output warped by the velocity (bilinear, clamped)
    const uint32_t vel = a.velocity[i];
    const float pu = (u - h2f_nn(vel & 0xffffu)) * W - 0.5f, pv = (v - h2f_nn(vel >> 16)) * H - 0.5f;
    const float fu = floorf(pu), fv = floorf(pv);
    const float au = pu - fu, av = pv - fv;
    const int i0 = min(max((int)fu, 0), W - 1), i1 = min(max((int)fu + 1, 0), W - 1);
    const int j0 = min(max((int)fv, 0), H - 1), j1 = min(max((int)fv + 1, 0), H - 1);
    const float4 p00 = unpack4(a.gi_prev[(size_t)j0 * W + i0]), p10 = unpack4(a.gi_prev[(size_t)j0 * W + i1]);
    const float4 p01 = unpack4(a.gi_prev[(size_t)j1 * W + i0]), p11 = unpack4(a.gi_prev[(size_t)j1 * W + i1]);
    const float w00 = (1 - au) * (1 - av), w10 = au * (1 - av), w01 = (1 - au) * av, w11 = au * av;
    float4 pr;
    pr.x = p00.x * w00 + p10.x * w10 + p01.x * w01 + p11.x * w11;
    pr.y = p00.y * w00 + p10.y * w10 + p01.y * w01 + p11.y * w11;
    pr.z = p00.z * w00 + p10.z * w10 + p01.z * w01 + p11.z * w11;
    pr.w = 1.0f;
    if (!a.have_history) pr = make_float4(nz.x, nz.y, nz.z, 1.0f);
    if (a.noisy) a.noisy[i] = make_float4(nz.x, nz.y, nz.z, 1.0f);
    a.prev[i] = pr;
    float f[16];
    f[0] = log1p_bf(nz.x); f[1] = log1p_bf(nz.y); f[2] = log1p_bf(nz.z);
    f[3] = fmaxf((alb & 0xffu) * k255, 0.01f); f[4] = fmaxf(((alb >> 8) & 0xffu) * k255, 0.01f);
    f[5] = fmaxf(((alb >> 16) & 0xffu) * k255, 0.01f);
    f[6] = g.x; f[7] = g.y; f[8] = g.z;
    f[9] = dist * 0.1f;
    f[10] = (rma & 0xffu) * k255;
    f[11] = log1p_bf(var);
    f[12] = log1p_bf(pr.x); f[13] = log1p_bf(pr.y); f[14] = log1p_bf(pr.z);
    f[15] = ((rma >> 8) & 0xffu) * k255;
    // the pixel's 32 bytes as two 16-byte stores (a warp then writes whole sectors)
    uint32_t w[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const __nv_bfloat162 b = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
        w[k] = *reinterpret_cast<const uint32_t*>(&b);
    }
    uint4* o = reinterpret_cast<uint4*>(a.features + i * 16);
    o[0] = make_uint4(w[0], w[1], w[2], w[3]);
    o[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

cudaError_t features(const FeatureArgs& a, cudaStream_t s) {
    dim3 block(32, 8), grid((a.W + 31) / 32, (a.H + 7) / 8);
    features_kernel<<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

// hdr = screen + gi * denoised, gi = RGB16F(max(albedo, 0.01) + 1e-5); history <- denoised
}  // namespace nn
}  // namespace sgi
