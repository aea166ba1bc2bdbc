// sgi_stats.cu - FP64 error statistics of a rendered frame against the
// converged target (sgi_gi_error_stats): the reductions behind every PSNR the
// benchmark and the tests report. No counterpart in StratusGFX.
//
// Per pixel, in binary64: the GI weight w = binary16(max(albedo / 255, 0.01) +
// 1e-5) (the gather's colour output, vpl_pbr_gi.fs:204, as the final pass
// reads it), the converged GI term r_gi = w * target, the converged frame
// r = direct + r_gi, and the errors of the frame (hdr - r) and of its GI term
// ((hdr - direct) - r_gi) over the three colour channels. Each block sums its
// pixels' squared errors and takes the maxima, then one block combines the
// blocks' values in block order: the result does not depend on scheduling.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/sgi.h"

namespace sgi {
namespace {

constexpr int kStatBlocks = 304;
constexpr int kStatThreads = 256;
constexpr int kStatFields = 6;   // sse frame, sse gi, peak frame, peak gi, max |err| frame, max |err| gi

__device__ double g_stat_partial[kStatBlocks * kStatFields];
__device__ double g_stat_out[kStatFields];

__device__ __forceinline__ double h2d(uint16_t h) { return (double)__half2float(__ushort_as_half(h)); }

__global__ void __launch_bounds__(kStatThreads) gi_error_partial_kernel(const uint32_t* __restrict__ albedo,
                                                                      const uint2* __restrict__ hdr,
                                                                      const uint2* __restrict__ direct,
                                                                      const float4* __restrict__ target,
                                                                      int64_t pixels) {
    double v[kStatFields] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * kStatThreads + threadIdx.x; i < pixels;
         i += (int64_t)gridDim.x * kStatThreads) {
        const uint32_t a = __ldg(albedo + i);
        const uint2 h = __ldg(hdr + i), d = __ldg(direct + i);
        const float4 t = __ldg(target + i);
        const uint16_t hs[3] = {(uint16_t)(h.x & 0xffffu), (uint16_t)(h.x >> 16), (uint16_t)(h.y & 0xffffu)};
        const uint16_t ds[3] = {(uint16_t)(d.x & 0xffffu), (uint16_t)(d.x >> 16), (uint16_t)(d.y & 0xffffu)};
        const double ts[3] = {(double)t.x, (double)t.y, (double)t.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double alb = (double)((a >> (8 * c)) & 0xffu) / 255.0;
            alb = alb < 0.01 ? 0.01 : alb;
            const double w = (double)__half2float(__double2half(alb + 1e-5));
            const double rgi = w * ts[c];
            const double dir = h2d(ds[c]);
            const double ref = dir + rgi;
            const double got = h2d(hs[c]);
            const double ef = got - ref, eg = (got - dir) - rgi;
            v[0] += ef * ef;
            v[1] += eg * eg;
            v[2] = fmax(v[2], fabs(ref));
            v[3] = fmax(v[3], fabs(rgi));
            v[4] = fmax(v[4], fabs(ef));
            v[5] = fmax(v[5], fabs(eg));
        }
    }
    __shared__ double red[kStatFields][kStatThreads];
#pragma unroll
    for (int f = 0; f < kStatFields; ++f) red[f][threadIdx.x] = v[f];
    __syncthreads();
    for (int w = kStatThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            red[0][threadIdx.x] += red[0][threadIdx.x + w];
            red[1][threadIdx.x] += red[1][threadIdx.x + w];
#pragma unroll
            for (int f = 2; f < kStatFields; ++f) red[f][threadIdx.x] = fmax(red[f][threadIdx.x], red[f][threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x < kStatFields) g_stat_partial[blockIdx.x * kStatFields + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void gi_error_final_kernel() {
    if (threadIdx.x >= kStatFields) return;
    const int f = threadIdx.x;
    double s = 0.0;
    for (int b = 0; b < kStatBlocks; ++b) {
        const double x = g_stat_partial[b * kStatFields + f];
        s = f < 2 ? s + x : fmax(s, x);
    }
    g_stat_out[f] = s;
}

std::mutex g_stat_mutex;   // the partial-sum array is shared by all callers of a device

}  // namespace
}  // namespace sgi

extern "C" sgi_status sgi_gi_error_stats(const sgi_gbuffer* g, const void* hdr, const void* direct, const float* target,
                                         int32_t width, int32_t height, sgi_error_stats* out, void* stream) {
    if (!g || !g->albedo || !hdr || !direct || !target || !out || width < 1 || height < 1) return SGI_ERR_ARG;
    const int64_t pixels = (int64_t)width * height;
    cudaStream_t s = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lock(sgi::g_stat_mutex);
    sgi::gi_error_partial_kernel<<<sgi::kStatBlocks, sgi::kStatThreads, 0, s>>>(
        g->albedo, (const uint2*)hdr, (const uint2*)direct, (const float4*)target, pixels);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        sgi::gi_error_final_kernel<<<1, 32, 0, s>>>();
        e = cudaGetLastError();
    }
    double host[sgi::kStatFields] = {};
    if (e == cudaSuccess) e = cudaMemcpyFromSymbolAsync(host, sgi::g_stat_out, sizeof(host), 0, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return SGI_ERR_CUDA;
    out->sse_frame = host[0];
    out->sse_gi = host[1];
    out->peak_frame = host[2];
    out->peak_gi = host[3];
    out->max_abs_frame = host[4];
    out->max_abs_gi = host[5];
    out->values = pixels * 3;
    return SGI_OK;
}
