// sgi_kernels.cu - the exact (bit-reproducible) kernels of the GI/lighting
// hot path on sm_103a that do not have a tolerance variant.
//
// Kernels (reference shader each restates, paths relative to the StratusGFX root):
//   vpl_vis_flags / vpl_compact  viscull_vpls.cs:47-120
//   tile_stage1                  vpl_tiled_deferred_culling_stage1.cs:50-90
//   tile_stage2                  vpl_tiled_deferred_culling_stage2.cs:61-129
//   vpl_color                    vpl_light_color.cs:41-75
//   post_fx                      taa.fs + gammaTonemap.fs
// The shading kernels (gather, denoise, deferred) are in sgi_shade.cu.
//
// Compiled with -fmad=false (see sgi_math.cuh): results are bit-reproducible.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "sgi_cull.cuh"
#include "sgi_internal.h"
#include "sgi_math.cuh"
#include "sgi_shade_common.cuh"

namespace sgi {

// ============================================================== post FX --
// taa.fs with aa_common.glsl's Reinhard tonemap, then gammaTonemap.fs (ACES film
// curve and gamma 2.2): the consumers of the stage's HDR frame
// (PerformTaaPostFx_ / PerformGammaTonemapPostFx_, StratusRendererBackend.cpp:2323-2360).
struct PostFxParams {
    int W, H;
    const uint2* hdr;            // RGBA16F frame
    const uint32_t* velocity;    // RG16F G-buffer velocity
    const uint2* hist_in;        // previous TAA output (RGBA16F), NULL on the first frame
    uint2* hist_out;             // this TAA output (RGBA16F)
    uint32_t* ldr;               // RGBA8 gamma-corrected output
    int taa;
};

SGI_D V3 h4rgb(uint2 t) {
    return v3(h2f((uint16_t)(t.x & 0xffffu)), h2f((uint16_t)(t.x >> 16)), h2f((uint16_t)(t.y & 0xffffu)));
}
SGI_D V3 reinhard(V3 c) { return c / (c + v3s(1.0f)); }
SGI_D V3 inverse_reinhard(V3 c) { return c / (v3s(1.0f) - c); }
SGI_D V3 vmin3(V3 a, V3 b) { return v3(gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)); }
SGI_D V3 vmax3(V3 a, V3 b) { return v3(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)); }
SGI_D float aces_film(float x) {
    return saturate((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f));
}

__global__ void __launch_bounds__(256) post_fx_kernel(PostFxParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.W || y >= p.H) return;
    const int W = p.W, H = p.H;
    const size_t i = (size_t)y * W + x;
    auto at = [&](int xx, int yy) {
        xx = xx < 0 ? 0 : (xx >= W ? W - 1 : xx);
        yy = yy < 0 ? 0 : (yy >= H ? H - 1 : yy);
        return h4rgb(__ldg(p.hdr + (size_t)yy * W + xx));
    };
    V3 outc = at(x, y);
    if (p.taa) {
        const uint32_t vel = __ldg(p.velocity + i);
        const float u = (float(x) + 0.5f) / float(W), v = (float(y) + 0.5f) / float(H);
        const float pu = u - h2f((uint16_t)(vel & 0xffffu)), pv = v - h2f((uint16_t)(vel >> 16));
        V3 currentColor = at(x, y);
        V3 prevColor = currentColor;
        if (p.hist_in) {
            const uint2* hp = p.hist_in;
            auto ch = [&](int ii, int jj, int c) {
                const uint2 t = __ldg(hp + (size_t)jj * W + ii);
                const uint32_t w = c < 2 ? t.x : t.y;
                return h2f((uint16_t)((c & 1) ? (w >> 16) : (w & 0xffffu)));
            };
            prevColor = v3(bilinear([&](int ii, int jj) { return ch(ii, jj, 0); }, W, H, pu, pv),
                           bilinear([&](int ii, int jj) { return ch(ii, jj, 1); }, W, H, pu, pv),
                           bilinear([&](int ii, int jj) { return ch(ii, jj, 2); }, W, H, pu, pv));
        }
        prevColor = reinhard(prevColor);
        const V3 c1 = at(x, y + 1), c2 = at(x, y - 1), c3 = at(x + 1, y), c4 = at(x - 1, y);
        const V3 minColor = reinhard(vmin3(currentColor, vmin3(c1, vmin3(c2, vmin3(c3, c4)))));
        const V3 maxColor = reinhard(vmax3(currentColor, vmax3(c1, vmax3(c2, vmax3(c3, c4)))));
        currentColor = reinhard(currentColor);
        prevColor = vmin3(vmax3(prevColor, minColor), maxColor);
        currentColor = inverse_reinhard(currentColor);
        prevColor = inverse_reinhard(prevColor);
        const V3 m = v3(mixf(currentColor.x, prevColor.x, 0.9f), mixf(currentColor.y, prevColor.y, 0.9f),
                        mixf(currentColor.z, prevColor.z, 0.9f));
        const uint2 h = pack_h4(m.x, m.y, m.z, 0.0625f);
        p.hist_out[i] = h;
        outc = h4rgb(h);   // the RGB16F TAA target is what the tonemap pass reads
    }
    const float inv_gamma = 1.0f / 2.2f;
    const float r = powf(aces_film(outc.x), inv_gamma);
    const float g = powf(aces_film(outc.y), inv_gamma);
    const float b = powf(aces_film(outc.z), inv_gamma);
    auto q = [](float c) { return (uint32_t)(saturate(c) * 255.0f + 0.5f); };
    p.ldr[i] = q(r) | (q(g) << 8) | (q(b) << 16) | 0xff000000u;
}

cudaError_t launch_post_fx(int32_t W, int32_t H, const uint2* hdr, const uint32_t* velocity, const uint2* hist_in,
                           uint2* hist_out, uint32_t* ldr, int32_t taa, cudaStream_t s) {
    PostFxParams p{W, H, hdr, velocity, hist_in, hist_out, ldr, taa};
    dim3 block(32, 8), grid((W + 31) / 32, (H + 7) / 8);
    post_fx_kernel<<<grid, block, 0, s>>>(p);
    return cudaGetLastError();
}

// ========================================================= VPL colouring --
// vpl_light_color.cs:41-75 over the compacted list (count = visible_index[0]).
__global__ void vpl_color_kernel(sgi_vpl* __restrict__ cv, const sgi_atlas_entry* __restrict__ ce,
                                 const int32_t* __restrict__ visible_index, int cap, sgi_cube_atlas cubes,
                                 sgi_diffuse_atlas diffuse, sgi_csm csm) {
    const int n = min(visible_index[0], cap);
    const V3 L = v3(csm.light_direction[0], csm.light_direction[1], csm.light_direction[2]);
    const V3 sun = v3(csm.light_color[0], csm.light_color[1], csm.light_color[2]);
    const V3 dir = v3(-L.x, -L.y, -L.z);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const sgi_atlas_entry e = ce[k];
        sgi_vpl v = cv[k];
        V3 diff = v3s(0.0f);
        if (e.index >= 0 && e.index < diffuse.num_atlases && e.layer >= 0 && e.layer < diffuse.layers_per_atlas) {
            const uint32_t t = __ldg((const uint32_t*)diffuse.atlas[e.index] + cube_texel(e.layer, diffuse.face_size, dir));
            diff = v3(unorm8(t, 0), unorm8(t, 1), unorm8(t, 2));
        }
        const V3 color = diff * sun;
        const float magnitude = v.radius * cube_fetch(cubes, e, dir);
        const float m = 1.1f * magnitude;
        const V3 spec = v3(v.position[0], v.position[1], v.position[2]) - L * m;
        const V3 c = ((color / 1.0f) * v.intensity) * 50000.0f;
        v.color[0] = c.x; v.color[1] = c.y; v.color[2] = c.z; v.color[3] = 1.0f;
        v.specular_position[0] = spec.x; v.specular_position[1] = spec.y; v.specular_position[2] = spec.z;
        v.specular_position[3] = 1.0f;
        cv[k] = v;
    }
}

cudaError_t launch_vpl_color(sgi_vpl* cv, const sgi_atlas_entry* ce, const int32_t* visible_index, int32_t cap,
                             const sgi_cube_atlas& cubes, const sgi_diffuse_atlas& diffuse, const sgi_csm& csm,
                             cudaStream_t s) {
    const int blocks = (cap + 255) / 256 < 152 ? (cap + 255) / 256 : 152;
    vpl_color_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(cv, ce, visible_index, cap, cubes, diffuse, csm);
    return cudaGetLastError();
}

// =========================================================== VPL vis cull --
// (the block-level passes are in sgi_cull.cuh)
__global__ void vpl_vis_flags_kernel(const sgi_vpl* __restrict__ vpls, int n, sgi_csm csm,
                                     uint8_t* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = vpl_visible(vpls, i, csm);
}

__global__ void __launch_bounds__(1024) vpl_compact_kernel(const sgi_vpl* __restrict__ vpls,
                                                           const sgi_atlas_entry* __restrict__ entries,
                                                           const uint8_t* __restrict__ flags, int n, int cap,
                                                           sgi_vpl* __restrict__ cv, sgi_atlas_entry* __restrict__ ce,
                                                           int32_t* __restrict__ visible_index,
                                                           float4* __restrict__ vpr) {
    compact_vpls<1024>(vpls, entries, flags, n, cap, cv, ce, visible_index, vpr, threadIdx.x);
}

// Both steps in one launch: every block flags its 256 VPLs, and the last block
// to finish (an atomic count of finished blocks, after a fence) compacts all
// of them in index order and returns the count to zero for the next launch.
// No block waits for another, and the compaction is the one above, so the
// result is that of the two kernels.
__global__ void __launch_bounds__(256) vpl_cull_kernel(const sgi_vpl* __restrict__ vpls,
                                                       const sgi_atlas_entry* __restrict__ entries, int n,
                                                       sgi_csm csm, uint8_t* __restrict__ flags, int cap,
                                                       sgi_vpl* __restrict__ cv, sgi_atlas_entry* __restrict__ ce,
                                                       int32_t* __restrict__ visible_index, float4* __restrict__ vpr,
                                                       unsigned* __restrict__ finished) {
    __shared__ bool last;
    const int i = blockIdx.x * 256 + threadIdx.x;
    if (i < n) flags[i] = vpl_visible(vpls, i, csm);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(finished, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    compact_vpls<256, true>(vpls, entries, flags, n, cap, cv, ce, visible_index, vpr, threadIdx.x);
    if (threadIdx.x == 0) *finished = 0u;
}

cudaError_t launch_vpl_cull(const sgi_vpl* vpls, const sgi_atlas_entry* entries, int32_t n, const sgi_csm& csm,
                            uint8_t* flags, int32_t cap, sgi_vpl* cv, sgi_atlas_entry* ce, int32_t* visible_index,
                            float4* vpr, unsigned* finished, cudaStream_t s) {
    if (n <= 0 || !finished) return cudaErrorInvalidValue;
    vpl_cull_kernel<<<(n + 255) / 256, 256, 0, s>>>(vpls, entries, n, csm, flags, cap, cv, ce, visible_index, vpr,
                                                    finished);
    return cudaGetLastError();
}

// Flag array of sgi_cull_vpls_noalloc (one byte per VPL). vpl_vis_flags_kernel
// writes every flag below the call's VPL count before vpl_compact_kernel reads
// it, so the array is never cleared.
static __device__ __align__(256) uint8_t g_noalloc_cull_flags[SGI_NOALLOC_CULL_MAX_VPLS];

cudaError_t noalloc_cull_flags(uint8_t** flags) {
    // looked up once per device, with that device current
    constexpr int kMaxDevices = 64;
    static std::mutex lock;
    static void* addr[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(lock);
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_cull_flags);
        if (e != cudaSuccess) return e;
        addr[dev] = p;
    }
    *flags = static_cast<uint8_t*>(addr[dev]);
    return cudaSuccess;
}

cudaError_t launch_vis_flags(const sgi_vpl* vpls, int32_t n, const sgi_csm& csm, uint8_t* flags, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    vpl_vis_flags_kernel<<<(n + 127) / 128, 128, 0, s>>>(vpls, n, csm, flags);
    return cudaGetLastError();
}

cudaError_t launch_compact(const sgi_vpl* vpls, const sgi_atlas_entry* entries, const uint8_t* flags, int32_t n,
                           int32_t cap, sgi_vpl* cv, sgi_atlas_entry* ce, int32_t* visible_index, float4* vpr,
                           cudaStream_t s) {
    vpl_compact_kernel<<<1, 1024, 0, s>>>(vpls, entries, flags, n, cap, cv, ce, visible_index, vpr);
    return cudaGetLastError();
}

// ============================================================ tile cull --
// Stage 1: one block per tile (tile_size^2 threads), tile_mean of sgi_cull.cuh.
__global__ void tile_stage1_kernel(int W, int H, int ts, int tiles_x, sgi_gbuffer g, sgi_camera cam,
                                   sgi_tile_stage1* __restrict__ out) {
    extern __shared__ float seq[];   // [tile_size^2][6], only for the sequential sum
    const int tile = blockIdx.x;
    tile_mean(W, H, ts, tile % tiles_x, tile / tiles_x, threadIdx.x, g, cam, seq, out + tile);
}

cudaError_t launch_tile_stage1(const sgi_config& cfg, const sgi_gbuffer& g, const sgi_camera& cam,
                               sgi_tile_stage1* out, cudaStream_t s) {
    const int ts = cfg.tile_size;
    const int tx = (cfg.width + ts - 1) / ts, ty = (cfg.height + ts - 1) / ts;
    const size_t seq_bytes = butterfly_tile_host(ts) ? 0 : sizeof(float) * 6 * ts * ts;
    tile_stage1_kernel<<<tx * ty, ts * ts, seq_bytes, s>>>(cfg.width, cfg.height, ts, tx, g, cam, out);
    return cudaGetLastError();
}

// Stage 2: one block of kTileCullThreads threads per tile, tile_cull of sgi_cull.cuh.
constexpr int kTileCullThreads = 128;
__global__ void __launch_bounds__(kTileCullThreads) tile_cull_kernel(int L, const sgi_tile_stage1* __restrict__ s1,
                                                                     const float4* __restrict__ vpr,
                                                                     const int32_t* __restrict__ visible_index,
                                                                     int32_t* __restrict__ lists) {
    extern __shared__ uint32_t cull_smem[];   // keys[count], then bin-b member indices[count]
    const int tile = blockIdx.x;
    const float4 p4 = __ldg(reinterpret_cast<const float4*>(s1 + tile));
    const float4 n4 = __ldg(reinterpret_cast<const float4*>(s1 + tile) + 1);
    tile_cull<kTileCullThreads>(L, v3(p4.x, p4.y, p4.z), v3(n4.x, n4.y, n4.z), vpr, __ldg(visible_index), cull_smem,
                                lists + (size_t)tile * (1 + L), threadIdx.x);
}

size_t tile_cull_smem(const sgi_config& cfg) { return (size_t)2 * sizeof(uint32_t) * (size_t)cfg.max_visible; }

cudaError_t launch_tile_stage2(const sgi_config& cfg, const sgi_tile_stage1* s1, const float4* vpr,
                               const int32_t* visible_index, int32_t* lists, cudaStream_t s) {
    const int ts = cfg.tile_size;
    const int T = ((cfg.width + ts - 1) / ts) * ((cfg.height + ts - 1) / ts);
    const size_t smem = tile_cull_smem(cfg);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(tile_cull_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    tile_cull_kernel<<<T, kTileCullThreads, smem, s>>>(cfg.max_vpls_per_tile, s1, vpr, visible_index, lists);
    return cudaGetLastError();
}

}  // namespace sgi
