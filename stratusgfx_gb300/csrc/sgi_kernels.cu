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
__global__ void vpl_vis_flags_kernel(const sgi_vpl* __restrict__ vpls, int n, sgi_csm csm,
                                     uint8_t* __restrict__ flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 pos = __ldg(reinterpret_cast<const float4*>(vpls + i));
    V3 p = v3(pos.x, pos.y, pos.z);
    V3 L = v3(csm.light_direction[0], csm.light_direction[1], csm.light_direction[2]);
    float shadowFactor = 1.0f - infinite_shadow(csm, p, L, false);
    flags[i] = shadowFactor < 1.0f ? 1 : 0;
}

// Stable compaction in ascending VPL index by one 1024-thread block: ballot
// prefix within each warp, exclusive scan of the 32 warp counts, running base
// across chunks of 1024 flags. Replaces the 8-thread atomicAdd loop of
// viscull_vpls.cs:85-98 (whose order is nondeterministic).
__global__ void __launch_bounds__(1024) vpl_compact_kernel(const sgi_vpl* __restrict__ vpls,
                                                           const sgi_atlas_entry* __restrict__ entries,
                                                           const uint8_t* __restrict__ flags, int n, int cap,
                                                           sgi_vpl* __restrict__ cv, sgi_atlas_entry* __restrict__ ce,
                                                           int32_t* __restrict__ visible_index) {
    __shared__ int warp_count[32];
    __shared__ int warp_base[32];
    __shared__ int chunk_total;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int base = 0;
    for (int start = 0; start < n; start += 1024) {
        int i = start + tid;
        bool f = i < n && flags[i] != 0;
        unsigned m = __ballot_sync(0xffffffffu, f);
        int within = __popc(m & ((1u << lane) - 1u));
        if (lane == 0) warp_count[warp] = __popc(m);
        __syncthreads();
        if (warp == 0) {
            int c = warp_count[lane];
            int incl = c;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += t;
            }
            warp_base[lane] = incl - c;
            if (lane == 31) chunk_total = incl;
        }
        __syncthreads();
        if (f) {
            int k = base + warp_base[warp] + within;
            if (k < cap) {
                const float4* src = reinterpret_cast<const float4*>(vpls + i);
                float4* dst = reinterpret_cast<float4*>(cv + k);
                dst[0] = __ldg(src); dst[1] = __ldg(src + 1); dst[2] = __ldg(src + 2); dst[3] = __ldg(src + 3);
                ce[k] = entries[i];
                visible_index[1 + k] = i;
            }
        }
        base += chunk_total;
        __syncthreads();
    }
    if (tid == 0) visible_index[0] = base < cap ? base : cap;
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
                           int32_t cap, sgi_vpl* cv, sgi_atlas_entry* ce, int32_t* visible_index, cudaStream_t s) {
    vpl_compact_kernel<<<1, 1024, 0, s>>>(vpls, entries, flags, n, cap, cv, ce, visible_index);
    return cudaGetLastError();
}

// ============================================================ tile cull --
// Stage 1: one block per tile (tile_size^2 threads). Per-tile mean world
// position and normalised mean normal. For tile sizes 8, 16 and 32 (a power of
// two number of warps) the sums use the warp butterfly order (xor 16, 8, 4, 2,
// 1, then xor nw/2 .. 1 over the warp totals); otherwise (e.g. the reference's
// 5x5 tiles) thread 0 adds the pixels in their order in the tile, as
// vpl_tiled_deferred_culling_stage1.cs:73-81 does. Pixels outside the image add 0 and are left out of the count.
// The kernel also packs (position, radius) of the compacted VPLs into `vpr`
// (16 bytes per VPL) for stage 2, which reads them once per tile.
SGI_D float butterfly(float v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__global__ void tile_stage1_kernel(int W, int H, int ts, int tiles_x, int num_tiles, sgi_gbuffer g, sgi_camera cam,
                                   sgi_tile_stage1* __restrict__ out, const sgi_vpl* __restrict__ cv,
                                   const int32_t* __restrict__ visible_index, float4* __restrict__ vpr) {
    __shared__ float wsum[32][6];
    extern __shared__ float seq[];   // [tile_size^2][6], only for the sequential sum
    const int tile = blockIdx.x;
    const int tx = tile % tiles_x, ty = tile / tiles_x;
    const int l = threadIdx.x;
    const int nthreads = ts * ts;
    {   // (position, radius) of the compacted VPLs, strided over all blocks
        const int count = __ldg(visible_index);
        for (int k = tile * nthreads + l; k < count; k += num_tiles * nthreads) {
            const float4 pos = __ldg(reinterpret_cast<const float4*>(cv + k));
            const float radius = __ldg(reinterpret_cast<const float*>(cv + k) + 12);
            vpr[k] = make_float4(pos.x, pos.y, pos.z, radius);
        }
    }
    const int x = tx * ts + l % ts, y = ty * ts + l / ts;
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (x < W && y < H) {
        size_t i = (size_t)y * W + x;
        float u = (float(x) + 0.5f) / float(W), vv = (float(y) + 0.5f) / float(H);
        V3 p = world_from_depth(u, vv, __ldg(g.depth + i), cam.inv_proj_view);
        V3 n = decode_normal(__ldg(g.normal + i));
        v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = n.x; v[4] = n.y; v[5] = n.z;
    }
    float w[6];
    bool have = false;
    const bool butterfly_order = (nthreads & 31) == 0 && (((nthreads >> 5) & ((nthreads >> 5) - 1)) == 0);
    if (butterfly_order) {
        const int lane = l & 31, warp = l >> 5, nw = nthreads >> 5;
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] = butterfly(v[c]);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c) wsum[warp][c] = v[c];
        }
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c) w[c] = lane < nw ? wsum[lane][c] : 0.0f;
            for (int off = nw >> 1; off >= 1; off >>= 1) {
#pragma unroll
                for (int c = 0; c < 6; ++c) w[c] = w[c] + __shfl_xor_sync(0xffffffffu, w[c], off);
            }
            have = lane == 0;
        }
    } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) seq[l * 6 + c] = v[c];
        __syncthreads();
        if (l == 0) {
#pragma unroll
            for (int c = 0; c < 6; ++c) w[c] = 0.0f;
            for (int j = 0; j < nthreads; ++j) {
#pragma unroll
                for (int c = 0; c < 6; ++c) w[c] = w[c] + seq[j * 6 + c];
            }
            have = true;
        }
    }
    if (have) {
        int cx = W - tx * ts < ts ? W - tx * ts : ts;
        int cy = H - ty * ts < ts ? H - ty * ts : ts;
        float cnt = float(cx * cy);
        V3 ap = v3(w[0], w[1], w[2]) / cnt;
        V3 an = v3(w[3], w[4], w[5]) / cnt;
        an = normalize(an);
        sgi_tile_stage1 o;
        o.average_position[0] = ap.x; o.average_position[1] = ap.y; o.average_position[2] = ap.z;
        o.average_position[3] = 1.0f;
        o.average_normal[0] = an.x; o.average_normal[1] = an.y; o.average_normal[2] = an.z;
        o.average_normal[3] = 1.0f;
        out[tile] = o;
    }
}

cudaError_t launch_tile_stage1(const sgi_config& cfg, const sgi_gbuffer& g, const sgi_camera& cam,
                               sgi_tile_stage1* out, const sgi_vpl* cv, const int32_t* visible_index, float4* vpr,
                               cudaStream_t s) {
    const int ts = cfg.tile_size;
    const int tx = (cfg.width + ts - 1) / ts, ty = (cfg.height + ts - 1) / ts;
    const int nw = (ts * ts) >> 5;
    const bool butterfly_order = ((ts * ts) & 31) == 0 && (nw & (nw - 1)) == 0;
    const size_t seq_bytes = butterfly_order ? 0 : sizeof(float) * 6 * ts * ts;
    tile_stage1_kernel<<<tx * ty, ts * ts, seq_bytes, s>>>(cfg.width, cfg.height, ts, tx, tx * ty, g, cam, out, cv,
                                                          visible_index, vpr);
    return cudaGetLastError();
}

// Stage 2, vpl_tiled_deferred_culling_stage2.cs:61-129: for each tile the
// shader inserts the visible VPLs, in order, into a list sorted by key =
// distance / radius with a strict '<' (ties keep the earlier VPL) and keeps
// the first L. The result is the L smallest candidates by (key, index), in
// that order. One 256-thread block per tile computes that set with the keys
// in shared memory (nothing per (tile, VPL) reaches global memory):
//   1. every visible VPL's key (kNoKey when it is not a candidate) goes to
//      shared memory, and each candidate counts into a 256-bin histogram of
//      floor(ratio * 256) (ratio <= 1; the bins are ordered like the keys);
//   2. with more than L candidates, a block scan of the histogram finds the
//      bin b where the count reaches L: every candidate of a lower bin is
//      kept, and from bin b the need = L - (candidates below b) smallest by
//      (key, index), found by ranking bin b's members against each other;
//   3. the kept (key, index) pairs, at most 64, are sorted by one warp.
constexpr uint32_t kNoKey = 0xffffffffu;

SGI_D uint32_t order_key(float k) {     // float order -> uint order (-0 == +0)
    const uint32_t b = __float_as_uint(k == 0.0f ? 0.0f : k);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// the histogram bin of a candidate's ratio (<= 1): non-decreasing in the ratio
SGI_D int ratio_bin(float ratio) {
    if (!(ratio > 0.0f)) return 0;
    const int b = (int)(ratio * 256.0f);
    return b > 255 ? 255 : b;
}

SGI_D unsigned long long pair_key(uint32_t key, int index) {
    return ((unsigned long long)key << 32) | (uint32_t)index;
}

// One compare-exchange stage of a bitonic network over 64 elements held as
// k0 at position lane and k1 at position lane + 32.
SGI_D void bitonic_stage64(unsigned long long& k0, unsigned long long& k1, int size, int j, int lane) {
    const unsigned FULL = 0xffffffffu;
    if (j == 32) {   // partners are the two registers of this lane; size == 64 -> ascending
        if (k1 < k0) { const unsigned long long t = k0; k0 = k1; k1 = t; }
        return;
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        unsigned long long& k = r ? k1 : k0;
        const int pos = lane + 32 * r;
        const unsigned long long o = __shfl_xor_sync(FULL, k, j);
        const bool ascending = (pos & size) == 0;
        const bool lower = (pos & j) == 0;
        // the lower position keeps the min when ascending, the max otherwise
        if ((lower == ascending) ? (o < k) : (k < o)) k = o;
    }
}

constexpr int kCullThreads = 256;

__global__ void __launch_bounds__(kCullThreads) tile_cull_kernel(int L, const sgi_tile_stage1* __restrict__ s1,
                                                                 const float4* __restrict__ vpr,
                                                                 const int32_t* __restrict__ visible_index,
                                                                 int32_t* __restrict__ lists) {
    extern __shared__ uint32_t cull_smem[];   // keys[count], then bin-b member indices[count]
    __shared__ uint32_t hist[256];
    __shared__ unsigned long long kept[64];
    __shared__ int warp_sum[kCullThreads / 32];
    __shared__ int s_bin, s_need, s_nkept, s_nb, s_mc;
    const int tile = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int count = __ldg(visible_index);
    uint32_t* keys = cull_smem;
    uint32_t* members = cull_smem + count;
    hist[tid] = 0u;
    if (tid == 0) { s_nkept = 0; s_nb = 0; }
    const float4 p4 = __ldg(reinterpret_cast<const float4*>(s1 + tile));
    const float4 n4 = __ldg(reinterpret_cast<const float4*>(s1 + tile) + 1);
    const V3 tp = v3(p4.x, p4.y, p4.z), tn = v3(n4.x, n4.y, n4.z);
    __syncthreads();
    int mine = 0;
    for (int k = tid; k < count; k += kCullThreads) {
        const float4 v = __ldg(vpr + k);
        const V3 lmf = v3(v.x, v.y, v.z) - tp;
        const float side = dot(tn, lmf);
        uint32_t u = kNoKey;
        if (!(side < 0.0f)) {
            const float ratio = length(lmf) / v.w;
            if (!(ratio > 1.0f) && ratio < kFloatMax) {
                u = order_key(ratio);
                ++mine;
                atomicAdd(&hist[ratio_bin(ratio)], 1u);
            }
        }
        keys[k] = u;
    }
    // candidates in the tile
    for (int off = 16; off >= 1; off >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, off);
    if (lane == 0) warp_sum[warp] = mine;
    __syncthreads();
    if (tid == 0) {
        int mc = 0;
        for (int w = 0; w < kCullThreads / 32; ++w) mc += warp_sum[w];
        s_mc = mc;
    }
    __syncthreads();
    const int mc = s_mc;
    const int take = mc < L ? mc : L;
    if (mc > L) {
        // inclusive scan of the histogram: bin b holds the L-th candidate
        const uint32_t h = hist[tid];
        uint32_t incl = h;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += t;
        }
        if (lane == 31) warp_sum[warp] = (int)incl;
        __syncthreads();
        uint32_t before = 0;
        for (int w = 0; w < warp; ++w) before += (uint32_t)warp_sum[w];
        incl += before;
        if (incl >= (uint32_t)L && incl - h < (uint32_t)L) { s_bin = tid; s_need = L - (int)(incl - h); }
        __syncthreads();
    } else if (tid == 0) {
        s_bin = 256;   // every candidate is kept
        s_need = 0;
    }
    __syncthreads();
    const int bin = s_bin;
    // kept: candidates of lower bins; bin b's members are ranked below
    for (int k = tid; k < count; k += kCullThreads) {
        const uint32_t u = keys[k];
        if (u == kNoKey) continue;
        const int b = ratio_bin(__uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u));
        if (b < bin) kept[atomicAdd(&s_nkept, 1)] = pair_key(u, k);
        else if (b == bin) members[atomicAdd(&s_nb, 1)] = (uint32_t)k;
    }
    __syncthreads();
    if (mc > L) {
        const int nb = s_nb, need = s_need;
        for (int m = tid; m < nb; m += kCullThreads) {
            const uint32_t k = members[m];
            const unsigned long long mk = pair_key(keys[k], (int)k);
            int rank = 0;
            for (int j = 0; j < nb; ++j) {
                const uint32_t kj = members[j];
                rank += pair_key(keys[kj], (int)kj) < mk ? 1 : 0;
            }
            if (rank < need) kept[atomicAdd(&s_nkept, 1)] = mk;
        }
        __syncthreads();
    }
    if (warp == 0) {
        unsigned long long k0 = lane < take ? kept[lane] : ~0ull;
        unsigned long long k1 = lane + 32 < take ? kept[lane + 32] : ~0ull;
        if (take > 1) {
            for (int size = 2; size <= 64; size <<= 1)
                for (int j = size >> 1; j >= 1; j >>= 1) bitonic_stage64(k0, k1, size, j, lane);
        }
        int32_t* o = lists + (size_t)tile * (1 + L);
        if (lane == 0) o[0] = take;
        if (lane < L) o[1 + lane] = lane < take ? (int32_t)(uint32_t)k0 : -1;
        if (lane + 32 < L) o[33 + lane] = lane + 32 < take ? (int32_t)(uint32_t)k1 : -1;
    }
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
    tile_cull_kernel<<<T, kCullThreads, smem, s>>>(cfg.max_vpls_per_tile, s1, vpr, visible_index, lists);
    return cudaGetLastError();
}

}  // namespace sgi
