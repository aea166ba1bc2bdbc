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
// position and normalised mean normal; the sums use the warp butterfly order
// (xor 16, 8, 4, 2, 1, then xor nw/2 .. 1 over the warp totals).
SGI_D float butterfly(float v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__global__ void tile_stage1_kernel(int W, int H, int ts, int tiles_x, sgi_gbuffer g, sgi_camera cam,
                                   sgi_tile_stage1* __restrict__ out) {
    __shared__ float wsum[32][6];
    const int tile = blockIdx.x;
    const int tx = tile % tiles_x, ty = tile / tiles_x;
    const int l = threadIdx.x;
    const int x = tx * ts + l % ts, y = ty * ts + l / ts;
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (x < W && y < H) {
        size_t i = (size_t)y * W + x;
        float u = (float(x) + 0.5f) / float(W), vv = (float(y) + 0.5f) / float(H);
        V3 p = world_from_depth(u, vv, __ldg(g.depth + i), cam.inv_proj_view);
        V3 n = decode_normal(__ldg(g.normal + i));
        v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = n.x; v[4] = n.y; v[5] = n.z;
    }
    const int lane = l & 31, warp = l >> 5, nw = (ts * ts) >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c) v[c] = butterfly(v[c]);
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < 6; ++c) wsum[warp][c] = v[c];
    }
    __syncthreads();
    if (warp == 0) {
        float w[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) w[c] = lane < nw ? wsum[lane][c] : 0.0f;
        for (int off = nw >> 1; off >= 1; off >>= 1) {
#pragma unroll
            for (int c = 0; c < 6; ++c) w[c] = w[c] + __shfl_xor_sync(0xffffffffu, w[c], off);
        }
        if (lane == 0) {
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
}

cudaError_t launch_tile_stage1(const sgi_config& cfg, const sgi_gbuffer& g, const sgi_camera& cam,
                               sgi_tile_stage1* out, cudaStream_t s) {
    const int ts = cfg.tile_size;
    const int tx = (cfg.width + ts - 1) / ts, ty = (cfg.height + ts - 1) / ts;
    tile_stage1_kernel<<<tx * ty, ts * ts, 0, s>>>(cfg.width, cfg.height, ts, tx, g, cam, out);
    return cudaGetLastError();
}

// Stage 2: one warp per tile. vpl_tiled_deferred_culling_stage2.cs:61-129
// inserts the visible VPLs, in order, into a list sorted by key =
// distance / radius with a strict '<' (ties keep the earlier VPL) and keeps
// the first L: the result is the first L entries of the stable sort of the
// candidates by key. This kernel computes that set without the sequential
// insertions, whose number depends on the VPL order:
//   1. every candidate's key (as an order-preserving uint) goes to shared memory;
//   2. if there are more than L candidates, a 4-round radix select (8 bits per
//      round) finds the L-th smallest key tau and how many keys equal to tau
//      are still needed;
//   3. keys < tau, then the needed keys == tau in index order, are compacted;
//   4. a 64-element warp bitonic sort orders them by (key, index).
constexpr uint32_t kNoKey = 0xffffffffu;

SGI_D uint32_t order_key(float k) {     // float order -> uint order (-0 == +0)
    const uint32_t b = __float_as_uint(k == 0.0f ? 0.0f : k);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

SGI_D bool key_less(uint32_t ka, int ia, uint32_t kb, int ib) { return ka < kb || (ka == kb && ia < ib); }

// One compare-exchange stage of a bitonic network over 64 elements held as
// (k0, i0) at position lane and (k1, i1) at position lane + 32.
SGI_D void bitonic_stage(uint32_t& k0, int& i0, uint32_t& k1, int& i1, int size, int j, int lane) {
    const unsigned FULL = 0xffffffffu;
    if (j == 32) {
        // partners are the two registers of this lane; size == 64 -> ascending
        if (key_less(k1, i1, k0, i0)) { uint32_t tk = k0; int ti = i0; k0 = k1; i0 = i1; k1 = tk; i1 = ti; }
        return;
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        uint32_t& k = r ? k1 : k0;
        int& id = r ? i1 : i0;
        const int pos = lane + 32 * r;
        const uint32_t ok = __shfl_xor_sync(FULL, k, j);
        const int oi = __shfl_xor_sync(FULL, id, j);
        const bool ascending = (pos & size) == 0;
        const bool lower = (pos & j) == 0;
        const bool other_less = key_less(ok, oi, k, id);
        // the lower position keeps the min when ascending, the max otherwise
        const bool take_other = (lower == ascending) ? other_less : !other_less;
        if (take_other) { k = ok; id = oi; }
    }
}

// 2a. keys: a block takes kKeyTiles tiles; its threads stride over the visible
// VPLs (the count lives on the device, so the grid cannot be sized by it), read
// each VPL's position and radius once and write its key for every tile of the
// block: keys[tile][k] in global memory (L2-resident), kNoKey when the VPL is
// not a candidate. Reading the VPL records once per block instead of once per
// tile cuts the L2 traffic of this pass by kKeyTiles.
constexpr int kKeyTiles = 8;
__global__ void __launch_bounds__(256) tile_keys_kernel(int num_tiles, int key_stride,
                                                        const sgi_tile_stage1* __restrict__ s1,
                                                        const sgi_vpl* __restrict__ cv,
                                                        const int32_t* __restrict__ visible_index,
                                                        uint32_t* __restrict__ keys) {
    __shared__ float4 tile_p[kKeyTiles], tile_n[kKeyTiles];
    const int count = __ldg(visible_index);
    const int t0 = blockIdx.x * kKeyTiles;
    const int nt = min(kKeyTiles, num_tiles - t0);
    if (threadIdx.x < nt) {
        tile_p[threadIdx.x] = __ldg(reinterpret_cast<const float4*>(s1 + t0 + threadIdx.x));
        tile_n[threadIdx.x] = __ldg(reinterpret_cast<const float4*>(s1 + t0 + threadIdx.x) + 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < count; k += blockDim.x) {
        const float* rec = reinterpret_cast<const float*>(cv + k);
        const V3 lp = v3(__ldg(rec + 0), __ldg(rec + 1), __ldg(rec + 2));
        const float radius = __ldg(rec + 12);
        for (int j = 0; j < nt; ++j) {
            const float4 p4 = tile_p[j], n4 = tile_n[j];
            const V3 lmf = lp - v3(p4.x, p4.y, p4.z);
            const float side = dot(v3(n4.x, n4.y, n4.z), lmf);
            uint32_t u = kNoKey;
            if (!(side < 0.0f)) {
                const float ratio = length(lmf) / radius;
                if (!(ratio > 1.0f) && ratio < kFloatMax) u = order_key(ratio);
            }
            keys[(size_t)(t0 + j) * key_stride + k] = u;
        }
    }
}

// 2b. select: one warp per tile over its keys.
__global__ void __launch_bounds__(256) tile_select_kernel(int num_tiles, int L, int key_stride,
                                                          const uint32_t* __restrict__ all_keys,
                                                          const int32_t* __restrict__ visible_index,
                                                          int32_t* __restrict__ lists) {
    __shared__ uint32_t hist_all[8][256];
    __shared__ uint32_t sel_all[8][128];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tile = blockIdx.x * 8 + warp;
    if (tile >= num_tiles) return;     // warps are independent: no block-wide barrier below
    uint32_t* hist = hist_all[warp];
    uint32_t* sel_k = sel_all[warp];
    int* sel_i = reinterpret_cast<int*>(sel_k + 64);
    const uint32_t* keys = all_keys + (size_t)tile * key_stride;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int count = __ldg(visible_index);

    int mc = 0;
    for (int base = 0; base < count; base += 32) {
        const int k = base + lane;
        const uint32_t u = k < count ? __ldg(keys + k) : kNoKey;
        mc += __popc(__ballot_sync(FULL, u != kNoKey));
    }
    const int take = mc < L ? mc : L;

    // radix select of the take-th smallest key
    uint32_t tau = kNoKey;
    int need_eq = 0;
    if (mc > L) {
        uint32_t prefix = 0u, mask = 0u;
        int remaining = L;
        for (int shift = 24; shift >= 0; shift -= 8) {
            for (int b = lane; b < 256; b += 32) hist[b] = 0u;
            __syncwarp();
            for (int k = lane; k < count; k += 32) {
                const uint32_t u = __ldg(keys + k);
                if (u != kNoKey && (u & mask) == prefix) atomicAdd(&hist[(u >> shift) & 0xffu], 1u);
            }
            __syncwarp();
            uint32_t hv[8];
            uint32_t sum = 0u;
#pragma unroll
            for (int j = 0; j < 8; ++j) { hv[j] = hist[lane * 8 + j]; sum += hv[j]; }
            uint32_t incl = sum;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t t = __shfl_up_sync(FULL, incl, off);
                if (lane >= off) incl += t;
            }
            const unsigned found = __ballot_sync(FULL, incl >= (uint32_t)remaining);
            const int src = __ffs(found) - 1;
            int bin = 0;
            uint32_t below = 0u;
            if (lane == src) {
                uint32_t c = incl - sum;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (c + hv[j] >= (uint32_t)remaining) { bin = lane * 8 + j; below = c; break; }
                    c += hv[j];
                }
            }
            bin = __shfl_sync(FULL, bin, src);
            below = __shfl_sync(FULL, below, src);
            remaining -= (int)below;
            prefix |= (uint32_t)bin << shift;
            mask |= 0xffu << shift;
            __syncwarp();
        }
        tau = prefix;
        need_eq = remaining;
    }

    // compaction in index order: keys < tau, then the first need_eq keys == tau
    int pos = 0, eq_seen = 0;
    for (int base = 0; base < count && pos < take; base += 32) {
        const int k = base + lane;
        const uint32_t u = k < count ? __ldg(keys + k) : kNoKey;
        const bool eq = u == tau && u != kNoKey;
        const unsigned meq = __ballot_sync(FULL, eq);
        const int eq_rank = eq_seen + __popc(meq & lt_mask);
        const bool sel = (u < tau) || (eq && eq_rank < need_eq);
        const unsigned ms = __ballot_sync(FULL, sel);
        if (sel) {
            const int p = pos + __popc(ms & lt_mask);
            sel_k[p] = u;
            sel_i[p] = k;
        }
        pos += __popc(ms);
        eq_seen += __popc(meq);
    }
    __syncwarp();

    // sort (key, index) ascending
    uint32_t k0 = lane < take ? sel_k[lane] : kNoKey;
    int i0 = lane < take ? sel_i[lane] : 0x7fffffff;
    uint32_t k1 = lane + 32 < take ? sel_k[lane + 32] : kNoKey;
    int i1 = lane + 32 < take ? sel_i[lane + 32] : 0x7fffffff;
    if (take > 1) {
        for (int size = 2; size <= 64; size <<= 1)
            for (int j = size >> 1; j >= 1; j >>= 1) bitonic_stage(k0, i0, k1, i1, size, j, lane);
    }
    int32_t* o = lists + (size_t)tile * (1 + L);
    if (lane == 0) o[0] = take;
    if (lane < L) o[1 + lane] = lane < take ? i0 : -1;
    if (lane + 32 < L) o[33 + lane] = lane + 32 < take ? i1 : -1;
}

cudaError_t launch_tile_stage2(const sgi_config& cfg, const sgi_tile_stage1* s1, const sgi_vpl* cv,
                               const int32_t* visible_index, uint32_t* keys, int32_t* lists, cudaStream_t s) {
    const int ts = cfg.tile_size;
    const int T = ((cfg.width + ts - 1) / ts) * ((cfg.height + ts - 1) / ts);
    const int key_stride = (cfg.max_visible + 31) & ~31;
    tile_keys_kernel<<<(T + kKeyTiles - 1) / kKeyTiles, 256, 0, s>>>(T, key_stride, s1, cv, visible_index, keys);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    tile_select_kernel<<<(T + 7) / 8, 256, 0, s>>>(T, cfg.max_vpls_per_tile, key_stride, keys, visible_index, lists);
    return cudaGetLastError();
}

}  // namespace sgi
