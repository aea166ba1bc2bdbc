// sgi_kernels.cu - the GI/lighting hot path on sm_103a.
//
// Kernels (reference shader each restates, paths relative to the StratusGFX root):
//   vpl_vis_flags / vpl_compact  viscull_vpls.cs:47-120
//   tile_stage1                  vpl_tiled_deferred_culling_stage1.cs:50-90
//   tile_stage2                  vpl_tiled_deferred_culling_stage2.cs:61-129
//   vpl_gather                   vpl_pbr_gi.fs:81-207
//   denoise_pass                 vpl_pbr_gi_denoise.fs:142-435
//   deferred_pbr_csm             pbr.fs:82-145 (+ pbr.glsl:158-227)
//
// Compiled with -fmad=false (see sgi_math.cuh): results are bit-reproducible.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "sgi_internal.h"
#include "sgi_math.cuh"

namespace sgi {

// ------------------------------------------------------------------ texels --
SGI_D uint2 ld_u2(const uint2* p, size_t i) { return __ldg(p + i); }
SGI_D void unpack_h4(uint2 t, float& a, float& b, float& c, float& d) {
    a = h2f((uint16_t)(t.x & 0xffffu)); b = h2f((uint16_t)(t.x >> 16));
    c = h2f((uint16_t)(t.y & 0xffffu)); d = h2f((uint16_t)(t.y >> 16));
}
SGI_D uint2 pack_h4(float a, float b, float c, float d) {
    return make_uint2((uint32_t)f2h(a) | ((uint32_t)f2h(b) << 16), (uint32_t)f2h(c) | ((uint32_t)f2h(d) << 16));
}

// The texels and weights of one bilinear sample: several channels sampled at
// the same uv share them (each channel then evaluates exactly the sum that
// bilinear() below forms).
struct Bilinear {
    size_t o00, o10, o01, o11;
    float w00, w10, w01, w11;
};
SGI_D Bilinear bilinear_at(int W, int H, float s, float t) {
    const float u = s * float(W) - 0.5f, v = t * float(H) - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const int i0 = tex_index(fu, W), i1 = tex_index(fu + 1.0f, W);
    const size_t r0 = (size_t)tex_index(fv, H) * W, r1 = (size_t)tex_index(fv + 1.0f, H) * W;
    Bilinear q;
    q.o00 = r0 + i0; q.o10 = r0 + i1; q.o01 = r1 + i0; q.o11 = r1 + i1;
    q.w00 = (1.0f - a) * (1.0f - b); q.w10 = a * (1.0f - b); q.w01 = (1.0f - a) * b; q.w11 = a * b;
    return q;
}
SGI_D float bilinear_sum(const Bilinear& q, float f00, float f10, float f01, float f11) {
    return __fmaf_rn(f11, q.w11, __fmaf_rn(f01, q.w01, __fmaf_rn(f10, q.w10, f00 * q.w00)));
}

// Bilinear sample (LINEAR, CLAMP_TO_EDGE) at uv of a scalar image.
template <class F> SGI_D float bilinear(F fetch, int W, int H, float s, float t) {
    float u = s * float(W) - 0.5f, v = t * float(H) - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    int i0 = tex_index(fu, W), i1 = tex_index(fu + 1.0f, W);
    int j0 = tex_index(fv, H), j1 = tex_index(fv + 1.0f, H);
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    return __fmaf_rn(fetch(i1, j1), w11, __fmaf_rn(fetch(i0, j1), w01, __fmaf_rn(fetch(i1, j0), w10, fetch(i0, j0) * w00)));
}

// ------------------------------------------------------------------- CSM --
// texture(sampler2DArrayShadow) with LINEAR + LEQUAL: bilinear weights over
// the four 0/1 compare results.
SGI_D float csm_pcf(const float* __restrict__ base, int R, float s, float t, float ref) {
    float u = s * float(R) - 0.5f, v = t * float(R) - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    float a = u - fu, b = v - fv;
    int i0 = tex_index(fu, R), i1 = tex_index(fu + 1.0f, R);
    int j0 = tex_index(fv, R), j1 = tex_index(fv + 1.0f, R);
    float c00 = ref <= __ldg(base + (size_t)j0 * R + i0) ? 1.0f : 0.0f;
    float c10 = ref <= __ldg(base + (size_t)j0 * R + i1) ? 1.0f : 0.0f;
    float c01 = ref <= __ldg(base + (size_t)j1 * R + i0) ? 1.0f : 0.0f;
    float c11 = ref <= __ldg(base + (size_t)j1 * R + i1) ? 1.0f : 0.0f;
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    return __fmaf_rn(c11, w11, __fmaf_rn(c01, w01, __fmaf_rn(c10, w10, c00 * w00)));
}

// calculateInfiniteShadowValue, pbr.glsl:158-227: lit fraction.
SGI_D float infinite_shadow(const sgi_csm& csm, V3 fragPos, V3 normal, bool useDepthBias) {
    V3 blends = v3(dot4(csm.cascade_planes[0], fragPos), dot4(csm.cascade_planes[1], fragPos),
                   dot4(csm.cascade_planes[2], fragPos));
    float bias = csm.depth_bias / (csm.zfar - csm.znear);
    if (!useDepthBias) bias = 0.0f;
    V3 L = v3(csm.light_direction[0], csm.light_direction[1], csm.light_direction[2]);
    V3 position = fragPos + normal * (1.0f - saturate(dot(normal, L))) * 1.0f;
    bool beyond2 = blends.y >= 0.0f;
    bool beyond3 = blends.z >= 0.0f;
    int index1 = beyond2 ? 2 : 0;
    int index2 = beyond3 ? 3 : 1;
    V4 c1 = mat4_mul(csm.cascade_proj_view[index1], position.x, position.y, position.z, 1.0f);
    V4 c2 = mat4_mul(csm.cascade_proj_view[index2], position.x, position.y, position.z, 1.0f);
    V3 cc1 = (v3(c1.x, c1.y, c1.z) / c1.w) * 0.5f + v3s(0.5f);
    V3 cc2 = (v3(c2.x, c2.y, c2.z) / c2.w) * 0.5f + v3s(0.5f);
    float depth1 = cc1.z;
    float depth2 = beyond3 ? saturate(cc2.z) : cc2.z;
    float weight = beyond2 ? saturate(blends.y) - saturate(blends.z) : 1.0f - saturate(blends.x);
    const int R = csm.resolution;
    float wh = 1.0f / float(R);
    const float* b1 = csm.depth + (size_t)index1 * R * R;
    const float* b2 = csm.depth + (size_t)index2 * R * R;
    float ref1 = depth1 - bias, ref2 = depth2 - bias;
    float light1 = 0.0f, light2 = 0.0f, samples = 0.0f;
#pragma unroll
    for (int yi = -1; yi <= 1; ++yi) {
#pragma unroll
        for (int xi = -1; xi <= 1; ++xi) {
            float ox = float(xi) * wh, oy = float(yi) * wh;
            light1 += csm_pcf(b1, R, cc1.x + ox, cc1.y + oy, ref1);
            light2 += csm_pcf(b2, R, cc2.x + ox, cc2.y + oy, ref2);
            samples += 1.0f;
        }
    }
    return mixf(light2, light1, weight) * (1.0f / samples);
}

// ------------------------------------------------------------- cube maps --
// Nearest texel of a cube face_size n in direction d: returns its offset within the layer stack.
SGI_D size_t cube_texel(int layer, int n, V3 d) {
    float ax = gabs(d.x), ay = gabs(d.y), az = gabs(d.z);
    int face; float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        if (d.x >= 0.0f) { face = 0; sc = -d.z; tc = -d.y; } else { face = 1; sc = d.z; tc = -d.y; }
    } else if (ay >= az) {
        ma = ay;
        if (d.y >= 0.0f) { face = 2; sc = d.x; tc = d.z; } else { face = 3; sc = d.x; tc = -d.z; }
    } else {
        ma = az;
        if (d.z >= 0.0f) { face = 4; sc = d.x; tc = -d.y; } else { face = 5; sc = -d.x; tc = -d.y; }
    }
    float s = 0.5f * (sc / ma + 1.0f);
    float t = 0.5f * (tc / ma + 1.0f);
    int i = nearest_index(s, n), j = nearest_index(t, n);
    return (((size_t)layer * 6 + face) * n + j) * n + i;
}

SGI_D float cube_fetch(const sgi_cube_atlas& at, sgi_atlas_entry e, V3 d) {
    if (e.index < 0 || e.index >= at.num_atlases || e.layer < 0 || e.layer >= at.layers_per_atlas) return 1.0f;
    float ax = gabs(d.x), ay = gabs(d.y), az = gabs(d.z);
    int face; float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        if (d.x >= 0.0f) { face = 0; sc = -d.z; tc = -d.y; } else { face = 1; sc = d.z; tc = -d.y; }
    } else if (ay >= az) {
        ma = ay;
        if (d.y >= 0.0f) { face = 2; sc = d.x; tc = d.z; } else { face = 3; sc = d.x; tc = -d.z; }
    } else {
        ma = az;
        if (d.z >= 0.0f) { face = 4; sc = d.x; tc = -d.y; } else { face = 5; sc = -d.x; tc = -d.y; }
    }
    float s = 0.5f * (sc / ma + 1.0f);
    float t = 0.5f * (tc / ma + 1.0f);
    const int n = at.face_size;
    int i = nearest_index(s, n), j = nearest_index(t, n);
    size_t off = (((size_t)e.layer * 6 + face) * n + j) * n + i;
    const void* base = at.atlas[e.index];
    if (at.format == SGI_CUBE_F16) return h2f(__ldg((const unsigned short*)base + off));
    if (at.format == SGI_CUBE_F32) return __ldg((const float*)base + off);
    return float(__ldg((const unsigned short*)base + off)) / 65535.0f;
}

// calculateShadowValue1Sample, pbr.glsl:116-136 (1 = occluded)
SGI_D float shadow_1sample(const sgi_cube_atlas& at, sgi_atlas_entry e, float farPlane, V3 fragPos, V3 lightPos,
                           float lightNormalDot, float minBias) {
    V3 fragDir = fragPos - lightPos;
    float currentDepth = length(fragDir);
    float bias = currentDepth * gmax(minBias, saturate(lightNormalDot) * 0.03f);
    float depth = cube_fetch(at, e, fragDir);
    depth = depth * farPlane;
    return (currentDepth - bias) > depth ? 1.0f : 0.0f;
}

// calculateShadowValue8Samples, pbr.glsl:81-113 (fraction occluded): eight taps at
// the direction offset by (+-0.3, +-0.3, +-0.3), x outermost.
SGI_D float shadow_8samples(const sgi_cube_atlas& at, sgi_atlas_entry e, float farPlane, V3 fragPos, V3 lightPos,
                            float lightNormalDot, float minBias) {
    V3 fragDir = fragPos - lightPos;
    float currentDepth = length(fragDir);
    float bias = currentDepth * gmax(minBias, saturate(lightNormalDot) * 0.03f);
    float shadow = 0.0f;
    const float offs[2] = {-0.3f, 0.3f};
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
            for (int z = 0; z < 2; ++z) {
                float depth = cube_fetch(at, e, fragDir + v3(offs[x], offs[y], offs[z]));
                depth = depth * farPlane;
                if ((currentDepth - bias) > depth) shadow = shadow + 1.0f;
            }
    return shadow / 8.0f;
}

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

// ================================================================ gather --
struct GatherParams {
    int W, H, ts, tiles_x, L, tiled, spp;
    ShadeConfig sc;
    sgi_gbuffer g;
    sgi_camera cam;
    const sgi_vpl* cv;
    const sgi_atlas_entry* ce;
    const int32_t* visible_index;
    const int32_t* lists;
    sgi_cube_atlas cubes;
    float time;
    GatherOut out;
};

// Per-pixel inputs of the gather (vpl_pbr_gi.fs:99-145).
struct PixelShade {
    V3 fragPos, viewDir, baseColor, normal, baseRefl;
    float distToCamera, roughness, metallic, ao, ambient;
    int sampleCount, candidates;
    const int32_t* list;
};

SGI_D PixelShade load_pixel(const GatherParams& p, int x, int y, size_t i) {
    PixelShade px;
    const float u = (float(x) + 0.5f) / float(p.W), v = (float(y) + 0.5f) / float(p.H);
    px.fragPos = world_from_depth(u, v, __ldg(p.g.depth + i), p.cam.inv_proj_view);
    const V3 viewPos = v3(p.cam.view_position[0], p.cam.view_position[1], p.cam.view_position[2]);
    px.viewDir = normalize(viewPos - px.fragPos);
    px.distToCamera = length(viewPos - px.fragPos);
    const uint32_t alb = __ldg(p.g.albedo + i);
    px.baseColor = v3(gmax(unorm8(alb, 0), 0.01f), gmax(unorm8(alb, 1), 0.01f), gmax(unorm8(alb, 2), 0.01f));
    px.normal = decode_normal(__ldg(p.g.normal + i));
    const uint32_t rma = __ldg(p.g.roughness_metallic_ambient + i);
    px.roughness = gmax(0.5f, unorm8(rma, 0));
    px.metallic = unorm8(rma, 1);
    px.ao = gclamp(h2f(__ldg(p.g.ssao + i)), 0.35f, 1.0f);
    px.ambient = unorm8(rma, 2);
    px.baseRefl = v3s(float(__ldg(p.g.base_reflectivity + i) & 0xffu) / 255.0f);
    const float roughnessWeight = 1.0f - px.roughness;
    const float distRatio = gmin(1.0f - px.distToCamera / 1000.0f, 1.0f);
    if (p.spp > 0) {
        px.sampleCount = p.spp;
    } else {
        int maxSamplesPerPixel = (int)mixf(2.0f, 10.0f, roughnessWeight);
        int samplesMax = (int)(float(maxSamplesPerPixel) * distRatio);
        px.sampleCount = samplesMax > 1 ? samplesMax : 1;
    }
    px.list = nullptr;
    if (p.tiled) {
        const int tile = (y / p.ts) * p.tiles_x + (x / p.ts);
        px.list = p.lists + (size_t)tile * (1 + p.L);
        px.candidates = __ldg(px.list);
    } else {
        px.candidates = __ldg(p.visible_index);
    }
    return px;
}

// The sample loop of vpl_pbr_gi.fs:148-200 with the seed z starting at seedZ.
SGI_D void sample_vpls(const GatherParams& p, const PixelShade& px, float seedX, float seedY, float seedZ,
                       V3& vplColor, float& validSamples) {
    ShadeParams sp{p.sc.min_roughness, p.sc.perceptual, p.sc.fog_density,
                   {p.sc.fog_color[0], p.sc.fog_color[1], p.sc.fog_color[2]}, p.sc.point_ambient};
    vplColor = v3s(0.0f);
    validSamples = 0.0f;
    const int candidates = px.candidates;
    if (candidates <= 0) return;
    const float minGi = p.sc.min_gi_occlusion;
    const V3 fragPos = px.fragPos, normal = px.normal;
    const VplPixel vp = vpl_pixel(fragPos, px.baseColor, normal, px.viewDir, px.distToCamera, px.roughness,
                                  px.metallic, px.ambient, px.baseRefl, sp);
    for (int s = 0, resamples = 0; s < px.sampleCount; ++s) {
        const float rnd = random3(seedX, seedY, seedZ);
        seedZ += 10000.0f;
        int lightIndex;
        if (px.list) {
            int r = (int)(float(candidates) * rnd);
            lightIndex = __ldg(px.list + 1 + (r < candidates - 1 ? r : candidates - 1));
        } else {
            lightIndex = (int)(float(candidates - 1) * rnd);
        }
        const float4* rec = reinterpret_cast<const float4*>(p.cv + lightIndex);
        const float4 pos = __ldg(rec);
        const float4 spec = __ldg(rec + 2);
        const float4 misc = __ldg(rec + 3);   // radius, farPlane, intensity
        const sgi_atlas_entry entry = p.ce[lightIndex];
        const V3 lightPosition = v3(pos.x, pos.y, pos.z);
        const V3 lmf = lightPosition - fragPos;
        const float lightRadius = misc.x;
        const float distance = length(lmf);
        if (resamples < 5) {
            float sideCheck = dot(normal, normalize(lmf));
            if (sideCheck < 0.0f || distance > lightRadius) { ++resamples; --s; continue; }
        }
        const float distanceRatio = gclamp((2.0f * distance) / lightRadius, 0.0f, 1.0f);
        const float distAttenuation = distanceRatio;
        const float4 col = __ldg(rec + 1);
        const V3 lightColor = v3(col.x, col.y, col.z);
        float shadowFactor = px.distToCamera < 500.0f
                                 ? shadow_1sample(p.cubes, entry, misc.y, fragPos, lightPosition,
                                                  dot(lightPosition - fragPos, normal), 0.1f)
                                 : 0.0f;
        shadowFactor = gmin(shadowFactor, mixf(minGi, 1.0f, distanceRatio));
        float reweight = 1.0f;
        if (shadowFactor > 0.0f) reweight = (1.0f - distAttenuation) * minGi + distAttenuation;
        validSamples += reweight;
        const V3 tmp = px.ao * vpl_lighting2_sample(vp, v3(spec.x, spec.y, spec.z), lightPosition, lightColor,
                                                    lightRadius);
        vplColor = vplColor + (1.0f - shadowFactor) * tmp;
    }
}

// vpl_pbr_gi.fs:81-207, one thread per pixel.
__global__ void __launch_bounds__(256, 4) vpl_gather_kernel(GatherParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.W || y >= p.H) return;
    const size_t i = (size_t)y * p.W + x;
    const PixelShade px = load_pixel(p, x, y, i);
    const V3 normal = px.normal;
    const float seedX = float(x) + 0.5f, seedY = float(y) + 0.5f;
    V3 vplColor;
    float validSamples;
    sample_vpls(p, px, seedX, seedY, p.time, vplColor, validSamples);
    validSamples = gmax(validSamples, 1.0f);
    const V3 b = vmin(vplColor, kHalfMax);
    // The reservoir as stored in its RGBA16F target (vpl_pbr_gi.fs:205).
    const float r0 = h2f(f2h(b.x)), r1 = h2f(f2h(b.y)), r2 = h2f(f2h(b.z)), r3 = h2f(f2h(validSamples));
    if (p.out.raw) p.out.raw[i] = pack_h4(r0, r1, r2, r3);
    // Denoise pass 0 for this pixel: computeMergedReservoir with minmaxNearest = 0
    // (vpl_pbr_gi_denoise.fs:192-273) reads only the centre texel, which is this one.
    const float depth = __ldg(p.g.depth + i);
    float cr0 = 0.0f, cr1 = 0.0f, cr2 = 0.0f, cr3 = 0.0f;
    const float depthCutoff = 0.1f * depth;
    float runningSum = 0.0f;
    const float probabilisticWeight = 1.0f / float(__ldg(p.visible_index));
    if (!(dot(normal, normal) < 0.906f)) {
        if (!(gabs(depth - depth) > depthCutoff)) {
            const float randUpdate = random3(seedX, seedY, p.time);
            const float probability = r3 * probabilisticWeight;
            cr3 += probability;
            if (randUpdate < (probability / cr3)) {
                cr0 += r0; cr1 += r1; cr2 += r2;
                runningSum += r3;
            }
        }
    }
    const float den = gmax(kEps, runningSum);
    p.out.merged[i] = pack_h4(cr0 / den, cr1 / den, cr2 / den, 1.0f);
    p.out.guide[i] = make_float4(normal.x, normal.y, normal.z, depth);
}

cudaError_t launch_gather(const sgi_config& cfg, const ShadeConfig& sc, const sgi_gbuffer& g, const sgi_camera& cam,
                          const sgi_vpl* cv, const sgi_atlas_entry* ce, const int32_t* visible_index,
                          const int32_t* lists, const sgi_cube_atlas& cubes, float time, const GatherOut& out,
                          cudaStream_t s, dim3 block) {
    GatherParams p;
    p.W = cfg.width; p.H = cfg.height; p.ts = cfg.tile_size;
    p.tiles_x = (cfg.width + cfg.tile_size - 1) / cfg.tile_size;
    p.L = cfg.max_vpls_per_tile; p.tiled = cfg.gi_mode == SGI_GI_TILED; p.spp = cfg.samples_per_pixel;
    p.sc = sc; p.g = g; p.cam = cam; p.cv = cv; p.ce = ce; p.visible_index = visible_index; p.lists = lists;
    p.cubes = cubes; p.time = time; p.out = out;
    if (block.x == 0) block = dim3(16, 16);
    dim3 grid((cfg.width + block.x - 1) / block.x, (cfg.height + block.y - 1) / block.y);
    vpl_gather_kernel<<<grid, block, 0, s>>>(p);
    return cudaGetLastError();
}

// Converged GI target: `batches` independent runs of the gather's sample loop
// per pixel (batch b seeds z at time + b * 2e5, far past the previous batch's
// draws), with sum(vplColor) and sum(validSamples) accumulated in FP64. Its
// ratio is the limit of the per-pixel estimate the K-sample path denoises;
// out = (sum vplColor / max(sum validSamples, 1), 1) as FP32.
__global__ void __launch_bounds__(256, 4) gi_target_kernel(GatherParams p, int batches, float4* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.W || y >= p.H) return;
    const size_t i = (size_t)y * p.W + x;
    const PixelShade px = load_pixel(p, x, y, i);
    const float seedX = float(x) + 0.5f, seedY = float(y) + 0.5f;
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, w = 0.0;
    for (int b = 0; b < batches; ++b) {
        V3 col;
        float valid;
        sample_vpls(p, px, seedX, seedY, p.time + float(b) * 200000.0f, col, valid);
        c0 += (double)col.x; c1 += (double)col.y; c2 += (double)col.z; w += (double)valid;
    }
    const double den = w < 1.0 ? 1.0 : w;
    out[i] = make_float4((float)(c0 / den), (float)(c1 / den), (float)(c2 / den), 1.0f);
}

cudaError_t launch_gi_target(const sgi_config& cfg, const ShadeConfig& sc, const sgi_gbuffer& g,
                             const sgi_camera& cam, const sgi_vpl* cv, const sgi_atlas_entry* ce,
                             const int32_t* visible_index, const int32_t* lists, const sgi_cube_atlas& cubes,
                             float time, int batches, float4* out, cudaStream_t s) {
    GatherParams p;
    p.W = cfg.width; p.H = cfg.height; p.ts = cfg.tile_size;
    p.tiles_x = (cfg.width + cfg.tile_size - 1) / cfg.tile_size;
    p.L = cfg.max_vpls_per_tile; p.tiled = cfg.gi_mode == SGI_GI_TILED; p.spp = cfg.samples_per_pixel;
    p.sc = sc; p.g = g; p.cam = cam; p.cv = cv; p.ce = ce; p.visible_index = visible_index; p.lists = lists;
    p.cubes = cubes; p.time = time;
    dim3 block(16, 16);
    dim3 grid((cfg.width + 15) / 16, (cfg.height + 15) / 16);
    gi_target_kernel<<<grid, block, 0, s>>>(p, batches, out);
    return cudaGetLastError();
}

// =============================================================== denoise --
// The 5x5 edge-stopping filter of vpl_pbr_gi_denoise.fs:307-327 with the
// weights of filterInput (:142-190): w = pow(max(0, n_c . n_q), 128) *
// exp(-|z_c - z_q|) / sigmaZ, centre weight 1, taps at stride 2^pass, clamped
// to the edge. Normals and depths come from the gather's guide (the same
// decoded values the shader computes per tap).
//
// The 24 off-centre taps run in pairs on the packed FP32 pipe
// (atrous_weight2, packed accumulation of the four channels): each lane
// performs the scalar operations of its tap with the same roundings, and the
// taps still accumulate one after another in the order dx = -2..2 (outer),
// dy = -2..2 (inner), so the sums are those of the one-tap-at-a-time loop
// (atrous_weight) bit for bit.
SGI_D void atrous_filter(int x, int y, int W, int H, int step, const float4* __restrict__ guide,
                         const uint2* __restrict__ res_in, V3 cn, float cd, float& rf0, float& rf1, float& rf2,
                         float& rf3) {
    int xs[5];
    size_t rows[5];
#pragma unroll
    for (int d = 0; d < 5; ++d) {
        const int xx = x + (d - 2) * step, yy = y + (d - 2) * step;
        xs[d] = xx < 0 ? 0 : (xx > W - 1 ? W - 1 : xx);
        rows[d] = (size_t)(yy < 0 ? 0 : (yy > H - 1 ? H - 1 : yy)) * W;
    }
    // the four channel sums, two per packed register
    float2 acc01 = make_float2(0.0f, 0.0f), acc23 = make_float2(0.0f, 0.0f);
    auto accumulate = [&](float f, uint2 t) {
        float a, b, c, e;
        unpack_h4(t, a, b, c, e);
        acc01 = fma2(f2s(f), make_float2(a, b), acc01);
        acc23 = fma2(f2s(f), make_float2(c, e), acc23);
    };
    const float ncd = -cd;
    const float2 cx = f2s(cn.x), cy = f2s(cn.y), cz = f2s(cn.z);
#pragma unroll
    for (int p = 0; p < 12; ++p) {   // taps t = 5 * (dx + 2) + (dy + 2); pairs (0,1) .. (10,11), (13,14) .. (23,24)
        if (p == 6) accumulate(1.0f, ld_u2(res_in, rows[2] + xs[2]));   // the centre tap, weight 1
        const int t = p < 6 ? 2 * p : 2 * p + 1;
        const size_t j0 = rows[t % 5] + xs[t / 5], j1 = rows[(t + 1) % 5] + xs[(t + 1) / 5];
        const float4 g0 = __ldg(guide + j0), g1 = __ldg(guide + j1);
        const uint2 r0 = ld_u2(res_in, j0), r1 = ld_u2(res_in, j1);
        const float2 f = atrous_weight2(cx, cy, cz, ncd, g0, g1);
        accumulate(f.x, r0);
        accumulate(f.y, r1);
    }
    rf0 = acc01.x; rf1 = acc01.y; rf2 = acc23.x; rf3 = acc23.y;
}

__global__ void __launch_bounds__(256, 5) atrous_kernel(int W, int H, int step, const float4* __restrict__ guide,
                                                     const uint2* __restrict__ res_in, uint2* __restrict__ res_out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    const float4 gc = __ldg(guide + i);
    float rf0, rf1, rf2, rf3;
    atrous_filter(x, y, W, H, step, guide, res_in, v3(gc.x, gc.y, gc.z), gc.w, rf0, rf1, rf2, rf3);
    const float den = gmax(kEps, rf3);
    res_out[i] = pack_h4(rf0 / den, rf1 / den, rf2 / den, 1.0f);
}

cudaError_t launch_atrous(int32_t W, int32_t H, int32_t pass, const float4* guide, const uint2* res_in,
                          uint2* res_out, cudaStream_t s, dim3 block) {
    if (block.x == 0) block = dim3(32, 8);
    dim3 grid((W + block.x - 1) / block.x, (H + block.y - 1) / block.y);
    atrous_kernel<<<grid, block, 0, s>>>(W, H, 1 << pass, guide, res_in, res_out);
    return cudaGetLastError();
}

// Final pass (final = true): the filter above, then temporal reprojection
// (vpl_pbr_gi_denoise.fs:336-429) and the composite screen + gi * illumAvg (:431).
__global__ void __launch_bounds__(256, 5) denoise_final_kernel(DenoiseLaunch d) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = d.width, H = d.height;
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    const float u = (float(x) + 0.5f) / float(W), v = (float(y) + 0.5f) / float(H);
    const float4 gc = __ldg(d.guide + i);
    const V3 centerNormal = v3(gc.x, gc.y, gc.z);
    const float centerDepth = gc.w;
    float rf0, rf1, rf2, rf3;
    atrous_filter(x, y, W, H, 1 << d.pass, d.guide, d.res_in, centerNormal, centerDepth, rf0, rf1, rf2, rf3);
    const float den = gmax(kEps, rf3);
    const V3 shadowFactor = v3(rf0 / den, rf1 / den, rf2 / den);
    if (d.res_out) d.res_out[i] = pack_h4(shadowFactor.x, shadowFactor.y, shadowFactor.z, 1.0f);
    // indirectIllumination: the gather colour output baseColor + 1e-5 as RGB16F
    const uint32_t alb = __ldg(d.cur.albedo + i);
    const V3 gi = v3(h2f(f2h(gmax(unorm8(alb, 0), 0.01f) + kEps)), h2f(f2h(gmax(unorm8(alb, 1), 0.01f) + kEps)),
                     h2f(f2h(gmax(unorm8(alb, 2), 0.01f) + kEps)));
    float s0, s1, s2, s3;
    unpack_h4(ld_u2(d.hdr_in, i), s0, s1, s2, s3);
    const V3 screen = v3(s0, s1, s2);
    const uint32_t vel = __ldg(d.cur.velocity + i);
    const float pu = u - h2f((uint16_t)(vel & 0xffffu)), pv = v - h2f((uint16_t)(vel >> 16));
    float historyAccum = h2f(__ldg(d.hist_prev + i));
    float accumMultiplier = 1.0f;
    const V3 currGi = shadowFactor;
    // previous depth, normal and GI bilinearly at the reprojected uv: one set of
    // texels and weights, each texel read once
    const Bilinear q = bilinear_at(W, H, pu, pv);
    const float* pd = d.prev_depth;
    const float prevCenterDepth = bilinear_sum(q, __ldg(pd + q.o00), __ldg(pd + q.o10), __ldg(pd + q.o01),
                                               __ldg(pd + q.o11));
    const uint32_t n00 = __ldg(d.prev_normal + q.o00), n10 = __ldg(d.prev_normal + q.o10),
                   n01 = __ldg(d.prev_normal + q.o01), n11 = __ldg(d.prev_normal + q.o11);
    V3 pnv;
    pnv.x = bilinear_sum(q, unorm8(n00, 0), unorm8(n10, 0), unorm8(n01, 0), unorm8(n11, 0));
    pnv.y = bilinear_sum(q, unorm8(n00, 1), unorm8(n10, 1), unorm8(n01, 1), unorm8(n11, 1));
    pnv.z = bilinear_sum(q, unorm8(n00, 2), unorm8(n10, 2), unorm8(n01, 2), unorm8(n11, 2));
    const V3 prevCenterNormal = normalize(pnv * 2.0f - v3s(1.0f));
    float g00[4], g10[4], g01[4], g11[4];
    unpack_h4(ld_u2(d.gi_prev, q.o00), g00[0], g00[1], g00[2], g00[3]);
    unpack_h4(ld_u2(d.gi_prev, q.o10), g10[0], g10[1], g10[2], g10[3]);
    unpack_h4(ld_u2(d.gi_prev, q.o01), g01[0], g01[1], g01[2], g01[3]);
    unpack_h4(ld_u2(d.gi_prev, q.o11), g11[0], g11[1], g11[2], g11[3]);
    const V3 prevGi = v3(bilinear_sum(q, g00[0], g10[0], g01[0], g11[0]), bilinear_sum(q, g00[1], g10[1], g01[1], g11[1]),
                         bilinear_sum(q, g00[2], g10[2], g01[2], g11[2]));
    const float currId = __ldg(d.cur.id + i);
    const float prevId = __ldg(d.prev_id + (size_t)nearest_index(pv, H) * W + nearest_index(pu, W));
    const float wn = gmax(0.0f, dot(centerNormal, prevCenterNormal));
    const float wz = expf_ieee(-gabs(centerDepth - prevCenterDepth));
    const float wid = currId != prevId ? 0.0f : 1.0f;
    float similarity = wn * wz * wid;
    if (similarity < 0.99f) { similarity = 0.0f; accumMultiplier = 0.0f; }
    historyAccum = gmin(1.0f + historyAccum * accumMultiplier, d.fps);
    const float maxAccumulationFactor = 1.0f / historyAccum;
    const V3 illumAvg = vmix(prevGi, currGi, maxAccumulationFactor);
    const V3 comb = screen + gi * illumAvg;
    d.hdr_out[i] = pack_h4(comb.x, comb.y, comb.z, 1.0f);
    d.gi_out[i] = pack_h4(illumAvg.x, illumAvg.y, illumAvg.z, 1.0f);
    d.hist_out[i] = f2h(historyAccum);
}

cudaError_t launch_denoise_final(const DenoiseLaunch& d, cudaStream_t s, dim3 block) {
    if (block.x == 0) block = dim3(32, 8);
    dim3 grid((d.width + block.x - 1) / block.x, (d.height + block.y - 1) / block.y);
    denoise_final_kernel<<<grid, block, 0, s>>>(d);
    return cudaGetLastError();
}

// ============================================================== deferred --
struct DeferredParams {
    int W, H;
    ShadeConfig sc;
    sgi_gbuffer g;
    sgi_camera cam;
    const sgi_point_light* points;
    int num_points;
    ShadowCasters casters;
    sgi_csm csm;
    uint2* out;
};

// pbr.fs:82-145: non-shadow-casting point lights + the directional light
// with its CSM (INFINITE_LIGHTING_ENABLED).
__global__ void __launch_bounds__(256, 4) deferred_pbr_csm_kernel(DeferredParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.W || y >= p.H) return;
    const size_t i = (size_t)y * p.W + x;
    ShadeParams sp{p.sc.min_roughness, p.sc.perceptual, p.sc.fog_density,
                   {p.sc.fog_color[0], p.sc.fog_color[1], p.sc.fog_color[2]}, p.sc.point_ambient};
    const float u = (float(x) + 0.5f) / float(p.W), v = (float(y) + 0.5f) / float(p.H);
    const V3 fragPos = world_from_depth(u, v, __ldg(p.g.depth + i), p.cam.inv_proj_view);
    const V3 viewPos = v3(p.cam.view_position[0], p.cam.view_position[1], p.cam.view_position[2]);
    const V3 viewMinusFrag = viewPos - fragPos;
    const V3 viewDir = normalize(viewMinusFrag);
    const float viewDist = length(viewMinusFrag);
    const uint32_t alb = __ldg(p.g.albedo + i);
    const V3 baseColor = v3(unorm8(alb, 0), unorm8(alb, 1), unorm8(alb, 2));
    const float albedoA = unorm8(alb, 3);
    const V3 normal = decode_normal(__ldg(p.g.normal + i));
    const uint32_t rma = __ldg(p.g.roughness_metallic_ambient + i);
    const float roughness = unorm8(rma, 0), metallic = unorm8(rma, 1), rmeB = unorm8(rma, 2);
    const float ambient = h2f(__ldg(p.g.ssao + i));
    const uint32_t br = __ldg(p.g.base_reflectivity + i);
    const float reflR = float(br & 0xffu) / 255.0f, reflG = float(br >> 8) / 255.0f;
    const V3 emissive = v3(albedoA, reflG, rmeB);
    V3 color = v3s(0.0f);
    for (int l = 0; l < p.num_points; ++l) {
        const float4* rec = reinterpret_cast<const float4*>(p.points + l);
        const float4 lp4 = __ldg(rec), lc4 = __ldg(rec + 1), m4 = __ldg(rec + 2);
        const V3 lp = v3(lp4.x, lp4.y, lp4.z), lc = v3(lc4.x, lc4.y, lc4.z);
        const float distance = length(lp - fragPos);
        if (distance < m4.x) {
            // calculatePointLighting2, pbr2.glsl:593-611
            const V3 lightDir = lp - fragPos;
            color = color + lighting_burley(lc, lightDir, viewDir, normal, baseColor, viewDist, length(lc) / 12.0f,
                                            roughness, metallic, ambient, 1.0f - 0.0f, v3s(reflR),
                                            quadratic_atten(lightDir), sp.point_ambient, sp);
        }
    }
    // shadowCasters, pbr.fs:116-131
    for (int l = 0; l < p.casters.count; ++l) {
        const float4* rec = reinterpret_cast<const float4*>(p.casters.lights + l);
        const float4 lp4 = __ldg(rec), lc4 = __ldg(rec + 1), m4 = __ldg(rec + 2);
        const V3 lp = v3(lp4.x, lp4.y, lp4.z), lc = v3(lc4.x, lc4.y, lc4.z);
        const float distance = length(lp - fragPos);
        if (distance < m4.x) {
            float shadowFactor = 0.0f;
            const sgi_atlas_entry entry = p.casters.entries[l];
            if (viewDist < 150.0f)
                shadowFactor = shadow_8samples(p.casters.atlas, entry, m4.y, fragPos, lp, dot(lp - fragPos, normal), 0.03f);
            else if (viewDist < 750.0f)
                shadowFactor = shadow_1sample(p.casters.atlas, entry, m4.y, fragPos, lp, dot(lp - fragPos, normal), 0.03f);
            const V3 lightDir = lp - fragPos;
            color = color + lighting_burley(lc, lightDir, viewDir, normal, baseColor, viewDist, length(lc) / 12.0f,
                                            roughness, metallic, ambient, 1.0f - shadowFactor, v3s(reflR),
                                            quadratic_atten(lightDir), sp.point_ambient, sp);
        }
    }
    const V3 lightDir = v3(p.csm.light_direction[0], p.csm.light_direction[1], p.csm.light_direction[2]);
    const V3 lightColor = v3(p.csm.light_color[0], p.csm.light_color[1], p.csm.light_color[2]);
    const float shadowFactor = infinite_shadow(p.csm, fragPos, normal, true);
    // calculateDirectionalLighting, pbr2.glsl:576-591, called with 1 - shadowFactor
    color = color + lighting_burley(lightColor, lightDir, viewDir, normal, baseColor, viewDist, 0.0f, roughness,
                                    metallic, ambient, 1.0f - (1.0f - shadowFactor), v3s(reflR), 1.0f, 0.0f, sp);
    const V3 o = vmin(color + emissive * p.sc.emission_strength, kHalfMax);
    p.out[i] = pack_h4(o.x, o.y, o.z, 1.0f);
}

cudaError_t launch_deferred(const sgi_config& cfg, const ShadeConfig& sc, const sgi_gbuffer& g,
                            const sgi_camera& cam, const sgi_point_light* points, int32_t num_points,
                            const ShadowCasters& casters, const sgi_csm& csm, uint2* hdr_out, cudaStream_t s,
                            dim3 block) {
    DeferredParams p;
    p.W = cfg.width; p.H = cfg.height; p.sc = sc; p.g = g; p.cam = cam; p.points = points;
    p.num_points = num_points; p.casters = casters; p.csm = csm; p.out = hdr_out;
    if (block.x == 0) block = dim3(32, 8);
    dim3 grid((cfg.width + block.x - 1) / block.x, (cfg.height + block.y - 1) / block.y);
    deferred_pbr_csm_kernel<<<grid, block, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace sgi
