// sgi_shade.cu - the shading kernels of the GI/lighting hot path on sm_103a:
//   vpl_gather        vpl_pbr_gi.fs:81-207 (+ denoise pass 0, the reservoir merge)
//   gi_target         the converged K-sample target (no reference counterpart)
//   atrous            vpl_pbr_gi_denoise.fs:142-327 (passes 1 .. n-2)
//   denoise_final     vpl_pbr_gi_denoise.fs:275-435 (last pass: filter, temporal, composite)
//   deferred_pbr_csm  pbr.fs:82-145 (+ pbr.glsl:158-227)
//
// This file is compiled twice into the library:
//   * as sgi_shade.cu with -fmad=false -prec-div=true -prec-sqrt=true: every
//     operation rounds as the CPU restatement of the shaders rounds, so the
//     results are bit-identical to it (namespace sgi::exact);
//   * through sgi_shade_fast.cu with SGI_FAST_MATH = 1 and contraction,
//     approximate division and square root, hardware reciprocal square root and
//     exponential (namespace sgi::fast): the tolerance mode, within 1e-3
//     relative error of the restatement outside the decision margins.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <cstring>
#include <mutex>

#include "sgi_cull.cuh"
#include "sgi_internal.h"
#include "sgi_math.cuh"
#include "sgi_shade_common.cuh"

#ifndef SGI_FAST_MATH
#define SGI_FAST_MATH 0
#endif
#if SGI_FAST_MATH
#define SGI_SHADE_NS fast
#else
#define SGI_SHADE_NS exact
#endif

namespace sgi {
namespace SGI_SHADE_NS {

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
    const float u = xdiv(float(x) + 0.5f, float(p.W)), v = xdiv(float(y) + 0.5f, float(p.H));
    px.fragPos = world_from_depth(u, v, __ldg(p.g.depth + i), p.cam.inv_proj_view);
    const V3 viewPos = v3(p.cam.view_position[0], p.cam.view_position[1], p.cam.view_position[2]);
    px.viewDir = normalize(viewPos - px.fragPos);
    px.distToCamera = xlength(xsub3(viewPos, px.fragPos));   // decides the shadow test and the sample count
    const uint32_t alb = __ldg(p.g.albedo + i);
    px.baseColor = v3(gmax(unorm8(alb, 0), 0.01f), gmax(unorm8(alb, 1), 0.01f), gmax(unorm8(alb, 2), 0.01f));
    px.normal = decode_normal(__ldg(p.g.normal + i));
    const uint32_t rma = __ldg(p.g.roughness_metallic_ambient + i);
    px.roughness = gmax(0.5f, unorm8(rma, 0));
    px.metallic = unorm8(rma, 1);
    px.ao = gclamp(h2f(__ldg(p.g.ssao + i)), 0.35f, 1.0f);
    px.ambient = unorm8(rma, 2);
    px.baseRefl = v3s(float(__ldg(p.g.base_reflectivity + i) & 0xffu) / 255.0f);
    const float roughnessWeight = xsub(1.0f, px.roughness);
    const float distRatio = gmin(xsub(1.0f, xdiv(px.distToCamera, 1000.0f)), 1.0f);
    if (p.spp > 0) {
        px.sampleCount = p.spp;
    } else {
        int maxSamplesPerPixel = (int)xmixf(2.0f, 10.0f, roughnessWeight);
        int samplesMax = (int)xmul(float(maxSamplesPerPixel), distRatio);
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

// A tile's VPL list staged in shared memory: the records and atlas slots of its
// L nearest VPLs, in list order. Used when a gather block covers exactly one
// tile (block = tile_size x tile_size), so that every sample of the block reads
// its VPL from shared memory instead of the compacted buffers in L2.
struct StagedList {
    float4 rec[SGI_MAX_TILE_LIST][4];   // position, colour, specular position, (radius, far, intensity, -)
    sgi_atlas_entry ent[SGI_MAX_TILE_LIST];
};

// dot(normal, normalize(lmf)) < 0 (vpl_pbr_gi.fs:171-172), evaluated as the
// shader evaluates it, but decided from the unnormalised product when its sign
// is certain: the dot product of the normalised vector is r * dot(N, lmf) with
// r = 1 / length(lmf) > 0 plus rounding errors below 4u r B (u = 2^-24,
// B = sum |N_i lmf_i|), and the rounded unnormalised product differs from the
// exact one by less than 3u B, so |dot(N, lmf)| > 2^-16 B fixes the sign of
// both. The guards keep every quantity normal and finite (no overflow of the
// length, no subnormal products); otherwise the full evaluation decides.
SGI_D bool side_negative(V3 N, V3 lmf) {
    const float d2 = xdot(lmf, lmf);
    const float du = xdot(N, lmf);
    const float b = __fmaf_rn(gabs(N.z), gabs(lmf.z), __fmaf_rn(gabs(N.y), gabs(lmf.y), xmul(gabs(N.x), gabs(lmf.x))));
    if (d2 >= 0x1p-100f && d2 <= 0x1p100f && b >= 0x1p-40f && b <= 0x1p100f && gabs(du) > xmul(b, 0x1p-16f))
        return du < 0.0f;
    return xdot(N, xnormalize(lmf)) < 0.0f;
}

// The sample loop of vpl_pbr_gi.fs:148-200 with the seed z starting at seedZ.
// kStaged: the list of the pixel's tile is in `staged` (list slot = array index).
template <bool kStaged>
SGI_D void sample_vpls(const GatherParams& p, const PixelShade& px, float seedX, float seedY, float seedZ,
                       V3& vplColor, float& validSamples, const StagedList* staged = nullptr) {
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
        float4 pos, col, spec, misc;
        sgi_atlas_entry entry;
        if (kStaged) {
            const int r = (int)xmul(float(candidates), rnd);
            const int slot = r < candidates - 1 ? r : candidates - 1;
            pos = staged->rec[slot][0];
            col = staged->rec[slot][1];
            spec = staged->rec[slot][2];
            misc = staged->rec[slot][3];
            entry = staged->ent[slot];
        } else {
            int lightIndex;
            if (px.list) {
                int r = (int)xmul(float(candidates), rnd);
                lightIndex = __ldg(px.list + 1 + (r < candidates - 1 ? r : candidates - 1));
            } else {
                lightIndex = (int)xmul(float(candidates - 1), rnd);
            }
            const float4* rec = reinterpret_cast<const float4*>(p.cv + lightIndex);
            pos = __ldg(rec);
            col = __ldg(rec + 1);
            spec = __ldg(rec + 2);
            misc = __ldg(rec + 3);   // radius, farPlane, intensity
            entry = p.ce[lightIndex];
        }
        const V3 lightPosition = v3(pos.x, pos.y, pos.z);
        const V3 lmf = xsub3(lightPosition, fragPos);
        const float lightRadius = misc.x;
        const float distance = xlength(lmf);
        if (resamples < 5) {
            if (side_negative(normal, lmf) || distance > lightRadius) { ++resamples; --s; continue; }
        }
        const float distanceRatio = gclamp((2.0f * distance) / lightRadius, 0.0f, 1.0f);
        const float distAttenuation = distanceRatio;
        const V3 lightColor = v3(col.x, col.y, col.z);
        // fragPos - lightPosition is -lmf exactly (a rounded difference changes sign with its operands),
        // so its length is `distance`
        float shadowFactor = px.distToCamera < 500.0f
                                 ? shadow_1sample_dir(p.cubes, entry, misc.y, v3(-lmf.x, -lmf.y, -lmf.z), distance,
                                                      xdot(lmf, normal), 0.1f)
                                 : 0.0f;
        shadowFactor = gmin(shadowFactor, mixf(minGi, 1.0f, distanceRatio));
        float reweight = 1.0f;
        if (shadowFactor > 0.0f) reweight = (1.0f - distAttenuation) * minGi + distAttenuation;
        validSamples += reweight;
        const V3 tmp = px.ao * vpl_lighting2_sample(vp, v3(spec.x, spec.y, spec.z), lightPosition, lightColor,
                                                    lightRadius, distance);
        vplColor = vplColor + (1.0f - shadowFactor) * tmp;
    }
}

// The block's tile list into shared memory (the block is tile `tile`).
SGI_D void stage_tile_list(const GatherParams& p, int tile, StagedList* staged, int tid, int nthreads) {
    const int32_t* list = p.lists + (size_t)tile * (1 + p.L);
    const int count = __ldg(list);
    for (int j = tid; j < count * 4; j += nthreads) {
        const int idx = __ldg(list + 1 + (j >> 2));
        staged->rec[j >> 2][j & 3] = __ldg(reinterpret_cast<const float4*>(p.cv + idx) + (j & 3));
    }
    for (int j = tid; j < count; j += nthreads) staged->ent[j] = p.ce[__ldg(list + 1 + j)];
}

// vpl_pbr_gi.fs:81-207 for pixel (x, y) inside the image, with denoise pass 0
// and the guide in its epilogue.
template <bool kStaged>
SGI_D void gather_pixel(const GatherParams& p, int x, int y, const StagedList* staged) {
    const size_t i = (size_t)y * p.W + x;
    const PixelShade px = load_pixel(p, x, y, i);
    const V3 normal = px.normal;
    const float seedX = float(x) + 0.5f, seedY = float(y) + 0.5f;
    V3 vplColor;
    float validSamples;
    sample_vpls<kStaged>(p, px, seedX, seedY, p.time, vplColor, validSamples, staged);
    validSamples = gmax(validSamples, 1.0f);
    const V3 b = vmin(vplColor, kHalfMax);
    // The reservoir as stored in its RGBA16F target (vpl_pbr_gi.fs:205).
    const float r0 = h2f(f2h(b.x)), r1 = h2f(f2h(b.y)), r2 = h2f(f2h(b.z)), r3 = h2f(f2h(validSamples));
    if (p.out.raw) p.out.raw[i] = pack_h4(r0, r1, r2, r3);
    // Denoise pass 0 for this pixel: computeMergedReservoir with minmaxNearest = 0
    // (vpl_pbr_gi_denoise.fs:192-273) reads only the centre texel, which is this one.
    const float depth = __ldg(p.g.depth + i);
    float cr0 = 0.0f, cr1 = 0.0f, cr2 = 0.0f, cr3 = 0.0f;
    float runningSum = 0.0f;
    const float probabilisticWeight = 1.0f / float(__ldg(p.visible_index));
    if (!(xdot(normal, normal) < 0.906f)) {
        if (!(gabs(xsub(depth, depth)) > xmul(0.1f, depth))) {
            const float randUpdate = random3(seedX, seedY, p.time);
            const float probability = r3 * probabilisticWeight;
            cr3 = xadd(cr3, probability);
            if (randUpdate < xdiv(probability, cr3)) {
                cr0 += r0; cr1 += r1; cr2 += r2;
                runningSum += r3;
            }
        }
    }
    const float den = gmax(kEps, runningSum);
    p.out.merged[i] = pack_h4(cr0 / den, cr1 / den, cr2 / den, 1.0f);
    p.out.guide[i] = make_float4(normal.x, normal.y, normal.z, depth);
}

// one thread per pixel; kStaged: the block is one tile and first stages the
// tile's list (StagedList, dynamic shared memory)
template <bool kStaged>
__global__ void __launch_bounds__(256, 4) vpl_gather_kernel(GatherParams p) {
    extern __shared__ float4 gather_smem[];
    StagedList* staged = reinterpret_cast<StagedList*>(gather_smem);
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (kStaged) {
        stage_tile_list(p, blockIdx.y * p.tiles_x + blockIdx.x, staged, threadIdx.y * blockDim.x + threadIdx.x,
                        blockDim.x * blockDim.y);
        __syncthreads();
    }
    if (x >= p.W || y >= p.H) return;
    gather_pixel<kStaged>(p, x, y, staged);
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
    // a block that is exactly one tile stages the tile's list in shared memory
    const bool staged = p.tiled && (int)block.x == cfg.tile_size && (int)block.y == cfg.tile_size;
    if (staged)
        vpl_gather_kernel<true><<<grid, block, sizeof(StagedList), s>>>(p);
    else
        vpl_gather_kernel<false><<<grid, block, 0, s>>>(p);
    return cudaGetLastError();
}

#if !SGI_FAST_MATH
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
        sample_vpls<false>(p, px, seedX, seedY, p.time + float(b) * 200000.0f, col, valid);
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
#endif  // !SGI_FAST_MATH

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
//
// The arithmetic takes its taps from two functors, guide_at(t) and res_at(t)
// for tap t = 5 * (dx + 2) + (dy + 2), so that the direct kernel (taps read
// from global memory, coordinates clamped per tap) and the staged kernel (taps
// read from a shared-memory lattice) run the same operations in the same order.
template <class GuideAt, class ResAt>
SGI_D void atrous_taps(GuideAt guide_at, ResAt res_at, V3 cn, float cd, float& rf0, float& rf1, float& rf2,
                       float& rf3) {
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
        if (p == 6) accumulate(1.0f, res_at(12));   // the centre tap, weight 1
        const int t = p < 6 ? 2 * p : 2 * p + 1;
        const float4 g0 = guide_at(t), g1 = guide_at(t + 1);
        const uint2 r0 = res_at(t), r1 = res_at(t + 1);
        const float2 f = atrous_weight2(cx, cy, cz, ncd, g0, g1);
        accumulate(f.x, r0);
        accumulate(f.y, r1);
    }
    rf0 = acc01.x; rf1 = acc01.y; rf2 = acc23.x; rf3 = acc23.y;
}

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
    atrous_taps([&](int t) { return __ldg(guide + rows[t % 5] + xs[t / 5]); },
                [&](int t) { return ld_u2(res_in, rows[t % 5] + xs[t / 5]); }, cn, cd, rf0, rf1, rf2, rf3);
}

SGI_D void atrous_pixel(int W, int H, int step, const float4* __restrict__ guide, const uint2* __restrict__ res_in,
                        uint2* __restrict__ res_out, int x, int y) {
    const size_t i = (size_t)y * W + x;
    const float4 gc = __ldg(guide + i);
    float rf0, rf1, rf2, rf3;
    atrous_filter(x, y, W, H, step, guide, res_in, v3(gc.x, gc.y, gc.z), gc.w, rf0, rf1, rf2, rf3);
    const float den = gmax(kEps, rf3);
    res_out[i] = pack_h4(rf0 / den, rf1 / den, rf2 / den, 1.0f);
}

__global__ void __launch_bounds__(256, 5) atrous_kernel(int W, int H, int step, const float4* __restrict__ guide,
                                                     const uint2* __restrict__ res_in, uint2* __restrict__ res_out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x < W && y < H) atrous_pixel(W, H, step, guide, res_in, res_out, x, y);
}

cudaError_t launch_atrous(int32_t W, int32_t H, int32_t pass, const float4* guide, const uint2* res_in,
                          uint2* res_out, cudaStream_t s, dim3 block) {
    if (block.x == 0) block = dim3(32, 8);
    dim3 grid((W + block.x - 1) / block.x, (H + block.y - 1) / block.y);
    atrous_kernel<<<grid, block, 0, s>>>(W, H, 1 << pass, guide, res_in, res_out);
    return cudaGetLastError();
}

// ------------------------------------------------- staged a-trous pass --
// At stride s the taps of pixel (x, y) are the pixels (x + i s, y + j s): the
// pixels whose coordinates leave the remainders (x mod s, y mod s) form a
// lattice on which the pass is a plain 5x5 stencil. A CTA of the staged kernel
// takes a 16 x 8 patch of two neighbouring lattices (x remainders 2k and
// 2k + 1, one lane each of a lane pair, so that a warp's shared-memory reads
// are contiguous) and stages the 20 x 12 lattice points its taps reach, as
// pixel pairs, with two TMA loads (guide and reservoir) whose traversal
// strides are s / 2 pixel pairs in x and s rows in y. Lattice points outside
// the image are filled by the copy with zeros and then replaced with the
// clamped pixel's values (plain loads, only in CTAs at the image border), so
// every tap reads what the direct kernel's clamped tap reads, and the
// arithmetic (atrous_taps) is the same: the results are bit-identical.
//
// Conditions (otherwise the caller runs the direct kernel): s = 2, 4 or 8
// (the copy's traversal stride is at most 8), an even width (pixel pairs; the
// reservoir's rows are then multiples of 16 bytes) and 16-byte aligned
// buffers. The wait for the copies is bounded: after `wait_ns` the CTA sets
// SGI_ERR_TIMEOUT in `status` and returns without writing. `skip_copies` (a test switch) issues no copy, so a
// wait runs out with nothing in flight.
constexpr int kLatX = 16, kLatY = 8, kLatHX = kLatX + 4, kLatHY = kLatY + 4;

struct AtrousStageWait {
    long long wait_ns;
    int32_t skip_copies;
    int32_t* status;
};

SGI_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

SGI_D bool stage_wait(uint32_t bar, uint32_t parity, const AtrousStageWait& w) {
    uint32_t done = 0;
    const long long t0 = global_ns();
    for (;;) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 20000;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > w.wait_ns) {
            atomicCAS(w.status, SGI_OK, SGI_ERR_TIMEOUT);
            return false;
        }
    }
}

// One CTA of the staged pass (256 threads): lattice patch (bx, by) of the grid
// (ntx * s / 2, nty * s). `bar` is an initialised mbarrier of this CTA whose
// phase `parity` the copies complete. Returns false (nothing written) when the
// wait ran out. The stand-alone kernel below and the persistent multi-view
// kernel (sgi_persistent.cuh) run it.
SGI_D bool atrous_staged_cta(const CUtensorMap* gmap, const CUtensorMap* rmap, int W, int H, int s, int ntx, int nty,
                             int bx, int by, const float4* __restrict__ guide, const uint2* __restrict__ res_in,
                             uint2* __restrict__ res_out, uint32_t bar, uint32_t parity, const AtrousStageWait& wt) {
    __shared__ __align__(128) float4 sg[kLatHY][kLatHX][2];
    __shared__ __align__(128) uint2 sr[kLatHY][kLatHX][2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tqx = bx % ntx, rp = bx / ntx;
    const int tqy = by % nty, ry = by / nty;
    const int qx0 = tqx * kLatX, qy0 = tqy * kLatY, rx = 2 * rp;
    if (tid == 0 && !wt.skip_copies) {
        constexpr uint32_t kBytes = sizeof(sg) + sizeof(sr);
        // the block's earlier accesses of sg / sr (a previous use) before the copies overwrite them
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(kBytes) : "memory");
        const int c1 = rp + (s >> 1) * (qx0 - 2), c2 = ry + s * (qy0 - 2);
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];\n" ::"r"(smem_u32(sg)),
            "l"(reinterpret_cast<uint64_t>(gmap)), "r"(0), "r"(c1), "r"(c2), "r"(bar)
            : "memory");
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];\n" ::"r"(smem_u32(sr)),
            "l"(reinterpret_cast<uint64_t>(rmap)), "r"(0), "r"(c1), "r"(c2), "r"(bar)
            : "memory");
    }
    const bool ok = __syncthreads_and(stage_wait(bar, parity, wt));
    if (!ok) return false;
    // lattice points outside the image: the clamped pixel's values (CTA-uniform test)
    if (qx0 < 2 || qy0 < 2 || rx + s * (qx0 + kLatHX - 3) >= W || ry + s * (qy0 + kLatHY - 3) >= H) {
        for (int e = tid; e < kLatHX * kLatHY; e += blockDim.x) {
            const int ex = e % kLatHX, ey = e / kLatHX;
            const int x0 = rx + s * (qx0 - 2 + ex), y = ry + s * (qy0 - 2 + ey);
            if (x0 >= 0 && x0 < W && y >= 0 && y < H) continue;   // x0 even, W even: x0 + 1 < W too
            const size_t row = (size_t)(y < 0 ? 0 : (y > H - 1 ? H - 1 : y)) * W;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int xx = x0 + h, cx = xx < 0 ? 0 : (xx > W - 1 ? W - 1 : xx);
                sg[ey][ex][h] = __ldg(guide + row + cx);
                sr[ey][ex][h] = ld_u2(res_in, row + cx);
            }
        }
    }
    __syncthreads();   // fix-ups written; also orders this use's reads before the next use's copies
    const int lx = lane >> 1, h = lane & 1, ly = warp;
    const int x = rx + h + s * (qx0 + lx), y = ry + s * (qy0 + ly);
    if (x < W && y < H) {
        const float4 gc = sg[ly + 2][lx + 2][h];
        float rf0, rf1, rf2, rf3;
        atrous_taps([&](int t) { return sg[ly + t % 5][lx + t / 5][h]; },
                    [&](int t) { return sr[ly + t % 5][lx + t / 5][h]; }, v3(gc.x, gc.y, gc.z), gc.w, rf0, rf1,
                    rf2, rf3);
        const float den = gmax(kEps, rf3);
        res_out[(size_t)y * W + x] = pack_h4(rf0 / den, rf1 / den, rf2 / den, 1.0f);
    }
    return true;
}

SGI_D void stage_barrier_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__global__ void __launch_bounds__(256, 5) atrous_staged_kernel(const __grid_constant__ CUtensorMap gmap,
                                                             const __grid_constant__ CUtensorMap rmap, int W,
                                                             int H, int s, int ntx, int nty,
                                                             const float4* __restrict__ guide,
                                                             const uint2* __restrict__ res_in,
                                                             uint2* __restrict__ res_out, AtrousStageWait wt) {
    __shared__ __align__(8) unsigned long long bar;
    const uint32_t b = smem_u32(&bar);
    if (threadIdx.x == 0) stage_barrier_init(b);
    __syncthreads();
    atrous_staged_cta(&gmap, &rmap, W, H, s, ntx, nty, blockIdx.x, blockIdx.y, guide, res_in, res_out, b, 0u, wt);
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// The two tensor maps of the staged pass at stride 2^pass over `guide` and `res_in` (pixel-pair views).
static cudaError_t encode_atrous_maps(int W, int H, int pass, const float4* guide, const uint2* res_in,
                                      CUtensorMap* gm, CUtensorMap* rm) {
    const int st = 1 << pass;
    auto encode = tensor_map_encoder();
    if (!encode) return cudaErrorNotSupported;
    const cuuint64_t dim[3] = {8, (cuuint64_t)W / 2, (cuuint64_t)H};
    const cuuint32_t box[3] = {8, (cuuint32_t)(kLatHX * st / 2), (cuuint32_t)(kLatHY * st)};
    const cuuint32_t stride[3] = {1, (cuuint32_t)(st / 2), (cuuint32_t)st};
    const cuuint64_t gstr[2] = {32, (cuuint64_t)W * 16};
    const cuuint64_t rstr[2] = {16, (cuuint64_t)W * 8};
    const bool ok = encode(gm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)guide, dim, gstr, box, stride,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS &&
                    encode(rm, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, (void*)res_in, dim, rstr, box, stride,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    return ok ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_atrous_staged(int32_t W, int32_t H, int32_t pass, const float4* guide, const uint2* res_in,
                                 uint2* res_out, long long wait_ns, int32_t skip_copies, int32_t* status,
                                 cudaStream_t s) {
    const int st = pass >= 1 && pass <= 3 ? 1 << pass : 0;
    if (!st || W < 2 || (W & 1) || H < 1 || ((uintptr_t)guide & 15) || ((uintptr_t)res_in & 15) || !status)
        return cudaErrorNotSupported;
    CUtensorMap gm, rm;
    const cudaError_t e = encode_atrous_maps(W, H, pass, guide, res_in, &gm, &rm);
    if (e != cudaSuccess) return e;
    int gx, gy, ntx, nty;
    atrous_lattice_grid(W, H, pass, &gx, &gy, &ntx, &nty);
    const AtrousStageWait wt{wait_ns > 0 ? wait_ns : 200000000LL, skip_copies, status};
    atrous_staged_kernel<<<dim3(gx, gy), 256, 0, s>>>(gm, rm, W, H, st, ntx, nty, guide, res_in, res_out, wt);
    return cudaGetLastError();
}

// Final pass (final = true): the filter above, then temporal reprojection
// (vpl_pbr_gi_denoise.fs:336-429) and the composite screen + gi * illumAvg (:431).
SGI_D void denoise_final_pixel(const DenoiseLaunch& d, int x, int y) {
    const int W = d.width, H = d.height;
    const size_t i = (size_t)y * W + x;
    const float u = xdiv(float(x) + 0.5f, float(W)), v = xdiv(float(y) + 0.5f, float(H));
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
    const float pu = xsub(u, h2f((uint16_t)(vel & 0xffffu))), pv = xsub(v, h2f((uint16_t)(vel >> 16)));
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
    const V3 prevCenterNormal = xnormalize(xsub3(xmul3(pnv, 2.0f), v3s(1.0f)));
    float g00[4], g10[4], g01[4], g11[4];
    unpack_h4(ld_u2(d.gi_prev, q.o00), g00[0], g00[1], g00[2], g00[3]);
    unpack_h4(ld_u2(d.gi_prev, q.o10), g10[0], g10[1], g10[2], g10[3]);
    unpack_h4(ld_u2(d.gi_prev, q.o01), g01[0], g01[1], g01[2], g01[3]);
    unpack_h4(ld_u2(d.gi_prev, q.o11), g11[0], g11[1], g11[2], g11[3]);
    const V3 prevGi = v3(bilinear_sum(q, g00[0], g10[0], g01[0], g11[0]), bilinear_sum(q, g00[1], g10[1], g01[1], g11[1]),
                         bilinear_sum(q, g00[2], g10[2], g01[2], g11[2]));
    const float currId = __ldg(d.cur.id + i);
    const float prevId = __ldg(d.prev_id + (size_t)nearest_index(pv, H) * W + nearest_index(pu, W));
    // the temporal decision: similarity against 0.99, exact in both builds
    const float wn = gmax(0.0f, xdot(centerNormal, prevCenterNormal));
    const float wz = expf_exact_near0(-gabs(xsub(centerDepth, prevCenterDepth)));
    const float wid = currId != prevId ? 0.0f : 1.0f;
    float similarity = xmul(xmul(wn, wz), wid);
    if (similarity < 0.99f) { similarity = 0.0f; accumMultiplier = 0.0f; }
    historyAccum = gmin(xadd(1.0f, xmul(historyAccum, accumMultiplier)), d.fps);
    const float maxAccumulationFactor = 1.0f / historyAccum;
    const V3 illumAvg = vmix(prevGi, currGi, maxAccumulationFactor);
    const V3 comb = screen + gi * illumAvg;
    d.hdr_out[i] = pack_h4(comb.x, comb.y, comb.z, 1.0f);
    d.gi_out[i] = pack_h4(illumAvg.x, illumAvg.y, illumAvg.z, 1.0f);
    d.hist_out[i] = f2h(historyAccum);
}

__global__ void __launch_bounds__(256, 5) denoise_final_kernel(DenoiseLaunch d) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x < d.width && y < d.height) denoise_final_pixel(d, x, y);
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
// Per-light constants of a block: the fog intensity length(colour) / 12 of
// the first kLightConst point lights and shadow casters (the same operations
// as per pixel, once per block).
constexpr int kLightConst = 32;
struct LightConst {
    float point_fog[kLightConst], caster_fog[kLightConst];
    int points, casters;   // how many of each are held
};
SGI_D void light_const_fill(const DeferredParams& p, LightConst& lc, int tid, int nthreads) {
    const int np = p.num_points < kLightConst ? p.num_points : kLightConst;
    const int nc = p.casters.count < kLightConst ? p.casters.count : kLightConst;
    for (int l = tid; l < np + nc; l += nthreads) {
        const bool caster = l >= np;
        const float4 c4 = __ldg(reinterpret_cast<const float4*>(caster ? p.casters.lights + (l - np) : p.points + l) + 1);
        const float f = length(v3(c4.x, c4.y, c4.z)) / 12.0f;
        if (caster) lc.caster_fog[l - np] = f;
        else lc.point_fog[l] = f;
    }
    if (tid == 0) { lc.points = np; lc.casters = nc; }
}

SGI_D void deferred_pixel(const DeferredParams& p, int x, int y, const LightConst* lcs = nullptr) {
    const size_t i = (size_t)y * p.W + x;
    ShadeParams sp{p.sc.min_roughness, p.sc.perceptual, p.sc.fog_density,
                   {p.sc.fog_color[0], p.sc.fog_color[1], p.sc.fog_color[2]}, p.sc.point_ambient};
    const float u = xdiv(float(x) + 0.5f, float(p.W)), v = xdiv(float(y) + 0.5f, float(p.H));
    const V3 fragPos = world_from_depth(u, v, __ldg(p.g.depth + i), p.cam.inv_proj_view);
    const V3 viewPos = v3(p.cam.view_position[0], p.cam.view_position[1], p.cam.view_position[2]);
    const V3 viewMinusFrag = xsub3(viewPos, fragPos);
    const V3 viewDir = normalize(viewMinusFrag);
    const float viewDist = xlength(viewMinusFrag);   // decides the caster shadow quality
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
    const BurleyPixel bp = burley_pixel(baseColor, v3s(reflR), roughness, metallic, viewDist, normal, viewDir, sp);
    V3 color = v3s(0.0f);
    for (int l = 0; l < p.num_points; ++l) {
        const float4* rec = reinterpret_cast<const float4*>(p.points + l);
        const float4 lp4 = __ldg(rec), lc4 = __ldg(rec + 1), m4 = __ldg(rec + 2);
        const V3 lp = v3(lp4.x, lp4.y, lp4.z), lc = v3(lc4.x, lc4.y, lc4.z);
        const float distance = xlength(xsub3(lp, fragPos));
        if (distance < m4.x) {
            // calculatePointLighting2, pbr2.glsl:593-611; |lightDir| is `distance`
            const V3 lightDir = lp - fragPos;
            const float fog = lcs && l < lcs->points ? lcs->point_fog[l] : length(lc) / 12.0f;
            color = color + lighting_burley_pxl(bp, lc, lightDir, distance, viewDir, normal, fog, ambient,
                                                1.0f - 0.0f, quadratic_atten_len(distance), sp.point_ambient, sp);
        }
    }
    // shadowCasters, pbr.fs:116-131
    for (int l = 0; l < p.casters.count; ++l) {
        const float4* rec = reinterpret_cast<const float4*>(p.casters.lights + l);
        const float4 lp4 = __ldg(rec), lc4 = __ldg(rec + 1), m4 = __ldg(rec + 2);
        const V3 lp = v3(lp4.x, lp4.y, lp4.z), lc = v3(lc4.x, lc4.y, lc4.z);
        const float distance = xlength(xsub3(lp, fragPos));
        if (distance < m4.x) {
            float shadowFactor = 0.0f;
            const sgi_atlas_entry entry = p.casters.entries[l];
            if (viewDist < 150.0f)
                shadowFactor = shadow_8samples(p.casters.atlas, entry, m4.y, fragPos, lp, xdot(xsub3(lp, fragPos), normal),
                                               0.03f);
            else if (viewDist < 750.0f)
                shadowFactor = shadow_1sample(p.casters.atlas, entry, m4.y, fragPos, lp, xdot(xsub3(lp, fragPos), normal),
                                              0.03f);
            const V3 lightDir = lp - fragPos;
            const float fog = lcs && l < lcs->casters ? lcs->caster_fog[l] : length(lc) / 12.0f;
            color = color + lighting_burley_pxl(bp, lc, lightDir, distance, viewDir, normal, fog, ambient,
                                                1.0f - shadowFactor, quadratic_atten_len(distance), sp.point_ambient,
                                                sp);
        }
    }
    const V3 lightDir = v3(p.csm.light_direction[0], p.csm.light_direction[1], p.csm.light_direction[2]);
    const V3 lightColor = v3(p.csm.light_color[0], p.csm.light_color[1], p.csm.light_color[2]);
    const float shadowFactor = infinite_shadow(p.csm, fragPos, normal, true);
    // calculateDirectionalLighting, pbr2.glsl:576-591, called with 1 - shadowFactor
    color = color + lighting_burley_px(bp, lightColor, lightDir, viewDir, normal, 0.0f, ambient,
                                       1.0f - (1.0f - shadowFactor), 1.0f, 0.0f, sp);
    const V3 o = vmin(color + emissive * p.sc.emission_strength, kHalfMax);
    p.out[i] = pack_h4(o.x, o.y, o.z, 1.0f);
}

__global__ void __launch_bounds__(256, 4) deferred_pbr_csm_kernel(DeferredParams p) {
    __shared__ LightConst lcs;
    light_const_fill(p, lcs, threadIdx.y * blockDim.x + threadIdx.x, blockDim.x * blockDim.y);
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x < p.W && y < p.H) deferred_pixel(p, x, y, &lcs);
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

// the persistent multi-view frame over the passes above
#include "sgi_persistent.cuh"

}  // namespace SGI_SHADE_NS
}  // namespace sgi
