// oracle/passes.hpp - TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// Per-pixel / per-tile / per-VPL restatements of the StratusGFX passes on the
// GI/lighting hot path, following the shader sources line by line (paths
// relative to the StratusGFX project root). Parity is UNPINNED by the
// reference (no golden vectors exist; GLSL cannot run here).
//
// Texture-sampling conventions this build defines (GL leaves them to the
// driver or the texture unit):
//   - a sample at a pixel centre, or at a centre plus an integer texel offset,
//     reads that texel exactly (LINEAR or NEAREST alike), clamped to the edge;
//   - bilinear (LINEAR) at an arbitrary uv: u = s*W - 0.5, i0 = floor(u),
//     a = u - i0, weights (1-a)(1-b), a(1-b), (1-a)b, ab accumulated in that
//     order, CLAMP_TO_EDGE, full FP32 weights;
//   - NEAREST at an arbitrary uv: texel floor(s*W), clamped;
//   - sampler2DArrayShadow LINEAR + LEQUAL: the same bilinear weights applied
//     to the four 0/1 results of (ref <= texel);
//   - samplerCube NEAREST: major-axis face rule of the GL spec with ties
//     resolved x, then y, then z; s = 0.5*(sc/|ma| + 1), texel floor(s*size).
#pragma once

#include <algorithm>
#include <vector>

#include "../include/sgi.h"
#include "counted.hpp"
#include "glsl.hpp"

namespace oracle {

inline int tex_index(double f, int n) {   // floor'ed coordinate -> clamped texel index (NaN -> 0)
    if (f >= double(n - 1)) return n - 1;
    if (f >= 0.0) return (int)f;
    return 0;
}

template <class T> inline T half_texel(const uint16_t* p, size_t i) { return T(f16_to_f32(p[i])); }

// Bilinear sample of a single-channel float image at uv (see header).
template <class T, class Fetch> inline T bilinear(Fetch fetch, int W, int H, T s, T t) {
    T u = s * T(W) - T(0.5), v = t * T(H) - T(0.5);
    T fu = gfloor(u), fv = gfloor(v);
    T a = u - fu, b = v - fv;
    int i0 = tex_index(double(fu), W), i1 = tex_index(double(fu + T(1)), W);
    int j0 = tex_index(double(fv), H), j1 = tex_index(double(fv + T(1)), H);
    T w00 = (T(1) - a) * (T(1) - b), w10 = a * (T(1) - b), w01 = (T(1) - a) * b, w11 = a * b;
    return gfma(fetch(i1, j1), w11, gfma(fetch(i0, j1), w01, gfma(fetch(i1, j0), w10, fetch(i0, j0) * w00)));
}
template <class T> inline int nearest_index(T s, int n) { return tex_index(double(gfloor(s * T(n))), n); }
// the margin-tracking instantiation also records how far the coordinate is from a texel boundary
inline int nearest_index(Tracked s, int n) {
    const double x = s.v * double(n);
    const double f = std::floor(x);
    record_margin(1, std::fmin(x - f, f + 1.0 - x) / std::fmax(std::fabs(x), 1.0));
    return tex_index(f, n);
}

// ------------------------------------------------------------------- CSM --
// texture(sampler2DArrayShadow, vec4(s, t, layer, ref)) with LINEAR + LEQUAL.
template <class T> inline T csm_pcf(const sgi_csm& csm, int layer, T s, T t, T ref) {
    const int R = csm.resolution;
    const float* base = csm.depth + (size_t)layer * R * R;
    auto fetch = [&](int i, int j) -> T { return ref <= T(base[(size_t)j * R + i]) ? T(1) : T(0); };
    return bilinear<T>(fetch, R, R, s, t);
}

// sampleShadowTexture, pbr.glsl:139-147
template <class T> inline T sample_shadow_tex(const sgi_csm& csm, V3<T> p, T depth, T ox, T oy, T bias) {
    T refv = depth - bias;
    return csm_pcf<T>(csm, (int)p.z, p.x + ox, p.y + oy, refv);
}

// calculateInfiniteShadowValue, pbr.glsl:158-227. Returns the lit fraction.
template <class T> inline T infinite_shadow(const sgi_csm& csm, V3<T> fragPos, V3<T> blends, V3<T> normal,
                                           bool useDepthBias) {
    T bias = T(csm.depth_bias) / (T(csm.zfar) - T(csm.znear));
    if (!useDepthBias) bias = T(0);
    V3<T> Ldir(T(csm.light_direction[0]), T(csm.light_direction[1]), T(csm.light_direction[2]));
    V3<T> position = fragPos + normal * (T(1) - saturate(dot(normal, Ldir))) * T(1);
    V3<T> cc[4];
    for (int i = 0; i < 4; ++i) {
        V4<T> c = mat4_mul<T>(csm.cascade_proj_view[i], position.x, position.y, position.z, T(1));
        V3<T> d = V3<T>(c.x, c.y, c.z) / c.w;
        cc[i] = d * T(0.5) + V3<T>(T(0.5));
    }
    bool beyond2 = blends.y >= T(0);
    bool beyond3 = blends.z >= T(0);
    int index1 = beyond2 ? 2 : 0;
    int index2 = beyond3 ? 3 : 1;
    V3<T> p1(cc[index1].x, cc[index1].y, T(index1));
    V3<T> p2(cc[index2].x, cc[index2].y, T(index2));
    T depth1 = cc[index1].z;
    T depth2 = cc[index2].z;
    depth2 = beyond3 ? saturate(depth2) : depth2;
    T weight = beyond2 ? saturate(blends.y) - saturate(blends.z) : T(1) - saturate(blends.x);
    T wh = T(1) / T(csm.resolution);   // computeTexelSize, common.glsl:117-121
    T light1 = 0, light2 = 0, samples = 0;
    const T bound = T(1);
    for (T y = -bound; y <= bound; y += T(1)) {
        for (T x = -bound; x <= bound; x += T(1)) {
            T ox = x * wh, oy = y * wh;
            light1 += sample_shadow_tex(csm, p1, depth1, ox, oy, bias);
            light2 += sample_shadow_tex(csm, p2, depth2, ox, oy, bias);
            samples += T(1);
        }
    }
    return mix(light2, light1, weight) * (T(1) / samples);
}

template <class T> inline V3<T> cascade_blends(const sgi_csm& csm, V3<T> p) {
    return V3<T>(dot4(csm.cascade_planes[0], p), dot4(csm.cascade_planes[1], p), dot4(csm.cascade_planes[2], p));
}

// ------------------------------------------------------------- cube maps --
template <class T> inline T cube_fetch(const sgi_cube_atlas& at, sgi_atlas_entry e, V3<T> d) {
    if (e.index < 0 || e.index >= at.num_atlases || e.layer < 0 || e.layer >= at.layers_per_atlas) return T(1);
    T ax = gabs(d.x), ay = gabs(d.y), az = gabs(d.z);
    int face; T sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        if (d.x >= T(0)) { face = 0; sc = -d.z; tc = -d.y; } else { face = 1; sc = d.z; tc = -d.y; }
    } else if (ay >= az) {
        ma = ay;
        if (d.y >= T(0)) { face = 2; sc = d.x; tc = d.z; } else { face = 3; sc = d.x; tc = -d.z; }
    } else {
        ma = az;
        if (d.z >= T(0)) { face = 4; sc = d.x; tc = -d.y; } else { face = 5; sc = -d.x; tc = -d.y; }
    }
    T s = T(0.5) * (sc / ma + T(1));
    T t = T(0.5) * (tc / ma + T(1));
    const int n = at.face_size;
    int i = nearest_index(s, n), j = nearest_index(t, n);
    size_t off = (((size_t)e.layer * 6 + face) * n + j) * n + i;
    switch (at.format) {
        case SGI_CUBE_F32: return T(((const float*)at.atlas[e.index])[off]);
        case SGI_CUBE_F16: return T(f16_to_f32(((const uint16_t*)at.atlas[e.index])[off]));
        default: return T(((const uint16_t*)at.atlas[e.index])[off]) / T(65535);
    }
}

// Nearest-texel offset of direction d in a cube stack of face size n (cube_fetch's selection).
template <class T> inline size_t cube_texel(int layer, int n, V3<T> d) {
    T ax = gabs(d.x), ay = gabs(d.y), az = gabs(d.z);
    int face; T sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        if (d.x >= T(0)) { face = 0; sc = -d.z; tc = -d.y; } else { face = 1; sc = d.z; tc = -d.y; }
    } else if (ay >= az) {
        ma = ay;
        if (d.y >= T(0)) { face = 2; sc = d.x; tc = d.z; } else { face = 3; sc = d.x; tc = -d.z; }
    } else {
        ma = az;
        if (d.z >= T(0)) { face = 4; sc = d.x; tc = -d.y; } else { face = 5; sc = -d.x; tc = -d.y; }
    }
    T s = T(0.5) * (sc / ma + T(1));
    T t = T(0.5) * (tc / ma + T(1));
    int i = nearest_index(s, n), j = nearest_index(t, n);
    return (((size_t)layer * 6 + face) * n + j) * n + i;
}

// vpl_light_color.cs:41-75 over the compacted list: colour from the diffuse cube
// and the sun, specular position from the distance cube, both in direction -L.
template <class T> void color_vpls(sgi_vpl* cv, const sgi_atlas_entry* ce, int count, const sgi_cube_atlas& cubes,
                                   const sgi_diffuse_atlas& diffuse, const sgi_csm& csm) {
    const V3<T> L(T(csm.light_direction[0]), T(csm.light_direction[1]), T(csm.light_direction[2]));
    const V3<T> sun(T(csm.light_color[0]), T(csm.light_color[1]), T(csm.light_color[2]));
    const V3<T> dir(-L.x, -L.y, -L.z);
    for (int k = 0; k < count; ++k) {
        const sgi_atlas_entry e = ce[k];
        sgi_vpl& v = cv[k];
        V3<T> diff(T(0), T(0), T(0));
        if (e.index >= 0 && e.index < diffuse.num_atlases && e.layer >= 0 && e.layer < diffuse.layers_per_atlas) {
            const uint32_t t = ((const uint32_t*)diffuse.atlas[e.index])[cube_texel(e.layer, diffuse.face_size, dir)];
            diff = V3<T>(T(t & 0xffu) / T(255), T((t >> 8) & 0xffu) / T(255), T((t >> 16) & 0xffu) / T(255));
        }
        const V3<T> color = diff * sun;
        const T magnitude = T(v.radius) * cube_fetch(cubes, e, dir);
        const T m = T(1.1f) * magnitude;
        const V3<T> spec = V3<T>(T(v.position[0]), T(v.position[1]), T(v.position[2])) - L * m;
        const V3<T> c = ((color / T(1)) * T(v.intensity)) * T(50000);
        v.color[0] = float(c.x); v.color[1] = float(c.y); v.color[2] = float(c.z); v.color[3] = 1.0f;
        v.specular_position[0] = float(spec.x); v.specular_position[1] = float(spec.y);
        v.specular_position[2] = float(spec.z); v.specular_position[3] = 1.0f;
    }
}

// calculateShadowValue1Sample, pbr.glsl:116-136 (1 = occluded)
template <class T> inline T shadow_1sample(const sgi_cube_atlas& at, sgi_atlas_entry e, T farPlane, V3<T> fragPos,
                                           V3<T> lightPos, T lightNormalDot, T minBias) {
    V3<T> fragDir = fragPos - lightPos;
    T currentDepth = length(fragDir);
    T bias = currentDepth * gmax(minBias, saturate(lightNormalDot) * T(0.03));
    T depth = cube_fetch(at, e, fragDir);
    depth = depth * farPlane;
    return (currentDepth - bias) > depth ? T(1) : T(0);
}

// calculateShadowValue8Samples, pbr.glsl:81-113 (fraction occluded)
template <class T> inline T shadow_8samples(const sgi_cube_atlas& at, sgi_atlas_entry e, T farPlane, V3<T> fragPos,
                                            V3<T> lightPos, T lightNormalDot, T minBias) {
    V3<T> fragDir = fragPos - lightPos;
    T currentDepth = length(fragDir);
    T bias = currentDepth * gmax(minBias, saturate(lightNormalDot) * T(0.03f));
    T shadow = T(0);
    const T offs[2] = {T(-0.3f), T(0.3f)};
    for (int x = 0; x < 2; ++x)
        for (int y = 0; y < 2; ++y)
            for (int z = 0; z < 2; ++z) {
                T depth = cube_fetch(at, e, fragDir + V3<T>(offs[x], offs[y], offs[z]));
                depth = depth * farPlane;
                if ((currentDepth - bias) > depth) shadow = shadow + T(1);
            }
    return shadow / T(8);
}

// ------------------------------------------------------------------ passes --
inline int tiles_x(const sgi_config& c) { return (c.width + c.tile_size - 1) / c.tile_size; }
inline int tiles_y(const sgi_config& c) { return (c.height + c.tile_size - 1) / c.tile_size; }

// viscull_vpls.cs:47-120. Stable compaction (ascending index), capped.
// visible_index[0] = count, visible_index[1+k] = original index of the k-th.
template <class T> int vis_cull(const sgi_vpl* vpls, int n, const sgi_csm& csm, int cap, int32_t* visible_index) {
    std::vector<char> vis(n, 0);
    V3<T> L(T(csm.light_direction[0]), T(csm.light_direction[1]), T(csm.light_direction[2]));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        V3<T> p(T(vpls[i].position[0]), T(vpls[i].position[1]), T(vpls[i].position[2]));
        V3<T> blends = cascade_blends(csm, p);
        T shadowFactor = T(1) - infinite_shadow(csm, p, blends, L, false);
        vis[i] = shadowFactor < T(1);
    }
    int k = 0;
    for (int i = 0; i < n; ++i) {
        if (!vis[i]) continue;
        if (k < cap) visible_index[1 + k] = i;
        ++k;
    }
    visible_index[0] = std::min(k, cap);
    return visible_index[0];
}

// The warp-butterfly reduction order the CUDA tile-cull kernel uses: lanes
// combine with xor partners 16, 8, 4, 2, 1 (all lanes end with the same sum),
// then warp totals combine with xor partners nw/2 .. 1.
template <class T> inline T butterfly_sum(T* a, int n) {
    std::vector<T> b(n);
    for (int off = n / 2; off >= 1; off /= 2) {
        for (int i = 0; i < n; ++i) b[i] = a[i] + a[i ^ off];
        for (int i = 0; i < n; ++i) a[i] = b[i];
    }
    return a[0];
}
// tile_size^2 = 32 x (a power of two) (tile sizes 8, 16, 32): the butterfly
// order above; otherwise (e.g. the reference's 5x5 tiles) the sequential sum of
// vpl_tiled_deferred_culling_stage1.cs:73-81, from 0 in the order of the pixels.
inline bool butterfly_tile(int n) { return n % 32 == 0 && ((n / 32) & (n / 32 - 1)) == 0; }
template <class T> inline T block_sum(std::vector<T>& vals) {
    int n = (int)vals.size();
    if (!butterfly_tile(n)) {
        T acc = T(0);
        for (int i = 0; i < n; ++i) acc = acc + vals[i];
        return acc;
    }
    int nw = n / 32;
    std::vector<T> w(nw);
    for (int k = 0; k < nw; ++k) w[k] = butterfly_sum(&vals[k * 32], 32);
    return nw == 1 ? w[0] : butterfly_sum(w.data(), nw);
}

// vpl_tiled_deferred_culling_stage1.cs:50-90, generalised to tile_size^2
// pixels; out-of-image pixels are excluded from the mean.
template <class T> void tile_stage1(const sgi_config& cfg, const sgi_gbuffer& g, const sgi_camera& cam, T* out) {
    const int W = cfg.width, H = cfg.height, ts = cfg.tile_size;
    const int TX = tiles_x(cfg), TY = tiles_y(cfg);
#pragma omp parallel for schedule(dynamic, 4)
    for (int tile = 0; tile < TX * TY; ++tile) {
        int tx = tile % TX, ty = tile / TX;
        std::vector<T> px(ts * ts), py(ts * ts), pz(ts * ts), nx(ts * ts), ny(ts * ts), nz(ts * ts);
        int count = 0;
        for (int l = 0; l < ts * ts; ++l) {
            int x = tx * ts + l % ts, y = ty * ts + l / ts;
            if (x >= W || y >= H) { px[l] = py[l] = pz[l] = nx[l] = ny[l] = nz[l] = T(0); continue; }
            ++count;
            size_t i = (size_t)y * W + x;
            T u = (T(x) + T(0.5)) / T(W), v = (T(y) + T(0.5)) / T(H);
            V3<T> p = world_from_depth<T>(u, v, T(g.depth[i]), cam.inv_proj_view);
            V3<T> n = decode_normal<T>(g.normal[i]);
            px[l] = p.x; py[l] = p.y; pz[l] = p.z; nx[l] = n.x; ny[l] = n.y; nz[l] = n.z;
        }
        V3<T> sp(block_sum(px), block_sum(py), block_sum(pz));
        V3<T> sn(block_sum(nx), block_sum(ny), block_sum(nz));
        T c = T(count);
        V3<T> ap = sp / c;
        V3<T> an = sn / c;
        an = normalize(an);
        T* o = out + (size_t)tile * 8;
        o[0] = ap.x; o[1] = ap.y; o[2] = ap.z; o[3] = T(1);
        o[4] = an.x; o[5] = an.y; o[6] = an.z; o[7] = T(1);
    }
}

// vpl_tiled_deferred_culling_stage2.cs:61-129 over the compacted list; the
// list holds compacted indices (== ascending original index). Equivalent to
// keeping the first L of a stable sort by distance/radius.
template <class T> void tile_stage2(const sgi_config& cfg, const T* stage1, const sgi_vpl* cv, int count,
                                    int32_t* lists) {
    const int TX = tiles_x(cfg), TY = tiles_y(cfg), L = cfg.max_vpls_per_tile;
#pragma omp parallel for schedule(dynamic, 8)
    for (int tile = 0; tile < TX * TY; ++tile) {
        const T* s = stage1 + (size_t)tile * 8;
        V3<T> fragPos(s[0], s[1], s[2]);
        V3<T> normal(s[4], s[5], s[6]);
        std::vector<int> idx(L, 0);
        std::vector<T> dist(L, T(3.402823466e+38));   // FLOAT_MAX
        int num = 0;
        for (int k = 0; k < count; ++k) {
            V3<T> lp(T(cv[k].position[0]), T(cv[k].position[1]), T(cv[k].position[2]));
            V3<T> lmf = lp - fragPos;
            T side = dot(normal, lmf);
            if (side < T(0)) continue;
            T radius = T(cv[k].radius);
            T d = length(lmf);
            T ratio = d / radius;
            if (ratio > T(1)) continue;
            for (int ii = 0; ii < L; ++ii) {
                if (ratio < dist[ii]) {
                    if (dist[ii] != T(3.402823466e+38)) {
                        for (int j = L - 2; j >= ii; --j) { idx[j + 1] = idx[j]; dist[j + 1] = dist[j]; }
                    }
                    idx[ii] = k;
                    dist[ii] = ratio;
                    if (num < L) ++num;
                    break;
                }
            }
        }
        int32_t* o = lists + (size_t)tile * (1 + L);
        o[0] = num;
        for (int i = 0; i < L; ++i) o[1 + i] = i < num ? idx[i] : -1;
    }
}

struct GatherArgs {
    const sgi_config* cfg;
    const sgi_gbuffer* g;
    const sgi_camera* cam;
    const sgi_vpl* cv;            // compacted VPLs
    const sgi_atlas_entry* ce;    // compacted atlas entries
    int count;                    // compacted count (numVisible[0])
    const int32_t* lists;         // tile lists (tiled mode)
    const sgi_cube_atlas* cubes;
    float time;
};

// vpl_pbr_gi.fs:81-200 for one pixel with the seed z starting at seedZ0:
// accumulates vplColor and validSamples over the sample loop.
template <class T> void gather_samples(const GatherArgs& a, int x, int y, float seedZ0, V3<T>& vplColorOut,
                                       T& validOut) {
    const sgi_config& cfg = *a.cfg;
    const sgi_gbuffer& g = *a.g;
    const int W = cfg.width, H = cfg.height;
    const size_t i = (size_t)y * W + x;
    BrdfParams bp{cfg.min_roughness, cfg.use_perceptual_roughness};
    FogParams fog{cfg.fog_density, {cfg.fog_color[0], cfg.fog_color[1], cfg.fog_color[2]}};
    T u = (T(x) + T(0.5)) / T(W), v = (T(y) + T(0.5)) / T(H);
    V3<T> fragPos = world_from_depth<T>(u, v, T(g.depth[i]), a.cam->inv_proj_view);
    V3<T> viewPos(T(a.cam->view_position[0]), T(a.cam->view_position[1]), T(a.cam->view_position[2]));
    V3<T> viewDir = normalize(viewPos - fragPos);
    T distToCamera = length(viewPos - fragPos);
    uint32_t alb = g.albedo[i];
    V3<T> baseColor(unorm8<T>(alb, 0), unorm8<T>(alb, 1), unorm8<T>(alb, 2));
    baseColor = V3<T>(gmax(baseColor.x, T(0.01)), gmax(baseColor.y, T(0.01)), gmax(baseColor.z, T(0.01)));
    V3<T> normal = decode_normal<T>(g.normal[i]);
    uint32_t rma = g.roughness_metallic_ambient[i];
    T roughness = gmax(T(0.5), unorm8<T>(rma, 0));
    T metallic = unorm8<T>(rma, 1);
    T ao = gclamp(half_texel<T>(g.ssao, i), T(0.35), T(1));
    T ambient = unorm8<T>(rma, 2);
    T refl = T(g.base_reflectivity[i] & 0xffu) / T(255);
    V3<T> baseRefl(refl);
    T roughnessWeight = T(1) - roughness;
    V3<T> vplColor(T(0));
    float seedX = float(x) + 0.5f, seedY = float(y) + 0.5f, seedZ = seedZ0;
    T validSamples = 0;
    T distRatio = gmin(T(1) - distToCamera / T(1000), T(1));
    int sampleCount;
    if (cfg.samples_per_pixel > 0) {
        sampleCount = cfg.samples_per_pixel;
    } else {
        int maxSamplesPerPixel = (int)mix(T(2), T(10), roughnessWeight);
        int samplesMax = maxSamplesPerPixel;
        samplesMax = std::max(1, (int)(T(samplesMax) * distRatio));
        sampleCount = samplesMax;
    }
    // candidate set
    const int32_t* list = nullptr;
    int candidates;
    if (cfg.gi_mode == SGI_GI_TILED) {
        int tile = (y / cfg.tile_size) * tiles_x(cfg) + (x / cfg.tile_size);
        list = a.lists + (size_t)tile * (1 + cfg.max_vpls_per_tile);
        candidates = list[0];
    } else {
        candidates = a.count;
    }
    if (candidates > 0) {
        const float minGi = cfg.min_gi_occlusion_factor;
        for (int s = 0, resamples = 0; s < sampleCount; ++s) {
            float rnd = random3(seedX, seedY, seedZ);
            seedZ += 10000.0f;
            int lightIndex;
            if (list) {
                int r = (int)(float(candidates) * rnd);
                lightIndex = list[1 + std::min(r, candidates - 1)];
            } else {
                lightIndex = (int)(float(candidates - 1) * rnd);   // maxRandomIndex = numVisible[0] - 1
            }
            const sgi_vpl& vp = a.cv[lightIndex];
            sgi_atlas_entry entry = a.ce[lightIndex];
            V3<T> lightPosition(T(vp.position[0]), T(vp.position[1]), T(vp.position[2]));
            V3<T> specPosition(T(vp.specular_position[0]), T(vp.specular_position[1]), T(vp.specular_position[2]));
            V3<T> lmf = lightPosition - fragPos;
            T lightRadius = T(vp.radius);
            T distance = length(lmf);
            if (resamples < 5) {
                T sideCheck = dot(normal, normalize(lmf));
                if (sideCheck < T(0) || distance > lightRadius) { ++resamples; --s; continue; }
            }
            T distanceRatio = gclamp((T(2) * distance) / lightRadius, T(0), T(1));
            T distAttenuation = distanceRatio;
            V3<T> lightColor(T(vp.color[0]), T(vp.color[1]), T(vp.color[2]));
            T shadowFactor = distToCamera < T(500)
                                 ? shadow_1sample<T>(*a.cubes, entry, T(vp.far_plane), fragPos, lightPosition,
                                                     dot(lightPosition - fragPos, normal), T(0.1))
                                 : T(0);
            shadowFactor = gmin(shadowFactor, mix(T(minGi), T(1), distanceRatio));
            T reweight = T(1);
            if (shadowFactor > T(0)) reweight = (T(1) - distAttenuation) * T(minGi) + distAttenuation;
            validSamples += reweight;
            V3<T> tmp = ao * vpl_lighting2<T>(fragPos, baseColor, normal, viewDir, specPosition, lightPosition,
                                             lightColor, distToCamera, lightRadius, roughness, metallic, ambient,
                                             T(0), baseRefl, bp, fog);
            vplColor = vplColor + (T(1) - shadowFactor) * tmp;
        }
    }
    vplColorOut = vplColor;
    validOut = validSamples;
}

// vpl_pbr_gi.fs:81-207 for one pixel. Writes (min(vplColor, 65504), validSamples).
template <class T> void gather_pixel(const GatherArgs& a, int x, int y, T* res) {
    V3<T> vplColor;
    T validSamples;
    gather_samples<T>(a, x, y, a.time, vplColor, validSamples);
    validSamples = gmax(validSamples, T(1));
    V3<T> bounded = vmin(vplColor, C<T>::HALF_MAX());
    res[0] = Prec<T>::store16(bounded.x);
    res[1] = Prec<T>::store16(bounded.y);
    res[2] = Prec<T>::store16(bounded.z);
    res[3] = Prec<T>::store16(validSamples);
}

template <class T> void gather(const GatherArgs& a, T* reservoir) {
    const int W = a.cfg->width, H = a.cfg->height;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            margin_begin<T>();
            gather_pixel<T>(a, x, y, reservoir + ((size_t)y * W + x) * 4);
            margin_end<T>((size_t)y * W + x);
        }
}

// Converged target: `batches` runs of the sample loop, batch b seeded at
// time + b * 2e5, binary32 samples summed in binary64 (the CUDA target kernel's
// definition). out[i] = (sum vplColor / max(sum valid, 1), 1).
inline void gi_target(const GatherArgs& a, int batches, float* out) {
    const int W = a.cfg->width, H = a.cfg->height;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            double c0 = 0, c1 = 0, c2 = 0, w = 0;
            for (int b = 0; b < batches; ++b) {
                V3<float> col;
                float valid;
                gather_samples<float>(a, x, y, a.time + float(b) * 200000.0f, col, valid);
                c0 += (double)col.x; c1 += (double)col.y; c2 += (double)col.z; w += (double)valid;
            }
            double den = w < 1.0 ? 1.0 : w;
            float* o = out + ((size_t)y * W + x) * 4;
            o[0] = (float)(c0 / den); o[1] = (float)(c1 / den); o[2] = (float)(c2 / den); o[3] = 1.0f;
        }
    }
}

template <class T> struct DenoiseArgs {
    const sgi_config* cfg;
    const sgi_gbuffer* cur;
    const sgi_gbuffer* prev;
    const T* hdr_in;            // [P][4] screen (RGB16F values)
    const T* gi_prev;           // [P][4] prevIndirectIllumination (RGB16F values)
    const T* hist_prev;         // [P]    historyDepth (R16F values)
    int num_visible;            // numVisible[0]
    float time;
    float fps;
};

// vpl_pbr_gi_denoise.fs:275-435, one pass for one pixel.
// res_in: previous reservoir [P][4]; outputs: res_out [P][4]; on the final
// pass also combined [P][4], gi [P][4], hist [P].
template <class T> void denoise_pixel(const DenoiseArgs<T>& a, int pass, const T* res_in, T* res_out, T* combined,
                                      T* gi_out, T* hist_out, int x, int y) {
    const sgi_config& cfg = *a.cfg;
    const int W = cfg.width, H = cfg.height;
    const size_t i = (size_t)y * W + x;
    const int multiplier = (1 << pass) - 1;
    const bool final = pass == cfg.denoise_passes - 1;
    const bool merge = pass == 0;
    const sgi_gbuffer& g = *a.cur;
    T u = (T(x) + T(0.5)) / T(W), v = (T(y) + T(0.5)) / T(H);
    auto cx = [&](int d) { return std::min(std::max(x + d, 0), W - 1); };
    auto cy = [&](int d) { return std::min(std::max(y + d, 0), H - 1); };

    V3<T> screen(T(a.hdr_in[i * 4 + 0]), T(a.hdr_in[i * 4 + 1]), T(a.hdr_in[i * 4 + 2]));
    uint32_t vel = g.velocity[i];
    T velx = T(f16_to_f32((uint16_t)(vel & 0xffffu))), vely = T(f16_to_f32((uint16_t)(vel >> 16)));
    T pu = u - velx, pv = v - vely;
    // indirectIllumination: the gather's colour output baseColor + 1e-5 stored
    // as RGB16F (vpl_pbr_gi.fs:204); later passes forward it unchanged.
    uint32_t alb = g.albedo[i];
    V3<T> bc(gmax(unorm8<T>(alb, 0), T(0.01)), gmax(unorm8<T>(alb, 1), T(0.01)), gmax(unorm8<T>(alb, 2), T(0.01)));
    V3<T> centerIllum(Prec<T>::store16(bc.x + C<T>::EPS()), Prec<T>::store16(bc.y + C<T>::EPS()),
                      Prec<T>::store16(bc.z + C<T>::EPS()));
    V3<T> centerNormal = decode_normal<T>(g.normal[i]);
    T centerDepth = T(g.depth[i]);
    T historyAccum = T(a.hist_prev[i]);
    T rf[4] = {0, 0, 0, 0};
    if (merge) {
        // computeMergedReservoir, vpl_pbr_gi_denoise.fs:192-273 (centre only, minmaxNearest = 0)
        float sx = float(x) + 0.5f, sy = float(y) + 0.5f, sz = a.time;
        T cr[4] = {0, 0, 0, 0};
        T depthCutoff = T(0.1) * centerDepth;
        T runningSum = 0;
        T probabilisticWeight = T(1) / T(a.num_visible);
        V3<T> currNormal = decode_normal<T>(g.normal[i]);
        if (!(dot(centerNormal, currNormal) < T(0.906))) {
            T currDepth = T(g.depth[i]);
            if (!(gabs(currDepth - centerDepth) > depthCutoff)) {
                const T* cur = res_in + i * 4;
                T randUpdate = T(random3(sx, sy, sz));
                sz += 10000.0f;
                T probability = cur[3] * probabilisticWeight;
                cr[3] += probability;
                if (randUpdate < (probability / cr[3])) {
                    cr[0] += cur[0]; cr[1] += cur[1]; cr[2] += cur[2];
                    runningSum += cur[3];
                }
            }
        }
        cr[3] = runningSum;
        for (int c = 0; c < 4; ++c) rf[c] = cr[c];
    } else {
        for (int dx = -2; dx <= 2; ++dx) {
            for (int dy = -2; dy <= 2; ++dy) {
                int ox = dx + dx * multiplier, oy = dy + dy * multiplier;
                size_t j = (size_t)cy(oy) * W + cx(ox);
                const T* r = res_in + j * 4;
                T filtered;
                if (dx == 0 && dy == 0) {
                    filtered = T(1);
                } else {   // filterInput, vpl_pbr_gi_denoise.fs:142-190
                    T currDepth = T(g.depth[j]);
                    T wz = Prec<T>::exp(-gabs(centerDepth - currDepth)) / T(1);   // sigmaZ = 1
                    V3<T> currNormal = decode_normal<T>(g.normal[j]);
                    T wn = gmax(T(0), dot(centerNormal, currNormal));
                    wn = Prec<T>::pow128(wn);                                       // sigmaN = 128
                    filtered = wn * wz * T(1);
                }
                for (int c = 0; c < 4; ++c) rf[c] = gfma(filtered, r[c], rf[c]);
            }
        }
    }
    T den = gmax(C<T>::EPS(), rf[3]);
    V3<T> shadowFactor(rf[0] / den, rf[1] / den, rf[2] / den);
    V3<T> gi = centerIllum;
    V3<T> illumAvg = gi;
    if (final) {
        T accumMultiplier = T(1);
        V3<T> currGi = shadowFactor;
        const sgi_gbuffer& pg = *a.prev;
        auto fdepth = [&](int ii, int jj) -> T { return T(pg.depth[(size_t)jj * W + ii]); };
        T prevCenterDepth = bilinear<T>(fdepth, W, H, pu, pv);
        V3<T> pn;
        {
            auto f0 = [&](int ii, int jj) -> T { return unorm8<T>(pg.normal[(size_t)jj * W + ii], 0); };
            auto f1 = [&](int ii, int jj) -> T { return unorm8<T>(pg.normal[(size_t)jj * W + ii], 1); };
            auto f2 = [&](int ii, int jj) -> T { return unorm8<T>(pg.normal[(size_t)jj * W + ii], 2); };
            pn = V3<T>(bilinear<T>(f0, W, H, pu, pv), bilinear<T>(f1, W, H, pu, pv), bilinear<T>(f2, W, H, pu, pv));
        }
        V3<T> prevCenterNormal = normalize(pn * T(2) - V3<T>(T(1)));
        V3<T> prevGi;
        {
            auto g0 = [&](int ii, int jj) -> T { return T(a.gi_prev[((size_t)jj * W + ii) * 4 + 0]); };
            auto g1 = [&](int ii, int jj) -> T { return T(a.gi_prev[((size_t)jj * W + ii) * 4 + 1]); };
            auto g2 = [&](int ii, int jj) -> T { return T(a.gi_prev[((size_t)jj * W + ii) * 4 + 2]); };
            prevGi = V3<T>(bilinear<T>(g0, W, H, pu, pv), bilinear<T>(g1, W, H, pu, pv), bilinear<T>(g2, W, H, pu, pv));
        }
        T currId = T(g.id[i]);
        T prevId = T(pg.id[(size_t)nearest_index(pv, H) * W + nearest_index(pu, W)]);
        T wn = gmax(T(0), dot(centerNormal, prevCenterNormal));
        T wz = Prec<T>::exp(-gabs(centerDepth - prevCenterDepth));
        T wid = currId != prevId ? T(0) : T(1);
        T similarity = wn * wz * wid;
        if (similarity < T(0.99)) { similarity = T(0); accumMultiplier = T(0); }
        historyAccum = gmin(T(1) + historyAccum * accumMultiplier, T(a.fps));
        T maxAccumulationFactor = T(1) / historyAccum;
        illumAvg = vmix(prevGi, currGi, maxAccumulationFactor);
    }
    T* ro = res_out + i * 4;
    ro[0] = Prec<T>::store16(shadowFactor.x);
    ro[1] = Prec<T>::store16(shadowFactor.y);
    ro[2] = Prec<T>::store16(shadowFactor.z);
    ro[3] = Prec<T>::store16(T(1));
    if (final) {
        V3<T> comb = screen + gi * illumAvg;
        T* co = combined + i * 4;
        co[0] = Prec<T>::store16(comb.x); co[1] = Prec<T>::store16(comb.y); co[2] = Prec<T>::store16(comb.z);
        co[3] = T(1);
        T* go = gi_out + i * 4;
        go[0] = Prec<T>::store16(illumAvg.x); go[1] = Prec<T>::store16(illumAvg.y);
        go[2] = Prec<T>::store16(illumAvg.z); go[3] = T(1);
        hist_out[i] = Prec<T>::store16(historyAccum);
    }
}

// Host loop of ComputeVirtualPointLightGlobalIllumination_,
// StratusRendererBackend.cpp:1912-1940: pass i uses multiplier 2^i - 1; pass 0
// merges reservoirs; the last pass is final.
template <class T> void denoise(const DenoiseArgs<T>& a, const T* reservoir, T* combined, T* gi_out, T* hist_out,
                                T* pass_out /* nullable [n][P][4] */, void (*after_pass)(int) = nullptr) {
    const int W = a.cfg->width, H = a.cfg->height, n = a.cfg->denoise_passes;
    const size_t P = (size_t)W * H;
    std::vector<T> bufA(P * 4), bufB(P * 4);
    const T* in = reservoir;
    for (int pass = 0; pass < n; ++pass) {
        T* out = (pass % 2 == 0) ? bufA.data() : bufB.data();
#pragma omp parallel for schedule(dynamic, 1)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                margin_begin<T>();
                denoise_pixel<T>(a, pass, in, out, combined, gi_out, hist_out, x, y);
                margin_end<T>((size_t)y * W + x);
            }
        if (pass_out) std::copy(out, out + P * 4, pass_out + (size_t)pass * P * 4);
        if (after_pass) after_pass(pass);
        in = out;
    }
}

// One denoise pass over the whole image (pass 0 merges, the last is final), from
// an arbitrary input reservoir: lets a pass of another implementation be
// checked on exactly the input it was given.
template <class T> void denoise_one_pass(const DenoiseArgs<T>& a, int pass, const T* res_in, T* res_out, T* combined,
                                         T* gi_out, T* hist_out) {
    const int W = a.cfg->width, H = a.cfg->height;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            margin_begin<T>();
            denoise_pixel<T>(a, pass, res_in, res_out, combined, gi_out, hist_out, x, y);
            margin_end<T>((size_t)y * W + x);
        }
}

struct DeferredArgs {
    const sgi_config* cfg;
    const sgi_gbuffer* g;
    const sgi_camera* cam;
    const sgi_point_light* points;
    int num_points;
    const sgi_csm* csm;
    // shadow-casting point lights (pbr.fs:116-131)
    const sgi_point_light* casters = nullptr;
    const sgi_atlas_entry* caster_entries = nullptr;
    int num_casters = 0;
    const sgi_cube_atlas* caster_atlas = nullptr;
};

// pbr.fs:82-145 (non-shadow-casting point lights + INFINITE_LIGHTING_ENABLED).
template <class T> void deferred_pixel(const DeferredArgs& a, int x, int y, T* out) {
    const sgi_config& cfg = *a.cfg;
    const sgi_gbuffer& g = *a.g;
    const sgi_csm& csm = *a.csm;
    const int W = cfg.width, H = cfg.height;
    const size_t i = (size_t)y * W + x;
    BrdfParams bp{cfg.min_roughness, cfg.use_perceptual_roughness};
    FogParams fog{cfg.fog_density, {cfg.fog_color[0], cfg.fog_color[1], cfg.fog_color[2]}};
    T u = (T(x) + T(0.5)) / T(W), v = (T(y) + T(0.5)) / T(H);
    V3<T> fragPos = world_from_depth<T>(u, v, T(g.depth[i]), a.cam->inv_proj_view);
    V3<T> viewPos(T(a.cam->view_position[0]), T(a.cam->view_position[1]), T(a.cam->view_position[2]));
    V3<T> viewMinusFrag = viewPos - fragPos;
    V3<T> viewDir = normalize(viewMinusFrag);
    T viewDist = length(viewMinusFrag);
    uint32_t alb = g.albedo[i];
    V3<T> baseColor(unorm8<T>(alb, 0), unorm8<T>(alb, 1), unorm8<T>(alb, 2));
    T albedoA = unorm8<T>(alb, 3);
    V3<T> normal = decode_normal<T>(g.normal[i]);
    uint32_t rma = g.roughness_metallic_ambient[i];
    T roughness = unorm8<T>(rma, 0), metallic = unorm8<T>(rma, 1), rmeB = unorm8<T>(rma, 2);
    T ambient = half_texel<T>(g.ssao, i);
    uint16_t br = g.base_reflectivity[i];
    T reflR = T(br & 0xffu) / T(255), reflG = T(br >> 8) / T(255);
    V3<T> emissive(albedoA, reflG, rmeB);
    V3<T> color(T(0));
    for (int l = 0; l < a.num_points; ++l) {
        const sgi_point_light& pl = a.points[l];
        V3<T> lp(T(pl.position[0]), T(pl.position[1]), T(pl.position[2]));
        V3<T> lc(T(pl.color[0]), T(pl.color[1]), T(pl.color[2]));
        T distance = length(lp - fragPos);
        if (distance < T(pl.radius)) {
            color = color + point_lighting2<T>(fragPos, baseColor, normal, viewDir, lp, lc, viewDist, roughness,
                                               metallic, ambient, T(0), V3<T>(reflR),
                                               T(cfg.point_light_ambient_intensity), bp, fog);
        }
    }
    for (int l = 0; l < a.num_casters; ++l) {
        const sgi_point_light& pl = a.casters[l];
        V3<T> lp(T(pl.position[0]), T(pl.position[1]), T(pl.position[2]));
        V3<T> lc(T(pl.color[0]), T(pl.color[1]), T(pl.color[2]));
        T distance = length(lp - fragPos);
        if (distance < T(pl.radius)) {
            T sf = T(0);
            const sgi_atlas_entry e = a.caster_entries[l];
            if (viewDist < T(150))
                sf = shadow_8samples<T>(*a.caster_atlas, e, T(pl.far_plane), fragPos, lp, dot(lp - fragPos, normal),
                                        T(0.03f));
            else if (viewDist < T(750))
                sf = shadow_1sample<T>(*a.caster_atlas, e, T(pl.far_plane), fragPos, lp, dot(lp - fragPos, normal),
                                       T(0.03f));
            color = color + point_lighting2<T>(fragPos, baseColor, normal, viewDir, lp, lc, viewDist, roughness,
                                               metallic, ambient, sf, V3<T>(reflR),
                                               T(cfg.point_light_ambient_intensity), bp, fog);
        }
    }
    V3<T> lightDir(T(csm.light_direction[0]), T(csm.light_direction[1]), T(csm.light_direction[2]));
    V3<T> lightColor(T(csm.light_color[0]), T(csm.light_color[1]), T(csm.light_color[2]));
    V3<T> blends = cascade_blends(csm, fragPos);
    T shadowFactor = infinite_shadow(csm, fragPos, blends, normal, true);
    color = color + directional_lighting<T>(lightColor, lightDir, viewDir, normal, baseColor, viewDist, roughness,
                                            metallic, ambient, T(1) - shadowFactor, V3<T>(reflR), T(0), bp, fog);
    V3<T> o = vmin(color + emissive * T(cfg.emission_strength), C<T>::HALF_MAX());
    out[0] = Prec<T>::store16(o.x);
    out[1] = Prec<T>::store16(o.y);
    out[2] = Prec<T>::store16(o.z);
    out[3] = T(1);
}

template <class T> void deferred(const DeferredArgs& a, T* out) {
    const int W = a.cfg->width, H = a.cfg->height;
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            margin_begin<T>();
            deferred_pixel<T>(a, x, y, out + ((size_t)y * W + x) * 4);
            margin_end<T>((size_t)y * W + x);
        }
}

// ----------------------------------------------------------------- post FX --
// taa.fs (aa_common.glsl Reinhard tonemap) + gammaTonemap.fs, as sgi_post_fx.
// hdr, hist_in, hist_out: [P][4] holding binary16 values; hist_in NULL on the
// first TAA frame; ldr: RGBA8.
template <class T> inline V3<T> reinhard(V3<T> c) { return c / (c + V3<T>(T(1))); }
template <class T> inline V3<T> inverse_reinhard(V3<T> c) { return c / (V3<T>(T(1)) - c); }
template <class T> inline V3<T> vmin3(V3<T> a, V3<T> b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
template <class T> inline V3<T> vmax3(V3<T> a, V3<T> b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
template <class T> inline T aces_film(T x) {
    return saturate((x * (T(2.51f) * x + T(0.03f))) / (x * (T(2.43f) * x + T(0.59f)) + T(0.14f)));
}

template <class T> void post_fx(int W, int H, const float* hdr, const uint32_t* velocity, const float* hist_in,
                                float* hist_out, uint32_t* ldr, int taa) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t)y * W + x;
            auto at = [&](int xx, int yy) {
                xx = xx < 0 ? 0 : (xx >= W ? W - 1 : xx);
                yy = yy < 0 ? 0 : (yy >= H ? H - 1 : yy);
                const float* p = hdr + ((size_t)yy * W + xx) * 4;
                return V3<T>(T(p[0]), T(p[1]), T(p[2]));
            };
            V3<T> outc = at(x, y);
            if (taa) {
                const uint32_t vel = velocity[i];
                T u = (T(x) + T(0.5)) / T(W), v = (T(y) + T(0.5)) / T(H);
                T pu = u - T(f16_to_f32(uint16_t(vel & 0xffffu))), pv = v - T(f16_to_f32(uint16_t(vel >> 16)));
                V3<T> currentColor = at(x, y);
                V3<T> prevColor = currentColor;
                if (hist_in) {
                    auto ch = [&](int c) {
                        return [&, c](int ii, int jj) -> T { return T(hist_in[((size_t)jj * W + ii) * 4 + c]); };
                    };
                    prevColor = V3<T>(bilinear<T>(ch(0), W, H, pu, pv), bilinear<T>(ch(1), W, H, pu, pv),
                                      bilinear<T>(ch(2), W, H, pu, pv));
                }
                prevColor = reinhard(prevColor);
                V3<T> c1 = at(x, y + 1), c2 = at(x, y - 1), c3 = at(x + 1, y), c4 = at(x - 1, y);
                V3<T> minColor = reinhard(vmin3(currentColor, vmin3(c1, vmin3(c2, vmin3(c3, c4)))));
                V3<T> maxColor = reinhard(vmax3(currentColor, vmax3(c1, vmax3(c2, vmax3(c3, c4)))));
                currentColor = reinhard(currentColor);
                prevColor = vmin3(vmax3(prevColor, minColor), maxColor);
                currentColor = inverse_reinhard(currentColor);
                prevColor = inverse_reinhard(prevColor);
                V3<T> m(mix(currentColor.x, prevColor.x, T(0.9f)), mix(currentColor.y, prevColor.y, T(0.9f)),
                        mix(currentColor.z, prevColor.z, T(0.9f)));
                float* ho = hist_out + i * 4;
                ho[0] = Prec<T>::store16(m.x); ho[1] = Prec<T>::store16(m.y); ho[2] = Prec<T>::store16(m.z);
                ho[3] = Prec<T>::store16(T(0.0625f));
                outc = V3<T>(T(ho[0]), T(ho[1]), T(ho[2]));
            }
            const T inv_gamma = T(1.0f / 2.2f);
            auto q = [&](T c) { return (uint32_t)(saturate(std::pow(aces_film(c), inv_gamma)) * T(255) + T(0.5)); };
            ldr[i] = q(outc.x) | (q(outc.y) << 8) | (q(outc.z) << 16) | 0xff000000u;
        }
    }
}

}  // namespace oracle
