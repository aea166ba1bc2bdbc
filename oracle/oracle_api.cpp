// oracle/oracle_api.cpp - TEST INFRASTRUCTURE ONLY.
//
// C entry points of the CPU oracle (FP32 parity / FP64 accuracy
// instantiations of the restated StratusGFX passes) and a CPU ray caster that
// checks the GPU scene generator. Called from tests/ and from bench.py's
// cpu_baseline leg through ctypes; nothing in the shipped library links it.
//
// Parity is UNPINNED by the reference (no golden vectors exist in
// StratusGFX, and its GLSL cannot run without an OpenGL driver).
//
// prec selects the instantiation: 32 -> float (buffers are float32),
// 64 -> double (buffers are float64), 0 -> Counted (float32 buffers; the same
// values as 32, with the operations tallied, see counted.hpp) for the passes
// that report algorithmic FLOPs, 1 -> Tracked (float64 buffers; the values of
// 64, plus each pixel's smallest decision margin written to the buffer given
// to oracle_set_margin_output) for the gather, denoise and deferred passes.
#include <cstdio>
#include <cstring>
#include <vector>

#include "../include/sgi.h"
#include "../include/sgi_scene.h"
#include "glsl.hpp"
#include "counted.hpp"
#include "passes.hpp"

using namespace oracle;

extern "C" {

int oracle_version(void) { return 1; }

// ---- operation tallies of the prec = 0 instantiation -----------------------
void oracle_count_reset(void) { tally_reset(); }
void oracle_count_read(uint64_t* out2) { tally_read(&out2[0], &out2[1]); }

// ---- decision margins of the prec = 1 instantiation ---------------------------
// margins: [H][W][2] float64 (comparison, texel-choice margins), or NULL to stop recording.
void oracle_set_margin_output(double* margins) { set_margin_output(margins); }

// ---- known-answer helpers ---------------------------------------------------
float oracle_random3(float x, float y, float z) { return random3(x, y, z); }
uint32_t oracle_hash(uint32_t x) { return ghash(x); }
float oracle_exp_f32(float x) { return exp_f32(x); }
float oracle_pow128_f32(float x) { return pow128_f32(x); }
uint16_t oracle_f32_to_f16(float x) { return f32_to_f16(x); }
float oracle_f16_to_f32(uint16_t h) { return f16_to_f32(h); }

void oracle_world_from_depth(int prec, double u, double v, double depth, const float* inv_pv, double* out3) {
    if (prec == 32) {
        V3<float> p = world_from_depth<float>((float)u, (float)v, (float)depth, inv_pv);
        out3[0] = p.x; out3[1] = p.y; out3[2] = p.z;
    } else {
        V3<double> p = world_from_depth<double>(u, v, depth, inv_pv);
        out3[0] = p.x; out3[1] = p.y; out3[2] = p.z;
    }
}

// One VPL BRDF evaluation (calculateVirtualPointLighting2 with shadowFactor 0)
// for known-answer tests. in: frag[3], n[3], v[3], spec[3], diff[3], color[3],
// scalars: viewDist, radius, roughness, metallic, ao, refl, base[3].
void oracle_vpl_brdf(int prec, const double* in, const sgi_config* cfg, double* out3) {
    BrdfParams bp{cfg->min_roughness, cfg->use_perceptual_roughness};
    FogParams fog{cfg->fog_density, {cfg->fog_color[0], cfg->fog_color[1], cfg->fog_color[2]}};
    auto run = [&](auto tag) {
        using T = decltype(tag);
        auto v3 = [&](int o) { return V3<T>(T(in[o]), T(in[o + 1]), T(in[o + 2])); };
        V3<T> r = vpl_lighting2<T>(v3(0), v3(24), v3(3), v3(6), v3(9), v3(12), v3(15), T(in[18]), T(in[19]),
                                   T(in[20]), T(in[21]), T(in[22]), T(0), V3<T>(T(in[23])), bp, fog);
        out3[0] = r.x; out3[1] = r.y; out3[2] = r.z;
    };
    if (prec == 32) run(float()); else run(double());
}

// Lit fraction of calculateInfiniteShadowValue for a set of points.
void oracle_infinite_shadow(int prec, const sgi_csm* csm, const double* pts, const double* normals, int n,
                            int use_bias, double* out) {
    for (int i = 0; i < n; ++i) {
        if (prec == 32) {
            V3<float> p((float)pts[3 * i], (float)pts[3 * i + 1], (float)pts[3 * i + 2]);
            V3<float> nn((float)normals[3 * i], (float)normals[3 * i + 1], (float)normals[3 * i + 2]);
            out[i] = infinite_shadow<float>(*csm, p, cascade_blends(*csm, p), nn, use_bias != 0);
        } else {
            V3<double> p(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
            V3<double> nn(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
            out[i] = infinite_shadow<double>(*csm, p, cascade_blends(*csm, p), nn, use_bias != 0);
        }
    }
}

// ---- passes ------------------------------------------------------------------
int oracle_vis_cull(int prec, const sgi_vpl* vpls, int n, const sgi_csm* csm, int cap, int32_t* visible_index) {
    if (prec == 0) return vis_cull<Counted>(vpls, n, *csm, cap, visible_index);
    return prec == 32 ? vis_cull<float>(vpls, n, *csm, cap, visible_index)
                      : vis_cull<double>(vpls, n, *csm, cap, visible_index);
}

// Recolours cv[0..count) in place (FP32 or FP64 arithmetic, stored as float).
void oracle_color_vpls(int prec, sgi_vpl* cv, const sgi_atlas_entry* ce, int count, const sgi_cube_atlas* cubes,
                       const sgi_diffuse_atlas* diffuse, const sgi_csm* csm) {
    if (prec == 32) color_vpls<float>(cv, ce, count, *cubes, *diffuse, *csm);
    else color_vpls<double>(cv, ce, count, *cubes, *diffuse, *csm);
}

// taa.fs + gammaTonemap.fs (sgi_post_fx); float buffers hold binary16 values.
void oracle_post_fx(int prec, int W, int H, const float* hdr, const uint32_t* velocity, const float* hist_in,
                    float* hist_out, uint32_t* ldr, int taa) {
    if (prec == 32) post_fx<float>(W, H, hdr, velocity, hist_in, hist_out, ldr, taa);
    else post_fx<double>(W, H, hdr, velocity, hist_in, hist_out, ldr, taa);
}

void oracle_tile_stage1(int prec, const sgi_config* cfg, const sgi_gbuffer* g, const sgi_camera* cam, void* out) {
    if (prec == 0) tile_stage1<Counted>(*cfg, *g, *cam, (Counted*)out);
    else if (prec == 32) tile_stage1<float>(*cfg, *g, *cam, (float*)out);
    else tile_stage1<double>(*cfg, *g, *cam, (double*)out);
}

void oracle_tile_stage2(int prec, const sgi_config* cfg, const void* stage1, const sgi_vpl* cv, int count,
                        int32_t* lists) {
    if (prec == 0) tile_stage2<Counted>(*cfg, (const Counted*)stage1, cv, count, lists);
    else if (prec == 32) tile_stage2<float>(*cfg, (const float*)stage1, cv, count, lists);
    else tile_stage2<double>(*cfg, (const double*)stage1, cv, count, lists);
}

void oracle_gather(int prec, const sgi_config* cfg, const sgi_gbuffer* g, const sgi_camera* cam, const sgi_vpl* cv,
                   const sgi_atlas_entry* ce, int count, const int32_t* lists, const sgi_cube_atlas* cubes, float time,
                   void* reservoir) {
    GatherArgs a{cfg, g, cam, cv, ce, count, lists, cubes, time};
    if (prec == 0) gather<Counted>(a, (Counted*)reservoir);
    else if (prec == 1) gather<Tracked>(a, (Tracked*)reservoir);
    else if (prec == 32) gather<float>(a, (float*)reservoir);
    else gather<double>(a, (double*)reservoir);
}

void oracle_gi_target(const sgi_config* cfg, const sgi_gbuffer* g, const sgi_camera* cam, const sgi_vpl* cv,
                      const sgi_atlas_entry* ce, int count, const int32_t* lists, const sgi_cube_atlas* cubes,
                      float time, int batches, float* out) {
    GatherArgs a{cfg, g, cam, cv, ce, count, lists, cubes, time};
    gi_target(a, batches, out);
}

// Cumulative tallied FLOPs after each denoise pass of a prec = 0 run.
static uint64_t* g_pass_flops = nullptr;
static void record_pass_flops(int pass) {
    uint64_t f, c;
    tally_read(&f, &c);
    g_pass_flops[pass] = f;
}

// hdr_in, gi_prev: [P][4]; hist_prev: [P]; all buffers of the precision's type.
// pass_flops (prec = 0 only, may be NULL): [denoise_passes] tallied FLOPs after each pass.
void oracle_denoise(int prec, const sgi_config* cfg, const sgi_gbuffer* cur, const sgi_gbuffer* prev,
                    const void* reservoir, const void* hdr_in, const void* gi_prev, const void* hist_prev,
                    int num_visible, const sgi_frame_params* params, void* combined, void* gi_out, void* hist_out,
                    void* pass_out, uint64_t* pass_flops) {
    g_pass_flops = pass_flops;
    if (prec == 0) {
        DenoiseArgs<Counted> a{cfg, cur, prev, (const Counted*)hdr_in, (const Counted*)gi_prev,
                               (const Counted*)hist_prev, num_visible, params->time, params->frames_per_second};
        denoise<Counted>(a, (const Counted*)reservoir, (Counted*)combined, (Counted*)gi_out, (Counted*)hist_out,
                         (Counted*)pass_out, pass_flops ? record_pass_flops : nullptr);
    } else if (prec == 32) {
        DenoiseArgs<float> a{cfg, cur, prev, (const float*)hdr_in, (const float*)gi_prev, (const float*)hist_prev,
                             num_visible, params->time, params->frames_per_second};
        denoise<float>(a, (const float*)reservoir, (float*)combined, (float*)gi_out, (float*)hist_out, (float*)pass_out);
    } else {
        DenoiseArgs<double> a{cfg, cur, prev, (const double*)hdr_in, (const double*)gi_prev, (const double*)hist_prev,
                              num_visible, params->time, params->frames_per_second};
        denoise<double>(a, (const double*)reservoir, (double*)combined, (double*)gi_out, (double*)hist_out,
                        (double*)pass_out);
    }
}

// One denoise pass `pass` from the reservoir res_in (prec 32, 64 or 1); the final
// pass also writes combined, gi_out and hist_out. Buffers as for oracle_denoise.
void oracle_denoise_pass(int prec, const sgi_config* cfg, const sgi_gbuffer* cur, const sgi_gbuffer* prev, int pass,
                         const void* res_in, const void* hdr_in, const void* gi_prev, const void* hist_prev,
                         int num_visible, const sgi_frame_params* params, void* res_out, void* combined,
                         void* gi_out, void* hist_out) {
    auto run = [&](auto zero) {
        using T = decltype(zero);
        DenoiseArgs<T> a{cfg, cur, prev, (const T*)hdr_in, (const T*)gi_prev, (const T*)hist_prev, num_visible,
                         params->time, params->frames_per_second};
        denoise_one_pass<T>(a, pass, (const T*)res_in, (T*)res_out, (T*)combined, (T*)gi_out, (T*)hist_out);
    };
    if (prec == 32) run(float());
    else if (prec == 1) run(Tracked());
    else run(double());
}

// casters / caster_entries / caster_atlas: shadow-casting point lights (num_casters may be 0).
void oracle_deferred(int prec, const sgi_config* cfg, const sgi_gbuffer* g, const sgi_camera* cam,
                     const sgi_point_light* points, int num_points, const sgi_csm* csm, void* out,
                     const sgi_point_light* casters, const sgi_atlas_entry* caster_entries, int num_casters,
                     const sgi_cube_atlas* caster_atlas) {
    DeferredArgs a{cfg, g, cam, points, num_points, csm, casters, caster_entries, num_casters, caster_atlas};
    if (prec == 0) deferred<Counted>(a, (Counted*)out);
    else if (prec == 1) deferred<Tracked>(a, (Tracked*)out);
    else if (prec == 32) deferred<float>(a, (float*)out);
    else deferred<double>(a, (double*)out);
}

// ---- CPU ray caster (checker of sgi_scene_*) -----------------------------------
// Slab test; returns entry t (may be negative) and the entry axis, or false.
static bool ray_box(const float* o, const float* d, const sgi_box& b, float& tnear, int& axis, float& tfar) {
    tnear = -INFINITY; tfar = INFINITY; axis = 0;
    for (int k = 0; k < 3; ++k) {
        if (d[k] == 0.0f) {
            if (o[k] < b.min[k] || o[k] > b.max[k]) return false;
            continue;
        }
        float t1 = (b.min[k] - o[k]) / d[k];
        float t2 = (b.max[k] - o[k]) / d[k];
        float lo = t1 < t2 ? t1 : t2, hi = t1 < t2 ? t2 : t1;
        if (lo > tnear) { tnear = lo; axis = k; }
        if (hi < tfar) tfar = hi;
    }
    return tnear <= tfar;
}

static inline uint32_t enc_unorm8(float v) {
    v = gclamp(v, 0.0f, 1.0f);
    return (uint32_t)(v * 255.0f + 0.5f);
}

static inline V4<float> mul4(const float* m, float x, float y, float z, float w) { return mat4_mul<float>(m, x, y, z, w); }

void oracle_scene_gbuffer(const sgi_box* boxes, int nb, const sgi_scene_camera* cam, int W, int H, float* depth,
                          uint32_t* normal, uint32_t* albedo, uint16_t* refl, uint32_t* rma, uint32_t* velocity,
                          float* id, uint16_t* ssao) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            size_t i = (size_t)y * W + x;
            float nx = ((float(x) + 0.5f) / float(W)) * 2.0f - 1.0f;
            float ny = ((float(y) + 0.5f) / float(H)) * 2.0f - 1.0f;
            V4<float> a = mul4(cam->inv_proj_view, nx, ny, -1.0f, 1.0f);
            V4<float> b = mul4(cam->inv_proj_view, nx, ny, 1.0f, 1.0f);
            float o[3] = {a.x / a.w, a.y / a.w, a.z / a.w};
            float e[3] = {b.x / b.w, b.y / b.w, b.z / b.w};
            float d[3] = {e[0] - o[0], e[1] - o[1], e[2] - o[2]};
            float best = INFINITY; int bi = -1, bax = 0;
            for (int k = 0; k < nb; ++k) {
                float tn, tf; int ax;
                if (!ray_box(o, d, boxes[k], tn, ax, tf)) continue;
                if (tn > 0.0f && tn < best) { best = tn; bi = k; bax = ax; }
            }
            if (bi < 0) {
                depth[i] = 1.0f; normal[i] = 0x00ff8080u; albedo[i] = 0; refl[i] = 0; rma[i] = 0;
                velocity[i] = 0; id[i] = 0.0f; ssao[i] = f32_to_f16(1.0f);
                continue;
            }
            const sgi_box& bx = boxes[bi];
            float p[3] = {o[0] + d[0] * best, o[1] + d[1] * best, o[2] + d[2] * best};
            float n[3] = {0.0f, 0.0f, 0.0f};
            n[bax] = d[bax] > 0.0f ? -1.0f : 1.0f;
            V4<float> c = mul4(cam->proj_view, p[0], p[1], p[2], 1.0f);
            V4<float> pc = mul4(cam->prev_proj_view, p[0], p[1], p[2], 1.0f);
            depth[i] = (c.z / c.w) * 0.5f + 0.5f;
            float cu = (c.x / c.w) * 0.5f + 0.5f, cv = (c.y / c.w) * 0.5f + 0.5f;
            float pu = (pc.x / pc.w) * 0.5f + 0.5f, pv = (pc.y / pc.w) * 0.5f + 0.5f;
            velocity[i] = (uint32_t)f32_to_f16(cu - pu) | ((uint32_t)f32_to_f16(cv - pv) << 16);
            normal[i] = enc_unorm8(n[0] * 0.5f + 0.5f) | (enc_unorm8(n[1] * 0.5f + 0.5f) << 8) |
                        (enc_unorm8(n[2] * 0.5f + 0.5f) << 16) | 0xff000000u;
            albedo[i] = enc_unorm8(bx.albedo[0]) | (enc_unorm8(bx.albedo[1]) << 8) | (enc_unorm8(bx.albedo[2]) << 16) |
                        (enc_unorm8(bx.albedo[3]) << 24);
            refl[i] = (uint16_t)enc_unorm8(bx.reflectance);
            rma[i] = enc_unorm8(bx.roughness) | (enc_unorm8(bx.metallic) << 8) | 0xff000000u;
            id[i] = bx.id;
            float h = p[1] < 0.0f ? 0.0f : p[1];
            ssao[i] = f32_to_f16(0.2f + 0.8f * (h / (h + 0.5f)));
        }
    }
}

void oracle_scene_csm(const sgi_box* boxes, int nb, const sgi_csm* csm, const float* inv_pv /*[4][16]*/,
                      float* depth_out) {
    const int R = csm->resolution;
    for (int c = 0; c < csm->num_cascades; ++c) {
        const float* M = csm->cascade_proj_view[c];
        const float* IM = inv_pv + 16 * c;
#pragma omp parallel for schedule(dynamic, 4)
        for (int j = 0; j < R; ++j) {
            for (int i = 0; i < R; ++i) {
                float nx = ((float(i) + 0.5f) / float(R)) * 2.0f - 1.0f;
                float ny = ((float(j) + 0.5f) / float(R)) * 2.0f - 1.0f;
                V4<float> a = mul4(IM, nx, ny, -1.0f, 1.0f);
                V4<float> b = mul4(IM, nx, ny, 1.0f, 1.0f);
                float o[3] = {a.x / a.w, a.y / a.w, a.z / a.w};
                float e[3] = {b.x / b.w, b.y / b.w, b.z / b.w};
                float d[3] = {e[0] - o[0], e[1] - o[1], e[2] - o[2]};
                float best = INFINITY; int bi = -1, bax = 0;
                for (int k = 0; k < nb; ++k) {
                    float tn, tf; int ax;
                    if (!ray_box(o, d, boxes[k], tn, ax, tf)) continue;
                    if (tn < best) { best = tn; bi = k; bax = ax; }
                }
                float out = 1.0f;
                if (bi >= 0) {
                    float p[3] = {o[0] + d[0] * best, o[1] + d[1] * best, o[2] + d[2] * best};
                    V4<float> cc = mul4(M, p[0], p[1], p[2], 1.0f);
                    float z = (cc.z / cc.w) * 0.5f + 0.5f;
                    // slope-scaled offset: clip-space normal = (M^-1)^T n (columns of IM dotted with n)
                    float ncx = IM[0 * 4 + bax], ncy = IM[1 * 4 + bax], ncz = IM[2 * 4 + bax];
                    float anz = gabs(ncz);
                    float slope = gmax(gabs(ncx), gabs(ncy)) / (anz * float(R));
                    if (!(slope < 1.0f)) slope = 1.0f;
                    out = gclamp(z + 2.0f * slope, 0.0f, 1.0f);
                }
                depth_out[((size_t)c * R + j) * R + i] = out;
            }
        }
    }
}

static inline void cube_dir(int face, float sc, float tc, float* d) {
    switch (face) {
        case 0: d[0] = 1.0f; d[1] = -tc; d[2] = -sc; break;
        case 1: d[0] = -1.0f; d[1] = -tc; d[2] = sc; break;
        case 2: d[0] = sc; d[1] = 1.0f; d[2] = tc; break;
        case 3: d[0] = sc; d[1] = -1.0f; d[2] = -tc; break;
        case 4: d[0] = sc; d[1] = -tc; d[2] = 1.0f; break;
        default: d[0] = -sc; d[1] = -tc; d[2] = -1.0f; break;
    }
}

void oracle_scene_cube_atlas(const sgi_box* boxes, int nb, const sgi_vpl* vpls, const sgi_atlas_entry* entries,
                             int count, const sgi_cube_atlas* atlas) {
    const int n = atlas->face_size;
#pragma omp parallel for schedule(dynamic, 1)
    for (int v = 0; v < count; ++v) {
        const sgi_vpl& vp = vpls[v];
        sgi_atlas_entry e = entries[v];
        for (int f = 0; f < 6; ++f) {
            for (int j = 0; j < n; ++j) {
                for (int i = 0; i < n; ++i) {
                    float sc = ((float(i) + 0.5f) / float(n)) * 2.0f - 1.0f;
                    float tc = ((float(j) + 0.5f) / float(n)) * 2.0f - 1.0f;
                    float d[3];
                    cube_dir(f, sc, tc, d);
                    float best = INFINITY;
                    for (int k = 0; k < nb; ++k) {
                        float tn, tf; int ax;
                        if (!ray_box(vp.position, d, boxes[k], tn, ax, tf)) continue;
                        if (tn > 0.0f && tn < best) best = tn;
                    }
                    float val = 1.0f;
                    if (best < INFINITY) {
                        float len = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
                        val = saturate((best * len) / vp.far_plane);
                    }
                    size_t off = (((size_t)e.layer * 6 + f) * n + j) * n + i;
                    if (atlas->format == SGI_CUBE_F32) ((float*)atlas->atlas[e.index])[off] = val;
                    else if (atlas->format == SGI_CUBE_F16) ((uint16_t*)atlas->atlas[e.index])[off] = f32_to_f16(val);
                    else ((uint16_t*)atlas->atlas[e.index])[off] = (uint16_t)(val * 65535.0f + 0.5f);
                }
            }
        }
    }
}

void oracle_scene_diffuse_atlas(const sgi_box* boxes, int nb, const sgi_vpl* vpls, const sgi_atlas_entry* entries,
                                int count, const sgi_diffuse_atlas* atlas) {
    const int n = atlas->face_size;
#pragma omp parallel for schedule(dynamic, 1)
    for (int v = 0; v < count; ++v) {
        const sgi_vpl& vp = vpls[v];
        sgi_atlas_entry e = entries[v];
        for (int f = 0; f < 6; ++f) {
            for (int j = 0; j < n; ++j) {
                for (int i = 0; i < n; ++i) {
                    float sc = ((float(i) + 0.5f) / float(n)) * 2.0f - 1.0f;
                    float tc = ((float(j) + 0.5f) / float(n)) * 2.0f - 1.0f;
                    float d[3];
                    cube_dir(f, sc, tc, d);
                    float best = INFINITY;
                    int bi = -1;
                    for (int k = 0; k < nb; ++k) {
                        float tn, tf; int ax;
                        if (!ray_box(vp.position, d, boxes[k], tn, ax, tf)) continue;
                        if (tn > 0.0f && tn < best) { best = tn; bi = k; }
                    }
                    uint32_t t = 0;
                    if (bi >= 0)
                        t = enc_unorm8(boxes[bi].albedo[0]) | (enc_unorm8(boxes[bi].albedo[1]) << 8) |
                            (enc_unorm8(boxes[bi].albedo[2]) << 16) | 0xff000000u;
                    size_t off = (((size_t)e.layer * 6 + f) * n + j) * n + i;
                    ((uint32_t*)atlas->atlas[e.index])[off] = t;
                }
            }
        }
    }
}

}  // extern "C"
