// sgi_api.cpp - C ABI of the GI/lighting stage (include/sgi.h) and of the
// scene generator (include/sgi_scene.h).
//
// Host orchestration that replaces, per frame and without any GPU->CPU sync:
//   RendererBackend::PerformVirtualPointLightCullingStage1_  StratusRendererBackend.cpp:1578-1661
//   RendererBackend::PerformVirtualPointLightCullingStage2_  :1666-1814 (the MapMemory readback
//       at :1675 is gone: atlas slots travel with the compacted list on the device)
//   RendererBackend::ComputeVirtualPointLightGlobalIllumination_ :1816-1952
//   the deferred lighting block of RenderScene               :2011-2038
// Status codes instead of exceptions (the reference throws at :70-72, :1083, :2659).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <new>
#include <mutex>
#include <string>

#include "../../include/sgi.h"
#include "../../include/sgi_nn.h"
#include "../../include/sgi_scene.h"
#include "sgi_ctx.h"
#include "sgi_internal.h"
#include "sgi_nn_internal.h"
#include "sgi_nn_net.h"


namespace {

// the log callback (sgi_set_log_callback); every failure of a context is reported through it
std::mutex g_log_lock;
sgi_log_fn g_log_fn = nullptr;
void* g_log_user = nullptr;

sgi_status fail(sgi_ctx* c, sgi_status s, const std::string& msg) {
    if (c) c->err = msg;
    sgi_log_message(SGI_LOG_ERROR, msg.c_str());
    return s;
}

sgi_status cuda_fail(sgi_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? SGI_ERR_OOM : SGI_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define SGI_CUDA(ctx, call, what)                           \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

template <class T> cudaError_t dalloc(T** p, size_t count) {
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T));
}

size_t pixels(const sgi_config& c) { return (size_t)c.width * (size_t)c.height; }

sgi_status validate_config(const sgi_config* cfg, std::string& why) {
    if (!cfg) { why = "config is NULL"; return SGI_ERR_ARG; }
    if (cfg->width < 1 || cfg->height < 1 || cfg->width > 16384 || cfg->height > 16384) {
        why = "width/height must be in [1, 16384]"; return SGI_ERR_ARG;
    }
    if (cfg->max_vpls < 1 || cfg->max_vpls > SGI_MAX_VPLS_BEFORE_CULL) {
        why = "max_vpls must be in [1, 10000]"; return SGI_ERR_ARG;
    }
    if (cfg->max_visible < 1 || cfg->max_visible > SGI_MAX_VPLS_BEFORE_CULL) {
        why = "max_visible must be in [1, 10000]"; return SGI_ERR_ARG;
    }
    if (cfg->tile_size < 4 || cfg->tile_size > 32) {
        why = "tile_size must be in [4, 32]"; return SGI_ERR_ARG;
    }
    if (cfg->max_vpls_per_tile < 1 || cfg->max_vpls_per_tile > SGI_MAX_TILE_LIST) {
        why = "max_vpls_per_tile must be in [1, 64]"; return SGI_ERR_ARG;
    }
    if (cfg->gi_mode != SGI_GI_REFERENCE && cfg->gi_mode != SGI_GI_TILED) { why = "bad gi_mode"; return SGI_ERR_ARG; }
    if (cfg->samples_per_pixel < 0 || cfg->samples_per_pixel > 1024) {
        why = "samples_per_pixel must be in [0, 1024]"; return SGI_ERR_ARG;
    }
    if (cfg->denoise_passes < 2 || cfg->denoise_passes > SGI_MAX_DENOISE_PASSES) {
        why = "denoise_passes must be in [2, 8]"; return SGI_ERR_ARG;
    }
    return SGI_OK;
}

bool gbuffer_ok(const sgi_gbuffer* g, bool need_all) {
    if (!g || !g->depth || !g->normal) return false;
    if (!need_all) return true;
    return g->albedo && g->base_reflectivity && g->roughness_metallic_ambient && g->velocity && g->id && g->ssao;
}

sgi::ShadeConfig make_shade(const sgi_config& c) {
    sgi::ShadeConfig s;
    s.min_roughness = c.min_roughness;
    s.perceptual = c.use_perceptual_roughness;
    s.fog_density = c.fog_density;
    for (int k = 0; k < 3; ++k) s.fog_color[k] = c.fog_color[k];
    s.point_ambient = c.point_light_ambient_intensity;
    s.min_gi_occlusion = c.min_gi_occlusion_factor;
    s.emission_strength = c.emission_strength;
    return s;
}

void free_all(sgi_ctx* c) {
    void* ptrs[] = {c->vpls, c->entries, c->points, c->shadow_points, c->shadow_entries, c->taa_hist[0],
                    c->taa_hist[1], c->flags, c->cv, c->ce, c->visible_index, c->stage1, c->lists,
                    c->vpr, c->reservoir, c->ping[0], c->ping[1], c->merged, c->direct, c->guide, c->gi_hist[0], c->gi_hist[1],
                    c->hist_depth[0], c->hist_depth[1], c->dev_status, c->cull_finished};
    for (void* p : ptrs) if (p) cudaFree(p);
    for (auto* p : c->pass_bufs) if (p) cudaFree(p);
    void* nnp[] = {c->nn_feat, c->nn_prev};
    for (void* p : nnp) if (p) cudaFree(p);
    for (auto& e : c->ev) if (e) cudaEventDestroy(e);
    if (c->ev_atrous_end) cudaEventDestroy(c->ev_atrous_end);
    if (c->fork) cudaEventDestroy(c->fork);
    if (c->join) cudaEventDestroy(c->join);
    if (c->side) cudaStreamDestroy(c->side);
}

inline void record(sgi_ctx* c, int k, cudaStream_t s) {
    if (c->timing) cudaEventRecord(c->ev[k], s);
}

// The context's build of a shading kernel: exact (bit-identical to the CPU
// restatement) or the tolerance mode (sgi_set_shading_precision).
#define SGI_SHADE(c, fn) ((c)->fast_shading ? sgi::fast::fn : sgi::exact::fn)

}  // namespace

extern "C" {

void sgi_set_log_callback(sgi_log_fn fn, void* user) {
    std::lock_guard<std::mutex> g(g_log_lock);
    g_log_fn = fn;
    g_log_user = user;
}

void sgi_log_message(int32_t level, const char* msg) {
    sgi_log_fn fn;
    void* user;
    {
        std::lock_guard<std::mutex> g(g_log_lock);
        fn = g_log_fn;
        user = g_log_user;
    }
    if (fn && msg) fn(level, msg, user);
}

int32_t sgi_abi_version(void) { return SGI_ABI_VERSION; }

const char* sgi_status_string(sgi_status s) {
    switch (s) {
        case SGI_OK: return "ok";
        case SGI_ERR_ARG: return "invalid argument";
        case SGI_ERR_OOM: return "out of device memory";
        case SGI_ERR_CUDA: return "CUDA error";
        case SGI_ERR_TIMEOUT: return "device wait timed out";
        case SGI_ERR_CAP: return "capacity exceeded";
        case SGI_ERR_STATE: return "invalid call order";
        default: return "unknown status";
    }
}

void sgi_config_defaults(sgi_config* cfg, int32_t width, int32_t height) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->width = width;
    cfg->height = height;
    cfg->max_vpls = SGI_MAX_VPLS_BEFORE_CULL;
    cfg->max_visible = SGI_MAX_VPLS_PER_FRAME;
    cfg->tile_size = 5;                 // VirtualPointLightData::tileXDivisor, StratusRendererBackend.h:346-347
    cfg->max_vpls_per_tile = 12;        // MAX_VPLS_PER_TILE, vpl_common.glsl:9
    cfg->gi_mode = SGI_GI_REFERENCE;
    cfg->samples_per_pixel = 0;
    cfg->denoise_passes = 4;
    cfg->debug_keep_passes = 0;
    cfg->min_roughness = 0.08f;
    cfg->use_perceptual_roughness = 1;
    cfg->min_gi_occlusion_factor = 0.95f;
    cfg->emission_strength = 0.0f;
    cfg->fog_density = 0.0f;
    cfg->fog_color[0] = cfg->fog_color[1] = cfg->fog_color[2] = 0.5f;
    cfg->point_light_ambient_intensity = 0.003f;
}

const char* sgi_last_error(const sgi_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int64_t sgi_launch_count(const sgi_ctx* ctx) { return ctx ? ctx->launches : 0; }

sgi_status sgi_create(const sgi_config* cfg, sgi_ctx** out) {
    if (!out) return SGI_ERR_ARG;
    *out = nullptr;
    std::string why;
    sgi_status st = validate_config(cfg, why);
    if (st != SGI_OK) sgi_log_message(SGI_LOG_ERROR, ("sgi_create: " + why).c_str());
    if (st != SGI_OK) return st;
    sgi_ctx* c = new (std::nothrow) sgi_ctx();
    if (!c) return SGI_ERR_OOM;
    c->cfg = *cfg;
    c->sc = make_shade(*cfg);
    std::memset(&c->csm, 0, sizeof(c->csm));
    std::memset(&c->cubes, 0, sizeof(c->cubes));
    cudaGetDevice(&c->device);
    const int ts = cfg->tile_size;
    c->num_tiles = ((cfg->width + ts - 1) / ts) * ((cfg->height + ts - 1) / ts);
    const size_t P = pixels(*cfg);
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t r) { if (e == cudaSuccess && r != cudaSuccess) e = r; };
    chk(dalloc(&c->vpls, cfg->max_vpls));
    chk(dalloc(&c->entries, cfg->max_vpls));
    chk(dalloc(&c->points, SGI_MAX_POINT_LIGHTS));
    chk(dalloc(&c->shadow_points, SGI_MAX_POINT_LIGHTS));
    chk(dalloc(&c->shadow_entries, SGI_MAX_POINT_LIGHTS));
    chk(dalloc(&c->flags, cfg->max_vpls));
    chk(dalloc(&c->cv, cfg->max_visible));
    chk(dalloc(&c->ce, cfg->max_visible));
    chk(dalloc(&c->visible_index, 1 + (size_t)cfg->max_vpls));
    chk(dalloc(&c->stage1, c->num_tiles));
    chk(dalloc(&c->lists, (size_t)c->num_tiles * (1 + cfg->max_vpls_per_tile)));
    chk(dalloc(&c->vpr, (size_t)cfg->max_visible));
    chk(dalloc(&c->reservoir, cfg->debug_keep_passes ? P : 1));
    chk(dalloc(&c->guide, P));
    chk(dalloc(&c->ping[0], P));
    chk(dalloc(&c->ping[1], P));
    chk(dalloc(&c->merged, P));
    chk(dalloc(&c->direct, P));
    chk(dalloc(&c->gi_hist[0], P));
    chk(dalloc(&c->gi_hist[1], P));
    chk(dalloc(&c->hist_depth[0], P));
    chk(dalloc(&c->hist_depth[1], P));
    chk(dalloc(&c->dev_status, 1));
    chk(dalloc(&c->cull_finished, 1));
    if (cfg->debug_keep_passes)
        for (int k = 0; k < cfg->denoise_passes; ++k) chk(dalloc(&c->pass_bufs[k], P));
    for (auto& ev : c->ev) chk(cudaEventCreate(&ev));
    chk(cudaEventCreate(&c->ev_atrous_end));
    chk(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    chk(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
    chk(cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming));
    if (e == cudaSuccess) chk(cudaMemset(c->visible_index, 0, sizeof(int32_t) * (1 + (size_t)cfg->max_vpls)));
    if (e == cudaSuccess) chk(cudaMemset(c->dev_status, 0, sizeof(int32_t)));
    if (e == cudaSuccess) chk(cudaMemset(c->cull_finished, 0, sizeof(unsigned)));
    if (e == cudaSuccess) chk(cudaMemset(c->gi_hist[0], 0, P * sizeof(uint2)));
    if (e == cudaSuccess) chk(cudaMemset(c->gi_hist[1], 0, P * sizeof(uint2)));
    if (e == cudaSuccess) chk(cudaMemset(c->hist_depth[0], 0, P * sizeof(uint16_t)));
    if (e == cudaSuccess) chk(cudaMemset(c->hist_depth[1], 0, P * sizeof(uint16_t)));
    if (e == cudaSuccess) chk(cudaDeviceSynchronize());
    if (e != cudaSuccess) {
        free_all(c);
        delete c;
        return e == cudaErrorMemoryAllocation ? SGI_ERR_OOM : SGI_ERR_CUDA;
    }
    *out = c;
    return SGI_OK;
}

sgi_status sgi_destroy(sgi_ctx* ctx) {
    if (!ctx) return SGI_ERR_ARG;
    cudaDeviceSynchronize();
    free_all(ctx);
    delete ctx;
    return SGI_OK;
}

sgi_status sgi_set_lights(sgi_ctx* ctx, const sgi_vpl* vpls, const sgi_atlas_entry* entries, int32_t num_vpls,
                          const sgi_point_light* points, int32_t num_points, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (num_vpls < 0 || num_points < 0) return fail(ctx, SGI_ERR_ARG, "negative light count");
    if (num_vpls > ctx->cfg.max_vpls) return fail(ctx, SGI_ERR_CAP, "num_vpls exceeds max_vpls");
    if (num_points > SGI_MAX_POINT_LIGHTS) return fail(ctx, SGI_ERR_CAP, "num_points exceeds 256");
    if (num_vpls > 0 && (!vpls || !entries)) return fail(ctx, SGI_ERR_ARG, "vpls/entries NULL");
    if (num_points > 0 && !points) return fail(ctx, SGI_ERR_ARG, "points NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (num_vpls > 0) {
        SGI_CUDA(ctx, cudaMemcpyAsync(ctx->vpls, vpls, sizeof(sgi_vpl) * num_vpls, cudaMemcpyDefault, s), "copy vpls");
        SGI_CUDA(ctx, cudaMemcpyAsync(ctx->entries, entries, sizeof(sgi_atlas_entry) * num_vpls, cudaMemcpyDefault, s),
                 "copy atlas entries");
    }
    if (num_points > 0)
        SGI_CUDA(ctx, cudaMemcpyAsync(ctx->points, points, sizeof(sgi_point_light) * num_points, cudaMemcpyDefault, s),
                 "copy point lights");
    ctx->num_vpls = num_vpls;
    ctx->num_points = num_points;
    ctx->lights_set = true;
    ctx->culled = false;
    return SGI_OK;
}

sgi_status sgi_set_shadow_maps(sgi_ctx* ctx, const sgi_csm* csm, const sgi_cube_atlas* cubes) {
    if (!ctx || !csm || !cubes) return fail(ctx, SGI_ERR_ARG, "NULL csm or cube atlas");
    if (!csm->depth || csm->resolution < 1 || csm->num_cascades != 4)
        return fail(ctx, SGI_ERR_ARG, "csm needs a depth pointer, resolution >= 1 and 4 cascades");
    if (cubes->num_atlases < 0 || cubes->num_atlases > SGI_MAX_ATLASES || cubes->face_size < 1 ||
        cubes->face_size > SGI_MAX_CUBE_FACE ||
        cubes->layers_per_atlas < 0 || cubes->format < SGI_CUBE_F32 || cubes->format > SGI_CUBE_UNORM16)
        return fail(ctx, SGI_ERR_ARG, "bad cube atlas description");
    for (int a = 0; a < cubes->num_atlases; ++a)
        if (!cubes->atlas[a]) return fail(ctx, SGI_ERR_ARG, "NULL cube atlas pointer");
    ctx->csm = *csm;
    ctx->cubes = *cubes;
    ctx->maps_set = true;
    return SGI_OK;
}

sgi_status sgi_cull_vpls(sgi_ctx* ctx, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (!ctx->lights_set || !ctx->maps_set) return fail(ctx, SGI_ERR_STATE, "set lights and shadow maps first");
    cudaStream_t s = (cudaStream_t)stream;
    if (ctx->num_vpls == 0) {
        SGI_CUDA(ctx, cudaMemsetAsync(ctx->visible_index, 0, sizeof(int32_t), s), "clear visible count");
    } else {
        SGI_CUDA(ctx, sgi::launch_vpl_cull(ctx->vpls, ctx->entries, ctx->num_vpls, ctx->csm, ctx->flags,
                                           ctx->cfg.max_visible, ctx->cv, ctx->ce, ctx->visible_index, ctx->vpr,
                                           ctx->cull_finished, s),
                 "vpl_cull");
        ctx->launches += 1;
        if (ctx->coloring) {
            SGI_CUDA(ctx, sgi::launch_vpl_color(ctx->cv, ctx->ce, ctx->visible_index, ctx->cfg.max_visible,
                                                ctx->cubes, ctx->diffuse, ctx->csm, s), "vpl_color");
            ctx->launches += 1;
        }
    }
    ctx->culled = true;
    return SGI_OK;
}

sgi_status sgi_cull_vpls_noalloc(const sgi_vpl* vpls, const sgi_atlas_entry* entries, int32_t num_vpls,
                                 const sgi_csm* csm, int32_t max_visible, sgi_vpl* visible_vpls,
                                 sgi_atlas_entry* visible_entries, int32_t* visible_index, void* stream) {
    if (!csm || !visible_vpls || !visible_entries || !visible_index || max_visible < 1 || num_vpls < 0)
        return SGI_ERR_ARG;
    if (num_vpls > SGI_NOALLOC_CULL_MAX_VPLS) return SGI_ERR_CAP;
    if (num_vpls > 0 && (!vpls || !entries)) return SGI_ERR_ARG;
    if (((uintptr_t)vpls & 15) || ((uintptr_t)visible_vpls & 15) || ((uintptr_t)entries & 7) ||
        ((uintptr_t)visible_entries & 7) || ((uintptr_t)visible_index & 3))
        return SGI_ERR_ARG;
    if (!csm->depth || csm->resolution < 1 || csm->num_cascades != 4) return SGI_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (num_vpls == 0) return cudaMemsetAsync(visible_index, 0, sizeof(int32_t), s) == cudaSuccess ? SGI_OK : SGI_ERR_CUDA;
    uint8_t* flags = nullptr;
    if (sgi::noalloc_cull_flags(&flags) != cudaSuccess) return SGI_ERR_CUDA;
    if (sgi::launch_vis_flags(vpls, num_vpls, *csm, flags, s) != cudaSuccess) return SGI_ERR_CUDA;
    if (sgi::launch_compact(vpls, entries, flags, num_vpls, max_visible, visible_vpls, visible_entries, visible_index,
                            nullptr, s) != cudaSuccess)
        return SGI_ERR_CUDA;
    return SGI_OK;
}

sgi_status sgi_cull_tiles(sgi_ctx* ctx, const sgi_gbuffer* gbuf, const sgi_camera* cam, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (!gbuffer_ok(gbuf, false) || !cam) return fail(ctx, SGI_ERR_ARG, "NULL G-buffer depth/normal or camera");
    if (!ctx->culled) return fail(ctx, SGI_ERR_STATE, "sgi_cull_vpls must run before sgi_cull_tiles");
    cudaStream_t s = (cudaStream_t)stream;
    SGI_CUDA(ctx, sgi::launch_tile_stage1(ctx->cfg, *gbuf, *cam, ctx->stage1, s), "tile_stage1");
    SGI_CUDA(ctx, sgi::launch_tile_stage2(ctx->cfg, ctx->stage1, ctx->vpr, ctx->visible_index, ctx->lists, s),
             "tile_stage2");
    ctx->launches += 2;
    return SGI_OK;
}

sgi_status sgi_direct_lighting(sgi_ctx* ctx, const sgi_gbuffer* gbuf, const sgi_camera* cam, void* hdr_out,
                               void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (!gbuffer_ok(gbuf, true) || !cam || !hdr_out) return fail(ctx, SGI_ERR_ARG, "NULL G-buffer, camera or output");
    if (!ctx->lights_set || !ctx->maps_set) return fail(ctx, SGI_ERR_STATE, "set lights and shadow maps first");
    sgi::ShadowCasters casters{ctx->shadow_points, ctx->shadow_entries, ctx->num_shadow_points, ctx->shadow_atlas};
    SGI_CUDA(ctx, SGI_SHADE(ctx, launch_deferred)(ctx->cfg, ctx->sc, *gbuf, *cam, ctx->points, ctx->num_points, casters, ctx->csm,
                                       (uint2*)hdr_out, (cudaStream_t)stream, ctx->block_dim(SGI_BLOCK_DIRECT)),
             "deferred_pbr_csm");
    ctx->launches += 1;
    return SGI_OK;
}

// vpl_pbr_gi.fs, with denoise pass 0 (the centre-only reservoir merge) in its epilogue
static sgi_status run_gather(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_camera* cam,
                             const sgi_frame_params* params, cudaStream_t s) {
    const sgi_config& cfg = ctx->cfg;
    const bool keep = cfg.debug_keep_passes != 0;
    sgi::GatherOut go;
    go.merged = keep ? ctx->pass_bufs[0] : ctx->merged;
    go.guide = ctx->guide;
    go.raw = keep ? ctx->reservoir : nullptr;
    SGI_CUDA(ctx, SGI_SHADE(ctx, launch_gather)(cfg, ctx->sc, *cur, *cam, ctx->cv, ctx->ce, ctx->visible_index, ctx->lists,
                                     ctx->cubes, params->time, go, s, ctx->block_dim(SGI_BLOCK_GATHER)),
             "vpl_gather");
    ctx->launches += 1;
    ctx->last_merged = go.merged;
    ctx->feat_hist = ctx->hist_cur;
    ctx->feat_have_history = ctx->have_history;
    return SGI_OK;
}

static sgi_status run_gi(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_gbuffer* prev, const sgi_camera* cam,
                         const void* hdr_in, void* hdr_out, const sgi_frame_params* params, cudaStream_t s,
                         int ev_gather, cudaEvent_t hdr_ready = nullptr) {
    const sgi_config& cfg = ctx->cfg;
    const bool keep = cfg.debug_keep_passes != 0;
    sgi_status st = run_gather(ctx, cur, cam, params, s);
    if (st != SGI_OK) return st;
    record(ctx, ev_gather + 1, s);
    // passes 1 .. n-2: a-trous at stride 2^pass (StratusRendererBackend.cpp:1912-1940)
    const uint2* in = ctx->last_merged;
    for (int pass = 1; pass < cfg.denoise_passes - 1; ++pass) {
        uint2* out = keep ? ctx->pass_bufs[pass] : ctx->ping[pass & 1];
        cudaError_t e = cudaErrorNotSupported;
        if (ctx->atrous_staged)
            e = SGI_SHADE(ctx, launch_atrous_staged)(cfg.width, cfg.height, pass, ctx->guide, in, out, ctx->wait_ns,
                                                     ctx->skip_copies, ctx->dev_status, s);
        if (e == cudaErrorNotSupported)   // strides above 8, odd widths: the direct kernel
            e = SGI_SHADE(ctx, launch_atrous)(cfg.width, cfg.height, pass, ctx->guide, in, out, s,
                                              ctx->block_dim(SGI_BLOCK_ATROUS));
        SGI_CUDA(ctx, e, "atrous");
        ctx->launches += 1;
        in = out;
    }
    if (ctx->timing) cudaEventRecord(ctx->ev_atrous_end, s);
    ctx->have_split = ctx->timing;
    // pass n-1: a-trous + temporal reprojection + composite
    sgi::DenoiseLaunch d;
    std::memset(&d, 0, sizeof(d));
    d.width = cfg.width; d.height = cfg.height; d.passes = cfg.denoise_passes; d.pass = cfg.denoise_passes - 1;
    d.time = params->time; d.fps = params->frames_per_second;
    d.cur = *cur;
    d.prev_depth = prev->depth; d.prev_normal = prev->normal; d.prev_id = prev->id;
    d.hdr_in = (const uint2*)hdr_in; d.hdr_out = (uint2*)hdr_out;
    d.gi_prev = ctx->gi_hist[ctx->hist_cur]; d.gi_out = ctx->gi_hist[1 - ctx->hist_cur];
    d.hist_prev = ctx->hist_depth[ctx->hist_cur]; d.hist_out = ctx->hist_depth[1 - ctx->hist_cur];
    d.visible_index = ctx->visible_index;
    d.guide = ctx->guide;
    d.res_in = in;
    d.res_out = keep ? ctx->pass_bufs[cfg.denoise_passes - 1] : nullptr;
    if (hdr_ready) SGI_CUDA(ctx, cudaStreamWaitEvent(s, hdr_ready, 0), "join direct lighting");
    SGI_CUDA(ctx, SGI_SHADE(ctx, launch_denoise_final)(d, s, ctx->block_dim(SGI_BLOCK_DENOISE_FINAL)), "denoise_final");
    ctx->launches += 1;
    ctx->hist_cur = 1 - ctx->hist_cur;
    ctx->have_history = true;
    return SGI_OK;
}

static bool frame_args_ok(const sgi_gbuffer* cur, const sgi_gbuffer* prev, const sgi_camera* cam,
                          const sgi_frame_params* params) {
    return gbuffer_ok(cur, true) && prev && prev->depth && prev->normal && prev->id && cam && params &&
           params->frames_per_second > 0.0f;
}

sgi_status sgi_global_illumination(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_gbuffer* prev,
                                   const sgi_camera* cam, const void* hdr_in, void* hdr_out,
                                   const sgi_frame_params* params, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (!frame_args_ok(cur, prev, cam, params) || !hdr_in || !hdr_out)
        return fail(ctx, SGI_ERR_ARG, "NULL frame argument or frames_per_second <= 0");
    if (!ctx->culled || !ctx->maps_set) return fail(ctx, SGI_ERR_STATE, "cull VPLs (and tiles) first");
    return run_gi(ctx, cur, prev, cam, hdr_in, hdr_out, params, (cudaStream_t)stream, 2);
}

sgi_status sgi_render_frame(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_gbuffer* prev, const sgi_camera* cam,
                            const sgi_frame_params* params, void* hdr_out, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (!frame_args_ok(cur, prev, cam, params) || !hdr_out)
        return fail(ctx, SGI_ERR_ARG, "NULL frame argument or frames_per_second <= 0");
    cudaStream_t s = (cudaStream_t)stream;
    // Without per-pass timing the direct lighting overlaps the culls and the gather
    // on the context's side stream (fork after the caller's prior work, join before
    // the composite); with timing the passes run in sequence so each can be timed.
    const bool overlap = !ctx->timing;
    if (overlap) {
        SGI_CUDA(ctx, cudaEventRecord(ctx->fork, s), "fork");
        SGI_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->fork, 0), "fork");
        sgi_status st0 = sgi_direct_lighting(ctx, cur, cam, ctx->direct, ctx->side);
        if (st0 != SGI_OK) return st0;
        SGI_CUDA(ctx, cudaEventRecord(ctx->join, ctx->side), "join");
    }
    record(ctx, 0, s);
    sgi_status st = sgi_cull_vpls(ctx, stream);
    if (st != SGI_OK) return st;
    record(ctx, 1, s);
    if (!overlap) {
        st = sgi_direct_lighting(ctx, cur, cam, ctx->direct, stream);
        if (st != SGI_OK) return st;
    }
    record(ctx, 2, s);
    if (ctx->cfg.gi_mode == SGI_GI_TILED) {
        st = sgi_cull_tiles(ctx, cur, cam, stream);
        if (st != SGI_OK) return st;
    }
    record(ctx, 3, s);
    st = run_gi(ctx, cur, prev, cam, ctx->direct, hdr_out, params, s, 3, overlap ? ctx->join : nullptr);
    if (st != SGI_OK) return st;
    record(ctx, 5, s);
    ctx->have_times = ctx->timing;
    return SGI_OK;
}

sgi_status sgi_gi_target(sgi_ctx* ctx, const sgi_gbuffer* gbuf, const sgi_camera* cam, float time, int32_t batches,
                         float* target, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (!gbuffer_ok(gbuf, true) || !cam || !target) return fail(ctx, SGI_ERR_ARG, "NULL G-buffer, camera or target");
    if (batches < 1 || batches > 65536) return fail(ctx, SGI_ERR_ARG, "batches must be in [1, 65536]");
    if (!ctx->culled || !ctx->maps_set) return fail(ctx, SGI_ERR_STATE, "cull VPLs (and tiles) first");
    SGI_CUDA(ctx, sgi::exact::launch_gi_target(ctx->cfg, ctx->sc, *gbuf, *cam, ctx->cv, ctx->ce, ctx->visible_index,
                                        ctx->lists, ctx->cubes, time, batches, (float4*)target, (cudaStream_t)stream),
             "gi_target");
    ctx->launches += 1;
    return SGI_OK;
}

sgi_status sgi_reset_history(sgi_ctx* ctx, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t P = pixels(ctx->cfg);
    for (int k = 0; k < 2; ++k) {
        SGI_CUDA(ctx, cudaMemsetAsync(ctx->gi_hist[k], 0, P * sizeof(uint2), s), "clear gi history");
        SGI_CUDA(ctx, cudaMemsetAsync(ctx->hist_depth[k], 0, P * sizeof(uint16_t), s), "clear history depth");
    }
    ctx->hist_cur = 0;
    ctx->have_history = false;
    ctx->have_taa = false;
    return SGI_OK;
}

sgi_status sgi_get_history(sgi_ctx* ctx, void* gi, void* history_length, int32_t* valid, void* stream) {
    if (!ctx || !gi || !history_length || !valid) return fail(ctx, SGI_ERR_ARG, "NULL history output");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t P = pixels(ctx->cfg);
    SGI_CUDA(ctx, cudaMemcpyAsync(gi, ctx->gi_hist[ctx->hist_cur], P * sizeof(uint2), cudaMemcpyDeviceToDevice, s),
             "copy gi history");
    SGI_CUDA(ctx, cudaMemcpyAsync(history_length, ctx->hist_depth[ctx->hist_cur], P * sizeof(uint16_t),
                                  cudaMemcpyDeviceToDevice, s), "copy history length");
    *valid = ctx->have_history ? 1 : 0;
    return SGI_OK;
}

sgi_status sgi_set_history(sgi_ctx* ctx, const void* gi, const void* history_length, int32_t valid, void* stream) {
    if (!ctx || !gi || !history_length) return fail(ctx, SGI_ERR_ARG, "NULL history input");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t P = pixels(ctx->cfg);
    SGI_CUDA(ctx, cudaMemcpyAsync(ctx->gi_hist[ctx->hist_cur], gi, P * sizeof(uint2), cudaMemcpyDeviceToDevice, s),
             "restore gi history");
    SGI_CUDA(ctx, cudaMemcpyAsync(ctx->hist_depth[ctx->hist_cur], history_length, P * sizeof(uint16_t),
                                  cudaMemcpyDeviceToDevice, s), "restore history length");
    ctx->have_history = valid != 0;
    return SGI_OK;
}

sgi_status sgi_post_fx(sgi_ctx* ctx, const void* hdr_in, const sgi_gbuffer* cur, int32_t taa, void* ldr_out,
                       void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (!hdr_in || !ldr_out || (taa && (!cur || !cur->velocity)))
        return fail(ctx, SGI_ERR_ARG, "NULL frame, output or velocity");
    const size_t P = pixels(ctx->cfg);
    if (taa && !ctx->taa_hist[0]) {
        SGI_CUDA(ctx, dalloc(&ctx->taa_hist[0], P), "alloc TAA history");
        SGI_CUDA(ctx, dalloc(&ctx->taa_hist[1], P), "alloc TAA history");
    }
    const uint2* hin = taa && ctx->have_taa ? ctx->taa_hist[ctx->taa_cur] : nullptr;
    uint2* hout = taa ? ctx->taa_hist[1 - ctx->taa_cur] : nullptr;
    SGI_CUDA(ctx, sgi::launch_post_fx(ctx->cfg.width, ctx->cfg.height, (const uint2*)hdr_in,
                                      taa ? cur->velocity : nullptr, hin, hout, (uint32_t*)ldr_out, taa ? 1 : 0,
                                      (cudaStream_t)stream), "post_fx");
    ctx->launches += 1;
    if (taa) {
        ctx->taa_cur = 1 - ctx->taa_cur;
        ctx->have_taa = true;
    }
    return SGI_OK;
}

sgi_status sgi_read_debug(sgi_ctx* ctx, int32_t which, void* host_dst, size_t bytes, size_t* needed) {
    if (!ctx) return SGI_ERR_ARG;
    const size_t P = pixels(ctx->cfg);
    const void* src = nullptr;
    size_t size = 0;
    switch (which) {
        case SGI_DEBUG_VISIBLE_INDEX: src = ctx->visible_index; size = sizeof(int32_t) * (1 + (size_t)ctx->cfg.max_vpls); break;
        case SGI_DEBUG_COMPACT_VPLS: src = ctx->cv; size = sizeof(sgi_vpl) * ctx->cfg.max_visible; break;
        case SGI_DEBUG_COMPACT_ENTRIES: src = ctx->ce; size = sizeof(sgi_atlas_entry) * ctx->cfg.max_visible; break;
        case SGI_DEBUG_TILE_STAGE1: src = ctx->stage1; size = sizeof(sgi_tile_stage1) * ctx->num_tiles; break;
        case SGI_DEBUG_TILE_LISTS:
            src = ctx->lists; size = sizeof(int32_t) * ctx->num_tiles * (1 + (size_t)ctx->cfg.max_vpls_per_tile); break;
        case SGI_DEBUG_RESERVOIR:
            if (!ctx->cfg.debug_keep_passes) return fail(ctx, SGI_ERR_ARG, "the raw reservoir needs debug_keep_passes");
            src = ctx->reservoir; size = P * sizeof(uint2); break;
        case SGI_DEBUG_GI_HISTORY: src = ctx->gi_hist[ctx->hist_cur]; size = P * sizeof(uint2); break;
        case SGI_DEBUG_HISTORY_DEPTH: src = ctx->hist_depth[ctx->hist_cur]; size = P * sizeof(uint16_t); break;
        case SGI_DEBUG_DIRECT: src = ctx->direct; size = P * sizeof(uint2); break;
        case SGI_DEBUG_TAA_HISTORY:
            if (!ctx->have_taa) return fail(ctx, SGI_ERR_STATE, "no TAA frame yet");
            src = ctx->taa_hist[ctx->taa_cur]; size = P * sizeof(uint2); break;
        default:
            if (which >= SGI_DEBUG_PASS_BASE && which < SGI_DEBUG_PASS_BASE + ctx->cfg.denoise_passes &&
                ctx->pass_bufs[which - SGI_DEBUG_PASS_BASE]) {
                src = ctx->pass_bufs[which - SGI_DEBUG_PASS_BASE];
                size = P * sizeof(uint2);
            } else {
                return fail(ctx, SGI_ERR_ARG, "unknown debug buffer (pass buffers need debug_keep_passes)");
            }
    }
    if (needed) *needed = size;
    if (!host_dst) return SGI_OK;
    SGI_CUDA(ctx, cudaDeviceSynchronize(), "synchronize before debug read");
    SGI_CUDA(ctx, cudaMemcpy(host_dst, src, bytes < size ? bytes : size, cudaMemcpyDeviceToHost), "debug read");
    return SGI_OK;
}

sgi_status sgi_set_shadow_point_lights(sgi_ctx* ctx, const sgi_point_light* lights, const sgi_atlas_entry* entries,
                                       int32_t n, const sgi_cube_atlas* atlas, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (n < 0) return fail(ctx, SGI_ERR_ARG, "negative light count");
    if (n > SGI_MAX_POINT_LIGHTS) return fail(ctx, SGI_ERR_CAP, "more than 256 shadow-casting point lights");
    if (n == 0) {
        ctx->num_shadow_points = 0;
        return SGI_OK;
    }
    if (!lights || !entries || !atlas) return fail(ctx, SGI_ERR_ARG, "NULL lights, entries or atlas");
    if (atlas->num_atlases < 1 || atlas->num_atlases > SGI_MAX_ATLASES || atlas->layers_per_atlas < 1 ||
        atlas->face_size < 1 || atlas->face_size > SGI_MAX_CUBE_FACE || atlas->format < SGI_CUBE_F32 ||
        atlas->format > SGI_CUBE_UNORM16)
        return fail(ctx, SGI_ERR_ARG, "shadow atlas: bad dimensions or format");
    cudaStream_t s = (cudaStream_t)stream;
    SGI_CUDA(ctx, cudaMemcpyAsync(ctx->shadow_points, lights, sizeof(sgi_point_light) * n, cudaMemcpyDefault, s),
             "copy shadow-casting lights");
    SGI_CUDA(ctx, cudaMemcpyAsync(ctx->shadow_entries, entries, sizeof(sgi_atlas_entry) * n, cudaMemcpyDefault, s),
             "copy shadow atlas entries");
    ctx->num_shadow_points = n;
    ctx->shadow_atlas = *atlas;
    return SGI_OK;
}

sgi_status sgi_set_vpl_coloring(sgi_ctx* ctx, const sgi_diffuse_atlas* diffuse) {
    if (!ctx) return SGI_ERR_ARG;
    if (!diffuse) {
        ctx->coloring = false;
        return SGI_OK;
    }
    if (diffuse->num_atlases < 1 || diffuse->num_atlases > SGI_MAX_ATLASES || diffuse->layers_per_atlas < 1 ||
        diffuse->face_size < 1 || diffuse->face_size > SGI_MAX_CUBE_FACE)
        return fail(ctx, SGI_ERR_ARG, "diffuse atlas: bad dimensions");
    for (int a = 0; a < diffuse->num_atlases; ++a)
        if (!diffuse->atlas[a] || ((uintptr_t)diffuse->atlas[a] & 3))
            return fail(ctx, SGI_ERR_ARG, "diffuse atlas: NULL or misaligned layer pointer");
    ctx->diffuse = *diffuse;
    ctx->coloring = true;
    return SGI_OK;
}

sgi_status sgi_set_block_shape(sgi_ctx* ctx, int32_t pass, int32_t bx, int32_t by) {
    if (!ctx) return SGI_ERR_ARG;
    if (pass < 0 || pass >= SGI_NUM_BLOCK_PASSES) return fail(ctx, SGI_ERR_ARG, "unknown pass");
    const bool dflt = bx == 0 && by == 0;
    if (!dflt && (bx < 1 || by < 1 || bx * by != 256 || bx % 8 != 0))
        return fail(ctx, SGI_ERR_ARG, "block shape must be 256 threads with a width that is a multiple of 8");
    ctx->block[pass][0] = bx;
    ctx->block[pass][1] = by;
    return SGI_OK;
}

sgi_status sgi_get_block_shape(const sgi_ctx* ctx, int32_t pass, int32_t* bx, int32_t* by) {
    if (!ctx || !bx || !by || pass < 0 || pass >= SGI_NUM_BLOCK_PASSES) return SGI_ERR_ARG;
    *bx = ctx->block[pass][0];
    *by = ctx->block[pass][1];
    return SGI_OK;
}

sgi_status sgi_set_shading_precision(sgi_ctx* ctx, int32_t mode) {
    if (!ctx) return SGI_ERR_ARG;
    if (mode != SGI_SHADING_EXACT && mode != SGI_SHADING_FAST)
        return fail(ctx, SGI_ERR_ARG, "shading precision must be SGI_SHADING_EXACT or SGI_SHADING_FAST");
    ctx->fast_shading = mode == SGI_SHADING_FAST;
    return SGI_OK;
}

int32_t sgi_get_shading_precision(const sgi_ctx* ctx) {
    return ctx && ctx->fast_shading ? SGI_SHADING_FAST : SGI_SHADING_EXACT;
}

sgi_status sgi_set_atrous_staging(sgi_ctx* ctx, int32_t mode) {
    if (!ctx) return SGI_ERR_ARG;
    if (mode != SGI_ATROUS_DIRECT && mode != SGI_ATROUS_STAGED)
        return fail(ctx, SGI_ERR_ARG, "a-trous staging must be SGI_ATROUS_DIRECT or SGI_ATROUS_STAGED");
    ctx->atrous_staged = mode == SGI_ATROUS_STAGED;
    return SGI_OK;
}

int32_t sgi_get_atrous_staging(const sgi_ctx* ctx) {
    return ctx && ctx->atrous_staged ? SGI_ATROUS_STAGED : SGI_ATROUS_DIRECT;
}

sgi_status sgi_set_wait_test(sgi_ctx* ctx, int64_t wait_ns, int32_t skip_copies) {
    if (!ctx || wait_ns < 0) return SGI_ERR_ARG;
    ctx->wait_ns = wait_ns;
    ctx->skip_copies = skip_copies != 0;
    return SGI_OK;
}

sgi_status sgi_device_status(sgi_ctx* ctx) {
    if (!ctx) return SGI_ERR_ARG;
    int32_t st = SGI_OK;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&st, ctx->dev_status, sizeof(st), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && st != SGI_OK) e = cudaMemset(ctx->dev_status, 0, sizeof(st));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "device status");
    return st == SGI_OK ? SGI_OK : fail(ctx, st, "a bounded device wait ran out (its pass wrote nothing)");
}

sgi_status sgi_set_timing(sgi_ctx* ctx, int32_t enabled) {
    if (!ctx) return SGI_ERR_ARG;
    ctx->timing = enabled != 0;
    ctx->have_times = false;
    return SGI_OK;
}

sgi_status sgi_get_pass_times(sgi_ctx* ctx, float* ms, int32_t n) {
    if (!ctx || !ms || n < 1) return SGI_ERR_ARG;
    if (!ctx->have_times) return fail(ctx, SGI_ERR_STATE, "no timed sgi_render_frame yet");
    SGI_CUDA(ctx, cudaEventSynchronize(ctx->ev[SGI_NUM_PASS_TIMES]), "event sync");
    for (int k = 0; k < SGI_NUM_PASS_TIMES && k < n; ++k) {
        float t = 0.0f;
        SGI_CUDA(ctx, cudaEventElapsedTime(&t, ctx->ev[k], ctx->ev[k + 1]), "event elapsed");
        ms[k] = t;
    }
    // the denoise pass split at its last a-trous pass (0 when the last timed frame had none)
    if (n > SGI_NUM_PASS_TIMES) {
        ms[5] = 0.0f;
        if (ctx->have_split) SGI_CUDA(ctx, cudaEventElapsedTime(&ms[5], ctx->ev[4], ctx->ev_atrous_end), "event elapsed");
    }
    if (n > SGI_NUM_PASS_TIMES + 1) {
        ms[6] = 0.0f;
        if (ctx->have_split) SGI_CUDA(ctx, cudaEventElapsedTime(&ms[6], ctx->ev_atrous_end, ctx->ev[5]), "event elapsed");
    }
    return SGI_OK;
}

// ---------------------------------------------------- learned denoiser --
static sgi_status nn_buffers(sgi_ctx* ctx) {
    if (ctx->nn_feat) return SGI_OK;
    const size_t P = pixels(ctx->cfg);
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t r) { if (e == cudaSuccess && r != cudaSuccess) e = r; };
    chk(dalloc(&ctx->nn_feat, P * 16));
    chk(dalloc(&ctx->nn_prev, P));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "allocate denoiser buffers");
    return SGI_OK;
}

static sgi_status run_features(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_camera* cam, __nv_bfloat16* feat,
                               float4* noisy, float4* prevw, cudaStream_t s) {
    sgi::nn::FeatureArgs a;
    a.W = ctx->cfg.width; a.H = ctx->cfg.height;
    a.inv_w = 1.0f / (float)a.W; a.inv_h = 1.0f / (float)a.H;
    a.merged = ctx->last_merged; a.guide = ctx->guide;
    a.albedo = cur->albedo; a.rma = cur->roughness_metallic_ambient; a.velocity = cur->velocity;
    a.gi_prev = ctx->gi_hist[ctx->feat_hist];
    a.have_history = ctx->feat_have_history ? 1 : 0;
    std::memcpy(a.inv_pv, cam->inv_proj_view, sizeof(a.inv_pv));
    for (int k = 0; k < 3; ++k) a.cam_pos[k] = cam->view_position[k];
    a.features = feat; a.noisy = noisy; a.prev = prevw;
    SGI_CUDA(ctx, sgi::nn::features(a, s), "kpcn_features");
    ctx->launches += 1;
    return SGI_OK;
}

sgi_status sgi_nn_features(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_camera* cam, void* features, float* noisy,
                           float* prev, void* stream) {
    if (!ctx) return SGI_ERR_ARG;
    if (!gbuffer_ok(cur, true) || !cam || !features || !noisy || !prev)
        return fail(ctx, SGI_ERR_ARG, "NULL G-buffer, camera or output");
    if (((uintptr_t)features | (uintptr_t)noisy | (uintptr_t)prev) & 15)
        return fail(ctx, SGI_ERR_ARG, "features, noisy and prev must be 16-byte aligned");
    if (!ctx->last_merged) return fail(ctx, SGI_ERR_STATE, "no gathered frame yet");
    return run_features(ctx, cur, cam, (__nv_bfloat16*)features, (float4*)noisy, (float4*)prev, (cudaStream_t)stream);
}

sgi_status sgi_render_frame_neural(sgi_ctx* ctx, sgi_nn* net, const sgi_gbuffer* cur, const sgi_gbuffer* prev,
                                   const sgi_camera* cam, const sgi_frame_params* params, void* hdr_out,
                                   void* stream) {
    if (!ctx || !net) return SGI_ERR_ARG;
    if (!frame_args_ok(cur, prev, cam, params) || !hdr_out)
        return fail(ctx, SGI_ERR_ARG, "NULL frame argument or frames_per_second <= 0");
    const int W = ctx->cfg.width, H = ctx->cfg.height;
    if (W % 4 || H % 4 || W > net->net.cfg.max_width * net->net.cfg.max_batch ||
        (size_t)W * H > (size_t)net->net.cfg.max_batch * net->net.cfg.max_height * net->net.cfg.max_width)
        return fail(ctx, SGI_ERR_CAP, "viewport exceeds the network's capacity (or is not a multiple of 4)");
    sgi_status st = nn_buffers(ctx);
    if (st != SGI_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const bool overlap = !ctx->timing;   // as in sgi_render_frame
    if (overlap) {
        SGI_CUDA(ctx, cudaEventRecord(ctx->fork, s), "fork");
        SGI_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->fork, 0), "fork");
        st = sgi_direct_lighting(ctx, cur, cam, ctx->direct, ctx->side);
        if (st != SGI_OK) return st;
        SGI_CUDA(ctx, cudaEventRecord(ctx->join, ctx->side), "join");
    }
    record(ctx, 0, s);
    st = sgi_cull_vpls(ctx, stream);
    if (st != SGI_OK) return st;
    record(ctx, 1, s);
    if (!overlap) {
        st = sgi_direct_lighting(ctx, cur, cam, ctx->direct, stream);
        if (st != SGI_OK) return st;
    }
    record(ctx, 2, s);
    if (ctx->cfg.gi_mode == SGI_GI_TILED) {
        st = sgi_cull_tiles(ctx, cur, cam, stream);
        if (st != SGI_OK) return st;
    }
    record(ctx, 3, s);
    st = run_gather(ctx, cur, cam, params, s);
    if (st != SGI_OK) return st;
    record(ctx, 4, s);
    st = run_features(ctx, cur, cam, ctx->nn_feat, nullptr, ctx->nn_prev, s);
    if (st != SGI_OK) return st;
    // the network's head applies the predicted kernels and writes the composite (HDR frame, GI history)
    // directly; it reads the direct lighting, so it waits for the side stream first
    st = nn_forward_composite(net, ctx->nn_feat, H, W, ctx->last_merged, (const float*)ctx->nn_prev, ctx->direct,
                              cur->albedo, (uint2*)hdr_out, ctx->gi_hist[1 - ctx->hist_cur],
                              ctx->hist_depth[1 - ctx->hist_cur], overlap ? ctx->join : nullptr, s);
    if (st != SGI_OK) return fail(ctx, st, std::string("denoiser: ") + sgi_nn_last_error(net));
    // the network: 11 convolutions (the head with the kernel apply) and 2 upsamplings on the tcgen05 path;
    // off it also 2 pooling launches and the separate kernel apply (the features kernel counts itself)
    ctx->launches += net->net.conv_path != SGI_NN_CONV_TCGEN05 ? 16 : net->net.head_fusion ? 13 : 14;
    ctx->hist_cur = 1 - ctx->hist_cur;
    ctx->have_history = true;
    record(ctx, 5, s);
    ctx->have_split = false;
    ctx->have_times = ctx->timing;
    return SGI_OK;
}

// ------------------------------------------------------------ scene ABI --
sgi_status sgi_scene_gbuffer(const sgi_box* boxes, int32_t num_boxes, const sgi_scene_camera* cam, int32_t width,
                             int32_t height, const sgi_gbuffer* out, void* stream) {
    if (!boxes || num_boxes < 1 || !cam || width < 1 || height < 1 || !gbuffer_ok(out, true)) return SGI_ERR_ARG;
    cudaError_t e = sgi::launch_scene_gbuffer(boxes, num_boxes, *cam, width, height, *out, (cudaStream_t)stream);
    return e == cudaSuccess ? SGI_OK : (e == cudaErrorInvalidValue ? SGI_ERR_CAP : SGI_ERR_CUDA);
}

sgi_status sgi_scene_csm(const sgi_box* boxes, int32_t num_boxes, const sgi_csm* csm,
                         const float inv_cascade_proj_view[4][16], void* stream) {
    if (!boxes || num_boxes < 1 || !csm || !csm->depth || csm->resolution < 1 || csm->num_cascades != 4 ||
        !inv_cascade_proj_view)
        return SGI_ERR_ARG;
    cudaError_t e = sgi::launch_scene_csm(boxes, num_boxes, *csm, inv_cascade_proj_view, (cudaStream_t)stream);
    return e == cudaSuccess ? SGI_OK : (e == cudaErrorInvalidValue ? SGI_ERR_CAP : SGI_ERR_CUDA);
}

sgi_status sgi_scene_diffuse_atlas(const sgi_box* boxes, int32_t num_boxes, const sgi_vpl* vpls,
                                   const sgi_atlas_entry* entries, int32_t count, const sgi_diffuse_atlas* atlas,
                                   void* stream) {
    if (!boxes || num_boxes < 1 || !vpls || !entries || count < 0 || !atlas || atlas->face_size < 1)
        return SGI_ERR_ARG;
    if (count == 0) return SGI_OK;
    cudaError_t e = sgi::launch_scene_diffuse(boxes, num_boxes, vpls, entries, count, *atlas, (cudaStream_t)stream);
    return e == cudaSuccess ? SGI_OK : (e == cudaErrorInvalidValue ? SGI_ERR_CAP : SGI_ERR_CUDA);
}

sgi_status sgi_scene_cube_atlas(const sgi_box* boxes, int32_t num_boxes, const sgi_vpl* vpls,
                                const sgi_atlas_entry* entries, int32_t count, const sgi_cube_atlas* atlas,
                                void* stream) {
    if (!boxes || num_boxes < 1 || !vpls || !entries || count < 0 || !atlas || atlas->face_size < 1)
        return SGI_ERR_ARG;
    if (count == 0) return SGI_OK;
    cudaError_t e = sgi::launch_scene_cubes(boxes, num_boxes, vpls, entries, count, *atlas, (cudaStream_t)stream);
    return e == cudaSuccess ? SGI_OK : (e == cudaErrorInvalidValue ? SGI_ERR_CAP : SGI_ERR_CUDA);
}

}  // extern "C"
