/*
 * sgi.h - C ABI of the GB300-native VPL global-illumination and deferred
 * lighting stage (StratusGFX RendererBackend GI/lighting drop-in).
 *
 * The reference stage is a set of private RendererBackend methods driven by
 * GL uniforms and SSBO bindings:
 *   PerformVirtualPointLightCullingStage1_   Source/Engine/StratusRendererBackend.cpp:1578-1661
 *   PerformVirtualPointLightCullingStage2_   Source/Engine/StratusRendererBackend.cpp:1666-1814
 *   ComputeVirtualPointLightGlobalIllumination_
 *                                            Source/Engine/StratusRendererBackend.cpp:1816-1952
 *   deferred lighting block of RenderScene   Source/Engine/StratusRendererBackend.cpp:2011-2038
 *   InitLights_ / InitCoreCSMData_           Source/Engine/StratusRendererBackend.cpp:2452-2604
 * What the drop-in keeps is the data contract: G-buffer formats
 * (StratusRendererBackend.cpp:384-424), GI/denoise buffer formats (:510-589),
 * the std430 structs (Source/Engine/StratusGpuCommon.h:217-307) and the
 * shadow-map conventions (:348-352, :2397-2449).
 *
 * Conventions
 *  - Every image is W*H texels, row-major, row 0 = bottom (GL window space):
 *    pixel (x, y) has fragment centre (x+0.5, y+0.5) and uv ((x+0.5)/W, (y+0.5)/H).
 *  - Formats: RGB8 textures are held in 4-byte RGBA8 texels (the alpha byte is
 *    ignored), RGB16F textures in 8-byte RGBA16F texels.
 *  - All buffer pointers passed to sgi_* are DEVICE pointers unless stated.
 *    The caller owns every input and output buffer; the context owns scratch
 *    (compacted VPL lists, per-tile lists, reservoirs, ping-pong targets and
 *    the denoiser history).
 *  - Calls are asynchronous on the given stream (a cudaStream_t passed as
 *    void*; NULL = legacy default stream). No call synchronises with the host
 *    except sgi_read_debug and sgi_get_pass_times. One context per stream.
 *  - Errors are status codes; nothing throws across the ABI. The text of the
 *    last error of a context is returned by sgi_last_error.
 */
#ifndef SGI_H_
#define SGI_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGI_ABI_VERSION 1

typedef int32_t sgi_status;
#define SGI_OK            0
#define SGI_ERR_ARG      (-1)  /* bad argument: null pointer, size, mode */
#define SGI_ERR_OOM      (-2)  /* device allocation failed */
#define SGI_ERR_CUDA     (-3)  /* CUDA runtime error (launch or copy) */
#define SGI_ERR_TIMEOUT  (-4)  /* a bounded device wait gave up */
#define SGI_ERR_CAP      (-5)  /* a size exceeds a configured capacity */
#define SGI_ERR_STATE    (-6)  /* call order: e.g. lighting before lights were set */

/* ------------------------------------------------------------------------ */
/* std430 records (byte-identical to the reference structs)                  */
/* ------------------------------------------------------------------------ */

/* GpuVplData, Source/Engine/StratusGpuCommon.h:217-232; VplData in
 * Source/Shaders/vpl_common.glsl:48-56. 64 bytes. */
typedef struct sgi_vpl {
    float position[4];
    float color[4];
    float specular_position[4];
    float radius;
    float far_plane;
    float intensity;
    float pad_;
} sgi_vpl;

/* GpuPointLight, Source/Engine/StratusGpuCommon.h:261-270; PointLight in
 * Source/Shaders/pbr.fs:16-22. 48 bytes. */
typedef struct sgi_point_light {
    float position[4];
    float color[4];
    float radius;
    float far_plane;
    float pad_[2];
} sgi_point_light;

/* GpuAtlasEntry, Source/Engine/StratusGpuCommon.h:274-277; AtlasEntry in
 * Source/Shaders/pbr.glsl:75-78. 8 bytes. */
typedef struct sgi_atlas_entry {
    int32_t index;   /* which cube-map atlas */
    int32_t layer;   /* cube layer inside that atlas */
} sgi_atlas_entry;

/* GpuVplStage1PerTileOutputs, Source/Engine/StratusGpuCommon.h:192-196. */
typedef struct sgi_tile_stage1 {
    float average_position[4];
    float average_normal[4];
} sgi_tile_stage1;

/* ------------------------------------------------------------------------ */
/* Configuration (RendererSettings subset, StratusRendererBackend.h:186-294) */
/* ------------------------------------------------------------------------ */

/* Which VPL set the GI gather samples from. */
#define SGI_GI_REFERENCE 0  /* global compacted list, vpl_pbr_gi.fs:145-151 */
#define SGI_GI_TILED     1  /* per-tile nearest-L list (culling stage 2) */

/* Storage format of the VPL distance cube maps. */
#define SGI_CUBE_F32     0
#define SGI_CUBE_F16     1
#define SGI_CUBE_UNORM16 2  /* the reference's GL_DEPTH_COMPONENT16 */

#define SGI_MAX_ATLASES          14   /* MAX_TOTAL_SHADOW_ATLASES, pbr.glsl:70 */
#define SGI_MAX_VPLS_BEFORE_CULL 10000 /* MAX_TOTAL_VPLS_BEFORE_CULLING, vpl_common.glsl:7 */
#define SGI_MAX_VPLS_PER_FRAME   4480 /* MAX_TOTAL_VPLS_PER_FRAME = 14*320, vpl_common.glsl:8 */
#define SGI_MAX_TILE_LIST        64
#define SGI_MAX_DENOISE_PASSES   8
#define SGI_MAX_POINT_LIGHTS     256
#define SGI_MAX_CUBE_FACE        16384 /* cube face size limit of the atlases (drivers allow 16384-32768) */

typedef struct sgi_config {
    int32_t width;                 /* viewport width in pixels  */
    int32_t height;                /* viewport height in pixels */
    int32_t max_vpls;              /* capacity of sgi_set_lights (<= 10000) */
    int32_t max_visible;           /* cap of the compacted list (reference 4480) */
    int32_t tile_size;             /* tile edge in pixels, 4..32 (reference and default 5, configs 16) */
    int32_t max_vpls_per_tile;     /* L, 1..64 (reference 12) */
    int32_t gi_mode;               /* SGI_GI_REFERENCE or SGI_GI_TILED */
    int32_t samples_per_pixel;     /* 0 = reference adaptive 2..10 (vpl_pbr_gi.fs:138-143), else fixed K */
    int32_t denoise_passes;        /* 2..8: pass 0 merges reservoirs, the last is final (reference 4) */
    int32_t debug_keep_passes;     /* nonzero: keep the raw reservoir and each denoise pass output for sgi_read_debug */
    float   min_roughness;         /* RendererSettings minRoughness_ = 0.08 */
    int32_t use_perceptual_roughness; /* RendererSettings usePerceptualRoughness = true */
    float   min_gi_occlusion_factor;  /* RendererSettings minGiOcclusionFactor_ = 0.95 */
    float   emission_strength;     /* RendererSettings emissionStrength_ = 0 */
    float   fog_density;           /* RendererSettings fogDensity_ = 0 */
    float   fog_color[3];          /* fog.glsl:3 default vec3(0.5) */
    float   point_light_ambient_intensity; /* pbr.glsl:66 default 0.003 */
} sgi_config;

/* Fills cfg with the reference defaults for a W x H viewport. */
void sgi_config_defaults(sgi_config* cfg, int32_t width, int32_t height);

/* ------------------------------------------------------------------------ */
/* Per-frame inputs                                                           */
/* ------------------------------------------------------------------------ */

/* G-buffer, formats of RendererBackend::InitGBuffer_ (StratusRendererBackend.cpp:384-424). */
typedef struct sgi_gbuffer {
    const float*    depth;      /* DEPTH FP32 window depth in [0,1] */
    const uint32_t* normal;     /* RGB8 0.5*n+0.5 */
    const uint32_t* albedo;     /* RGBA8 base colour, alpha = emissive.r */
    const uint16_t* base_reflectivity; /* RG8 (reflectance, emissive.g) */
    const uint32_t* roughness_metallic_ambient; /* RGB8 (roughness, metallic, emissive.b) */
    const uint32_t* velocity;   /* RG16F uv(current) - uv(previous) */
    const float*    id;         /* R32F draw id */
    const uint16_t* ssao;       /* R16F blurred occlusion */
} sgi_gbuffer;

/* RendererFrame camera fields (StratusRendererBackend.h:297-323). Matrices are
 * column-major (glm), GL clip conventions (NDC z in [-1,1]). */
typedef struct sgi_camera {
    float inv_proj_view[16];
    float view_position[4];
} sgi_camera;

/* Directional light + cascaded shadow map (pbr.glsl:53-63, set by
 * InitCoreCSMData_ StratusRendererBackend.cpp:2452-2474 and InitLights_ :2583-2596). */
typedef struct sgi_csm {
    const float* depth;            /* DEVICE [num_cascades][resolution][resolution] FP32 window depth */
    int32_t resolution;
    int32_t num_cascades;          /* must be 4 */
    float   cascade_proj_view[4][16];  /* cascadeProjViews[i] (projectionViewSample) */
    float   cascade_planes[3][4];      /* cascadePlanes[i] = cascades[i+1].cascadePlane */
    float   light_direction[4];    /* infiniteLightDirection (unit, towards the light) */
    float   light_color[4];        /* infiniteLightColor = luminance */
    float   znear;                 /* infiniteLightZnear */
    float   zfar;                  /* infiniteLightZfar */
    float   depth_bias;            /* infiniteLightDepthBias */
    float   pad_;
} sgi_csm;

/* VPL distance cube maps: samplerCubeArray shadowCubeMaps[MAX_TOTAL_SHADOW_ATLASES]
 * (vpl_pbr_gi.fs:69). Atlas a holds layers_per_atlas cubes laid out
 * [layer][face +X,-X,+Y,-Y,+Z,-Z][t][s], texel = saturate(distance / farPlane)
 * (shadowVpl.fs:26-34). */
typedef struct sgi_cube_atlas {
    const void* atlas[SGI_MAX_ATLASES];  /* DEVICE pointers */
    int32_t num_atlases;
    int32_t layers_per_atlas;
    int32_t face_size;
    int32_t format;                      /* SGI_CUBE_* */
} sgi_cube_atlas;

/* Diffuse colour cubes of the VPLs: the RGB each VPL's shadow pass renders
 * (shadowVpl.fs:34 into an RGB8 attachment with nearest filtering,
 * StratusRendererBackend.cpp:2397-2430), stored as RGBA8 texels (A unused) with
 * the addressing of sgi_cube_atlas: [layer][face][row][col]. */
typedef struct sgi_diffuse_atlas {
    const void* atlas[SGI_MAX_ATLASES];  /* DEVICE pointers */
    int32_t num_atlases;
    int32_t layers_per_atlas;
    int32_t face_size;
    int32_t reserved;
} sgi_diffuse_atlas;

typedef struct sgi_frame_params {
    float time;               /* RNG seed z (uniform float time), milliseconds */
    float frames_per_second;  /* uniform framesPerSecond = 1 / deltaSeconds */
} sgi_frame_params;

/* ------------------------------------------------------------------------ */
/* Context                                                                    */
/* ------------------------------------------------------------------------ */

typedef struct sgi_ctx sgi_ctx;

int32_t     sgi_abi_version(void);
const char* sgi_status_string(sgi_status s);

/* Allocates the context and its scratch on the current CUDA device.
 * Replaces the buffer setup of RendererBackend::UpdateWindowDimensions_
 * (StratusRendererBackend.cpp:437-589). */
sgi_status sgi_create(const sgi_config* cfg, sgi_ctx** out);
sgi_status sgi_destroy(sgi_ctx* ctx);
const char* sgi_last_error(const sgi_ctx* ctx);

/* Uploads this frame's VPL records (and their cube-atlas slots) and point
 * lights. Replaces InitVplFrameData_ (StratusRendererBackend.cpp:1281-1292)
 * and the point-light SSBO uploads of InitLights_ (:2535-2552). `entries` is
 * indexed like `vpls`. Device pointers; copied device-to-device on `stream`. */
sgi_status sgi_set_lights(sgi_ctx* ctx,
                          const sgi_vpl* vpls, const sgi_atlas_entry* entries, int32_t num_vpls,
                          const sgi_point_light* points, int32_t num_points,
                          void* stream);

/* Shadow-casting point lights of sgi_direct_lighting (the shadowCasters loop of
 * pbr.fs:116-131): each light within its radius adds calculatePointLighting2
 * with a shadow factor from its distance cube (slot entries[i] of `atlas`):
 * calculateShadowValue8Samples (pbr.glsl:81-113, 8 taps at +-0.3 offsets of the
 * direction) when the view distance is below 150, calculateShadowValue1Sample
 * (:116-136) below 750, none beyond. Records and entries are copied (device or
 * host pointers) on `stream`; the atlas (caller-owned device memory, any
 * SGI_CUBE_* format, nearest texel) must stay valid while set. n = 0 removes
 * them. At most 256. */
sgi_status sgi_set_shadow_point_lights(sgi_ctx* ctx, const sgi_point_light* lights, const sgi_atlas_entry* entries,
                                       int32_t n, const sgi_cube_atlas* atlas, void* stream);

/* Binds the directional light's CSM and the VPL cube atlases (caller-owned
 * device memory; pointers and matrices are copied into the context). */
sgi_status sgi_set_shadow_maps(sgi_ctx* ctx, const sgi_csm* csm, const sgi_cube_atlas* cubes);

/* VPL visibility cull: viscull_vpls.cs dispatched by
 * PerformVirtualPointLightCullingStage1_ (StratusRendererBackend.cpp:1578-1661).
 * Stable compaction in ascending VPL index; no host readback. */
sgi_status sgi_cull_vpls(sgi_ctx* ctx, void* stream);

/* The VPL visibility cull without a context and without allocating anything.
 * No counterpart in StratusGFX (its culling pass always owns its buffers); it
 * runs the kernels of sgi_cull_vpls on caller-owned device buffers:
 *   vpls, entries        [num_vpls] (16-byte aligned), csm: the directional CSM;
 *   visible_vpls         [max_visible], visible_entries [max_visible];
 *   visible_index        int32 [1 + max_visible]: the visible count (capped at
 *                        max_visible), then the original indices, ascending.
 * The per-VPL visibility flags live in a fixed 16384-byte array inside the
 * library (one per device), so num_vpls may not exceed
 * SGI_NOALLOC_CULL_MAX_VPLS: larger counts return SGI_ERR_CAP and launch nothing.
 * Every flag a call reads is written by the same call first; nothing has to
 * start at zero. Calls that overlap on one device (two streams, or two host
 * threads, with work in flight at the same time) share that array and race:
 * order them on one stream or with events. The first call on each device looks
 * up the array's address (cudaGetSymbolAddress, no allocation) and keeps it for
 * the life of the process; make that call before any stream capture begins. A
 * cudaDeviceReset destroys the array with the context, so the kept address is
 * stale after one: do not call this entry point again in that process. */
#define SGI_NOALLOC_CULL_MAX_VPLS 16384
sgi_status sgi_cull_vpls_noalloc(const sgi_vpl* vpls, const sgi_atlas_entry* entries, int32_t num_vpls,
                                 const sgi_csm* csm, int32_t max_visible, sgi_vpl* visible_vpls,
                                 sgi_atlas_entry* visible_entries, int32_t* visible_index, void* stream);

/* Per-tile culling: vpl_tiled_deferred_culling_stage1.cs + _stage2.cs
 * (dispatch at StratusRendererBackend.cpp:1733-1783). */
sgi_status sgi_cull_tiles(sgi_ctx* ctx, const sgi_gbuffer* gbuf, const sgi_camera* cam, void* stream);

/* Deferred PBR + CSM lighting: pbr.fs with INFINITE_LIGHTING_ENABLED, the
 * RenderScene block at StratusRendererBackend.cpp:2011-2038.
 * hdr_out: RGB16F (8-byte texels) W*H. */
sgi_status sgi_direct_lighting(sgi_ctx* ctx, const sgi_gbuffer* gbuf, const sgi_camera* cam,
                               void* hdr_out, void* stream);

/* GI gather + spatiotemporal denoise + composite:
 * ComputeVirtualPointLightGlobalIllumination_ (StratusRendererBackend.cpp:1816-1952).
 * hdr_in = lighting colour buffer ("screen"), hdr_out = lightingFbo colour
 * (both RGB16F 8-byte texels). `prev` is the previous frame's G-buffer (only
 * normal, depth and id are read). Updates the context's history. */
sgi_status sgi_global_illumination(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_gbuffer* prev,
                                   const sgi_camera* cam, const void* hdr_in, void* hdr_out,
                                   const sgi_frame_params* params, void* stream);

/* The whole stage in reference order: VPL cull, direct lighting, tile cull,
 * GI gather, denoise, composite (RenderScene :1982-1987 and :2011-2045). */
sgi_status sgi_render_frame(sgi_ctx* ctx, const sgi_gbuffer* cur, const sgi_gbuffer* prev,
                            const sgi_camera* cam, const sgi_frame_params* params,
                            void* hdr_out, void* stream);

/* Converged GI target (no counterpart in the reference; the reference of the
 * denoisers' error): `batches` independent runs of the gather's per-pixel
 * sample loop (batch b starts its seed z at time + b * 2e5) with the sums of
 * vplColor and validSamples accumulated in FP64. Writes per pixel the float4
 * (sum vplColor / max(sum validSamples, 1), 1) to `target` (device, W*H
 * float4): the value the K-sample estimate plus denoiser approximates. Uses
 * this frame's culled lists: call after sgi_cull_vpls (and sgi_cull_tiles in
 * tiled mode). 64 batches of K = 8 give the K = 512 target. */
sgi_status sgi_gi_target(sgi_ctx* ctx, const sgi_gbuffer* gbuf, const sgi_camera* cam, float time,
                         int32_t batches, float* target, void* stream);

/* FP64 error statistics of a rendered frame against the converged target
 * (no counterpart in the reference; the reductions behind the reported PSNRs).
 * With w = binary16(max(albedo / 255, 0.01) + 1e-5) per colour channel (the GI
 * weight the final denoise pass composites with), the converged GI term is
 * r_gi = w * target and the converged frame r = direct + r_gi; the statistics
 * cover the errors hdr - r (frame) and (hdr - direct) - r_gi (GI term) over the
 * three colour channels of every pixel, computed and reduced in binary64 on the
 * device in a fixed order. hdr, direct: RGBA16F (8 bytes a pixel), target: the
 * float4 output of sgi_gi_target; all device memory. Synchronises `stream`.
 * PSNR = 10 log10(peak^2 / (sse / values)). */
typedef struct sgi_error_stats {
    double sse_frame, sse_gi;         /* sums of squared errors */
    double peak_frame, peak_gi;       /* max |r|, max |r_gi| */
    double max_abs_frame, max_abs_gi; /* largest absolute errors */
    int64_t values;                   /* 3 * width * height */
} sgi_error_stats;
sgi_status sgi_gi_error_stats(const sgi_gbuffer* gbuf, const void* hdr, const void* direct, const float* target,
                              int32_t width, int32_t height, sgi_error_stats* out, void* stream);

/* Clears the denoiser history (vplGIDenoisedPrevFrameFbo). */
sgi_status sgi_reset_history(sgi_ctx* ctx, void* stream);

/* Snapshot and restore of the denoiser history (no counterpart in StratusGFX,
 * whose history lives only in its FBOs): the GI the next frame reprojects
 * (RGBA16F, width x height x 8 bytes) and the accumulated history length
 * (R16F, width x height x 2 bytes), device buffers, copied on `stream`;
 * *valid / valid say whether a frame has written them (before the first frame
 * the final pass starts from zero history). A restored context renders its next
 * frame exactly as the context the snapshot came from would have. */
sgi_status sgi_get_history(sgi_ctx* ctx, void* gi, void* history_length, int32_t* valid, void* stream);
sgi_status sgi_set_history(sgi_ctx* ctx, const void* gi, const void* history_length, int32_t valid, void* stream);

/* Log callback (the counterpart of STRATUS_LOG / STRATUS_ERROR, StratusLog.h:8-10):
 * every failure a call returns is also reported with its message, level
 * SGI_LOG_ERROR; NULL removes the callback. The callback may run on any thread
 * that calls the library and must not call back into it. */
#define SGI_LOG_INFO  0
#define SGI_LOG_ERROR 1
typedef void (*sgi_log_fn)(int32_t level, const char* message, void* user);
void sgi_set_log_callback(sgi_log_fn fn, void* user);
/* Sends one message through the callback (used by the library's own modules). */
void sgi_log_message(int32_t level, const char* message);

/* Synchronous copies of context scratch for parity tests.
 * which: SGI_DEBUG_*; writes at most `bytes` to host_dst; *needed (if not
 * NULL) receives the full size. */
#define SGI_DEBUG_VISIBLE_INDEX   0  /* int32 [1 + max_vpls]: count, then original indices */
#define SGI_DEBUG_COMPACT_VPLS    1  /* sgi_vpl [max_visible] */
#define SGI_DEBUG_COMPACT_ENTRIES 2  /* sgi_atlas_entry [max_visible] */
#define SGI_DEBUG_TILE_STAGE1     3  /* sgi_tile_stage1 [tiles] */
#define SGI_DEBUG_TILE_LISTS      4  /* int32 [tiles][1 + L]: count, compacted indices */
#define SGI_DEBUG_RESERVOIR       5  /* RGBA16F [W*H]: gather output (vplColor, validSamples); needs debug_keep_passes */
#define SGI_DEBUG_GI_HISTORY      6  /* RGB16F [W*H]: this frame's denoised GI (giColor) */
#define SGI_DEBUG_HISTORY_DEPTH   7  /* R16F [W*H]: accumulated history length */
#define SGI_DEBUG_DIRECT          8  /* RGB16F [W*H]: direct lighting of sgi_render_frame */
#define SGI_DEBUG_TAA_HISTORY     9  /* RGBA16F [W*H]: the last TAA output of sgi_post_fx */
#define SGI_DEBUG_PASS_BASE      16  /* + k: RGBA16F [W*H] reservoir output of denoise pass k */
sgi_status sgi_read_debug(sgi_ctx* ctx, int32_t which, void* host_dst, size_t bytes, size_t* needed);

/* Arithmetic of the shading kernels (gather, denoise, deferred lighting) of a
 * context; no counterpart in StratusGFX, whose GLSL leaves the precision of
 * division, sqrt, exp and multiply-add fusion to the driver.
 *   SGI_SHADING_EXACT (default): correctly rounded operations in a fixed order,
 *     bit-identical to the CPU restatement of the shaders.
 *   SGI_SHADING_FAST: the same expressions with approximate division and square
 *     root, hardware reciprocal square root and exponential and multiply-add
 *     contraction. Each pass stays within 1e-3 relative error of the exact one
 *     (denominator at least 2^-14, the smallest normal binary16) wherever no
 *     branch decision of the pass lies within its decision margin; the VPL and
 *     tile culls are exact in both modes, so the per-tile lists are identical. */
#define SGI_SHADING_EXACT 0
#define SGI_SHADING_FAST  1
sgi_status sgi_set_shading_precision(sgi_ctx* ctx, int32_t mode);
int32_t    sgi_get_shading_precision(const sgi_ctx* ctx);

/* Where the a-trous passes 1 .. n-2 (vpl_pbr_gi_denoise.fs:307-327 at stride
 * 2^pass) take their taps; no counterpart in StratusGFX (a fragment shader
 * samples textures). Both modes give bit-identical results.
 *   SGI_ATROUS_DIRECT: every tap is a clamped load from global memory.
 *   SGI_ATROUS_STAGED (default): a CTA stages the lattice of pixels its taps
 *     reach in shared memory with strided TMA copies (strides 2, 4 and 8 on
 *     even widths; other passes run direct). */
#define SGI_ATROUS_DIRECT 0
#define SGI_ATROUS_STAGED 1
sgi_status sgi_set_atrous_staging(sgi_ctx* ctx, int32_t mode);
int32_t    sgi_get_atrous_staging(const sgi_ctx* ctx);

/* Bounded device waits of a context's kernels (the staged a-trous pass waits
 * for its copies): wait_ns limits each wait (0 = the default, 200 ms);
 * skip_copies != 0 is a test switch under which no copy is issued, so that
 * every wait runs out with nothing in flight. A wait that runs out leaves its
 * pixels unwritten and sets SGI_ERR_TIMEOUT in the context's device status,
 * which sgi_device_status returns (after synchronising the device) and clears. */
sgi_status sgi_set_wait_test(sgi_ctx* ctx, int64_t wait_ns, int32_t skip_copies);
sgi_status sgi_device_status(sgi_ctx* ctx);

/* Per-pass GPU times (ms) of the last sgi_render_frame when timing is on:
 * [0] vpl cull, [1] direct lighting, [2] tile cull, [3] gather, [4] denoise;
 * with n >= 7 also the denoise pass split into [5] its a-trous passes and
 * [6] its final pass (temporal reprojection and composite). */
#define SGI_NUM_PASS_TIMES 5
#define SGI_NUM_PASS_TIMES_SPLIT 7
sgi_status sgi_set_timing(sgi_ctx* ctx, int32_t enabled);
sgi_status sgi_get_pass_times(sgi_ctx* ctx, float* ms, int32_t n);

/* Kernel launches the context issued since creation (all sgi_* calls). */
int64_t sgi_launch_count(const sgi_ctx* ctx);

/* Self-check of the packed FP32 arithmetic (no StratusGFX counterpart). The
 * a-trous passes evaluate two filter taps per instruction on the packed FP32
 * pipe; each lane must equal the scalar arithmetic bit for bit. Runs n
 * threads, each evaluating SGI_LANE_CHECKS checks both ways on hashed
 * operands: 0-2 packed add, multiply, multiply-add; 3-5 the same on exact
 * rounding ties; 6 exp over its whole range; 7 x^128; 8 a pair of a-trous tap
 * weights; 9 their accumulation into the channel sums; 10-11 multiply-add
 * with a subnormal multiplicand onto zero and onto normal sums. counts[k] = threads
 * whose check k differed; `first` (optional, SGI_LANE_CHECKS * 16 floats)
 * receives for each failing check the packed results, the scalar results and
 * the operands of one failing thread. Synchronous; uses the current device. */
#define SGI_LANE_CHECKS 12
sgi_status sgi_lane_selftest(int32_t n, uint32_t* counts, float* first);

/* Post-processing consumers of the HDR frame (no part of the GI stage in
 * StratusGFX, which runs them later in the frame: PerformTaaPostFx_ and
 * PerformGammaTonemapPostFx_, StratusRendererBackend.cpp:2323-2360):
 *   taa != 0: taa.fs - the previous TAA output, bilinearly reprojected by the
 *     G-buffer velocity, clamped in Reinhard space to the min/max of the pixel
 *     and its 4 neighbours, blended 90 % with the current colour; the result
 *     (RGBA16F, alpha 0.0625) becomes the context's TAA history (the first
 *     frame after creation or sgi_reset_history uses the current colour);
 *   then gammaTonemap.fs: ACES film curve (2.51, 0.03, 2.43, 0.59, 0.14),
 *     gamma 1/2.2, written as RGBA8 (A = 255) to ldr_out [height][width].
 * hdr_in: RGBA16F [height][width] (sgi_render_frame's output). */
sgi_status sgi_post_fx(sgi_ctx* ctx, const void* hdr_in, const sgi_gbuffer* cur, int32_t taa, void* ldr_out,
                       void* stream);

/* VPL colouring (vpl_light_color.cs:41-75, dispatched after the visibility cull
 * by PerformVirtualPointLightCullingStage1_, StratusRendererBackend.cpp:1703-1731).
 * Once set (NULL turns it off; the atlas must stay valid while set), every
 * sgi_cull_vpls also recolours the visible VPLs of the compacted list in place:
 *   color             = (diffuse(-L).rgb * sun colour) * intensity * 50000, w = 1
 *   specularPosition  = position.xyz - (1.1 * radius * depth(-L)) * L, w = 1
 * with L the CSM's light direction and sun colour its light colour, both cubes
 * read at the nearest texel in direction -L (the distance cube of
 * sgi_set_shadow_maps as a normalised depth). */
sgi_status sgi_set_vpl_coloring(sgi_ctx* ctx, const sgi_diffuse_atlas* diffuse);

/* Thread-block shape of a per-pixel pass (no counterpart in StratusGFX, whose
 * fragment shaders have no block shape). Every shape computes the same pixels
 * bit for bit; the fastest depends on the viewport, which is what
 * sgi_batch_create's autotuner (sgi_batch.h) measures. bx * by must be 256 with
 * bx a multiple of 8; (0, 0) restores the pass's default (gather 16x16, the
 * others 32x8). */
enum { SGI_BLOCK_GATHER = 0, SGI_BLOCK_ATROUS = 1, SGI_BLOCK_DENOISE_FINAL = 2, SGI_BLOCK_DIRECT = 3,
       SGI_NUM_BLOCK_PASSES = 4 };
sgi_status sgi_set_block_shape(sgi_ctx* ctx, int32_t pass, int32_t bx, int32_t by);
sgi_status sgi_get_block_shape(const sgi_ctx* ctx, int32_t pass, int32_t* bx, int32_t* by);

#ifdef __cplusplus
}
#endif

#endif /* SGI_H_ */
