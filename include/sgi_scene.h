/*
 * sgi_scene.h - GPU generation of the GI stage's inputs for synthetic box
 * scenes: G-buffer, cascaded shadow map and VPL distance cube atlases.
 *
 * In StratusGFX these inputs come from rasterisation passes upstream of the
 * GI/lighting stage: the G-buffer pass (pbr_geometry_pass.fs:95-141), the CSM
 * depth pass (RenderCSMDepth_, StratusRendererBackend.cpp:1081-1158; csm.vs,
 * csm.fs) and the VPL cube shadow pass (shadowVpl.fs:26-34, host
 * StratusRendererBackend.cpp:1426-1575). Here they are produced by ray casting
 * axis-aligned boxes on the GPU, in the same formats and conventions, so that
 * the stage's inputs never pass through a CPU.
 *
 * All buffer pointers are DEVICE pointers; matrices are host values.
 */
#ifndef SGI_SCENE_H_
#define SGI_SCENE_H_

#include "sgi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One axis-aligned box with a constant material. 64 bytes. */
typedef struct sgi_box {
    float min[4];
    float max[4];
    float albedo[4];     /* rgb base colour; a = emissive r (G-buffer albedo alpha) */
    float roughness;
    float metallic;
    float reflectance;   /* written to base_reflectivity.r */
    float id;            /* written to the id buffer */
} sgi_box;

/* Camera of the G-buffer pass: column-major GL matrices. */
typedef struct sgi_scene_camera {
    float proj_view[16];
    float inv_proj_view[16];
    float prev_proj_view[16];   /* for the velocity buffer (calculateVelocity, common.glsl:157-167) */
    float position[4];
} sgi_scene_camera;

/* Writes every plane of `out` (W*H each; the pointers are written through). */
sgi_status sgi_scene_gbuffer(const sgi_box* boxes, int32_t num_boxes, const sgi_scene_camera* cam,
                             int32_t width, int32_t height, const sgi_gbuffer* out, void* stream);

/* Depth of the nearest surface towards the light per CSM texel, depth clamp
 * on, slope-scaled polygon offset factor 2 (StratusRendererBackend.cpp:1089-1091).
 * csm->depth is the output [num_cascades][res][res]; inv_cascade_proj_view
 * holds the 4 inverse matrices (column-major). */
sgi_status sgi_scene_csm(const sgi_box* boxes, int32_t num_boxes, const sgi_csm* csm,
                         const float inv_cascade_proj_view[4][16], void* stream);

/* Distance cube maps for VPLs [first, first + count): texel = saturate(d / far_plane),
 * written into slot (index, layer) = entries[v] of `atlas` (layout of sgi_cube_atlas). */
sgi_status sgi_scene_cube_atlas(const sgi_box* boxes, int32_t num_boxes, const sgi_vpl* vpls,
                                const sgi_atlas_entry* entries, int32_t count,
                                const sgi_cube_atlas* atlas, void* stream);

/* Diffuse colour cubes for the same VPLs and texel directions: the RGB8 albedo of
 * the first box the texel's ray hits (A = 255), 0 where it hits none (the colour
 * attachment shadowVpl.fs writes). */
sgi_status sgi_scene_diffuse_atlas(const sgi_box* boxes, int32_t num_boxes, const sgi_vpl* vpls,
                                   const sgi_atlas_entry* entries, int32_t count, const sgi_diffuse_atlas* atlas,
                                   void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SGI_SCENE_H_ */
