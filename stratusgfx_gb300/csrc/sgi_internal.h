// sgi_internal.h - launch wrappers shared by the host layer (sgi_api.cpp) and
// the CUDA translation units. Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sgi.h"
#include "../../include/sgi_scene.h"

namespace sgi {

#ifdef __CUDACC__
#define SGI_HD_INLINE __host__ __device__ __forceinline__
#else
#define SGI_HD_INLINE inline
#endif

// Device-side constants of the shading passes (RendererSettings subset).
struct ShadeConfig {
    float min_roughness;
    int32_t perceptual;
    float fog_density;
    float fog_color[3];
    float point_ambient;
    float min_gi_occlusion;
    float emission_strength;
};

// Outputs of the gather kernel. Its epilogue also performs denoise pass 0
// (the centre-only reservoir merge) and records the per-pixel guide that the
// later passes read instead of re-decoding normals.
struct GatherOut {
    uint2* merged;           // RGBA16F pass-0 output (shadowFactor, 1)
    float4* guide;           // decoded centre normal (xyz) and window depth (w)
    uint2* raw;              // RGBA16F raw reservoir (vplColor, validSamples); may be null
};

struct DenoiseLaunch {
    int32_t width, height;
    int32_t pass;            // 1 .. passes-1
    int32_t passes;
    float time;
    float fps;
    sgi_gbuffer cur;         // depth, normal, albedo, velocity, id of this frame
    const float* prev_depth;
    const uint32_t* prev_normal;
    const float* prev_id;
    const uint2* res_in;     // RGBA16F reservoir of the previous pass (gather output for pass 0)
    uint2* res_out;          // RGBA16F (may be null on the final pass)
    const uint2* hdr_in;     // screen, RGB16F
    uint2* hdr_out;          // combined, RGB16F (final pass)
    const uint2* gi_prev;    // prevIndirectIllumination, RGB16F
    uint2* gi_out;           // giColor, RGB16F (final pass)
    const uint16_t* hist_prev;  // historyDepth, R16F
    uint16_t* hist_out;         // newHistoryDepth, R16F (final pass)
    const int32_t* visible_index;  // [0] = numVisible
    const float4* guide;     // from the gather
};

cudaError_t launch_vis_flags(const sgi_vpl* vpls, int32_t n, const sgi_csm& csm, uint8_t* flags, cudaStream_t s);
// Device address of the fixed flag array of sgi_cull_vpls_noalloc on the current device.
cudaError_t noalloc_cull_flags(uint8_t** flags);
// taa.fs + gammaTonemap.fs: hist_in NULL on the first TAA frame; taa = 0 tonemaps hdr directly
cudaError_t launch_post_fx(int32_t W, int32_t H, const uint2* hdr, const uint32_t* velocity, const uint2* hist_in,
                           uint2* hist_out, uint32_t* ldr, int32_t taa, cudaStream_t s);
// vpl_light_color.cs over the compacted list (recolours cv in place)
cudaError_t launch_vpl_color(sgi_vpl* cv, const sgi_atlas_entry* ce, const int32_t* visible_index, int32_t cap,
                             const sgi_cube_atlas& cubes, const sgi_diffuse_atlas& diffuse, const sgi_csm& csm,
                             cudaStream_t s);
// vpr (may be null): (position, radius) of the kept VPLs for the tile cull
// visibility flags and compaction in one launch (the last block compacts); `finished` is a zeroed device
// counter owned by the caller, zero again after the launch
cudaError_t launch_vpl_cull(const sgi_vpl* vpls, const sgi_atlas_entry* entries, int32_t n, const sgi_csm& csm,
                            uint8_t* flags, int32_t cap, sgi_vpl* cv, sgi_atlas_entry* ce, int32_t* visible_index,
                            float4* vpr, unsigned* finished, cudaStream_t s);
cudaError_t launch_compact(const sgi_vpl* vpls, const sgi_atlas_entry* entries, const uint8_t* flags, int32_t n,
                           int32_t cap, sgi_vpl* cv, sgi_atlas_entry* ce, int32_t* visible_index, float4* vpr,
                           cudaStream_t s);
cudaError_t launch_tile_stage1(const sgi_config& cfg, const sgi_gbuffer& g, const sgi_camera& cam,
                               sgi_tile_stage1* out, cudaStream_t s);
// stage 2: one block per tile, keys in shared memory (tile_cull_smem bytes)
cudaError_t launch_tile_stage2(const sgi_config& cfg, const sgi_tile_stage1* s1, const float4* vpr,
                               const int32_t* visible_index, int32_t* lists, cudaStream_t s);
size_t tile_cull_smem(const sgi_config& cfg);
// shadow-casting point lights of the deferred pass (pbr.fs:116-131)
struct ShadowCasters {
    const sgi_point_light* lights;
    const sgi_atlas_entry* entries;
    int32_t count;
    sgi_cube_atlas atlas;
};

// ------------------------------------------------ persistent multi-view frame --
// One launch renders a plain frame of many views: persistent CTAs take work
// items (view, level, index) from a queue in dependency order and wait, with a
// time limit, until the levels an item depends on are complete for its view.
enum PLevel : int {
    kPVis = 0,        // VPL visibility flags, 256 VPLs per item
    kPCompact = 1,    // stable compaction of the visible VPLs, one item
    kPDirect = 2,     // deferred lighting, kPBlocksPerItem 16x16 pixel blocks per item
    kPTile = 3,       // tile mean + tile cull, kPBlocksPerItem 16x16 tiles per item
    kPGather = 4,     // gather + denoise pass 0, kPBlocksPerItem tiles per item
    kPAtrous = 5,     // + (pass - 1): a-trous pass 1 .. n-2; the final pass follows the last one
};
constexpr int kPMaxLevels = kPAtrous + SGI_MAX_DENOISE_PASSES - 1;
constexpr int kPBlocksPerItem = 4;   // 16x16 pixel blocks of one item of the pixel passes
constexpr int kPMaxViews = 256;
SGI_HD_INLINE uint32_t pitem(int view, int level, int index) {
    return (uint32_t)view | ((uint32_t)level << 8) | ((uint32_t)index << 13);
}

// Work-queue state in device memory: zero before the first launch; the last
// CTA of every launch returns it to zero.
struct PQueue {
    unsigned int next;        // items taken
    unsigned int finished;    // CTAs that left the loop
    int done[kPMaxViews][kPMaxLevels];
};

// What a view's passes need, gathered from its context (host side).
struct PViewDesc {
    sgi_config cfg;
    ShadeConfig sc;
    const sgi_vpl* vpls; const sgi_atlas_entry* entries; int32_t num_vpls;
    sgi_csm csm;
    sgi_cube_atlas cubes;
    const sgi_point_light* points; int32_t num_points;
    const sgi_point_light* casters; const sgi_atlas_entry* caster_entries; int32_t num_casters;
    sgi_cube_atlas caster_atlas;
    uint8_t* flags; sgi_vpl* cv; sgi_atlas_entry* ce; int32_t* visible_index; float4* vpr;
    sgi_tile_stage1* stage1; int32_t* lists;
    sgi_gbuffer cur; sgi_camera cam; const sgi_gbuffer* prev_ptr; sgi_gbuffer prev;
    sgi_frame_params params;
    float4* guide; uint2* raw;
    uint2* pass_buf[SGI_MAX_DENOISE_PASSES];   // output of every denoise pass
    uint2* direct;
    const uint2* gi_prev; uint2* gi_out; const uint16_t* hist_prev; uint16_t* hist_out;
    void* hdr_out;
    int32_t atrous_staged;   // the context's a-trous staging (sgi_set_atrous_staging)
};

struct PPlan {
    const uint32_t* items;     // dispatch order
    int32_t num_items;
    int32_t num_views;
    const int32_t* counts;     // [num_views][kPMaxLevels] items per level
    PQueue* q;
    int32_t* status;           // SGI_OK, or SGI_ERR_TIMEOUT after a wait gave up (the host clears it)
    const int32_t* skip;       // [num_views][kPMaxLevels]: nonzero = the level's items do nothing (test switch)
    const long long* wait_ns;  // limit of every wait (device memory, so that a captured launch sees changes)
    const unsigned char* views;  // per-view parameter blocks of view_bytes each
    int32_t view_bytes;
};

// The CTA grid of the staged a-trous pass at stride 2^pass (sgi_shade.cu): lattice patches of 16 x 8 points
// per two x remainders, (ntx * s / 2) x (nty * s) CTAs; 0 (no staged pass) for strides above 8 or odd widths.
inline int atrous_lattice_grid(int W, int H, int pass, int* gx, int* gy, int* ntx, int* nty) {
    const int st = pass >= 1 && pass <= 3 ? 1 << pass : 0;
    if (!st || W < 2 || (W & 1) || H < 1) { *gx = *gy = *ntx = *nty = 0; return 0; }
    *ntx = ((W + st - 1) / st + 15) / 16;
    *nty = ((H + st - 1) / st + 7) / 8;
    *gx = *ntx * (st / 2);
    *gy = *nty * st;
    return *gx * *gy;
}

// The shading kernels (sgi_shade.cu) exist twice: sgi::exact is bit-identical to
// the CPU restatement of the shaders, sgi::fast is the tolerance mode (fast
// division, square root, exponential and contraction; see sgi_shade.cu).
#define SGI_SHADE_LAUNCHERS \
    cudaError_t launch_gather(const sgi_config& cfg, const ShadeConfig& sc, const sgi_gbuffer& g, const sgi_camera& cam, \
                              const sgi_vpl* cv, const sgi_atlas_entry* ce, const int32_t* visible_index, \
                              const int32_t* lists, const sgi_cube_atlas& cubes, float time, const GatherOut& out, \
                              cudaStream_t s, dim3 block = dim3(0, 0, 0)); \
    /* a-trous pass `pass` (1 .. passes-2): 5x5 taps at stride 2^pass */ \
    cudaError_t launch_atrous(int32_t W, int32_t H, int32_t pass, const float4* guide, const uint2* res_in, \
                              uint2* res_out, cudaStream_t s, dim3 block = dim3(0, 0, 0)); \
    /* the same pass from a TMA-staged shared-memory lattice (strides 2, 4, 8; even width; */ \
    /* cudaErrorNotSupported otherwise); a wait that runs out sets SGI_ERR_TIMEOUT in *status */ \
    cudaError_t launch_atrous_staged(int32_t W, int32_t H, int32_t pass, const float4* guide, const uint2* res_in, \
                                     uint2* res_out, long long wait_ns, int32_t skip_copies, int32_t* status, \
                                     cudaStream_t s); \
    /* last pass: a-trous filter + temporal reprojection + composite */ \
    cudaError_t launch_denoise_final(const DenoiseLaunch& d, cudaStream_t s, dim3 block = dim3(0, 0, 0)); \
    cudaError_t launch_deferred(const sgi_config& cfg, const ShadeConfig& sc, const sgi_gbuffer& g, \
                                const sgi_camera& cam, const sgi_point_light* points, int32_t num_points, \
                                const ShadowCasters& casters, const sgi_csm& csm, uint2* hdr_out, cudaStream_t s, \
                                dim3 block = dim3(0, 0, 0)); \
    /* persistent multi-view frame: bytes of one view's parameter block, filling it, the launch */ \
    int32_t persistent_view_bytes(); \
    bool persistent_fill_view(const PViewDesc& d, unsigned char* out); /* false: a tensor map failed */ \
    size_t persistent_smem(int32_t max_visible); \
    /* variant 0: registers for 4 CTAs per SM, 1: for 2 */ \
    cudaError_t persistent_occupancy(int variant, size_t smem, int* blocks_per_sm); \
    cudaError_t launch_persistent(const PPlan& plan, int variant, int grid, size_t smem, cudaStream_t s);

namespace exact {
SGI_SHADE_LAUNCHERS
// converged target: `batches` runs of the sample loop, sums in FP64 -> float4 (rgb, 1)
cudaError_t launch_gi_target(const sgi_config& cfg, const ShadeConfig& sc, const sgi_gbuffer& g,
                             const sgi_camera& cam, const sgi_vpl* cv, const sgi_atlas_entry* ce,
                             const int32_t* visible_index, const int32_t* lists, const sgi_cube_atlas& cubes,
                             float time, int batches, float4* out, cudaStream_t s);
}  // namespace exact
namespace fast {
SGI_SHADE_LAUNCHERS
}  // namespace fast
#undef SGI_SHADE_LAUNCHERS

// Thread-block shapes of the per-pixel passes: any shape of 256 threads gives the
// same results (every pixel is computed by one thread, independently); a zero
// shape selects the pass's default.

// scene generation (sgi_scene.cu)
cudaError_t launch_scene_gbuffer(const sgi_box* boxes, int32_t nb, const sgi_scene_camera& cam, int32_t W,
                                 int32_t H, const sgi_gbuffer& out, cudaStream_t s);
cudaError_t launch_scene_csm(const sgi_box* boxes, int32_t nb, const sgi_csm& csm, const float (*inv)[16],
                             cudaStream_t s);
cudaError_t launch_scene_diffuse(const sgi_box* boxes, int32_t nb, const sgi_vpl* vpls,
                                 const sgi_atlas_entry* entries, int32_t count, const sgi_diffuse_atlas& atlas,
                                 cudaStream_t s);
cudaError_t launch_scene_cubes(const sgi_box* boxes, int32_t nb, const sgi_vpl* vpls, const sgi_atlas_entry* entries,
                               int32_t count, const sgi_cube_atlas& atlas, cudaStream_t s);

}  // namespace sgi
