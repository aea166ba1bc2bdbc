// sgi_ctx.h - the GI/lighting stage context behind sgi_ctx (host side, internal).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/sgi.h"
#include "sgi_internal.h"

struct sgi_ctx {
    sgi_config cfg;
    sgi::ShadeConfig sc;
    std::string err;
    int64_t launches = 0;
    int device = 0;

    // lights
    sgi_vpl* vpls = nullptr;
    sgi_atlas_entry* entries = nullptr;
    int32_t num_vpls = 0;
    sgi_point_light* points = nullptr;
    int32_t num_points = 0;
    bool lights_set = false;
    bool maps_set = false;
    sgi_csm csm;
    sgi_cube_atlas cubes;

    // culling scratch
    uint8_t* flags = nullptr;
    sgi_vpl* cv = nullptr;
    sgi_atlas_entry* ce = nullptr;
    int32_t* visible_index = nullptr;
    sgi_tile_stage1* stage1 = nullptr;
    int32_t* lists = nullptr;
    float4* vpr = nullptr;            // (position, radius) of the compacted VPLs, for the tile cull
    int32_t num_tiles = 0;
    bool culled = false;

    // GI scratch
    uint2* reservoir = nullptr;
    uint2* ping[2] = {nullptr, nullptr};
    uint2* merged = nullptr;                // denoise pass-0 output (kept for the learned denoiser)
    uint2* pass_bufs[SGI_MAX_DENOISE_PASSES] = {};
    uint2* direct = nullptr;
    float4* guide = nullptr;
    uint2* gi_hist[2] = {nullptr, nullptr};
    uint16_t* hist_depth[2] = {nullptr, nullptr};
    int hist_cur = 0;
    bool have_history = false;
    const uint2* last_merged = nullptr;   // pass-0 output of the last gather
    int feat_hist = 0;                    // history slot that was "previous" for the last gather
    bool feat_have_history = false;

    // learned-denoiser inputs/outputs (allocated on first use)
    __nv_bfloat16* nn_feat = nullptr;
    float4* nn_prev = nullptr;

    // shading kernels: exact (false) or the tolerance mode (true)
    bool fast_shading = false;
    // a-trous passes from the TMA-staged lattice (true, the default: 9-11 % faster at
    // 1080p) or with direct tap loads
    bool atrous_staged = true;
    // bounded device waits: limit (0 = the kernels' default), test switch, status word
    long long wait_ns = 0;
    int32_t skip_copies = 0;
    int32_t* dev_status = nullptr;
    unsigned* cull_finished = nullptr;   // finished-block count of the one-launch VPL cull (zero between launches)

    // timing
    bool timing = false;
    cudaEvent_t ev[SGI_NUM_PASS_TIMES + 1] = {};
    cudaEvent_t ev_atrous_end = nullptr;   // between the last a-trous pass and the final denoise pass
    bool have_split = false;               // the last timed frame recorded ev_atrous_end
    bool have_times = false;

    // direct lighting runs on a side stream, concurrently with the VPL and tile
    // culls and the GI gather, and joins before the final composite
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;

    // shadow-casting point lights of the direct lighting (sgi_set_shadow_point_lights)
    sgi_point_light* shadow_points = nullptr;
    sgi_atlas_entry* shadow_entries = nullptr;
    int32_t num_shadow_points = 0;
    sgi_cube_atlas shadow_atlas = {};

    // TAA history of sgi_post_fx (RGBA16F ping-pong, allocated on first use)
    uint2* taa_hist[2] = {nullptr, nullptr};
    int taa_cur = 0;
    bool have_taa = false;

    // VPL colouring after the cull (sgi_set_vpl_coloring)
    bool coloring = false;
    sgi_diffuse_atlas diffuse = {};

    // thread-block shapes of the per-pixel passes (SGI_BLOCK_*; {0, 0} = default)
    int32_t block[SGI_NUM_BLOCK_PASSES][2] = {};
    dim3 block_dim(int pass) const {
        return block[pass][0] ? dim3((unsigned)block[pass][0], (unsigned)block[pass][1], 1) : dim3(0, 0, 0);
    }
};
