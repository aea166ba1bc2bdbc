// sgi_persistent.cuh - one launch that renders a plain frame of many views
// (included at the end of sgi_shade.cu, so it exists in the exact and in the
// tolerance build of the shading kernels).
//
// The frame of a view is a chain of passes, each a set of independent work
// items: VPL visibility flags (256 VPLs an item) -> stable compaction (one
// item) -> per tile: mean position/normal and VPL list (one 16x16 tile an
// item) -> gather + denoise pass 0 (one tile, its list staged in shared
// memory) -> a-trous passes -> final pass (which also needs the view's direct
// lighting, a set of items of its own). The host lists every view's items in
// an order that respects these dependencies (all items of a pass before the
// next pass's, views interleaved within a pass). The grid is no larger than
// the number of CTAs that fit on the GPU at once; each CTA takes the next item
// from the queue, waits until the passes it depends on are complete for its
// view, runs it and counts it done. Every item a CTA waits for was taken
// earlier by a running CTA, so the waits end, except when the test switch
// `skip` holds a pass back: then a wait gives up after `wait_ns`, sets
// SGI_ERR_TIMEOUT in the status word and raises the abort flag (the same
// word), every CTA leaves at its next wait or fetch, and the last CTA to leave
// returns the queue to zero for the next launch.
//
// Every buffer a launch writes is written once and read only after its
// writers are counted done (each denoise pass has its own output buffer), so
// reads through the read-only data path never see a line from before the
// write.
#pragma once

// One view's parameters in device memory.
struct PView {
    // culls
    const sgi_vpl* vpls;
    const sgi_atlas_entry* entries;
    int32_t num_vpls, max_visible, L;
    int32_t width, height, tiles_x, blocks, passes;
    uint8_t* flags;
    sgi_vpl* cv;
    sgi_atlas_entry* ce;
    int32_t* visible_index;
    float4* vpr;
    sgi_tile_stage1* stage1;
    int32_t* lists;
    sgi_csm csm;
    sgi_gbuffer g;
    sgi_camera cam;
    // shading
    GatherParams gp;
    DeferredParams dp;
    DenoiseLaunch dl;                            // the final pass
    const float4* guide;
    uint2* pass_buf[SGI_MAX_DENOISE_PASSES];     // output of each denoise pass
    // a-trous passes 1..3 from the TMA-staged lattice (atrous_staged_cta): CTA grid per pass (gx = 0: the
    // direct per-pixel filter) and the tensor maps of guide and input reservoir
    int32_t lat_gx[3], lat_gy[3], lat_ntx[3], lat_nty[3];
    CUtensorMap amap[3][2];                      // CUtensorMap is 128-byte aligned
};

int32_t persistent_view_bytes() { return (int32_t)((sizeof(PView) + 255) & ~(size_t)255); }

bool persistent_fill_view(const PViewDesc& d, unsigned char* out) {
    PView v;
    memset(&v, 0, sizeof(v));
    const sgi_config& cfg = d.cfg;
    v.vpls = d.vpls; v.entries = d.entries; v.num_vpls = d.num_vpls; v.max_visible = cfg.max_visible;
    v.L = cfg.max_vpls_per_tile;
    v.width = cfg.width; v.height = cfg.height; v.tiles_x = (cfg.width + 15) / 16; v.passes = cfg.denoise_passes;
    v.blocks = v.tiles_x * ((cfg.height + 15) / 16);
    v.flags = d.flags; v.cv = d.cv; v.ce = d.ce; v.visible_index = d.visible_index; v.vpr = d.vpr;
    v.stage1 = d.stage1; v.lists = d.lists; v.csm = d.csm; v.g = d.cur; v.cam = d.cam;
    GatherParams& p = v.gp;
    p.W = cfg.width; p.H = cfg.height; p.ts = cfg.tile_size; p.tiles_x = v.tiles_x;
    p.L = cfg.max_vpls_per_tile; p.tiled = 1; p.spp = cfg.samples_per_pixel;
    p.sc = d.sc; p.g = d.cur; p.cam = d.cam; p.cv = d.cv; p.ce = d.ce; p.visible_index = d.visible_index;
    p.lists = d.lists; p.cubes = d.cubes; p.time = d.params.time;
    p.out.merged = d.pass_buf[0]; p.out.guide = d.guide; p.out.raw = d.raw;
    DeferredParams& q = v.dp;
    q.W = cfg.width; q.H = cfg.height; q.sc = d.sc; q.g = d.cur; q.cam = d.cam; q.points = d.points;
    q.num_points = d.num_points;
    q.casters = ShadowCasters{d.casters, d.caster_entries, d.num_casters, d.caster_atlas};
    q.csm = d.csm; q.out = d.direct;
    DenoiseLaunch& l = v.dl;
    l.width = cfg.width; l.height = cfg.height; l.passes = cfg.denoise_passes; l.pass = cfg.denoise_passes - 1;
    l.time = d.params.time; l.fps = d.params.frames_per_second;
    l.cur = d.cur;
    l.prev_depth = d.prev.depth; l.prev_normal = d.prev.normal; l.prev_id = d.prev.id;
    l.res_in = d.pass_buf[cfg.denoise_passes - 2];
    l.res_out = d.pass_buf[cfg.denoise_passes - 1];
    l.hdr_in = d.direct; l.hdr_out = (uint2*)d.hdr_out;
    l.gi_prev = d.gi_prev; l.gi_out = d.gi_out; l.hist_prev = d.hist_prev; l.hist_out = d.hist_out;
    l.visible_index = d.visible_index;
    l.guide = d.guide;
    v.guide = d.guide;
    for (int k = 0; k < SGI_MAX_DENOISE_PASSES; ++k) v.pass_buf[k] = d.pass_buf[k];
    bool ok = true;
    for (int pass = 1; pass <= 3 && pass < cfg.denoise_passes - 1; ++pass) {
        int gx = 0, gy = 0, ntx = 0, nty = 0;
        if (d.atrous_staged && atrous_lattice_grid(cfg.width, cfg.height, pass, &gx, &gy, &ntx, &nty) > 0) {
            if (encode_atrous_maps(cfg.width, cfg.height, pass, d.guide, d.pass_buf[pass - 1], &v.amap[pass - 1][0],
                                   &v.amap[pass - 1][1]) != cudaSuccess) {
                ok = false;
                gx = gy = 0;
            }
        }
        v.lat_gx[pass - 1] = gx; v.lat_gy[pass - 1] = gy; v.lat_ntx[pass - 1] = ntx; v.lat_nty[pass - 1] = nty;
    }
    memcpy(out, &v, sizeof(v));
    return ok;
}

size_t persistent_smem(int32_t max_visible) {
    const size_t cull = (size_t)2 * sizeof(uint32_t) * (size_t)max_visible;
    return cull > sizeof(StagedList) ? cull : sizeof(StagedList);
}

// Waits until the pass `level` of view `v` has all its items done. Returns
// false when the launch was aborted or this wait gave up (after setting the
// status word).
SGI_D bool wait_level(const PPlan& plan, int v, int level) {
    const int need = plan.counts[v * kPMaxLevels + level];
    volatile int* done = &plan.q->done[v][level];
    volatile int* status = plan.status;
    if (*done >= need) {
        __threadfence();
        return true;
    }
    const long long t0 = global_ns();
    const long long limit = *(volatile const long long*)plan.wait_ns;
    for (;;) {
        if (*done >= need) break;
        if (*status != SGI_OK) return false;
        if (global_ns() - t0 > limit) {
            atomicCAS(plan.status, SGI_OK, SGI_ERR_TIMEOUT);
            return false;
        }
        __nanosleep(256);
    }
    __threadfence();
    return true;
}

SGI_D bool wait_deps(const PPlan& plan, const PView& pv, int v, int level) {
    const int final_level = kPAtrous + pv.passes - 2;
    switch (level) {
        case kPVis:
        case kPDirect: return true;
        case kPCompact: return wait_level(plan, v, kPVis);
        case kPTile: return wait_level(plan, v, kPCompact);
        case kPGather: return wait_level(plan, v, kPTile);
        default:
            if (level == final_level && !wait_level(plan, v, kPDirect)) return false;
            return wait_level(plan, v, level - 1);
    }
}

// kMinBlocks: the CTAs per SM the registers are budgeted for (4: 64 registers a
// thread, 2: 128); the batch's tuner times both.
template <int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks) persistent_frame_kernel(PPlan plan) {
    extern __shared__ float4 persistent_smem_buf[];
    __shared__ uint32_t s_item;
    __shared__ int s_go;
    __shared__ sgi_tile_stage1 s_tile;
    __shared__ LightConst s_lc;
    __shared__ __align__(8) unsigned long long s_bar;   // the staged a-trous copies
    const int tid = threadIdx.x;
    const uint32_t bar = smem_u32(&s_bar);
    uint32_t stage_uses = 0;   // completed phases of s_bar
    if (tid == 0) stage_barrier_init(bar);
    __syncthreads();
    // thread 0 takes the next queue position while the CTA works on the current item
    unsigned next = tid == 0 ? atomicAdd(&plan.q->next, 1u) : 0u;
    for (;;) {
        if (tid == 0) {
            uint32_t it = 0xffffffffu;
            int go = 0;
            if (*(volatile int*)plan.status == SGI_OK && next < (unsigned)plan.num_items) {
                it = plan.items[next];
                const int v = (int)(it & 0xffu), level = (int)((it >> 8) & 0x1fu);
                const PView& pv = *reinterpret_cast<const PView*>(plan.views + (size_t)v * plan.view_bytes);
                go = wait_deps(plan, pv, v, level) ? 1 : 0;
                if (go) next = atomicAdd(&plan.q->next, 1u);
            }
            s_item = it;
            s_go = go;
        }
        __syncthreads();
        const uint32_t it = s_item;
        if (!s_go) break;
        const int v = (int)(it & 0xffu), level = (int)((it >> 8) & 0x1fu), index = (int)(it >> 13);
        const PView& pv = *reinterpret_cast<const PView*>(plan.views + (size_t)v * plan.view_bytes);
        if (!plan.skip[v * kPMaxLevels + level]) {
            if (level == kPVis) {
                const int i = index * 256 + tid;
                if (i < pv.num_vpls) pv.flags[i] = vpl_visible(pv.vpls, i, pv.csm);
            } else if (level == kPCompact) {
                compact_vpls<256>(pv.vpls, pv.entries, pv.flags, pv.num_vpls, pv.max_visible, pv.cv, pv.ce,
                                  pv.visible_index, pv.vpr, tid);
            } else if (level >= kPAtrous && level - kPAtrous < 3 && level < kPAtrous + pv.passes - 2 &&
                       pv.lat_gx[level - kPAtrous] > 0) {
                // a-trous pass 1..3 from the staged lattice: kPBlocksPerItem lattice CTAs an item
                const int k = level - kPAtrous, pass = k + 1;
                const int n = pv.lat_gx[k] * pv.lat_gy[k];
                const int c1 = min((index + 1) * kPBlocksPerItem, n);
                const AtrousStageWait wt{*(volatile const long long*)plan.wait_ns, 0, plan.status};
                for (int c = index * kPBlocksPerItem; c < c1; ++c) {
                    const bool ok = atrous_staged_cta(&pv.amap[k][0], &pv.amap[k][1], pv.width, pv.height, 1 << pass,
                                                      pv.lat_ntx[k], pv.lat_nty[k], c % pv.lat_gx[k], c / pv.lat_gx[k],
                                                      pv.guide, pv.pass_buf[pass - 1], pv.pass_buf[pass], bar,
                                                      stage_uses & 1u, wt);
                    ++stage_uses;
                    __syncthreads();   // this use's reads of the staged lattice before the next use's copies
                    if (!ok) break;    // the status word says so; every CTA leaves at its next fetch
                }
            } else {
                // the pixel passes: kPBlocksPerItem consecutive 16x16 blocks (tiles) an item
                if (level == kPDirect) {   // the light constants of this view, once per item
                    light_const_fill(pv.dp, s_lc, tid, 256);
                    __syncthreads();
                }
                const int b1 = min((index + 1) * kPBlocksPerItem, pv.blocks);
                for (int b = index * kPBlocksPerItem; b < b1; ++b) {
                    const int bx = b % pv.tiles_x, by = b / pv.tiles_x;
                    const int x = bx * 16 + (tid & 15), y = by * 16 + (tid >> 4);
                    const bool inside = x < pv.width && y < pv.height;
                    if (level == kPDirect) {
                        if (inside) deferred_pixel(pv.dp, x, y, &s_lc);
                    } else if (level == kPTile) {
                        tile_mean(pv.width, pv.height, 16, bx, by, tid, pv.g, pv.cam, nullptr, &s_tile);
                        __syncthreads();
                        if (tid == 0) pv.stage1[b] = s_tile;
                        const V3 tp = v3(s_tile.average_position[0], s_tile.average_position[1],
                                         s_tile.average_position[2]);
                        const V3 tn = v3(s_tile.average_normal[0], s_tile.average_normal[1], s_tile.average_normal[2]);
                        tile_cull(pv.L, tp, tn, pv.vpr, __ldg(pv.visible_index),
                                  reinterpret_cast<uint32_t*>(persistent_smem_buf), pv.lists + (size_t)b * (1 + pv.L),
                                  tid);
                    } else if (level == kPGather) {
                        StagedList* staged = reinterpret_cast<StagedList*>(persistent_smem_buf);
                        stage_tile_list(pv.gp, b, staged, tid, 256);
                        __syncthreads();
                        if (inside) gather_pixel<true>(pv.gp, x, y, staged);
                        __syncthreads();   // the staged list is rewritten by the next block
                    } else if (level < kPAtrous + pv.passes - 2) {
                        const int pass = level - kPAtrous + 1;
                        if (inside)
                            atrous_pixel(pv.width, pv.height, 1 << pass, pv.guide, pv.pass_buf[pass - 1],
                                         pv.pass_buf[pass], x, y);
                    } else {
                        if (inside) denoise_final_pixel(pv.dl, x, y);
                    }
                }
            }
        }
        __syncthreads();
        if (tid == 0 && !plan.skip[v * kPMaxLevels + level]) {
            __threadfence();
            atomicAdd(&plan.q->done[v][level], 1);
        }
    }
    // the last CTA to leave returns the queue to zero
    if (tid == 0) {
        __threadfence();
        const unsigned f = atomicAdd(&plan.q->finished, 1u);
        if (f == gridDim.x - 1) {
            for (int v = 0; v < plan.num_views; ++v)
                for (int l = 0; l < kPMaxLevels; ++l) plan.q->done[v][l] = 0;
            plan.q->next = 0u;
            plan.q->finished = 0u;
            __threadfence();
        }
    }
}

template <int kMinBlocks> cudaError_t persistent_occupancy_of(size_t smem, int* blocks_per_sm) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(persistent_frame_kernel<kMinBlocks>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, persistent_frame_kernel<kMinBlocks>, 256, smem);
}

cudaError_t persistent_occupancy(int variant, size_t smem, int* blocks_per_sm) {
    return variant == 0 ? persistent_occupancy_of<4>(smem, blocks_per_sm) : persistent_occupancy_of<2>(smem, blocks_per_sm);
}

cudaError_t launch_persistent(const PPlan& plan, int variant, int grid, size_t smem, cudaStream_t s) {
    if (variant == 0)
        persistent_frame_kernel<4><<<grid, 256, smem, s>>>(plan);
    else
        persistent_frame_kernel<2><<<grid, 256, smem, s>>>(plan);
    return cudaGetLastError();
}
