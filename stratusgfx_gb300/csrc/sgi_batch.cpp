// sgi_batch.cpp - C ABI of include/sgi_batch.h: block-shape autotuning and CUDA
// graph capture of one frame of many views.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/sgi_batch.h"
#include "sgi_ctx.h"

struct sgi_batch {
    std::vector<sgi_view> views;
    sgi_nn* net = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int next = 0;                 // graph of the next replay (history parity)
    int64_t kernels = 0;          // kernel nodes per graph
    std::string err;
    // persistent mode (sgi_batch_create_persistent): one kernel per frame
    bool persistent = false;
    bool fast = false;
    unsigned char* d_views = nullptr;     // [2 parities][views][view_bytes]
    uint32_t* d_items = nullptr;
    int32_t* d_counts = nullptr;
    sgi::PQueue* d_queue = nullptr;
    int32_t* d_status = nullptr;
    int32_t* d_skip = nullptr;
    long long* d_wait = nullptr;
    std::vector<void*> scratch;           // per-view denoise pass buffers
    sgi::PPlan plan[2] = {};
    int variant = 0;                      // register budget of the persistent kernel (tuned)
    int grid = 0;
    size_t smem = 0;
};

namespace {

constexpr int kShapes[5][2] = {{32, 8}, {16, 16}, {64, 4}, {128, 2}, {8, 32}};

sgi_status bfail(sgi_batch* b, sgi_status s, const std::string& msg) {
    if (b) b->err = msg;
    sgi_log_message(SGI_LOG_ERROR, msg.c_str());
    return s;
}

sgi_status render(const sgi_view& v, sgi_nn* net, cudaStream_t s) {
    if (net)
        return sgi_render_frame_neural(v.ctx, net, v.cur, v.prev, v.cam, &v.params, v.hdr_out, (void*)s);
    return sgi_render_frame(v.ctx, v.cur, v.prev, v.cam, &v.params, v.hdr_out, (void*)s);
}

// Per pass, the candidate shape with the smallest total time over `frames` timed frames.
// Pass times: [1] direct lighting, [3] gather, [4] denoise (a-trous + final, tuned together).
sgi_status tune(sgi_batch* b, const sgi_view& v, int frames, cudaStream_t s) {
    const bool timing = v.ctx->timing;
    sgi_set_timing(v.ctx, 1);
    float best[3] = {1e30f, 1e30f, 1e30f};
    int pick[3] = {0, 0, 0};
    for (int c = 0; c < 5; ++c) {
        for (int p = 0; p < SGI_NUM_BLOCK_PASSES; ++p) sgi_set_block_shape(v.ctx, p, kShapes[c][0], kShapes[c][1]);
        float sum[3] = {0.0f, 0.0f, 0.0f};
        for (int f = 0; f < frames + 1; ++f) {   // one untimed frame per candidate
            sgi_status st = render(v, b->net, s);
            if (st != SGI_OK) return bfail(b, st, std::string("tuning frame: ") + sgi_last_error(v.ctx));
            float ms[SGI_NUM_PASS_TIMES];
            st = sgi_get_pass_times(v.ctx, ms, SGI_NUM_PASS_TIMES);
            if (st != SGI_OK) return bfail(b, st, std::string("pass times: ") + sgi_last_error(v.ctx));
            if (f == 0) continue;
            sum[0] += ms[1];
            sum[1] += ms[3];
            sum[2] += ms[4];
        }
        for (int k = 0; k < 3; ++k)
            if (sum[k] < best[k]) { best[k] = sum[k]; pick[k] = c; }
    }
    sgi_set_block_shape(v.ctx, SGI_BLOCK_DIRECT, kShapes[pick[0]][0], kShapes[pick[0]][1]);
    sgi_set_block_shape(v.ctx, SGI_BLOCK_GATHER, kShapes[pick[1]][0], kShapes[pick[1]][1]);
    sgi_set_block_shape(v.ctx, SGI_BLOCK_ATROUS, kShapes[pick[2]][0], kShapes[pick[2]][1]);
    sgi_set_block_shape(v.ctx, SGI_BLOCK_DENOISE_FINAL, kShapes[pick[2]][0], kShapes[pick[2]][1]);
    sgi_set_timing(v.ctx, timing ? 1 : 0);
    return SGI_OK;
}

// One frame of every view captured on `s` (a non-default stream) into an executable graph.
sgi_status capture(sgi_batch* b, cudaStream_t s, cudaGraphExec_t* exec, int64_t* kernels) {
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return bfail(b, SGI_ERR_CUDA, std::string("begin capture: ") + cudaGetErrorString(e));
    sgi_status st = SGI_OK;
    for (const sgi_view& v : b->views) {
        st = render(v, b->net, s);
        if (st != SGI_OK) {
            b->err = std::string("captured frame: ") + sgi_last_error(v.ctx);
            break;
        }
    }
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(s, &g);
    if (st != SGI_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return bfail(b, SGI_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e));
    size_t n = 0;
    cudaGraphGetNodes(g, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) cudaGraphGetNodes(g, nodes.data(), &n);
    int64_t k = 0;
    for (cudaGraphNode_t node : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(node, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    *kernels = k;
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, SGI_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    return SGI_OK;
}

void release(sgi_batch* b) {
    for (auto& x : b->exec)
        if (x) cudaGraphExecDestroy(x);
    b->exec[0] = b->exec[1] = nullptr;
    void* bufs[] = {b->d_views, b->d_items, b->d_counts, b->d_queue, b->d_status, b->d_skip, b->d_wait};
    for (void* p : bufs)
        if (p) cudaFree(p);
    for (void* p : b->scratch)
        if (p) cudaFree(p);
    b->scratch.clear();
    b->d_views = nullptr; b->d_items = nullptr; b->d_counts = nullptr; b->d_queue = nullptr;
    b->d_status = nullptr; b->d_skip = nullptr; b->d_wait = nullptr;
}

// ---------------------------------------------------------- persistent mode --
sgi_status pcheck(sgi_batch* b, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return SGI_OK;
    return bfail(b, e == cudaErrorMemoryAllocation ? SGI_ERR_OOM : SGI_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

// One persistent launch of plan p on s.
cudaError_t persistent_launch(sgi_batch* b, int p, int variant, int grid, cudaStream_t s) {
    return b->fast ? sgi::fast::launch_persistent(b->plan[p], variant, grid, b->smem, s)
                   : sgi::exact::launch_persistent(b->plan[p], variant, grid, b->smem, s);
}

// The view's passes as the persistent kernel reads them, for history parity `parity`
// (0: the context's current history slot is the previous frame's, as in sgi_render_frame).
sgi::PViewDesc view_desc(const sgi_view& v, uint2** pass_buf, int parity) {
    const sgi_ctx* c = v.ctx;
    sgi::PViewDesc d;
    std::memset(&d, 0, sizeof(d));
    d.cfg = c->cfg;
    d.sc = c->sc;
    d.vpls = c->vpls; d.entries = c->entries; d.num_vpls = c->num_vpls;
    d.csm = c->csm; d.cubes = c->cubes;
    d.points = c->points; d.num_points = c->num_points;
    d.casters = c->shadow_points; d.caster_entries = c->shadow_entries; d.num_casters = c->num_shadow_points;
    d.caster_atlas = c->shadow_atlas;
    d.flags = c->flags; d.cv = c->cv; d.ce = c->ce; d.visible_index = c->visible_index; d.vpr = c->vpr;
    d.stage1 = c->stage1; d.lists = c->lists;
    d.cur = *v.cur; d.cam = *v.cam; d.prev = *v.prev;
    d.params = v.params;
    d.guide = c->guide;
    d.raw = c->cfg.debug_keep_passes ? c->reservoir : nullptr;
    for (int k = 0; k < c->cfg.denoise_passes; ++k) d.pass_buf[k] = pass_buf[k];
    d.direct = c->direct;
    const int cur = parity == 0 ? c->hist_cur : 1 - c->hist_cur;
    d.gi_prev = c->gi_hist[cur]; d.gi_out = c->gi_hist[1 - cur];
    d.hist_prev = c->hist_depth[cur]; d.hist_out = c->hist_depth[1 - cur];
    d.hdr_out = v.hdr_out;
    d.atrous_staged = v.ctx->atrous_staged ? 1 : 0;
    return d;
}

sgi_status build_persistent(sgi_batch* b, int32_t tune_frames, cudaStream_t s) {
    const int n = (int)b->views.size();
    const int vb = b->fast ? sgi::fast::persistent_view_bytes() : sgi::exact::persistent_view_bytes();
    std::vector<unsigned char> host_views((size_t)2 * n * vb, 0);
    std::vector<int32_t> counts((size_t)n * sgi::kPMaxLevels, 0);
    std::vector<uint32_t> items;
    int32_t max_visible = 1;
    for (int i = 0; i < n; ++i) {
        const sgi_view& v = b->views[i];
        const sgi_config& cfg = v.ctx->cfg;
        uint2* pass_buf[SGI_MAX_DENOISE_PASSES] = {};
        for (int k = 0; k < cfg.denoise_passes; ++k) {
            void* p = nullptr;
            sgi_status st = pcheck(b, cudaMalloc(&p, sizeof(uint2) * (size_t)cfg.width * cfg.height), "pass buffers");
            if (st != SGI_OK) return st;
            b->scratch.push_back(p);
            pass_buf[k] = (uint2*)p;
        }
        for (int parity = 0; parity < 2; ++parity) {
            const sgi::PViewDesc d = view_desc(v, pass_buf, parity);
            unsigned char* out = host_views.data() + ((size_t)parity * n + i) * vb;
            const bool filled = b->fast ? sgi::fast::persistent_fill_view(d, out) : sgi::exact::persistent_fill_view(d, out);
            if (!filled) return bfail(b, SGI_ERR_CUDA, "tensor maps of the staged a-trous passes");
        }
        const int blocks = ((cfg.width + 15) / 16) * ((cfg.height + 15) / 16);
        const int chunks = (blocks + sgi::kPBlocksPerItem - 1) / sgi::kPBlocksPerItem;
        int32_t* c = counts.data() + (size_t)i * sgi::kPMaxLevels;
        c[sgi::kPVis] = (v.ctx->num_vpls + 255) / 256;
        c[sgi::kPCompact] = 1;
        c[sgi::kPDirect] = chunks;
        c[sgi::kPTile] = chunks;
        c[sgi::kPGather] = chunks;
        for (int pass = 1; pass < cfg.denoise_passes; ++pass) {
            // staged a-trous passes (1..3, the context's staging on, even width) have lattice CTAs as items
            int gx, gy, ntx, nty;
            const int lat = pass < cfg.denoise_passes - 1 && v.ctx->atrous_staged
                                ? sgi::atrous_lattice_grid(cfg.width, cfg.height, pass, &gx, &gy, &ntx, &nty)
                                : 0;
            c[sgi::kPAtrous + pass - 1] = lat > 0 ? (lat + sgi::kPBlocksPerItem - 1) / sgi::kPBlocksPerItem : chunks;
        }
        if (cfg.max_visible > max_visible) max_visible = cfg.max_visible;
    }
    // dispatch order: pass by pass, every view's items of a pass before the next pass
    const int levels[] = {sgi::kPVis, sgi::kPCompact, sgi::kPDirect, sgi::kPTile, sgi::kPGather};
    for (int level : levels)
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < counts[(size_t)i * sgi::kPMaxLevels + level]; ++k) items.push_back(sgi::pitem(i, level, k));
    for (int level = sgi::kPAtrous; level < sgi::kPMaxLevels; ++level)
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < counts[(size_t)i * sgi::kPMaxLevels + level]; ++k) items.push_back(sgi::pitem(i, level, k));
    sgi_status st = SGI_OK;
    if ((st = pcheck(b, cudaMalloc(&b->d_views, host_views.size()), "views")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMalloc(&b->d_items, sizeof(uint32_t) * items.size()), "items")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMalloc(&b->d_counts, sizeof(int32_t) * counts.size()), "counts")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMalloc(&b->d_queue, sizeof(sgi::PQueue)), "queue")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMalloc(&b->d_status, sizeof(int32_t)), "status")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMalloc(&b->d_skip, sizeof(int32_t) * counts.size()), "skip")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMalloc(&b->d_wait, sizeof(long long)), "wait limit")) != SGI_OK) return st;
    const long long wait_default = 1000000000ll;   // 1 s
    if ((st = pcheck(b, cudaMemcpyAsync(b->d_wait, &wait_default, sizeof(long long), cudaMemcpyHostToDevice, s),
                     "wait limit")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMemcpyAsync(b->d_views, host_views.data(), host_views.size(), cudaMemcpyHostToDevice, s),
                     "views")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMemcpyAsync(b->d_items, items.data(), sizeof(uint32_t) * items.size(),
                                        cudaMemcpyHostToDevice, s), "items")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMemcpyAsync(b->d_counts, counts.data(), sizeof(int32_t) * counts.size(),
                                        cudaMemcpyHostToDevice, s), "counts")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMemsetAsync(b->d_queue, 0, sizeof(sgi::PQueue), s), "queue")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMemsetAsync(b->d_status, 0, sizeof(int32_t), s), "status")) != SGI_OK) return st;
    if ((st = pcheck(b, cudaMemsetAsync(b->d_skip, 0, sizeof(int32_t) * counts.size(), s), "skip")) != SGI_OK) return st;
    for (int p = 0; p < 2; ++p) {
        sgi::PPlan& pl = b->plan[p];
        pl.items = b->d_items; pl.num_items = (int32_t)items.size(); pl.num_views = n;
        pl.counts = b->d_counts; pl.q = b->d_queue; pl.status = b->d_status; pl.skip = b->d_skip;
        pl.wait_ns = b->d_wait;
        pl.views = b->d_views + (size_t)p * n * vb;
        pl.view_bytes = vb;
    }
    b->smem = b->fast ? sgi::fast::persistent_smem(max_visible) : sgi::exact::persistent_smem(max_visible);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm[2] = {0, 0};
    for (int var = 0; var < 2; ++var) {
        cudaError_t e = b->fast ? sgi::fast::persistent_occupancy(var, b->smem, &per_sm[var])
                                : sgi::exact::persistent_occupancy(var, b->smem, &per_sm[var]);
        if ((st = pcheck(b, e, "occupancy")) != SGI_OK) return st;
    }
    if (per_sm[0] < 1) return bfail(b, SGI_ERR_CUDA, "the persistent kernel does not fit on an SM");
    // register budget (64 or 128 per thread) and CTAs per SM: without tuning, 64 registers and the most CTAs
    // that fit; with tuning, every pair is timed over tune_frames launches and the fastest is kept
    b->variant = 0;
    b->grid = per_sm[0] * sms;
    cudaError_t e = cudaSuccess;
    if (tune_frames > 0) {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = 1e30f;
        for (int var = 0; var < 2 && st == SGI_OK; ++var) {
            for (int c = 1; c <= per_sm[var]; ++c) {
                float total = 0.0f;
                for (int f = 0; f < tune_frames + 1; ++f) {
                    cudaEventRecord(e0, s);
                    e = persistent_launch(b, b->next, var, c * sms, s);
                    cudaEventRecord(e1, s);
                    b->next ^= 1;
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    if (e != cudaSuccess) break;
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (f > 0) total += ms;
                }
                if ((st = pcheck(b, e, "tuning launch")) != SGI_OK) break;
                if (total < best) { best = total; b->variant = var; b->grid = c * sms; }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (st != SGI_OK) return st;
        int32_t status = 0;
        if ((st = pcheck(b, cudaMemcpy(&status, b->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost), "status")) !=
            SGI_OK) return st;
        if (status != SGI_OK) return bfail(b, status, "a tuning launch gave up waiting");
    }
    // one graph per history parity, each holding the single kernel launch
    for (int p = 0; p < 2; ++p) {
        const int par = (b->next + p) & 1;
        e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            cudaError_t le = persistent_launch(b, par, b->variant, b->grid, s);
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(s, &g);
            if (e == cudaSuccess) e = le;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec[par], g, 0);
            if (g) cudaGraphDestroy(g);
        }
        if ((st = pcheck(b, e, "capture")) != SGI_OK) return st;
    }
    b->kernels = 1;
    return SGI_OK;
}

}  // namespace

extern "C" {

sgi_status sgi_batch_create(const sgi_view* views, int32_t num_views, sgi_nn* net, int32_t tune_frames,
                            void* stream, sgi_batch** out) {
    if (!views || num_views < 1 || !out || tune_frames < 0 || tune_frames > 64) return SGI_ERR_ARG;
    for (int i = 0; i < num_views; ++i) {
        const sgi_view& v = views[i];
        if (!v.ctx || !v.cur || !v.prev || !v.cam || !v.hdr_out) return SGI_ERR_ARG;
        if (!v.ctx->have_history) return SGI_ERR_STATE;   // render one frame of every view first
    }
    sgi_batch* b = new (std::nothrow) sgi_batch;
    if (!b) return SGI_ERR_OOM;
    b->views.assign(views, views + num_views);
    b->net = net;
    cudaStream_t user = (cudaStream_t)stream;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamSynchronize(user);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete b;
        return SGI_ERR_CUDA;
    }
    sgi_status st = SGI_OK;
    if (tune_frames > 0)
        for (const sgi_view& v : b->views)
            if ((st = tune(b, v, tune_frames, s)) != SGI_OK) break;
    // two graphs: the first captures the current history parity, the second the other
    int64_t k0 = 0, k1 = 0;
    if (st == SGI_OK) st = capture(b, s, &b->exec[0], &k0);
    if (st == SGI_OK) st = capture(b, s, &b->exec[1], &k1);
    b->kernels = k0;
    e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (st == SGI_OK && e != cudaSuccess) st = bfail(b, SGI_ERR_CUDA, cudaGetErrorString(e));
    if (st != SGI_OK) {
        release(b);
        delete b;
        return st;
    }
    *out = b;
    return SGI_OK;
}

sgi_status sgi_batch_create_persistent(const sgi_view* views, int32_t num_views, int32_t tune_frames, void* stream,
                                       sgi_batch** out) {
    if (!views || num_views < 1 || num_views > sgi::kPMaxViews || !out || tune_frames < 0 || tune_frames > 64)
        return SGI_ERR_ARG;
    *out = nullptr;
    const bool fast = views[0].ctx && views[0].ctx->fast_shading;
    for (int i = 0; i < num_views; ++i) {
        const sgi_view& v = views[i];
        if (!v.ctx || !v.cur || !v.prev || !v.cam || !v.hdr_out) return SGI_ERR_ARG;
        const sgi_ctx* c = v.ctx;
        if (c->cfg.gi_mode != SGI_GI_TILED || c->cfg.tile_size != 16 || c->coloring || c->fast_shading != fast)
            return SGI_ERR_ARG;   // tiled mode with 16x16 tiles, no VPL colouring, one shading mode
        if (!c->have_history || !c->lights_set || !c->maps_set) return SGI_ERR_STATE;
        if (v.params.frames_per_second <= 0.0f) return SGI_ERR_ARG;
    }
    sgi_batch* b = new (std::nothrow) sgi_batch;
    if (!b) return SGI_ERR_OOM;
    b->views.assign(views, views + num_views);
    b->persistent = true;
    b->fast = fast;
    cudaStream_t user = (cudaStream_t)stream;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamSynchronize(user);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete b;
        return SGI_ERR_CUDA;
    }
    sgi_status st = build_persistent(b, tune_frames, s);
    e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (st == SGI_OK && e != cudaSuccess) st = bfail(b, SGI_ERR_CUDA, cudaGetErrorString(e));
    if (st != SGI_OK) {
        // keep the message for the caller? the batch is gone: report through the status only
        release(b);
        delete b;
        return st;
    }
    *out = b;
    return SGI_OK;
}

sgi_status sgi_batch_persistent_shape(const sgi_batch* b, int32_t* registers, int32_t* ctas) {
    if (!b || !b->persistent || !registers || !ctas) return SGI_ERR_ARG;
    *registers = b->variant == 0 ? 64 : 128;
    *ctas = b->grid;
    return SGI_OK;
}

sgi_status sgi_batch_status(sgi_batch* b) {
    if (!b) return SGI_ERR_ARG;
    if (!b->persistent) return SGI_OK;
    int32_t status = 0;
    if (cudaMemcpy(&status, b->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        return bfail(b, SGI_ERR_CUDA, "status read");
    if (status != SGI_OK) {
        cudaMemset(b->d_status, 0, sizeof(int32_t));
        cudaDeviceSynchronize();
        return bfail(b, status, "a persistent launch gave up waiting for a pass (SGI_ERR_TIMEOUT)");
    }
    return SGI_OK;
}

sgi_status sgi_batch_set_wait_limit(sgi_batch* b, int64_t nanoseconds) {
    if (!b || !b->persistent || nanoseconds < 1000 || nanoseconds > 60000000000ll) return SGI_ERR_ARG;
    const long long ns = nanoseconds;
    if (cudaMemcpy(b->d_wait, &ns, sizeof(long long), cudaMemcpyHostToDevice) != cudaSuccess)
        return bfail(b, SGI_ERR_CUDA, "wait limit");
    return SGI_OK;
}

sgi_status sgi_batch_skip_pass(sgi_batch* b, int32_t view, int32_t level, int32_t skip) {
    if (!b || !b->persistent || view < 0 || view >= (int32_t)b->views.size() || level < 0 ||
        level >= sgi::kPMaxLevels)
        return SGI_ERR_ARG;
    const int32_t v = skip ? 1 : 0;
    if (cudaMemcpy(b->d_skip + (size_t)view * sgi::kPMaxLevels + level, &v, sizeof(int32_t),
                   cudaMemcpyHostToDevice) != cudaSuccess)
        return bfail(b, SGI_ERR_CUDA, "skip switch");
    return SGI_OK;
}

sgi_status sgi_batch_launch(sgi_batch* b, void* stream) {
    if (!b || !b->exec[b->next]) return SGI_ERR_ARG;
    cudaError_t e = cudaGraphLaunch(b->exec[b->next], (cudaStream_t)stream);
    if (e != cudaSuccess) return bfail(b, SGI_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    b->next ^= 1;
    return SGI_OK;
}

int64_t sgi_batch_kernel_count(const sgi_batch* b) { return b ? b->kernels : 0; }

sgi_status sgi_batch_destroy(sgi_batch* b) {
    if (!b) return SGI_ERR_ARG;
    // the capture left each context on the parity of graph 0; after an odd
    // number of replays the history the device holds is the other one
    if (b->next == 1)
        for (const sgi_view& v : b->views) v.ctx->hist_cur = 1 - v.ctx->hist_cur;
    release(b);
    delete b;
    return SGI_OK;
}

const char* sgi_batch_last_error(const sgi_batch* b) { return b ? b->err.c_str() : "NULL batch"; }

}  // extern "C"
