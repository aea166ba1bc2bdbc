// sgi_batch.cpp - C ABI of include/sgi_batch.h: block-shape autotuning and CUDA
// graph capture of one frame of many views.
#include <cuda_runtime.h>

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
};

namespace {

constexpr int kShapes[5][2] = {{32, 8}, {16, 16}, {64, 4}, {128, 2}, {8, 32}};

sgi_status bfail(sgi_batch* b, sgi_status s, const std::string& msg) {
    if (b) b->err = msg;
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
