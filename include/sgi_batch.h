/*
 * sgi_batch.h - many views of the GI stage replayed as one CUDA graph.
 *
 * No counterpart in StratusGFX, which renders one view per frame
 * (RendererBackend::RenderScene, StratusRendererBackend.cpp:2011-2045). A batch
 * holds n views, each an sgi_ctx sized for its own viewport with lights and
 * shadow maps set, plus the frame inputs it renders. sgi_batch_create can tune
 * every view's thread-block shapes (sgi_set_block_shape) by timing them, then
 * captures one frame of every view - sgi_render_frame, or
 * sgi_render_frame_neural when a network is given - into a CUDA graph;
 * sgi_batch_launch replays all views' culls, gathers, denoisers and
 * composites with one graph launch. Views run in order on the launching
 * stream (each view's direct lighting on its context's side stream), so one
 * network serves views of any size up to its capacity.
 */
#ifndef SGI_BATCH_H_
#define SGI_BATCH_H_

#include "sgi.h"
#include "sgi_nn.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgi_view {
    sgi_ctx* ctx;
    const sgi_gbuffer* cur;
    const sgi_gbuffer* prev;
    const sgi_camera* cam;
    sgi_frame_params params;
    void* hdr_out;            /* RGBA16F [height][width] of the view's context */
} sgi_view;

typedef struct sgi_batch sgi_batch;

/* Builds the batch (synchronises `stream`). Every view's context must already
 * have rendered one frame of the same kind (plain, or neural with `net`), so
 * that its history and scratch exist.
 *   tune_frames > 0: for every view and each candidate block shape (32x8,
 *     16x16, 64x4, 128x2, 8x32; results do not depend on the shape) renders
 *     tune_frames frames with per-pass timing and keeps, per pass, the shape
 *     of the smallest total time.
 * The graph fixes the frame inputs (G-buffers, camera, frame parameters):
 * every replay renders the same frame of each view and advances its history.
 * Two graphs alternate between the history buffers. While the batch exists the
 * contexts must not be driven by other calls; sgi_batch_destroy leaves their
 * host state matching the history the replays wrote. */
sgi_status sgi_batch_create(const sgi_view* views, int32_t num_views, sgi_nn* net, int32_t tune_frames,
                            void* stream, sgi_batch** out);
/* One frame of every view: a single CUDA graph launch on `stream`. */
sgi_status sgi_batch_launch(sgi_batch* batch, void* stream);
/* Kernel nodes of one replay (the kernel launches it performs). */
int64_t sgi_batch_kernel_count(const sgi_batch* batch);
sgi_status sgi_batch_destroy(sgi_batch* batch);
const char* sgi_batch_last_error(const sgi_batch* batch);

#ifdef __cplusplus
}
#endif

#endif /* SGI_BATCH_H_ */
