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
/* The same batch as ONE persistent kernel per frame (no counterpart in
 * StratusGFX): plain frames (sgi_render_frame's passes, in the context's
 * shading precision) of up to 256 views, each in tiled mode with 16x16 tiles
 * and without VPL colouring, all in one shading precision. A grid of
 * persistent 256-thread CTAs - as many as fit on the GPU at once, or with
 * tune_frames > 0 the fastest CTA count per SM over tune_frames launches -
 * takes work items from a device queue in pass order: per view the VPL
 * visibility flags (256 VPLs an item), the stable compaction, the direct
 * lighting, per 16x16 tile the mean and VPL list, the gather (the tile's list
 * staged in shared memory) and each denoise pass (one 16x16 block an item).
 * An item waits, on the GPU, until the passes it depends on are complete for
 * its view; every wait gives up after the batch's wait limit (1 s unless
 * sgi_batch_set_wait_limit says otherwise), which sets SGI_ERR_TIMEOUT for
 * sgi_batch_status and ends the launch early (no later item runs). The launch
 * is captured in a CUDA graph (one kernel node; two graphs alternate between
 * the history buffers) and replayed by sgi_batch_launch. Results are those of
 * sgi_render_frame on each view, bit for bit in the exact precision. Each view
 * gets its own denoise pass buffers (width x height x 8 bytes per pass). */
sgi_status sgi_batch_create_persistent(const sgi_view* views, int32_t num_views, int32_t tune_frames, void* stream,
                                       sgi_batch** out);
/* The shape the persistent batch launches with: registers per thread the
 * kernel is built for (64 or 128) and the number of CTAs. */
sgi_status sgi_batch_persistent_shape(const sgi_batch* batch, int32_t* registers, int32_t* ctas);
/* SGI_OK, or the status a persistent launch set (SGI_ERR_TIMEOUT when a wait
 * gave up); reading it clears it. Synchronous. SGI_OK for graph batches. */
sgi_status sgi_batch_status(sgi_batch* batch);
/* The limit of every wait of a persistent batch, in nanoseconds (1e3 .. 6e10). */
sgi_status sgi_batch_set_wait_limit(sgi_batch* batch, int64_t nanoseconds);
/* Test switch of a persistent batch: while set, the items of pass `level` of
 * view `view` do nothing and are never counted done, so the passes after it
 * wait until the limit. Levels: 0 visibility flags, 1 compaction, 2 direct
 * lighting, 3 tile lists, 4 gather, 5 + k the (k + 1)-th denoise pass after the
 * gather's. Synchronous. */
sgi_status sgi_batch_skip_pass(sgi_batch* batch, int32_t view, int32_t level, int32_t skip);

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
