"""Block shapes of the per-pixel passes and the multi-view CUDA graph batch.

Every thread-block shape computes each pixel with the same arithmetic, so frames
rendered with any shape must be bit-identical; a batch replay must produce the
same frames, bit for bit, as rendering each view in turn through the C ABI the
same number of times (the captured launches are the same kernels with the same
arguments), and its host state must stay in step with the history it wrote.
"""
import ctypes as C

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from stratusgfx_gb300 import abi, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402
from stratusgfx_gb300.denoiser import KpcnDenoiser  # noqa: E402

SHAPES = [(32, 8), (16, 16), (64, 4), (128, 2), (8, 32)]


def view_scene(W, H, seed, K=4):
    w = S.Workload(f"room12_{W}x{H}", W, H, 12, 48, 2, 512, 32, abi.SGI_CUBE_F16, K, 5, 2)
    return w, stage.DeviceScene(S.workload_scene(w, seed), w)


class View:
    """One view: a context with lights and maps set, frame 1 of its scene."""

    def __init__(self, w, ds):
        self.w, self.ds = w, ds
        self.st = stage.GiStage(stage.workload_config(w))
        self.st.set_lights(ds.vpls, ds.entries, ds.points)
        self.st.set_shadow_maps(ds.csms[1], ds.cubes)
        self.out = torch.zeros((w.height, w.width, 4), dtype=torch.float16, device="cuda")
        self.cur, self.prev = ds.gbuffers[1].struct(), ds.gbuffers[0].struct()
        self.cam = ds.camera(1)
        self.params = abi.FrameParams(1016.0, 60.0)

    def frame(self, net=None):
        lib = self.st.lib
        if net is None:
            st = lib.sgi_render_frame(self.st.ctx, C.byref(self.cur), C.byref(self.prev), C.byref(self.cam),
                                      C.byref(self.params), C.c_void_p(self.out.data_ptr()), None)
        else:
            st = lib.sgi_render_frame_neural(self.st.ctx, net.h, C.byref(self.cur), C.byref(self.prev),
                                             C.byref(self.cam), C.byref(self.params),
                                             C.c_void_p(self.out.data_ptr()), None)
        abi.check(st, self.st.ctx)

    def struct(self):
        return abi.View(self.st.ctx.value, C.addressof(self.cur), C.addressof(self.prev), C.addressof(self.cam),
                        self.params, self.out.data_ptr())


def test_block_shapes_are_bit_identical():
    w, ds = view_scene(200, 120, 71)
    ref = View(w, ds)
    for _ in range(3):
        ref.frame()
    torch.cuda.synchronize()
    lib = abi.load()
    for bx, by in SHAPES:
        v = View(w, ds)
        for p in range(4):
            assert lib.sgi_set_block_shape(v.st.ctx, p, bx, by) == abi.SGI_OK
        for _ in range(3):
            v.frame()
        torch.cuda.synchronize()
        assert torch.equal(v.out.view(torch.int16), ref.out.view(torch.int16)), (bx, by)
        v.st.close()
    gx, gy = C.c_int32(), C.c_int32()
    assert lib.sgi_get_block_shape(ref.st.ctx, abi.SGI_BLOCK_GATHER, C.byref(gx), C.byref(gy)) == abi.SGI_OK
    assert (gx.value, gy.value) == (0, 0)
    for bad in ((16, 8), (12, 21), (256, 2), (4, 64)):
        assert lib.sgi_set_block_shape(ref.st.ctx, 0, *bad) == abi.SGI_ERR_ARG
    assert lib.sgi_set_block_shape(ref.st.ctx, 4, 32, 8) == abi.SGI_ERR_ARG


def run_batch(net, tune):
    lib = abi.load()
    sizes = [(96, 64, 11), (160, 96, 12), (64, 64, 13)]
    scenes = [view_scene(W, H, seed) for W, H, seed in sizes]
    seq = [View(w, ds) for w, ds in scenes]
    bat = [View(w, ds) for w, ds in scenes]
    for v in seq + bat:
        v.frame(net)            # history and scratch exist before the capture
    arr = (abi.View * len(bat))(*[v.struct() for v in bat])
    h = C.c_void_p()
    st = lib.sgi_batch_create(arr, len(bat), net.h if net else None, tune, None, C.byref(h))
    assert st == abi.SGI_OK, lib.sgi_batch_last_error(h)
    # per view: the one-launch VPL cull, direct lighting, tile means, tile cull, gather, then 3 a-trous passes
    # and the final pass (plain: 9) or the features and the network's 13 launches (neural: 19)
    assert lib.sgi_batch_kernel_count(h) >= 3 * (19 if net else 9)
    tuned_frames = 5 * (tune + 1) if tune else 0
    for v in seq:
        for _ in range(tuned_frames):
            v.frame(net)
    for _ in range(3):
        assert lib.sgi_batch_launch(h, None) == abi.SGI_OK
    for v in seq:
        for _ in range(3):
            v.frame(net)
    torch.cuda.synchronize()
    for a, b in zip(seq, bat):
        assert torch.equal(a.out.view(torch.int16), b.out.view(torch.int16)), a.w.name
    # an odd number of replays: destroy puts the host state on the history the replays wrote
    assert lib.sgi_batch_destroy(h) == abi.SGI_OK
    for v in seq + bat:
        v.frame(net)
    torch.cuda.synchronize()
    for a, b in zip(seq, bat):
        assert torch.equal(a.out.view(torch.int16), b.out.view(torch.int16)), a.w.name
    for v in seq + bat:
        v.st.close()


def test_batch_replay_matches_per_view_frames_plain():
    run_batch(None, tune=1)


def test_batch_replay_matches_per_view_frames_neural():
    net = KpcnDenoiser(1, 96, 160, seed=5)
    try:
        run_batch(net, tune=0)
    finally:
        net.close()


def test_batch_create_rejects_views_without_a_first_frame():
    lib = abi.load()
    w, ds = view_scene(64, 64, 21)
    v = View(w, ds)
    arr = (abi.View * 1)(v.struct())
    h = C.c_void_p()
    assert lib.sgi_batch_create(arr, 1, None, 0, None, C.byref(h)) == abi.SGI_ERR_STATE
    assert lib.sgi_batch_create(arr, 0, None, 0, None, C.byref(h)) == abi.SGI_ERR_ARG
    v.st.close()


def run_persistent(fast=False):
    """The persistent batch (one kernel per frame over all views' passes) against each view rendered in turn:
    bit for bit in the exact precision; in the tolerance precision within its 1e-3 relative error (the two
    kernels may fuse multiply-adds differently)."""
    lib = abi.load()
    sizes = [(96, 64, 11), (160, 96, 12), (64, 64, 13), (200, 120, 14)]
    scenes = [view_scene(W, H, seed) for W, H, seed in sizes]
    seq = [View(w, ds) for w, ds in scenes]
    bat = [View(w, ds) for w, ds in scenes]
    for v in seq + bat:
        if fast:
            assert lib.sgi_set_shading_precision(v.st.ctx, abi.SGI_SHADING_FAST) == abi.SGI_OK
        v.frame()
    arr = (abi.View * len(bat))(*[v.struct() for v in bat])
    h = C.c_void_p()
    st = lib.sgi_batch_create_persistent(arr, len(bat), 0, None, C.byref(h))
    assert st == abi.SGI_OK, lib.sgi_batch_last_error(h)
    assert lib.sgi_batch_kernel_count(h) == 1

    def compare():
        for a, b in zip(seq, bat):
            if fast:
                x, y = a.out.float(), b.out.float()
                rel = ((x - y).abs() / y.abs().clamp(min=2.0 ** -14)).max().item()
                assert rel <= 1e-3, (a.w.name, rel)
            else:
                assert torch.equal(a.out.view(torch.int16), b.out.view(torch.int16)), a.w.name

    for _ in range(3):
        assert lib.sgi_batch_launch(h, None) == abi.SGI_OK
    for v in seq:
        for _ in range(3):
            v.frame()
    torch.cuda.synchronize()
    assert lib.sgi_batch_status(h) == abi.SGI_OK
    compare()
    assert lib.sgi_batch_destroy(h) == abi.SGI_OK
    for v in seq + bat:
        v.frame()
    torch.cuda.synchronize()
    compare()
    for v in seq + bat:
        v.st.close()


def test_persistent_batch_matches_per_view_frames():
    run_persistent(fast=False)


def test_persistent_batch_in_the_tolerance_precision():
    run_persistent(fast=True)


def test_persistent_batch_views_bit_exact_against_the_oracle():
    """The persistent kernel's views against the FP32 oracle directly: each view renders its first frame
    through the C ABI, then one launch of the persistent batch renders the next; the oracle runs the same
    two frames (the second reading the first's history) and every view's HDR output must equal it."""
    import numpy as np

    from helpers import assert_bit_exact, host_scene_from_device
    from oracle import binding as O
    lib = abi.load()
    sizes = [(96, 64, 51), (160, 96, 52), (200, 120, 53)]
    views = [View(*view_scene(W, H, seed)) for W, H, seed in sizes]
    for v in views:
        v.frame()
    arr = (abi.View * len(views))(*[v.struct() for v in views])
    h = C.c_void_p()
    assert lib.sgi_batch_create_persistent(arr, len(views), 0, None, C.byref(h)) == abi.SGI_OK
    assert lib.sgi_batch_launch(h, None) == abi.SGI_OK
    torch.cuda.synchronize()
    assert lib.sgi_batch_status(h) == abi.SGI_OK
    for v in views:
        w = v.w
        hs = host_scene_from_device(v.ds, (0, 1))
        cfg = stage.workload_config(w)
        gi = np.zeros((w.height, w.width, 4), np.float32)
        hist = np.zeros((w.height, w.width), np.float32)
        for _ in range(2):
            ref = O.frame(32, cfg, hs, 1, gi, hist, v.params.time, v.params.frames_per_second)
            gi, hist = ref["gi"], ref["hist"]
        got = v.out.cpu().numpy().astype(np.float32)[..., :3]
        assert_bit_exact(got, ref["combined"][..., :3], f"{w.name}: persistent batch frame")
    assert lib.sgi_batch_destroy(h) == abi.SGI_OK
    for v in views:
        v.st.close()


def test_persistent_batch_wait_gives_up_and_the_next_launch_succeeds():
    """The test switch holds back view 0's VPL compaction: the tile passes that wait for it give up after the
    batch's 20 ms limit, the launch ends with SGI_ERR_TIMEOUT, and with the switch cleared the next launch
    completes (status OK, every view's output finite)."""
    lib = abi.load()
    views = [View(*view_scene(W, H, seed)) for W, H, seed in ((96, 64, 31), (128, 96, 32))]
    for v in views:
        v.frame()
    arr = (abi.View * 2)(*[v.struct() for v in views])
    h = C.c_void_p()
    assert lib.sgi_batch_create_persistent(arr, 2, 2, None, C.byref(h)) == abi.SGI_OK   # tuned CTA count
    assert lib.sgi_batch_set_wait_limit(h, 20_000_000) == abi.SGI_OK
    assert lib.sgi_batch_skip_pass(h, 0, 1, 1) == abi.SGI_OK
    assert lib.sgi_batch_launch(h, None) == abi.SGI_OK
    torch.cuda.synchronize()
    assert lib.sgi_batch_status(h) == abi.SGI_ERR_TIMEOUT
    assert b"gave up" in lib.sgi_batch_last_error(h)
    assert lib.sgi_batch_skip_pass(h, 0, 1, 0) == abi.SGI_OK
    for _ in range(2):
        assert lib.sgi_batch_launch(h, None) == abi.SGI_OK
    torch.cuda.synchronize()
    assert lib.sgi_batch_status(h) == abi.SGI_OK
    for v in views:
        assert torch.isfinite(v.out.float()).all()
    assert lib.sgi_batch_skip_pass(h, 2, 1, 1) == abi.SGI_ERR_ARG
    assert lib.sgi_batch_destroy(h) == abi.SGI_OK
    for v in views:
        v.st.close()


def test_persistent_batch_rejects_unsupported_views():
    lib = abi.load()
    w, ds = view_scene(64, 64, 41)
    v = View(w, ds)
    arr = (abi.View * 1)(v.struct())
    h = C.c_void_p()
    assert lib.sgi_batch_create_persistent(arr, 1, 0, None, C.byref(h)) == abi.SGI_ERR_STATE   # no first frame
    v.frame()
    assert lib.sgi_batch_create_persistent(arr, 257, 0, None, C.byref(h)) == abi.SGI_ERR_ARG
    w8 = S.Workload("room12_64x64_t8", 64, 64, 12, 48, 2, 512, 32, abi.SGI_CUBE_F16, 4, 5, 2, tile_size=8)
    v8 = View(w8, stage.DeviceScene(S.workload_scene(w8, 42), w8))
    v8.frame()
    arr8 = (abi.View * 1)(v8.struct())
    assert lib.sgi_batch_create_persistent(arr8, 1, 0, None, C.byref(h)) == abi.SGI_ERR_ARG   # 8x8 tiles
    v.st.close()
    v8.st.close()


def test_tuner_choices_are_cached_per_viewport(tmp_path):
    """stratusgfx_gb300.tuning: the first batch tunes and records every view's block shapes by viewport; a
    second batch of views with those viewports applies them and builds without tuning."""
    from stratusgfx_gb300 import tuning
    lib = abi.load()
    cache = str(tmp_path / "shapes.json")
    sizes = [(96, 64, 51), (160, 96, 52)]
    runs = []
    for _ in range(2):
        views = [View(*view_scene(W, H, seed)) for W, H, seed in sizes]
        for v in views:
            v.frame()
        arr = (abi.View * len(views))(*[v.struct() for v in views])
        h, tuned = tuning.create_batch(arr, [(v.w.width, v.w.height) for v in views], cache=cache, tune_frames=1)
        assert lib.sgi_batch_launch(h, None) == abi.SGI_OK
        torch.cuda.synchronize()
        runs.append((tuned, views, h))
    assert runs[0][0] and not runs[1][0]
    import json
    entries = json.load(open(cache))
    assert set(entries) == {"96x64:plain", "160x96:plain"}
    gx, gy = C.c_int32(), C.c_int32()
    for v in runs[1][1]:
        lib.sgi_get_block_shape(v.st.ctx, abi.SGI_BLOCK_GATHER, C.byref(gx), C.byref(gy))
        assert [gx.value, gy.value] == entries[f"{v.w.width}x{v.w.height}:plain"]["gather"]
    for _, views, h in runs:
        assert lib.sgi_batch_destroy(h) == abi.SGI_OK
        for v in views:
            v.st.close()
