"""Parity of every CUDA pass with the FP32 oracle, through the C ABI (libsgi.so).

Inputs are produced once by the oracle's CPU ray caster and uploaded, so the
kernels and the oracle see identical bytes. Both evaluate the same binary32
expression trees without FMA contraction, so the expected result is bit-exact;
each test asserts exact equality (NaN == NaN) and, as the stated tolerance of
the FP32 path, a max relative error <= 1e-3 is implied by it.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import GpuSetup, assert_bit_exact, half4_to_f32, half_bits_equal, psnr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402

TIME = 1000.0
FPS = 60.0


Setup = GpuSetup


@pytest.fixture(scope="module")
def small():
    return Setup(S.SMALL, 1235, debug_keep_passes=1)


def test_scene_generator_matches_cpu_raycaster(small):
    lib = abi.load()
    sc, w = small.sc, small.w
    boxes = torch.from_numpy(sc.boxes).cuda()
    for k in range(len(sc.cameras)):
        g = stage.GBufferTensors(w.height, w.width, "cuda")
        abi.check(lib.sgi_scene_gbuffer(C.c_void_p(boxes.data_ptr()), sc.boxes.shape[0],
                                        C.byref(stage.scene_camera_struct(sc, k)), w.width, w.height,
                                        C.byref(g.struct()), None))
        torch.cuda.synchronize()
        got = g.numpy()
        for name in O.HostGBuffer.NAMES:
            ref = getattr(small.hs.gbuffers[k], name)
            assert np.array_equal(got[name].view(np.uint8), ref.view(np.uint8)), f"gbuffer plane {name} frame {k}"
    # CSM
    d = torch.empty((4, w.csm_resolution, w.csm_resolution), dtype=torch.float32, device="cuda")
    cs = stage.csm_struct(sc, 1, d.data_ptr(), w.csm_resolution)
    abi.check(lib.sgi_scene_csm(C.c_void_p(boxes.data_ptr()), sc.boxes.shape[0], C.byref(cs),
                                C.byref(stage.inv_cascade_array(sc, 1)), None))
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy().view(np.uint32), small.hs.csm_depth[1].view(np.uint32))
    # cube atlas
    st = torch.zeros_like(small.cube_t)
    at = abi.CubeAtlas()
    for a in range(st.shape[0]):
        at.atlas[a] = st[a].data_ptr()
    at.num_atlases, at.layers_per_atlas, at.face_size, at.format = st.shape[0], 320, w.cube_size, w.cube_format
    abi.check(lib.sgi_scene_cube_atlas(C.c_void_p(boxes.data_ptr()), sc.boxes.shape[0],
                                       C.c_void_p(small.vpls.data_ptr()), C.c_void_p(small.entries.data_ptr()),
                                       sc.vpls.shape[0], C.byref(at), None))
    torch.cuda.synchronize()
    n = sc.vpls.shape[0]
    assert np.array_equal(st.cpu().numpy()[0, :n].view(np.uint32), small.hs.cube_storage[0, :n].view(np.uint32))


def _run_frame(s: Setup, k=1, **cfgkw):
    st, cfg = s.stage(k, **cfgkw)
    out = torch.empty((cfg.height, cfg.width, 4), dtype=torch.float16, device="cuda")
    st.render_frame(s.g[k], s.g[k - 1], s.hs.camera(k), out, TIME, FPS)
    torch.cuda.synchronize()
    return st, cfg, out


def test_vpl_visibility_cull_bit_exact(small):
    st, cfg, _ = _run_frame(small)
    n = small.sc.vpls.shape[0]
    got = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    ref = O.vis_cull(32, small.sc.vpls, small.hs.csms[1], cfg.max_visible)
    cnt = int(ref[0])
    assert got[0] == cnt
    assert np.array_equal(got[1:1 + cnt], ref[1:1 + cnt])
    cv = st.read_debug(abi.SGI_DEBUG_COMPACT_VPLS, np.float32).reshape(-1, 16)[:cnt]
    assert np.array_equal(cv.view(np.uint32), small.sc.vpls[ref[1:1 + cnt]].view(np.uint32))
    ce = st.read_debug(abi.SGI_DEBUG_COMPACT_ENTRIES, np.int32).reshape(-1, 2)[:cnt]
    assert np.array_equal(ce, small.sc.entries[ref[1:1 + cnt]])
    assert cnt <= n


def test_vpl_cull_with_shadowed_vpls_and_cap():
    """Half of the VPLs are moved under the floor (CSM-occluded); the cap truncates in index order."""
    w = S.Workload("room12_96x64_vpl200", 96, 64, 12, 200, 0, 512, 16, abi.SGI_CUBE_F32, 4, 3, 1)
    s = Setup(w, 77)
    v = s.sc.vpls.copy()
    v[1::2, 1] = -0.25          # inside the floor slab
    s.vpls = torch.from_numpy(v).cuda()
    for cap in (200, 37):
        st, cfg = s.stage(1, max_visible=cap)
        st.cull_vpls()
        torch.cuda.synchronize()
        got = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
        ref = O.vis_cull(32, v, s.hs.csms[1], cap)
        cnt = int(ref[0])
        assert got[0] == cnt and cnt <= cap
        assert np.array_equal(got[1:1 + cnt], ref[1:1 + cnt])
        assert np.all(np.diff(got[1:1 + cnt]) > 0)
        st.close()


def test_tile_cull_bit_exact(small):
    st, cfg, _ = _run_frame(small)
    s1 = st.read_debug(abi.SGI_DEBUG_TILE_STAGE1, np.float32).reshape(-1, 8)
    ref1 = O.tile_stage1(32, cfg, small.hs.gbuffers[1], small.hs.camera(1))
    assert_bit_exact(s1, ref1, "tile stage 1 (mean position / normal)")
    idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    cnt = int(idx[0])
    cv = small.sc.vpls[idx[1:1 + cnt]]
    lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + cfg.max_vpls_per_tile)
    ref2 = O.tile_stage2(32, cfg, ref1, cv, cnt)
    assert np.array_equal(lists, ref2), "tile stage 2 lists"


@pytest.mark.parametrize("L,ts", [(1, 16), (12, 8), (33, 32), (64, 16), (12, 5), (64, 4), (20, 24)])
def test_tile_lists_variants(small, L, ts):
    st, cfg = small.stage(1, max_vpls_per_tile=L, tile_size=ts)
    st.cull_vpls()
    st.cull_tiles(small.g[1], small.hs.camera(1))
    torch.cuda.synchronize()
    ref1 = O.tile_stage1(32, cfg, small.hs.gbuffers[1], small.hs.camera(1))
    idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    cnt = int(idx[0])
    ref2 = O.tile_stage2(32, cfg, ref1, small.sc.vpls[idx[1:1 + cnt]], cnt)
    lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + L)
    assert np.array_equal(lists, ref2)
    st.close()


def test_tile_lists_with_tied_keys():
    """Groups of VPLs at the same position with the same radius: equal keys, which the
    reference's strict '<' insertion keeps in index order; with L = 12 the cut falls
    inside a group of ties."""
    w = S.Workload("room12_128x96_vpl600", 128, 96, 12, 600, 0, 512, 16, abi.SGI_CUBE_F32, 4, 3, 1)
    s = Setup(w, 91)
    v = s.sc.vpls.copy()
    v[1::3, :3] = v[0::3, :3][: len(v[1::3])]    # every group of three shares one position
    v[2::3, :3] = v[0::3, :3][: len(v[2::3])]
    s.vpls = torch.from_numpy(v).cuda()
    for L, ts in ((12, 16), (7, 5)):
        st, cfg = s.stage(1, max_vpls_per_tile=L, tile_size=ts)
        st.cull_vpls()
        st.cull_tiles(s.g[1], s.hs.camera(1))
        torch.cuda.synchronize()
        idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
        cnt = int(idx[0])
        ref1 = O.tile_stage1(32, cfg, s.hs.gbuffers[1], s.hs.camera(1))
        ref2 = O.tile_stage2(32, cfg, ref1, v[idx[1:1 + cnt]], cnt)
        lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + L)
        assert (ref2[:, 0] == L).mean() > 0.5
        assert np.array_equal(lists, ref2)
        st.close()


def test_reference_tile_preset_frame_bit_exact(small):
    """The reference's tile constants: 5x5 tiles (StratusRendererBackend.h:346-347), 12 VPLs per tile
    (vpl_common.glsl:9), the per-tile mean by the sequential sum of stage 1; tiled gather, whole frame."""
    st, cfg, out = _run_frame(small, tile_size=5, max_vpls_per_tile=12)
    H, W = cfg.height, cfg.width
    ref = O.frame(32, cfg, small.hs, 1, np.zeros((H, W, 4), np.float32), np.zeros((H, W), np.float32), TIME, FPS)
    lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + 12)
    assert lists.shape[0] == 64 * 36
    assert np.array_equal(lists, ref["lists"])
    assert_bit_exact(out.cpu().numpy().astype(np.float32)[..., :3], ref["combined"][..., :3], "5x5-tile frame HDR")
    st.close()


def _gather_ref(s, st, cfg, k=1):
    idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    cnt = int(idx[0])
    cv = s.sc.vpls[idx[1:1 + cnt]]
    ce = s.sc.entries[idx[1:1 + cnt]]
    lists = None
    if cfg.gi_mode == abi.SGI_GI_TILED:
        lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + cfg.max_vpls_per_tile)
    return O.gather(32, cfg, s.hs.gbuffers[k], s.hs.camera(k), cv, ce, cnt, lists, s.hs.cubes, TIME), cnt


@pytest.mark.parametrize("mode,spp", [(abi.SGI_GI_TILED, 8), (abi.SGI_GI_REFERENCE, 0), (abi.SGI_GI_REFERENCE, 8),
                                      (abi.SGI_GI_TILED, 0)])
def test_gather_bit_exact(small, mode, spp):
    st, cfg, _ = _run_frame(small, gi_mode=mode, samples_per_pixel=spp)
    got = st.read_debug(abi.SGI_DEBUG_RESERVOIR, np.uint16).view(np.float16).reshape(cfg.height, cfg.width, 4)
    ref, _ = _gather_ref(small, st, cfg)
    assert_bit_exact(got.astype(np.float32), ref, f"gather reservoir mode={mode} spp={spp}")
    assert np.isfinite(got).all()


def test_denoise_passes_bit_exact(small):
    st, cfg, out = _run_frame(small)
    H, W = cfg.height, cfg.width
    res = st.read_debug(abi.SGI_DEBUG_RESERVOIR, np.uint16)
    res32 = half4_to_f32(res, H, W)
    direct = half4_to_f32(st.read_debug(abi.SGI_DEBUG_DIRECT, np.uint16), H, W)
    idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    comb, gi, hist, passes = O.denoise(32, cfg, small.hs.gbuffers[1], small.hs.gbuffers[0], res32, direct,
                                       np.zeros((H, W, 4), np.float32), np.zeros((H, W), np.float32), int(idx[0]),
                                       TIME, FPS, keep_passes=True)
    for p in range(cfg.denoise_passes):
        gp = half4_to_f32(st.read_debug(abi.SGI_DEBUG_PASS_BASE + p, np.uint16), H, W)
        assert_bit_exact(gp, passes[p], f"denoise pass {p} reservoir")
    assert_bit_exact(out.cpu().numpy().astype(np.float32)[..., :3], comb[..., :3], "combined HDR output")
    gh = half4_to_f32(st.read_debug(abi.SGI_DEBUG_GI_HISTORY, np.uint16), H, W)
    assert_bit_exact(gh[..., :3], gi[..., :3], "GI history (giColor)")
    hd = st.read_debug(abi.SGI_DEBUG_HISTORY_DEPTH, np.uint16).view(np.float16).reshape(H, W).astype(np.float32)
    assert_bit_exact(hd, hist, "history depth")


def test_deferred_bit_exact():
    w = S.Workload("room12_200x120_pts4", 200, 120, 12, 32, 4, 1024, 16, abi.SGI_CUBE_F32, 4, 3, 1)
    s = Setup(w, 4242)
    st, cfg = s.stage(1)
    out = torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda")
    st.direct_lighting(s.g[1], s.hs.camera(1), out)
    torch.cuda.synchronize()
    ref = O.deferred(32, cfg, s.hs.gbuffers[1], s.hs.camera(1), s.sc.points, s.hs.csms[1])
    got = out.cpu().numpy().astype(np.float32)
    assert_bit_exact(got[..., :3], ref[..., :3], "deferred PBR + CSM")
    assert (got[..., :3] > 0).mean() > 0.2


def test_two_frame_sequence_with_history(small):
    """Frame 1 then frame 2 on one context: history from frame 1 feeds the temporal pass of frame 2."""
    st, cfg = small.stage(1)
    H, W = cfg.height, cfg.width
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    gi_prev = np.zeros((H, W, 4), np.float32)
    hist_prev = np.zeros((H, W), np.float32)
    for k in (1, 2):
        st.set_shadow_maps(small.csm[k], small.cubes)
        st.render_frame(small.g[k], small.g[k - 1], small.hs.camera(k), out, TIME + 16.0 * k, FPS)
        torch.cuda.synchronize()
        ref = O.frame(32, cfg, small.hs, k, gi_prev, hist_prev, TIME + 16.0 * k, FPS)
        assert_bit_exact(out.cpu().numpy().astype(np.float32)[..., :3], ref["combined"][..., :3], f"frame {k} HDR")
        gi_prev, hist_prev = ref["gi"], ref["hist"]
    # history accumulated beyond one frame on static, well-matched pixels
    hd = st.read_debug(abi.SGI_DEBUG_HISTORY_DEPTH, np.uint16).view(np.float16).astype(np.float32)
    assert hd.max() >= 2.0


def test_fp32_path_psnr_vs_fp64_oracle(small):
    _, cfg, out = _run_frame(small)
    H, W = cfg.height, cfg.width
    ref64 = O.frame(64, cfg, small.hs, 1, np.zeros((H, W, 4)), np.zeros((H, W)), TIME, FPS)
    p = psnr(out.cpu().numpy().astype(np.float64)[..., :3], ref64["combined"][..., :3])
    assert p > 50.0, p


@pytest.mark.parametrize("W,H", [(1, 1), (17, 9), (33, 31)])
def test_tiny_and_ragged_viewports(W, H):
    w = S.Workload(f"room12_{W}x{H}", W, H, 12, 24, 2, 256, 8, abi.SGI_CUBE_F16, 4, 3, 1, tile_size=16,
                   max_per_tile=8)
    s = Setup(w, 9 + W)
    st, cfg, out = _run_frame(s)
    ref = O.frame(32, cfg, s.hs, 1, np.zeros((H, W, 4), np.float32), np.zeros((H, W), np.float32), TIME, FPS)
    assert_bit_exact(out.cpu().numpy().astype(np.float32)[..., :3], ref["combined"][..., :3], f"{W}x{H} HDR")
    lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + cfg.max_vpls_per_tile)
    assert np.array_equal(lists, ref["lists"])


def test_no_vpls_visible():
    """All VPLs occluded: the gather adds nothing and the merge pass divides by a zero count."""
    w = S.Workload("room12_64x48_novis", 64, 48, 12, 16, 0, 256, 8, abi.SGI_CUBE_F32, 4, 3, 1)
    s = Setup(w, 5)
    v = s.sc.vpls.copy()
    rng = np.random.default_rng(0)
    v[:, 0] = rng.uniform(4.0, 6.0, len(v))   # 1 m under the middle of the floor slab: the sun ray is blocked
    v[:, 1] = -1.0
    v[:, 2] = rng.uniform(4.0, 6.0, len(v))
    s.vpls = torch.from_numpy(v).cuda()
    s.sc.vpls = v
    assert O.vis_cull(32, v, s.hs.csms[1], 16)[0] == 0
    st, cfg, out = _run_frame(s)
    assert st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)[0] == 0
    ref = O.frame(32, cfg, s.hs, 1, np.zeros((48, 64, 4), np.float32), np.zeros((48, 64), np.float32), TIME, FPS)
    got = out.cpu().numpy().astype(np.float32)[..., :3]
    assert np.all(half_bits_equal(got.astype(np.float16), ref["combined"][..., :3].astype(np.float16)))


def test_abi_rejects_bad_arguments():
    lib = abi.load()
    cfg = stage.default_config(64, 48)
    h = C.c_void_p()
    bad = stage.default_config(64, 48, tile_size=40)
    assert lib.sgi_create(C.byref(bad), C.byref(h)) == abi.SGI_ERR_ARG
    abi.check(lib.sgi_create(C.byref(cfg), C.byref(h)))
    try:
        assert lib.sgi_cull_vpls(h, None) == abi.SGI_ERR_STATE
        v = torch.zeros((cfg.max_vpls + 1, 16), device="cuda")
        e = torch.zeros((cfg.max_vpls + 1, 2), dtype=torch.int32, device="cuda")
        assert lib.sgi_set_lights(h, C.c_void_p(v.data_ptr()), C.c_void_p(e.data_ptr()), cfg.max_vpls + 1, None, 0,
                                  None) == abi.SGI_ERR_CAP
        assert b"max_vpls" in lib.sgi_last_error(h)
        # cube faces above SGI_MAX_CUBE_FACE are refused (the texel offsets assume 6 n^2 < 2^31)
        d = torch.zeros(16, device="cuda")
        csm = abi.Csm()
        csm.depth = d.data_ptr()
        csm.resolution = 1
        csm.num_cascades = 4
        cubes = abi.CubeAtlas()
        cubes.atlas[0] = d.data_ptr()
        cubes.num_atlases, cubes.layers_per_atlas, cubes.format = 1, 1, abi.SGI_CUBE_F32
        cubes.face_size = abi.SGI_MAX_CUBE_FACE + 1
        assert lib.sgi_set_shadow_maps(h, C.byref(csm), C.byref(cubes)) == abi.SGI_ERR_ARG
        cubes.face_size = abi.SGI_MAX_CUBE_FACE
        assert lib.sgi_set_shadow_maps(h, C.byref(csm), C.byref(cubes)) == abi.SGI_OK
        # the denoiser inputs are written with 16-byte stores: misaligned outputs are refused
        g = abi.GBuffer(*([d.data_ptr()] * 8))
        cam = abi.Camera()
        buf = torch.zeros(64, device="cuda")
        p0, p4 = buf.data_ptr(), buf.data_ptr() + 4
        assert lib.sgi_nn_features(h, C.byref(g), C.byref(cam), p4, p0, p0, None) == abi.SGI_ERR_ARG
        assert lib.sgi_nn_features(h, C.byref(g), C.byref(cam), p0, p4, p0, None) == abi.SGI_ERR_ARG
        assert b"16-byte aligned" in lib.sgi_last_error(h)
        assert lib.sgi_nn_features(h, C.byref(g), C.byref(cam), p0, p0, p0, None) == abi.SGI_ERR_STATE   # no frame
    finally:
        lib.sgi_destroy(h)


@pytest.mark.parametrize("mode", [abi.SGI_GI_TILED, abi.SGI_GI_REFERENCE])
def test_converged_target_bit_exact(small, mode):
    """sgi_gi_target: batches of the sample loop summed in FP64 must equal the oracle's."""
    st, cfg = small.stage(1, gi_mode=mode)
    st.cull_vpls()
    if mode == abi.SGI_GI_TILED:
        st.cull_tiles(small.g[1], small.hs.camera(1))
    out = torch.empty((cfg.height, cfg.width, 4), dtype=torch.float32, device="cuda")
    st.gi_target(small.g[1], small.hs.camera(1), TIME, 6, out)
    torch.cuda.synchronize()
    idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    cnt = int(idx[0])
    lists = None
    if mode == abi.SGI_GI_TILED:
        lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + cfg.max_vpls_per_tile)
    ref = O.gi_target(cfg, small.hs.gbuffers[1], small.hs.camera(1), small.sc.vpls[idx[1:1 + cnt]],
                      small.sc.entries[idx[1:1 + cnt]], cnt, lists, small.hs.cubes, TIME, 6)
    assert_bit_exact(out.cpu().numpy(), ref, f"converged target mode={mode}")
    st.close()


def test_history_snapshot_restores_the_next_frame(small):
    """sgi_get_history after frame 1 on one context, sgi_set_history on a fresh one: frame 2 of both is
    bit-identical (the temporal pass reads only the history and the inputs)."""
    lib = abi.load()
    H, W = small.w.height, small.w.width
    a, _ = small.stage(1)
    b, _ = small.stage(1)
    out_a = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    out_b = torch.empty_like(out_a)
    a.render_frame(small.g[1], small.g[0], small.hs.camera(1), out_a, TIME + 16.0, FPS)
    gi = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    hl = torch.empty((H, W), dtype=torch.float16, device="cuda")
    valid = C.c_int32(-1)
    abi.check(lib.sgi_get_history(a.ctx, C.c_void_p(gi.data_ptr()), C.c_void_p(hl.data_ptr()), C.byref(valid),
                                  None), a.ctx)
    assert valid.value == 1
    abi.check(lib.sgi_set_history(b.ctx, C.c_void_p(gi.data_ptr()), C.c_void_p(hl.data_ptr()), 1, None), b.ctx)
    for st, out in ((a, out_a), (b, out_b)):
        st.set_shadow_maps(small.csm[2], small.cubes)
        st.render_frame(small.g[2], small.g[1], small.hs.camera(2), out, TIME + 32.0, FPS)
    torch.cuda.synchronize()
    assert torch.equal(out_a.view(torch.int16), out_b.view(torch.int16))
    assert lib.sgi_get_history(a.ctx, None, None, C.byref(valid), None) == abi.SGI_ERR_ARG
    a.close()
    b.close()
