"""Parity at the workloads the benchmark times, through the C ABI.

The 1920x1080 workload (40-box room, 2048 VPLs with 6x128^2 FP16 distance
cubes, 4 point lights, 4x2048^2 CSM, <= 64 VPLs per 16x16 tile, K = 8, 5
denoise passes) renders two consecutive frames on one context, the second
reading the first's history; the visible-VPL list, every per-tile list
(vpl_tiled_deferred_culling_stage2.cs:61-129) and the HDR output must equal
the FP32 oracle's bit for bit. The 3840x2160 workload (4096 VPLs, K = 4)
checks the visibility cull and the 32,400 per-tile lists, and two whole
frames the same way (the second reading the first's history).

Inputs come from the device scene generator and are copied to the host for the
oracle (the generator equals the oracle's CPU ray caster bit for bit, see
test_scene_generator_matches_cpu_raycaster). The tolerance is exact equality
(NaN == NaN), stronger than the stated 1e-3 relative tolerance of the FP32 path.
"""
import numpy as np
import pytest

from helpers import assert_bit_exact, host_scene_from_device

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402

FPS = 60.0


def test_hd_workload_two_frames_bit_exact():
    w = S.HD
    sc = S.workload_scene(w, 1234 + 2)          # the benchmark's scene
    ds = stage.DeviceScene(sc, w)
    hs = host_scene_from_device(ds, (0, 1, 2))
    cfg = stage.workload_config(w)
    L = cfg.max_vpls_per_tile
    st = stage.GiStage(cfg)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    out = torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda")
    gi = np.zeros((w.height, w.width, 4), np.float32)
    hist = np.zeros((w.height, w.width), np.float32)
    for k in (1, 2):
        t = 1000.0 + 16.0 * k
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        st.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, t, FPS)
        torch.cuda.synchronize()
        ref = O.frame(32, cfg, hs, k, gi, hist, t, FPS)
        idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
        cnt = ref["count"]
        assert idx[0] == cnt and cnt > 1000, (idx[0], cnt)
        assert np.array_equal(idx[1:1 + cnt], ref["visible_index"][1:1 + cnt])
        lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + L)
        assert lists.shape == ref["lists"].shape == (8160, 1 + L)
        full = int((ref["lists"][:, 0] == L).sum())
        assert full > 100, f"only {full} tiles reach the cap: the selection path is not exercised"
        assert np.array_equal(lists, ref["lists"]), f"frame {k}: {int((lists != ref['lists']).any(1).sum())} tiles differ"
        got = out.cpu().numpy().astype(np.float32)[..., :3]
        assert_bit_exact(got, ref["combined"][..., :3], f"1920x1080 frame {k} HDR")
        gi, hist = ref["gi"], ref["hist"]
    st.close()


def test_uhd_workload_tile_lists_bit_exact():
    w = S.UHD
    sc = S.workload_scene(w, 1234 + 4)          # the 3840x2160 comparison's scene
    ds = stage.DeviceScene(sc, w)
    hs = host_scene_from_device(ds, (1,), cubes=False)
    cfg = stage.workload_config(w)
    L = cfg.max_vpls_per_tile
    st = stage.GiStage(cfg)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    st.set_shadow_maps(ds.csms[1], ds.cubes)
    st.cull_vpls()
    st.cull_tiles(ds.gbuffers[1], ds.camera(1))
    torch.cuda.synchronize()
    idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    ref_idx = O.vis_cull(32, sc.vpls, hs.csms[1], cfg.max_visible)
    cnt = int(ref_idx[0])
    assert idx[0] == cnt and cnt > 2000
    assert np.array_equal(idx[1:1 + cnt], ref_idx[1:1 + cnt])
    s1 = O.tile_stage1(32, cfg, hs.gbuffers[1], hs.camera(1))
    assert_bit_exact(st.read_debug(abi.SGI_DEBUG_TILE_STAGE1, np.float32).reshape(-1, 8), s1, "4K tile stage 1")
    ref = O.tile_stage2(32, cfg, s1, sc.vpls[ref_idx[1:1 + cnt]], cnt)
    lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + L)
    assert lists.shape == (32400, 1 + L)
    assert int((ref[:, 0] == L).sum()) > 100
    assert np.array_equal(lists, ref), f"{int((lists != ref).any(1).sum())} of 32400 tile lists differ"
    st.close()


def test_uhd_workload_two_frames_bit_exact():
    w = S.UHD
    sc = S.workload_scene(w, 1234 + 4)
    ds = stage.DeviceScene(sc, w)
    hs = host_scene_from_device(ds, (0, 1, 2))
    cfg = stage.workload_config(w)
    L = cfg.max_vpls_per_tile
    st = stage.GiStage(cfg)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    out = torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda")
    gi = np.zeros((w.height, w.width, 4), np.float32)
    hist = np.zeros((w.height, w.width), np.float32)
    for k in (1, 2):
        t = 1000.0 + 16.0 * k
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        st.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, t, FPS)
        torch.cuda.synchronize()
        assert st.lib.sgi_device_status(st.ctx) == abi.SGI_OK
        ref = O.frame(32, cfg, hs, k, gi, hist, t, FPS)
        idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
        cnt = ref["count"]
        assert idx[0] == cnt and cnt > 2000
        lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + L)
        assert np.array_equal(lists, ref["lists"]), f"frame {k}"
        got = out.cpu().numpy().astype(np.float32)[..., :3]
        assert_bit_exact(got, ref["combined"][..., :3], f"3840x2160 frame {k} HDR")
        gi, hist = ref["gi"], ref["hist"]
    st.close()
