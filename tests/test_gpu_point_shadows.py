"""Shadow-casting point lights of the direct lighting (pbr.fs:116-131 with
calculateShadowValue8Samples) on the GPU against the FP32 oracle. The lights'
distance cubes come from the scene generator (sgi_scene_cube_atlas with the
lights' positions and far planes) and are checked byte for byte against the CPU
ray caster first; the lit frame must then match the oracle bit for bit in every
cube format (exact equality: same binary32 expression trees, no contraction).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import assert_bit_exact, upload_cubes, upload_gbuffer

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402


def caster_records(sc, far):
    """Point lights as shadow casters, and the VPL-shaped records that make their distance cubes."""
    lights = sc.points.copy()
    lights[:, 9] = far                                   # far plane of each light's cube
    as_vpl = np.zeros((lights.shape[0], 16), np.float32)
    as_vpl[:, 0:4] = lights[:, 0:4]
    as_vpl[:, 13] = far
    entries = np.array([[0, k] for k in range(lights.shape[0])], np.int32)
    return lights, as_vpl, entries


@pytest.mark.parametrize("fmt", [abi.SGI_CUBE_UNORM16, abi.SGI_CUBE_F16, abi.SGI_CUBE_F32])
def test_shadowed_point_lights_bit_exact(fmt):
    w = S.Workload("room12_128x80_pts3", 128, 80, 12, 16, 3, 512, 32, fmt, 4, 3, 1)
    sc = S.workload_scene(w, 61)
    hs = O.HostScene(sc, w)
    lights, as_vpl, entries = caster_records(sc, 14.0)
    # the lights' distance cubes: GPU generator vs CPU ray caster
    ref_store, ref_atlas = O.scene_cubes(sc.boxes, as_vpl, entries, 32, fmt)
    cube_t, atlas = upload_cubes(np.zeros_like(ref_store), fmt)
    lib = abi.load()
    boxes = torch.from_numpy(sc.boxes).cuda()
    v = torch.from_numpy(as_vpl).cuda()
    e = torch.from_numpy(entries).cuda()
    abi.check(lib.sgi_scene_cube_atlas(C.c_void_p(boxes.data_ptr()), sc.boxes.shape[0], C.c_void_p(v.data_ptr()),
                                       C.c_void_p(e.data_ptr()), lights.shape[0], C.byref(atlas), None))
    torch.cuda.synchronize()
    got_store = cube_t.cpu().numpy()
    if ref_store.dtype == np.uint16:
        got_store = got_store.view(np.uint16)
    assert np.array_equal(got_store, ref_store)
    # direct lighting: two plain point lights + the three casters (+ the sun with its CSM)
    cfg = stage.workload_config(w)
    st = stage.GiStage(cfg)
    st.set_lights(torch.from_numpy(sc.vpls).cuda(), torch.from_numpy(sc.entries).cuda(),
                  torch.from_numpy(sc.points[:2]).cuda())
    csm_t = torch.from_numpy(hs.csm_depth[1]).cuda()
    st.set_shadow_maps(stage.csm_struct(sc, 1, csm_t.data_ptr(), w.csm_resolution), atlas)
    lt = torch.from_numpy(lights).cuda()
    assert lib.sgi_set_shadow_point_lights(st.ctx, C.c_void_p(lt.data_ptr()), C.c_void_p(e.data_ptr()),
                                           lights.shape[0], C.byref(atlas), None) == abi.SGI_OK
    g = upload_gbuffer(hs.gbuffers[1])
    out = torch.zeros((w.height, w.width, 4), dtype=torch.float16, device="cuda")
    st.direct_lighting(g, hs.camera(1), out)
    torch.cuda.synchronize()
    ref = O.deferred(32, cfg, hs.gbuffers[1], hs.camera(1), sc.points[:2], hs.csms[1], lights, entries, ref_atlas)
    got = out.cpu().numpy().astype(np.float32)
    assert_bit_exact(got[..., :3], ref[..., :3], "direct lighting with shadowed point lights")
    # the casters' shadows matter: without them the frame differs
    plain = O.deferred(32, cfg, hs.gbuffers[1], hs.camera(1), sc.points[:2], hs.csms[1])
    assert not np.array_equal(ref, plain)
    # limits
    assert lib.sgi_set_shadow_point_lights(st.ctx, C.c_void_p(lt.data_ptr()), C.c_void_p(e.data_ptr()), 257,
                                           C.byref(atlas), None) == abi.SGI_ERR_CAP
    assert lib.sgi_set_shadow_point_lights(st.ctx, None, None, 0, None, None) == abi.SGI_OK
    st.close()
