"""VPL colouring (vpl_light_color.cs) and the diffuse cubes it reads, on the GPU
against the FP32 oracle: the scene generator's diffuse cubes byte for byte
against the CPU ray caster, and the recoloured compacted VPL list of
sgi_cull_vpls (with sgi_set_vpl_coloring) bit for bit against the oracle's
visibility cull followed by its colouring pass. Same inputs, same binary32
expression trees without contraction: the tolerance is exact equality.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import assert_bit_exact, upload_cubes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402


def diffuse_on_gpu(sc, face):
    lib = abi.load()
    n = sc.vpls.shape[0]
    layers = sc.layers_per_atlas
    na = max(1, (n + layers - 1) // layers)
    t = torch.zeros((na, layers, 6, face, face), dtype=torch.int32, device="cuda")
    at = abi.DiffuseAtlas()
    for a in range(na):
        at.atlas[a] = t[a].data_ptr()
    at.num_atlases, at.layers_per_atlas, at.face_size = na, layers, face
    boxes = torch.from_numpy(sc.boxes).cuda()
    vpls = torch.from_numpy(sc.vpls).cuda()
    entries = torch.from_numpy(sc.entries).cuda()
    abi.check(lib.sgi_scene_diffuse_atlas(C.c_void_p(boxes.data_ptr()), sc.boxes.shape[0],
                                          C.c_void_p(vpls.data_ptr()), C.c_void_p(entries.data_ptr()), n,
                                          C.byref(at), None))
    torch.cuda.synchronize()
    return t, at


@pytest.mark.parametrize("fmt", [abi.SGI_CUBE_F16, abi.SGI_CUBE_F32])
def test_vpl_coloring_bit_exact(fmt):
    w = S.Workload("room12_96x64_vpl96", 96, 64, 12, 96, 2, 512, 16, fmt, 4, 3, 2)
    sc = S.workload_scene(w, 51)
    sc.vpls[::4, 1] = -1.0                         # some VPLs below the floor: culled by the CSM
    sc.vpls[:, 14] = np.linspace(0.0005, 0.002, sc.vpls.shape[0], dtype=np.float32)   # varied intensities
    hs = O.HostScene(sc, w)
    # diffuse cubes: GPU generator vs the CPU ray caster
    dt, dat = diffuse_on_gpu(sc, w.cube_size)
    dref, dref_at = O.scene_diffuse(sc.boxes, sc.vpls, sc.entries, w.cube_size, sc.layers_per_atlas)
    assert np.array_equal(dt.cpu().numpy().view(np.uint32), dref)
    assert (dref != 0).any() and (dref == 0).any()
    # cull + colouring on the GPU
    csm_t = torch.from_numpy(hs.csm_depth[1]).cuda()
    csm = stage.csm_struct(sc, 1, csm_t.data_ptr(), w.csm_resolution)
    cube_t, cubes = upload_cubes(hs.cube_storage, fmt, sc.layers_per_atlas)
    cfg = stage.workload_config(w)
    st = stage.GiStage(cfg)
    st.set_lights(torch.from_numpy(sc.vpls).cuda(), torch.from_numpy(sc.entries).cuda(),
                  torch.from_numpy(sc.points).cuda())
    st.set_shadow_maps(csm, cubes)
    lib = abi.load()
    assert lib.sgi_set_vpl_coloring(st.ctx, C.byref(dat)) == abi.SGI_OK
    st.cull_vpls()
    torch.cuda.synchronize()
    idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    cnt = int(idx[0])
    cv = st.read_debug(abi.SGI_DEBUG_COMPACT_VPLS, np.float32).reshape(-1, 16)[:cnt]
    ce = st.read_debug(abi.SGI_DEBUG_COMPACT_ENTRIES, np.int32).reshape(-1, 2)[:cnt]
    # oracle: visibility cull, then the colouring pass on the compacted list
    ref_idx = O.vis_cull(32, sc.vpls, hs.csms[1], cfg.max_visible)
    assert np.array_equal(idx[:1 + cnt], ref_idx[:1 + cnt]) and 0 < cnt < sc.vpls.shape[0]
    sel = ref_idx[1:1 + cnt]
    ref = O.color_vpls(32, sc.vpls[sel], sc.entries[sel], cnt, hs.cubes, dref_at, hs.csms[1])
    assert np.array_equal(ce, sc.entries[sel])
    assert_bit_exact(cv, ref, "recoloured VPLs")
    assert not np.array_equal(ref[:, 4:12], sc.vpls[sel][:, 4:12])   # the pass changed colour and specular position
    # colouring off again: the compacted list carries the input records
    assert lib.sgi_set_vpl_coloring(st.ctx, None) == abi.SGI_OK
    st.cull_vpls()
    torch.cuda.synchronize()
    cv0 = st.read_debug(abi.SGI_DEBUG_COMPACT_VPLS, np.float32).reshape(-1, 16)[:cnt]
    assert np.array_equal(cv0.view(np.uint32), sc.vpls[sel].view(np.uint32))
    bad = abi.DiffuseAtlas()
    assert lib.sgi_set_vpl_coloring(st.ctx, C.byref(bad)) == abi.SGI_ERR_ARG
    st.close()
