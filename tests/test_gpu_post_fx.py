"""Post-processing of the HDR frame (taa.fs + gammaTonemap.fs through sgi_post_fx)
on the GPU against the FP32 oracle, over three frames of a moving camera so the
TAA history is reprojected by the G-buffer velocity. The TAA output (RGBA16F) is
pure binary32 arithmetic and must match bit for bit; the RGBA8 output goes
through pow(x, 1/2.2), where the device powf and the host's may differ in the
last place, so its tolerance is 1 in 255 per channel (and most pixels exact).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import upload_gbuffer

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402


def test_post_fx_matches_oracle():
    w = S.Workload("room12_120x72_vpl32", 120, 72, 12, 32, 2, 512, 16, abi.SGI_CUBE_F16, 4, 3, 3)
    sc = S.workload_scene(w, 91)
    ds = stage.DeviceScene(sc, w)
    st = stage.GiStage(stage.workload_config(w))
    st.set_lights(ds.vpls, ds.entries, ds.points)
    lib = abi.load()
    hist = None
    H, W = w.height, w.width
    for k in range(1, 4):
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        hdr = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
        st.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), hdr, 1000.0 + 16.0 * k, 60.0)
        ldr = torch.zeros((H, W), dtype=torch.int32, device="cuda")
        abi.check(lib.sgi_post_fx(st.ctx, C.c_void_p(hdr.data_ptr()), C.byref(ds.gbuffers[k].struct()), 1,
                                  C.c_void_p(ldr.data_ptr()), None), st.ctx)
        torch.cuda.synchronize()
        vel = ds.gbuffers[k].velocity.cpu().numpy().view(np.uint32).reshape(H, W)
        ref_ldr, ref_taa = O.post_fx(32, hdr.cpu().numpy(), vel, hist, taa=True)
        got = ldr.cpu().numpy().view(np.uint32)
        diff = np.abs((got[..., None] >> np.array([0, 8, 16]) & 0xff).astype(int) -
                      (ref_ldr[..., None] >> np.array([0, 8, 16]) & 0xff).astype(int))
        assert diff.max() <= 1 and (diff == 0).mean() > 0.99, (k, diff.max(), (diff == 0).mean())
        assert ((got >> 24) == 255).all()
        taa = st.read_debug(abi.SGI_DEBUG_TAA_HISTORY, np.uint16).view(np.float16).reshape(H, W, 4)
        assert np.array_equal(taa.astype(np.float32).view(np.uint32), ref_taa.view(np.uint32)), k
        hist = ref_taa
    # the TAA history the context keeps equals the oracle's (RGBA16F, bit for bit): tonemap-only
    # output of a frame equal to that history reproduces the oracle's LDR of it
    ldr2 = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    h16 = torch.from_numpy(hist.astype(np.float16)).cuda()
    abi.check(lib.sgi_post_fx(st.ctx, C.c_void_p(h16.data_ptr()), None, 0, C.c_void_p(ldr2.data_ptr()), None), st.ctx)
    torch.cuda.synchronize()
    ref2, _ = O.post_fx(32, hist.astype(np.float16), np.zeros((H, W), np.uint32), None, taa=False)
    d2 = np.abs((ldr2.cpu().numpy().view(np.uint32) & 0xff).astype(int) - (ref2 & 0xff).astype(int))
    assert d2.max() <= 1
    assert lib.sgi_post_fx(st.ctx, None, None, 0, C.c_void_p(ldr2.data_ptr()), None) == abi.SGI_ERR_ARG
    assert lib.sgi_post_fx(st.ctx, C.c_void_p(h16.data_ptr()), None, 1, C.c_void_p(ldr2.data_ptr()), None) == \
        abi.SGI_ERR_ARG
    st.close()
