"""What the trained network gains over the method without it.

A 480x272 room (40 boxes, 512 VPLs, 4 point lights) is rendered for four
frames three ways: the plain a-trous path at K = 8, the neural path with the
committed trained weights at K = 1, and the neural path with an untrained
(randomly initialised) network at K = 1. Each frame's GI term is compared with
the converged K = 512 GI (FP64 accumulation); the trained network must beat
both the a-trous filter and the untrained network by a clear margin.
"""
import ctypes as C
import os

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from stratusgfx_gb300 import abi, denoiser, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402

W_ = S.Workload("room40_480x272_vpl512_k8", 480, 272, 40, 512, 4, 1024, 64, abi.SGI_CUBE_F16, 8, 5, 4)


def gi_psnr(render, ds, w, cfg, targets):
    st = stage.GiStage(cfg)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    H, W = w.height, w.width
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    direct = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    vals = []
    for k in range(1, len(targets) + 1):
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        render(st, k, out)
        st.direct_lighting(ds.gbuffers[k], ds.camera(k), direct)
        torch.cuda.synchronize()
        alb = ds.gbuffers[k].albedo[..., :3].double() / 255.0
        ref = (torch.clamp(alb, min=0.01) + 1e-5).half().double() * targets[k - 1][..., :3].double()
        got = out[..., :3].double() - direct[..., :3].double()
        mse = torch.mean((got - ref) ** 2)
        vals.append(float(10.0 * torch.log10(torch.max(torch.abs(ref)) ** 2 / mse)))
    st.close()
    return sum(vals) / len(vals)


@pytest.mark.skipif(not os.path.exists(denoiser.WEIGHTS), reason="no trained weights")
def test_trained_network_beats_atrous_and_untrained_network():
    w = W_
    sc = S.workload_scene(w, 4321)
    ds = stage.DeviceScene(sc, w)
    # converged GI: 64 batches of 8 samples, FP64 sums, seeded apart from the frames
    tcfg = stage.workload_config(w, samples_per_pixel=8)
    ts = stage.GiStage(tcfg)
    ts.set_lights(ds.vpls, ds.entries, ds.points)
    targets = []
    for k in range(1, len(sc.cameras)):
        ts.set_shadow_maps(ds.csms[k], ds.cubes)
        cam = ds.camera(k)
        ts.cull_vpls()
        ts.cull_tiles(ds.gbuffers[k], cam)
        t = torch.empty((w.height, w.width, 4), dtype=torch.float32, device="cuda")
        ts.gi_target(ds.gbuffers[k], cam, 1000.0 + 16.0 * k + 7.0e6, 64, t)
        targets.append(t)
    torch.cuda.synchronize()
    ts.close()

    def plain(st, k, out):
        st.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, 1000.0 + 16.0 * k, 60.0)

    def neural_with(net):
        def render(st, k, out):
            fp = abi.FrameParams(1000.0 + 16.0 * k, 60.0)
            abi.check(st.lib.sgi_render_frame_neural(st.ctx, net.h, C.byref(ds.gbuffers[k].struct()),
                                                     C.byref(ds.gbuffers[k - 1].struct()), C.byref(ds.camera(k)),
                                                     C.byref(fp), C.c_void_p(out.data_ptr()), None), st.ctx)
        return render

    p_plain = gi_psnr(plain, ds, w, stage.workload_config(w), targets)
    k1 = stage.workload_config(w, samples_per_pixel=1)
    trained = denoiser.KpcnDenoiser(1, w.height, w.width)
    trained.load(denoiser.WEIGHTS)
    untrained = denoiser.KpcnDenoiser(1, w.height, w.width, seed=3)
    try:
        p_trained = gi_psnr(neural_with(trained), ds, w, k1, targets)
        p_untrained = gi_psnr(neural_with(untrained), ds, w, k1, targets)
    finally:
        trained.close()
        untrained.close()
    print(f"GI PSNR: a-trous K=8 {p_plain:.2f} dB, trained K=1 {p_trained:.2f} dB, untrained K=1 {p_untrained:.2f} dB")
    assert p_trained > p_plain + 1.0, (p_plain, p_trained)
    assert p_trained > p_untrained + 3.0, (p_untrained, p_trained)
