"""The TMA-staged a-trous passes (sgi_set_atrous_staging(SGI_ATROUS_STAGED)).

A CTA of the staged kernel stages the lattice of pixels its taps reach (stride
2^pass: 2, 4, 8) in shared memory with strided TMA copies and fixes up the
lattice points outside the image with the clamped pixels; the filter
arithmetic is the direct kernel's. Both modes must give bit-identical passes
(vpl_pbr_gi_denoise.fs:307-327, the restatement in oracle/passes.hpp) on
viewports whose lattices end anywhere in a CTA, on an odd width (the staged
path does not apply: every pass runs direct) and with 7 passes (strides 16
and 32 run direct). The wait for the copies is bounded: with the copies
switched off it runs out, reports SGI_ERR_TIMEOUT and the next frame is whole.
"""
import numpy as np
import pytest

from helpers import GpuSetup, assert_bit_exact, half4_to_f32, half_bits_equal

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402

TIME, FPS = 1000.0, 60.0

CASES = {
    "320x180": (S.SMALL, 1235, {}),
    # even width that is no multiple of 16 * 8 pixels, height no multiple of 8 * 8
    "198x94": (S.Workload("room12_198x94", 198, 94, 12, 48, 2, 512, 32, abi.SGI_CUBE_F16, 4, 5, 2), 77, {}),
    # odd width: the staged path does not apply
    "201x57": (S.Workload("room12_201x57", 201, 57, 12, 48, 0, 512, 32, abi.SGI_CUBE_F32, 4, 5, 2), 78, {}),
    # smaller than one CTA's lattice in both directions
    "6x4": (S.Workload("room12_6x4", 6, 4, 12, 16, 0, 256, 16, abi.SGI_CUBE_F32, 4, 5, 2, tile_size=4,
                       max_per_tile=8), 79, {}),
    # 7 passes: strides 2 .. 32, the staged kernel for 2, 4, 8
    "7passes": (S.Workload("room12_256x128_p7", 256, 128, 12, 48, 0, 512, 32, abi.SGI_CUBE_F32, 4, 7, 2), 80, {}),
}


def _frame(s, staged, fast=False):
    st, cfg = s.stage(1)
    if fast:
        assert st.lib.sgi_set_shading_precision(st.ctx, abi.SGI_SHADING_FAST) == abi.SGI_OK
    assert st.lib.sgi_set_atrous_staging(st.ctx, abi.SGI_ATROUS_STAGED if staged else abi.SGI_ATROUS_DIRECT) \
        == abi.SGI_OK
    H, W = cfg.height, cfg.width
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    st.render_frame(s.g[1], s.g[0], s.hs.camera(1), out, TIME, FPS)
    torch.cuda.synchronize()
    assert st.lib.sgi_device_status(st.ctx) == abi.SGI_OK
    passes = [st.read_debug(abi.SGI_DEBUG_PASS_BASE + p, np.uint16).view(np.float16)
              for p in range(cfg.denoise_passes)]
    r = dict(st=st, cfg=cfg, out=out.cpu().numpy(), passes=passes,
             raw=st.read_debug(abi.SGI_DEBUG_RESERVOIR, np.uint16),
             direct=st.read_debug(abi.SGI_DEBUG_DIRECT, np.uint16),
             idx=st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32))
    return r


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    w, seed, kw = CASES[request.param]
    return GpuSetup(w, seed, **kw)


@pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])
def test_staged_passes_equal_direct_passes(case, fast):
    a = _frame(case, staged=False, fast=fast)
    b = _frame(case, staged=True, fast=fast)
    assert b["st"].lib.sgi_get_atrous_staging(b["st"].ctx) == abi.SGI_ATROUS_STAGED
    for p, (pa, pb) in enumerate(zip(a["passes"], b["passes"])):
        m = half_bits_equal(pa, pb)
        assert m.all(), f"pass {p}: {(~m).sum()} of {m.size} values differ"
    assert half_bits_equal(a["out"], b["out"]).all(), "HDR output"
    a["st"].close()
    b["st"].close()


def test_staged_passes_bit_exact_against_the_oracle(case):
    r = _frame(case, staged=True)
    cfg, st = r["cfg"], r["st"]
    H, W = cfg.height, cfg.width
    res32 = half4_to_f32(r["raw"], H, W)
    direct = half4_to_f32(r["direct"], H, W)
    comb, _, _, passes = O.denoise(32, cfg, case.hs.gbuffers[1], case.hs.gbuffers[0], res32, direct,
                                   np.zeros((H, W, 4), np.float32), np.zeros((H, W), np.float32), int(r["idx"][0]),
                                   TIME, FPS, keep_passes=True)
    for p in range(cfg.denoise_passes):
        assert_bit_exact(r["passes"][p].reshape(H, W, 4).astype(np.float32), passes[p], f"denoise pass {p}")
    assert_bit_exact(r["out"].astype(np.float32)[..., :3], comb[..., :3], "combined HDR output")
    st.close()


def test_staged_wait_runs_out_and_the_next_frame_is_whole():
    s = GpuSetup(S.SMALL, 1235)
    ref = _frame(s, staged=True)
    st, cfg = s.stage(1)
    assert st.lib.sgi_set_atrous_staging(st.ctx, abi.SGI_ATROUS_STAGED) == abi.SGI_OK
    H, W = cfg.height, cfg.width
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    # no copy is issued: every staged CTA's wait runs out after 1 ms with nothing in flight
    assert st.lib.sgi_set_wait_test(st.ctx, 1_000_000, 1) == abi.SGI_OK
    st.render_frame(s.g[1], s.g[0], s.hs.camera(1), out, TIME, FPS)
    assert st.lib.sgi_device_status(st.ctx) == abi.SGI_ERR_TIMEOUT
    assert st.lib.sgi_device_status(st.ctx) == abi.SGI_OK, "the status is cleared once read"
    # the next frame, from the same history state as the reference context's first frame
    assert st.lib.sgi_reset_history(st.ctx, None) == abi.SGI_OK
    assert st.lib.sgi_set_wait_test(st.ctx, 0, 0) == abi.SGI_OK
    st.render_frame(s.g[1], s.g[0], s.hs.camera(1), out, TIME, FPS)
    torch.cuda.synchronize()
    assert st.lib.sgi_device_status(st.ctx) == abi.SGI_OK
    assert half_bits_equal(out.cpu().numpy(), ref["out"]).all()
    assert st.lib.sgi_set_wait_test(st.ctx, -1, 0) == abi.SGI_ERR_ARG
    assert st.lib.sgi_set_atrous_staging(st.ctx, 2) == abi.SGI_ERR_ARG
    st.close()
    ref["st"].close()
