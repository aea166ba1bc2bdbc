"""The tolerance mode of the shading kernels (sgi_set_shading_precision FAST).

The fast build evaluates the gather, the denoise passes and the deferred pass
with approximate division and square root, the hardware exponential and
multiply-add contraction, but computes everything a branch decision or a texel
choice depends on with correctly rounded operations, so it takes the same
branches as the exact build. Each pass is checked on exactly the input it was
given (the fast run's previous pass) against the FP32 oracle:

    relative error = |gpu - oracle| / max(|oracle|, 2^-14)   (2^-14: the
    smallest normal binary16, the storage format of every pass output)
    max relative error <= 1e-3  (the stated tolerance of the FP32 path)

The decision-margin mask of the FP64 oracle (pixels where some comparison lies
within 1e-4 relative of its threshold, or some nearest-texel coordinate within
1e-5 relative of a texel boundary) is reported beside the unmasked error; the
assertion holds on every pixel, masked or not. The culls are exact in both
modes: the tile lists must be identical.
"""
import numpy as np
import pytest

from helpers import GpuSetup, half4_to_f32, psnr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402

TIME, FPS = 1000.0, 60.0
REL_FLOOR = 2.0 ** -14
MAX_REL = 1e-3
CMP_MARGIN, TEX_MARGIN = 1e-4, 1e-5


def rel_err(got, ref):
    g = np.asarray(got, np.float64)
    r = np.asarray(ref, np.float64)
    both_nan = np.isnan(g) & np.isnan(r)
    e = np.abs(g - r) / np.maximum(np.abs(r), REL_FLOOR)
    e[both_nan] = 0.0
    e[np.isnan(e)] = np.inf
    return e


def check(name, got, ref, margins=None):
    e = rel_err(got, ref)
    per_px = e.reshape(e.shape[0], e.shape[1], -1).max(axis=2)
    masked = np.zeros(per_px.shape, bool)
    if margins is not None:
        masked = (margins[..., 0] < CMP_MARGIN) | (margins[..., 1] < TEX_MARGIN)
    outside = float(per_px[~masked].max()) if (~masked).any() else 0.0
    print(f"{name}: max rel err {per_px.max():.3e} (outside the decision-margin mask {outside:.3e}, "
          f"mask {masked.mean():.4%} of pixels)")
    assert per_px.max() <= MAX_REL, f"{name}: max relative error {per_px.max():.3e} at {np.unravel_index(per_px.argmax(), per_px.shape)}"
    return per_px.max()


WORKLOADS = {
    "small": (S.SMALL, 1235),
    # 480x272 with 4 point lights and FP16 cubes (the 1080p configuration's formats)
    "points_f16": (S.Workload("room40_480x272_vpl256_pts4", 480, 272, 40, 256, 4, 1024, 64, abi.SGI_CUBE_F16, 8, 5, 2),
                   4321),
}


@pytest.fixture(scope="module", params=sorted(WORKLOADS))
def fast_frame(request):
    w, seed = WORKLOADS[request.param]
    s = GpuSetup(w, seed, debug_keep_passes=1)
    st, cfg = s.stage(1)
    assert st.lib.sgi_set_shading_precision(st.ctx, abi.SGI_SHADING_FAST) == abi.SGI_OK
    assert st.lib.sgi_get_shading_precision(st.ctx) == abi.SGI_SHADING_FAST
    H, W = cfg.height, cfg.width
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    st.render_frame(s.g[1], s.g[0], s.hs.camera(1), out, TIME, FPS)
    torch.cuda.synchronize()
    r = dict(s=s, cfg=cfg, out=out.cpu().numpy().astype(np.float32))
    r["idx"] = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
    r["lists"] = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + cfg.max_vpls_per_tile)
    r["raw"] = half4_to_f32(st.read_debug(abi.SGI_DEBUG_RESERVOIR, np.uint16), H, W)
    r["direct"] = half4_to_f32(st.read_debug(abi.SGI_DEBUG_DIRECT, np.uint16), H, W)
    r["passes"] = [half4_to_f32(st.read_debug(abi.SGI_DEBUG_PASS_BASE + p, np.uint16), H, W)
                   for p in range(cfg.denoise_passes)]
    r["gi"] = half4_to_f32(st.read_debug(abi.SGI_DEBUG_GI_HISTORY, np.uint16), H, W)
    r["hist"] = st.read_debug(abi.SGI_DEBUG_HISTORY_DEPTH, np.uint16).view(np.float16).reshape(H, W).astype(np.float32)
    st.close()
    return r


def test_fast_mode_keeps_the_culled_lists(fast_frame):
    s, cfg = fast_frame["s"], fast_frame["cfg"]
    ref = O.frame(32, cfg, s.hs, 1, np.zeros((cfg.height, cfg.width, 4), np.float32),
                  np.zeros((cfg.height, cfg.width), np.float32), TIME, FPS)
    cnt = ref["count"]
    assert fast_frame["idx"][0] == cnt
    assert np.array_equal(fast_frame["idx"][1:1 + cnt], ref["visible_index"][1:1 + cnt])
    assert np.array_equal(fast_frame["lists"], ref["lists"])


def _compacted(s, idx):
    cnt = int(idx[0])
    return s.sc.vpls[idx[1:1 + cnt]], s.sc.entries[idx[1:1 + cnt]], cnt


def test_fast_gather_within_tolerance(fast_frame):
    s, cfg = fast_frame["s"], fast_frame["cfg"]
    cv, ce, cnt = _compacted(s, fast_frame["idx"])
    ref = O.gather(32, cfg, s.hs.gbuffers[1], s.hs.camera(1), cv, ce, cnt, fast_frame["lists"], s.hs.cubes, TIME)
    with O.margins(cfg.height, cfg.width) as m:
        O.gather(1, cfg, s.hs.gbuffers[1], s.hs.camera(1), cv, ce, cnt, fast_frame["lists"], s.hs.cubes, TIME)
    check("gather reservoir", fast_frame["raw"], ref, m.m)


def test_fast_deferred_within_tolerance(fast_frame):
    s, cfg = fast_frame["s"], fast_frame["cfg"]
    pts = s.sc.points if len(s.sc.points) else None
    ref = O.deferred(32, cfg, s.hs.gbuffers[1], s.hs.camera(1), pts, s.hs.csms[1])
    with O.margins(cfg.height, cfg.width) as m:
        O.deferred(1, cfg, s.hs.gbuffers[1], s.hs.camera(1), pts, s.hs.csms[1])
    check("deferred PBR + CSM", fast_frame["direct"][..., :3], ref[..., :3], m.m)


def test_fast_denoise_passes_within_tolerance(fast_frame):
    s, cfg = fast_frame["s"], fast_frame["cfg"]
    H, W = cfg.height, cfg.width
    cnt = int(fast_frame["idx"][0])
    z4, z1 = np.zeros((H, W, 4), np.float32), np.zeros((H, W), np.float32)
    n = cfg.denoise_passes
    for p in range(n):
        src = fast_frame["raw"] if p == 0 else fast_frame["passes"][p - 1]
        res, comb, gi, hist = O.denoise_pass(32, cfg, s.hs.gbuffers[1], s.hs.gbuffers[0], p, src,
                                             fast_frame["direct"], z4, z1, cnt, TIME, FPS)
        with O.margins(H, W) as m:
            O.denoise_pass(1, cfg, s.hs.gbuffers[1], s.hs.gbuffers[0], p, src, fast_frame["direct"], z4, z1, cnt,
                           TIME, FPS)
        check(f"denoise pass {p}", fast_frame["passes"][p][..., :3], res[..., :3], m.m)
        if p == n - 1:
            check("combined HDR", fast_frame["out"][..., :3], comb[..., :3], m.m)
            check("GI history", fast_frame["gi"][..., :3], gi[..., :3], m.m)
            assert np.array_equal(fast_frame["hist"], hist), "history length is a decision: identical in both modes"


def test_fast_frame_psnr_against_fp64(fast_frame):
    s, cfg = fast_frame["s"], fast_frame["cfg"]
    H, W = cfg.height, cfg.width
    ref64 = O.frame(64, cfg, s.hs, 1, np.zeros((H, W, 4)), np.zeros((H, W)), TIME, FPS)
    p = psnr(fast_frame["out"][..., :3].astype(np.float64), ref64["combined"][..., :3])
    print(f"fast frame PSNR vs the FP64 oracle: {p:.1f} dB")
    assert p > 50.0
