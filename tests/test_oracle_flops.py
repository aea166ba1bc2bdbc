"""The oracle's operation-counting instantiation (oracle/counted.hpp), which
gives the algorithmic FLOPs behind the FP32 roofline of the shading kernels.

It must follow the FP32 oracle exactly (same branches, same values), and its
tally must equal a count worked out by hand from the restated shader lines for
a pass whose work does not depend on the data.
"""
import numpy as np
import pytest

from oracle import binding as O
from stratusgfx_gb300 import scene as S
from stratusgfx_gb300 import stage

TIME, FPS = 1000.0, 60.0


@pytest.fixture(scope="module")
def small():
    w = S.SMALL
    sc = S.workload_scene(w, 1235)
    return w, sc, O.HostScene(sc, w), stage.workload_config(w)


def test_counting_instantiation_equals_fp32(small):
    w, sc, hs, cfg = small
    H, W = w.height, w.width
    z4, z1 = np.zeros((H, W, 4), np.float32), np.zeros((H, W), np.float32)
    r = O.frame(32, cfg, hs, 1, z4, z1, TIME, FPS, keep=True)
    idx = O.vis_cull(0, sc.vpls, hs.csms[1], cfg.max_visible)
    assert np.array_equal(idx, r["visible_index"])
    cnt = int(idx[0])
    cv, ce = sc.vpls[idx[1:1 + cnt]], sc.entries[idx[1:1 + cnt]]
    s1 = O.tile_stage1(0, cfg, hs.gbuffers[1], hs.camera(1))
    assert np.array_equal(s1.view(np.uint32), r["stage1"].view(np.uint32))
    assert np.array_equal(O.tile_stage2(0, cfg, s1, cv, cnt), r["lists"])
    g = O.gather(0, cfg, hs.gbuffers[1], hs.camera(1), cv, ce, cnt, r["lists"], hs.cubes, TIME)
    assert np.array_equal(g.view(np.uint32), r["reservoir"].view(np.uint32))
    d = O.deferred(0, cfg, hs.gbuffers[1], hs.camera(1), None, hs.csms[1])
    assert np.array_equal(d.view(np.uint32), r["direct"].view(np.uint32))
    comb, gi, hist, _ = O.denoise(0, cfg, hs.gbuffers[1], hs.gbuffers[0], g, d, z4, z1, cnt, TIME, FPS)
    for a, b in ((comb, r["combined"]), (gi, r["gi"]), (hist, r["hist"])):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_tile_stage1_count_matches_the_hand_count(small):
    """Per pixel: uv 2 x (add, div) = 4; worldPositionFromDepth: 2 (depth*2-1) + 4 (uv*2-1) + 4 rows x
    (mul + 3 fma) = 28 + the divide by w (reciprocal + 3 mul) = 4, i.e. 38; the normal decode: 3 divides
    by 255, 3 mul + 3 sub, normalize = dot (mul + 2 fma = 5) + sqrt + reciprocal + 3 mul = 10, i.e. 19.
    61 per pixel inside the image. Per 16x16 tile: six butterfly sums over 8 warps (5 x 32 adds per warp,
    then 3 x 8 over the warp totals: 1304 each) and the two means (4 each) plus a normalize (10)."""
    w, sc, hs, cfg = small
    O.count_reset()
    O.tile_stage1(0, cfg, hs.gbuffers[1], hs.camera(1))
    flops, cmps = O.count_read()
    T = ((w.width + 15) // 16) * ((w.height + 15) // 16)
    assert flops == w.width * w.height * 61 + T * (6 * 1304 + 18)
    assert cmps == 0


def test_frame_flops_reports_every_kernel(small):
    w, sc, hs, cfg = small
    H, W = w.height, w.width
    fl = O.frame_flops(cfg, hs, 1, np.zeros((H, W, 4), np.float32), np.zeros((H, W), np.float32), TIME, FPS)
    assert set(fl) == {"vpl_cull", "direct", "tile_stage1", "tile_stage2", "gather", "denoise_pass0", "atrous",
                       "denoise_final"}
    P = W * H
    # a-trous: 3 passes x 24 weighted taps, each with an exp, a pow(x, 128) and a 3-term dot product
    assert 3 * 24 * 20 * P < fl["atrous"][0] < 3 * 25 * 80 * P
    assert fl["gather"][0] > 8 * 100 * P * 0.5
