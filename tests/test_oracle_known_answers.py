"""Known answers of the oracle's denoise and tile-cull passes (no GPU).

StratusGFX has no shader tests, so these pin the restated passes to properties
that follow from the shader formulas alone, with answers computed here
independently:

* an a-trous pass (vpl_pbr_gi_denoise.fs:142-190, :307-327) leaves a constant
  reservoir unchanged: every tap is the same value, and the result is the
  weighted sum divided by the sum of the weights;
* across opposite normals the edge-stopping weight max(0, n_c . n_q)^128 is
  zero, so a step edge between two such regions stays sharp;
* the temporal pass (:336-429) with zero motion over an unchanged surface
  counts the history up by one per frame until it reaches the frame rate, and
  blends previous and current GI with weight 1 / history; a changed object id
  resets the history to 1;
* the stage-2 tile lists (vpl_tiled_deferred_culling_stage2.cs:61-129) of a
  hand-built VPL grid with integer coordinates hold the VPLs in front of the
  tile's plane within their radius, nearest first, ties in index order.
"""
import numpy as np
import pytest

from oracle import binding as O
from stratusgfx_gb300 import abi

W, H = 24, 16
FPS = 30.0


def encode_normal(n):
    """RGB8 bytes of a unit normal as pbr_geometry_pass.fs stores it (n * 0.5 + 0.5)."""
    return np.clip(np.round((np.asarray(n, np.float64) * 0.5 + 0.5) * 255.0), 0, 255).astype(np.uint8)


def gbuffer(rng, normals=None, depth=None, ids=None):
    g = O.HostGBuffer(H, W)
    g.depth[:] = rng.uniform(0.2, 0.9, (H, W)).astype(np.float32) if depth is None else depth
    if normals is None:
        v = rng.normal(0, 1, (H, W, 3))
        v /= np.linalg.norm(v, axis=2, keepdims=True)
        normals = v
    g.normal[..., :3] = encode_normal(normals)
    g.albedo[:] = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    g.rma[:] = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    g.id[:] = 7.0 if ids is None else ids
    return g


def config(passes=4):
    cfg = abi.config_defaults(W, H)
    cfg.denoise_passes = passes
    return cfg


def run_pass(prec, cfg, cur, prev, p, res, gi_prev=None, hist_prev=None):
    z4 = np.zeros((H, W, 4), np.float64)
    return O.denoise_pass(prec, cfg, cur, prev, p, res, z4, z4 if gi_prev is None else gi_prev,
                          np.zeros((H, W)) if hist_prev is None else hist_prev, 64, 1000.0, FPS)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("p", [1, 2])
def test_atrous_pass_leaves_a_constant_reservoir_unchanged(prec, p):
    rng = np.random.default_rng(10 + p)
    cfg = config()
    g = gbuffer(rng)
    c = np.array([0.75, 1.5, 0.125, 1.0])   # binary16 values
    res = np.broadcast_to(c, (H, W, 4)).copy()
    out = run_pass(prec, cfg, g, g, p, res)[0]
    if prec == 64:
        assert np.abs(out[..., :3] - c[:3]).max() <= 1e-12
    else:   # the float32 quotient is within an ulp of c, and the binary16 store rounds it to c
        assert np.array_equal(out[..., :3], np.broadcast_to(c[:3], (H, W, 3)).astype(np.float32))
    assert np.all(out[..., 3] == 1.0)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("p", [1, 2])
def test_atrous_pass_keeps_a_step_edge_between_opposite_normals(prec, p):
    rng = np.random.default_rng(20 + p)
    cfg = config()
    n = np.zeros((H, W, 3))
    n[:, : W // 2, 0] = 1.0
    n[:, W // 2:, 0] = -1.0
    g = gbuffer(rng, normals=n, depth=np.full((H, W), 0.5, np.float32))
    res = np.zeros((H, W, 4))
    res[:, : W // 2] = (0.5, 0.5, 0.5, 1.0)
    res[:, W // 2:] = (2.0, 2.0, 2.0, 1.0)
    out = run_pass(prec, cfg, g, g, p, res)[0]
    assert np.all(out[:, : W // 2, :3] == 0.5)
    assert np.all(out[:, W // 2:, :3] == 2.0)


@pytest.mark.parametrize("prec", [32, 64])
def test_temporal_pass_counts_history_to_the_frame_rate_and_blends(prec):
    rng = np.random.default_rng(30)
    cfg = config()
    final = cfg.denoise_passes - 1
    n = np.zeros((H, W, 3))
    n[..., 2] = 1.0
    g = gbuffer(rng, normals=n, depth=np.full((H, W), 0.5, np.float32))   # cur == prev, zero velocity
    c = np.array([0.75, 1.5, 0.125, 1.0])
    res = np.broadcast_to(c, (H, W, 4)).copy()
    gprev = np.broadcast_to(np.array([0.25, 0.5, 1.0, 1.0]), (H, W, 4)).copy()
    tol = 1e-12 if prec == 64 else 2e-3   # binary16 outputs in the FP32 oracle
    for h in (0.0, 1.0, 5.0, FPS - 1.0, FPS, FPS + 3.0):
        _, comb, gi, hist = run_pass(prec, cfg, g, g, final, res, gprev, np.full((H, W), h))
        want_h = min(h + 1.0, FPS)
        assert np.all(hist == np.float32(want_h)), (h, np.unique(hist))
        want = gprev[..., :3] * (1.0 - 1.0 / want_h) + c[:3] / want_h
        assert np.abs(gi[..., :3] - want).max() <= tol * np.abs(want).max(), h
        # combined = screen (zero here) + (max(albedo, 0.01) + 1e-5 as binary16) * gi
        alb = np.maximum(g.albedo[..., :3].astype(np.float64) / 255.0, 0.01) + 1e-5
        alb16 = alb.astype(np.float16).astype(np.float64) if prec == 32 else alb
        assert np.abs(comb[..., :3] - alb16 * gi[..., :3]).max() <= tol * max(1.0, np.abs(comb).max())
    # another object id at the same place: no history, the current estimate alone
    prev = gbuffer(np.random.default_rng(30), normals=n, depth=np.full((H, W), 0.5, np.float32), ids=9.0)
    _, _, gi, hist = run_pass(prec, cfg, g, prev, final, res, gprev, np.full((H, W), 12.0))
    assert np.all(hist == 1.0)
    assert np.abs(gi[..., :3] - c[:3]).max() <= tol


def grid_vpls():
    pts = np.array([(x, y, z) for z in (-1, 0, 1, 2) for y in range(-3, 4) for x in range(-3, 4)], np.float32)
    v = np.zeros((len(pts), 16), np.float32)
    v[:, :3] = pts
    v[:, 3] = 1.0
    v[:, 12] = 4.0    # radius: ratio <= 1 <=> |L - p|^2 <= 16
    v[:, 13] = 100.0
    v[:, 14] = 1.0
    return v


def expected_list(vpls, pos, normal, L):
    lmf = vpls[:, :3].astype(np.float64) - np.asarray(pos, np.float64)
    side = lmf @ np.asarray(normal, np.float64)
    d2 = (lmf ** 2).sum(axis=1)
    keep = [k for k in range(len(vpls)) if side[k] >= 0 and d2[k] <= 16.0]
    keep.sort(key=lambda k: (d2[k], k))
    return keep[:L], len(keep)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("L", [12, 64])
def test_tile_lists_of_a_hand_built_vpl_grid(prec, L):
    cfg = abi.config_defaults(32, 16)
    cfg.tile_size = 16
    cfg.max_vpls_per_tile = L
    tiles = [((0.0, 0.0, 0.0), (0.0, 0.0, 1.0)),    # floor tile at the origin
             ((1.0, 0.0, 0.0), (1.0, 0.0, 0.0))]    # wall tile facing +x
    stage1 = np.array([[*p, 1.0, *n, 1.0] for p, n in tiles])
    vpls = grid_vpls()
    lists = O.tile_stage2(prec, cfg, stage1, vpls, len(vpls))
    for t, (p, n) in enumerate(tiles):
        want, candidates = expected_list(vpls, p, n, L)
        assert candidates > 12   # more candidates than the reference cap: the list is a selection
        assert lists[t, 0] == len(want)
        assert list(lists[t, 1:1 + len(want)]) == want
        assert np.all(lists[t, 1 + len(want):] == -1)
