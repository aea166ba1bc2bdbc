"""Known-answer tests of the CPU oracle's built-ins and shading formulas (no GPU).

StratusGFX ships no shader tests or golden vectors, so these pin the oracle to
independent evaluations of the shader formulas (Python, float64) and to
properties that follow from them.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import binding as O
from stratusgfx_gb300 import abi


def py_hash(x):
    """common.glsl:183-190 on uint32."""
    m = 0xFFFFFFFF
    x = (x + (x << 10)) & m
    x ^= x >> 6
    x = (x + (x << 3)) & m
    x ^= x >> 11
    x = (x + (x << 15)) & m
    return x


def py_random3(x, y, z):
    b = lambda f: int(np.float32(f).view(np.uint32))  # noqa: E731
    h = py_hash(b(x) ^ py_hash(b(y)) ^ py_hash(b(z)))
    m = (h & 0x007FFFFF) | 0x3F800000
    return float(np.uint32(m).view(np.float32)) - 1.0


def test_hash_and_random_match_independent_python():
    lib = O.load()
    rng = np.random.default_rng(0)
    for x in list(rng.integers(0, 2**32, 200)) + [0, 1, 0xFFFFFFFF]:
        assert lib.oracle_hash(int(x)) == py_hash(int(x))
    for (x, y, z) in [(0.5, 0.5, 0.0), (1919.5, 1079.5, 1000.0), (17.5, 3.5, 11000.0)] + \
            [tuple(rng.uniform(0, 4000, 3)) for _ in range(100)]:
        r = lib.oracle_random3(x, y, z)
        assert r == np.float32(py_random3(x, y, z))
        assert 0.0 <= r < 1.0


def test_seed_step_is_absorbed_at_epoch_millisecond_times():
    """vpl_pbr_gi.fs:132-150 seeds z with milliseconds since the epoch (~1.7e12): in binary32
    seed.z += 10000.0 rounds back to seed.z, so all draws of a pixel repeat. Small times do not."""
    t = np.float32(1.7e12)
    assert np.float32(t + np.float32(10000.0)) == t
    assert np.float32(np.float32(1000.0) + np.float32(10000.0)) != np.float32(1000.0)


def test_exp_is_accurate_and_exact_at_zero():
    lib = O.load()
    assert lib.oracle_exp_f32(0.0) == 1.0
    assert lib.oracle_exp_f32(-0.0) == 1.0
    xs = np.concatenate([np.linspace(-87, 88, 20001), -np.abs(np.random.default_rng(1).normal(size=2000))])
    worst = 0.0
    for x in xs:
        x = float(np.float32(x))
        got = lib.oracle_exp_f32(x)
        ref = math.exp(x)
        worst = max(worst, abs(got - ref) / ref)
    assert worst < 5e-7, worst     # a few binary32 ulps
    assert lib.oracle_exp_f32(-200.0) == 0.0
    assert math.isinf(lib.oracle_exp_f32(100.0))


def test_pow128_accuracy():
    lib = O.load()
    for x in np.linspace(0.0, 1.0, 1001):
        x = float(np.float32(x))
        ref = x ** 128
        got = lib.oracle_pow128_f32(x)
        assert abs(got - ref) <= 2e-5 * ref + 1e-38


def test_float_to_half_rounding_matches_ieee_rne():
    lib = O.load()
    rng = np.random.default_rng(3)
    vals = np.concatenate([rng.normal(scale=s, size=3000) for s in (1e-6, 1e-3, 1.0, 100.0, 3e4)]).astype(np.float32)
    specials = np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, 7e4, 2.0**-24, 2.0**-25, 1.5 * 2.0**-25,
                         2.0**-14, 2.0**-14 - 2.0**-25, 1.0 + 2.0**-11, 1.0 + 3 * 2.0**-11, np.inf, -np.inf],
                        dtype=np.float32)
    for v in np.concatenate([vals, specials]):
        assert lib.oracle_f32_to_f16(float(v)) == int(np.float16(v).view(np.uint16)), v
        h = np.float16(v)
        if np.isfinite(h):
            assert lib.oracle_f16_to_f32(int(h.view(np.uint16))) == float(h)


def test_world_position_round_trip():
    from stratusgfx_gb300 import scene as S
    proj = S.perspective(math.radians(60.0), 16 / 9, 0.1, 30.0)
    view = S.look_at((1.0, 2.0, 3.0), (8.0, 0.5, 5.0), (0.0, 1.0, 0.0))
    pv = proj @ view
    inv = S.colmajor(np.linalg.inv(pv))
    out = np.zeros(3)
    for p in [(5.0, 0.0, 4.0), (9.9, 3.0, 6.0), (4.0, 1.0, 2.5)]:
        c = pv @ np.array([*p, 1.0])
        ndc = c[:3] / c[3]
        u, v, d = ndc[0] * 0.5 + 0.5, ndc[1] * 0.5 + 0.5, ndc[2] * 0.5 + 0.5
        for prec, tol in ((64, 1e-4), (32, 2e-3)):   # the matrix itself is binary32
            O.load().oracle_world_from_depth(prec, u, v, d, inv.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p))
            assert np.allclose(out, p, atol=tol), (prec, out, p)


def py_vpl_lighting(frag, n, v, spec, diff, color, dist, radius, rough, metal, ao, refl, base, min_r=0.08):
    """calculateVirtualPointLighting2 (pbr2.glsl:613-657) evaluated independently in float64."""
    frag, n, v, spec, diff, color, base = map(np.asarray, (frag, n, v, spec, diff, color, base))
    eps, pi = 1e-5, 3.14159265359
    sdir, ddir = spec - frag, diff - frag

    def atten(d):
        L = np.linalg.norm(d)
        ratio = min(L / radius, 1.0)
        md = (10 * (1 - math.exp(-3 * ratio)) + 1 * math.exp(-3 * ratio)) * radius
        return 1.0 / (md + L * L)

    rr = max(max(0.0, min_r), rough * rough)
    dc = (1 - metal) * base / (base + eps)
    f0 = (0.16 * refl * refl * (1 - metal) + base * metal) * (1.0 / (base + eps))

    def dots(ld):
        L = ld / np.linalg.norm(ld)
        H = (v + L) / np.linalg.norm(v + L)
        sat = lambda x: min(max(x, 0.0), 1.0)  # noqa: E731
        return sat(n @ v), sat(n @ L), sat(n @ H), sat(L @ H)

    NdV, NdL, NdH, LdH = dots(sdir)
    r2 = rr * rr
    fq = (NdH * r2 - NdH) * NdH + 1
    ndf = r2 / max(pi * fq * fq, eps)
    vis = 0.5 / max(NdL * math.sqrt((NdV - r2 * NdV) * NdV + r2) + NdV * math.sqrt((NdL - r2 * NdL) * NdL + r2), eps)
    fr = (1 - LdH) ** 5
    fres = fr + f0 * (1 - fr)
    spec_t = ndf * vis * fres * NdL
    _, NdL2, _, _ = dots(ddir)
    diff_t = dc / pi * NdL2
    brdf = atten(sdir) * spec_t + atten(ddir) * diff_t
    return brdf * color


@pytest.mark.parametrize("case", range(6))
def test_vpl_brdf_matches_independent_evaluation(case):
    rng = np.random.default_rng(100 + case)
    frag = rng.uniform(0, 10, 3)
    n = rng.normal(size=3); n /= np.linalg.norm(n)
    cam = frag + n * 3 + rng.normal(size=3)
    v = (cam - frag) / np.linalg.norm(cam - frag)
    diff = frag + n * 2 + rng.normal(size=3) * 0.5
    spec = diff + rng.normal(size=3) * 0.01
    color = rng.uniform(1, 100, 3)
    base = rng.uniform(0.05, 0.95, 3)
    rough, metal, refl = rng.uniform(0.5, 1.0), float(case % 2), 0.5
    inp = np.zeros(27)
    inp[0:3], inp[3:6], inp[6:9], inp[9:12], inp[12:15], inp[15:18] = frag, n, v, spec, diff, color
    inp[18], inp[19], inp[20], inp[21], inp[22], inp[23] = np.linalg.norm(cam - frag), 8.0, rough, metal, 1.0, refl
    inp[24:27] = base
    cfg = abi.Config()
    O.load()
    lib = abi.load(build_if_missing=True)
    lib.sgi_config_defaults(C.byref(cfg), 8, 8)
    ref = py_vpl_lighting(frag, n, v, spec, diff, color, inp[18], 8.0, rough, metal, 1.0, refl, base)
    for prec, tol in ((64, 1e-12), (32, 2e-5)):
        out = np.zeros(3)
        O.load().oracle_vpl_brdf(prec, inp.ctypes.data_as(C.c_void_p), C.byref(cfg), out.ctypes.data_as(C.c_void_p))
        assert np.allclose(out, ref, rtol=tol, atol=1e-12), (prec, out, ref)


def test_vpl_coloring_known_answer():
    """vpl_light_color.cs on one VPL 0.25 m above a floor box, sun straight overhead:
    the diffuse cube in direction -L sees the floor's albedo and the distance cube
    the floor, so color = albedo * sun * intensity * 50000 and the specular position
    lies 1.1 * radius * depth below the VPL."""
    box = np.zeros((1, 16), np.float32)
    box[0, 0:3], box[0, 4:7] = (-5.0, -1.0, -5.0), (5.0, 0.0, 5.0)
    box[0, 8:12] = (0.5, 0.25, 1.0, 1.0)                  # albedo rgba
    vpl = np.zeros((1, 16), np.float32)
    vpl[0, 0:4] = (0.3, 0.25, -0.2, 1.0)
    vpl[0, 12], vpl[0, 13], vpl[0, 14] = 2.0, 4.0, 0.001  # radius, far plane, intensity
    entries = np.zeros((1, 2), np.int32)
    storage, cubes = O.scene_cubes(box, vpl, entries, 8, abi.SGI_CUBE_F32)
    dstore, diffuse = O.scene_diffuse(box, vpl, entries, 8)
    csm = abi.Csm()
    csm.light_direction[0:4] = [0.0, 1.0, 0.0, 0.0]
    csm.light_color[0:4] = [3.0, 2.0, 1.0, 1.0]
    out = O.color_vpls(64, vpl, entries, 1, cubes, diffuse, csm)
    alb = np.array([round(0.5 * 255) / 255, round(0.25 * 255) / 255, 1.0])
    np.testing.assert_allclose(out[0, 4:7], alb * [3.0, 2.0, 1.0] * 0.001 * 50000, rtol=1e-6)
    assert out[0, 7] == 1.0
    # the nearest texel to straight down (face -y, texel (4, 4) of 8) looks along (1/8, -1, -1/8)
    depth = 0.25 * math.sqrt(1.0 + 2.0 / 64.0) / 4.0        # distance along that ray / far plane
    np.testing.assert_allclose(out[0, 8:11], [0.3, 0.25 - 1.1 * 2.0 * depth, -0.2], rtol=1e-5, atol=1e-6)
    assert out[0, 11] == 1.0
    # the texel straight down holds the floor's colour; straight up sees nothing (0)
    assert dstore[0, 0, 3].max() == (128 | (64 << 8) | (255 << 16) | (255 << 24))
    assert dstore[0, 0, 2].max() == 0


def _kat_scene():
    from stratusgfx_gb300 import scene as S
    from stratusgfx_gb300 import stage
    w = S.Workload("room12_48x32_kat", 48, 32, 12, 8, 2, 256, 8, abi.SGI_CUBE_F32, 4, 3, 1)
    sc = S.workload_scene(w, 77)
    hs = O.HostScene(sc, w)
    return w, sc, hs, stage.workload_config(w)


def test_shadow_caster_with_empty_cube_equals_plain_point_light():
    """A shadow-casting point light whose distance cube is all 1.0 (nothing within its
    far plane) gets shadow factor 0 from both the 8-sample and the 1-sample filter, so
    pbr.fs adds exactly what the same light adds as a non-shadow caster."""
    w, sc, hs, cfg = _kat_scene()
    lights = sc.points.copy()
    empty = np.ones((1, 320, 6, 8, 8), np.float32)
    atlas = O.cube_struct(empty, abi.SGI_CUBE_F32)
    entries = np.array([[0, k] for k in range(lights.shape[0])], np.int32)
    ref = O.deferred(32, cfg, hs.gbuffers[1], hs.camera(1), lights, hs.csms[1])
    got = O.deferred(32, cfg, hs.gbuffers[1], hs.camera(1), None, hs.csms[1], lights, entries, atlas)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    # a cube at depth 0 everywhere occludes every tap: the lights then add less
    full = O.cube_struct(np.zeros((1, 320, 6, 8, 8), np.float32), abi.SGI_CUBE_F32)
    dark = O.deferred(32, cfg, hs.gbuffers[1], hs.camera(1), None, hs.csms[1], lights, entries, full)
    none = O.deferred(32, cfg, hs.gbuffers[1], hs.camera(1), None, hs.csms[1])
    lit = ref[..., :3].sum()
    assert none[..., :3].sum() <= dark[..., :3].sum() < lit


def test_post_fx_known_answers():
    """gammaTonemap.fs: ACES film then gamma 1/2.2 to RGBA8 (0 -> 0, 1 -> 231, saturating
    colours -> 255); taa.fs: a history far outside the current pixel's neighbourhood is
    clamped to it, so on a flat image the TAA output is the image itself."""
    H, W = 6, 8
    vel = np.zeros((H, W), np.uint32)
    for val, want in ((0.0, 0), (1.0, 231), (500.0, 255)):
        hdr = np.full((H, W, 4), val, np.float16)
        ldr, _ = O.post_fx(64, hdr, vel, None, taa=False)
        assert (ldr & 0xff).max() == want and (ldr & 0xff).min() == want, (val, ldr & 0xff)
        assert ((ldr >> 24) == 255).all()
    aces1 = 2.54 / 3.16
    assert round(aces1 ** (1 / 2.2) * 255) == 231
    hdr = np.full((H, W, 4), 0.75, np.float16)
    hist = np.full((H, W, 4), 40.0, np.float32)
    ldr, taa = O.post_fx(64, hdr, vel, hist, taa=True)
    np.testing.assert_allclose(taa[..., :3], 0.75, rtol=1e-3)
    assert (taa[..., 3] == 0.0625).all()
    ref, _ = O.post_fx(64, hdr, vel, None, taa=False)
    assert np.array_equal(ldr, ref)
