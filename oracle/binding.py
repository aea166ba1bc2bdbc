"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as the
checker / CPU baseline. Parity of the oracle itself is UNPINNED by the
reference (StratusGFX has no golden vectors; its GLSL needs an OpenGL driver).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from oracle import build as _build  # noqa: E402
from stratusgfx_gb300 import abi  # noqa: E402  (struct layouts of include/sgi.h only)

_lib = None


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(_build.build())
        P = C.c_void_p
        sig = {
            "oracle_version": (C.c_int, []),
            "oracle_random3": (C.c_float, [C.c_float, C.c_float, C.c_float]),
            "oracle_hash": (C.c_uint32, [C.c_uint32]),
            "oracle_exp_f32": (C.c_float, [C.c_float]),
            "oracle_pow128_f32": (C.c_float, [C.c_float]),
            "oracle_f32_to_f16": (C.c_uint16, [C.c_float]),
            "oracle_f16_to_f32": (C.c_float, [C.c_uint16]),
            "oracle_world_from_depth": (None, [C.c_int, C.c_double, C.c_double, C.c_double, P, P]),
            "oracle_vpl_brdf": (None, [C.c_int, P, C.POINTER(abi.Config), P]),
            "oracle_infinite_shadow": (None, [C.c_int, C.POINTER(abi.Csm), P, P, C.c_int, C.c_int, P]),
            "oracle_vis_cull": (C.c_int, [C.c_int, P, C.c_int, C.POINTER(abi.Csm), C.c_int, P]),
            "oracle_tile_stage1": (None, [C.c_int, C.POINTER(abi.Config), C.POINTER(abi.GBuffer), C.POINTER(abi.Camera), P]),
            "oracle_tile_stage2": (None, [C.c_int, C.POINTER(abi.Config), P, P, C.c_int, P]),
            "oracle_gather": (None, [C.c_int, C.POINTER(abi.Config), C.POINTER(abi.GBuffer), C.POINTER(abi.Camera), P,
                                     P, C.c_int, P, C.POINTER(abi.CubeAtlas), C.c_float, P]),
            "oracle_gi_target": (None, [C.POINTER(abi.Config), C.POINTER(abi.GBuffer), C.POINTER(abi.Camera), P, P,
                                        C.c_int, P, C.POINTER(abi.CubeAtlas), C.c_float, C.c_int, P]),
            "oracle_denoise": (None, [C.c_int, C.POINTER(abi.Config), C.POINTER(abi.GBuffer), C.POINTER(abi.GBuffer),
                                      P, P, P, P, C.c_int, C.POINTER(abi.FrameParams), P, P, P, P, P]),
            "oracle_count_reset": (None, []),
            "oracle_set_margin_output": (None, [P]),
            "oracle_denoise_pass": (None, [C.c_int, C.POINTER(abi.Config), C.POINTER(abi.GBuffer),
                                           C.POINTER(abi.GBuffer), C.c_int, P, P, P, P, C.c_int,
                                           C.POINTER(abi.FrameParams), P, P, P, P]),
            "oracle_count_read": (None, [P]),
            "oracle_deferred": (None, [C.c_int, C.POINTER(abi.Config), C.POINTER(abi.GBuffer), C.POINTER(abi.Camera),
                                       P, C.c_int, C.POINTER(abi.Csm), P, P, P, C.c_int, C.POINTER(abi.CubeAtlas)]),
            "oracle_scene_gbuffer": (None, [P, C.c_int, C.POINTER(abi.SceneCamera), C.c_int, C.c_int, P, P, P, P, P,
                                            P, P, P]),
            "oracle_scene_csm": (None, [P, C.c_int, C.POINTER(abi.Csm), P, P]),
            "oracle_scene_cube_atlas": (None, [P, C.c_int, P, P, C.c_int, C.POINTER(abi.CubeAtlas)]),
            "oracle_scene_diffuse_atlas": (None, [P, C.c_int, P, P, C.c_int, C.POINTER(abi.DiffuseAtlas)]),
            "oracle_post_fx": (None, [C.c_int, C.c_int, C.c_int, P, P, P, P, P, C.c_int]),
            "oracle_color_vpls": (None, [C.c_int, P, P, C.c_int, C.POINTER(abi.CubeAtlas), C.POINTER(abi.DiffuseAtlas),
                                         C.POINTER(abi.Csm)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _dt(prec):
    """Buffer dtype of an instantiation: 32 float, 64 double, 0 the counting float instantiation,
    1 the margin-tracking double instantiation."""
    return np.float64 if prec in (64, 1) else np.float32


class margins:
    """Context manager: prec = 1 passes run inside it write each pixel's smallest decision margins
    (see oracle/counted.hpp, Tracked) into self.m ([H, W, 2] float64: comparisons, texel choices)."""

    def __init__(self, H, W):
        self.m = np.full((H, W, 2), np.inf)

    def __enter__(self):
        load().oracle_set_margin_output(_p(self.m))
        return self

    def __exit__(self, *exc):
        load().oracle_set_margin_output(None)
        return False


def denoise_pass(prec, cfg, cur: HostGBuffer, prev: HostGBuffer, pass_index, res_in, hdr_in, gi_prev, hist_prev,
                 num_visible, time, fps):
    """One denoise pass from res_in: returns (res_out, combined, gi, hist) (the last three only filled on
    the final pass)."""
    H, W = cfg.height, cfg.width
    dt = _dt(prec)
    keep = [np.ascontiguousarray(a, dtype=dt) for a in (res_in, hdr_in, gi_prev, hist_prev)]
    res_out = np.zeros((H, W, 4), dt)
    comb = np.zeros((H, W, 4), dt)
    gi = np.zeros((H, W, 4), dt)
    hist = np.zeros((H, W), dt)
    fp = abi.FrameParams(time, fps)
    load().oracle_denoise_pass(prec, C.byref(cfg), C.byref(cur.struct()), C.byref(prev.struct()), pass_index,
                               *[_p(a) for a in keep], num_visible, C.byref(fp), _p(res_out), _p(comb), _p(gi),
                               _p(hist))
    return res_out, comb, gi, hist


class HostGBuffer:
    """numpy G-buffer planes (same shapes/dtypes as stage.GBufferTensors)."""

    NAMES = ("depth", "normal", "albedo", "base_reflectivity", "rma", "velocity", "id", "ssao")

    def __init__(self, H, W, arrays=None):
        if arrays is None:
            arrays = dict(depth=np.zeros((H, W), np.float32), normal=np.zeros((H, W, 4), np.uint8),
                          albedo=np.zeros((H, W, 4), np.uint8), base_reflectivity=np.zeros((H, W, 2), np.uint8),
                          rma=np.zeros((H, W, 4), np.uint8), velocity=np.zeros((H, W, 2), np.float16),
                          id=np.zeros((H, W), np.float32), ssao=np.zeros((H, W), np.float16))
        for k in self.NAMES:
            setattr(self, k, np.ascontiguousarray(arrays[k]))

    def struct(self) -> abi.GBuffer:
        return abi.GBuffer(*[getattr(self, k).ctypes.data for k in self.NAMES])

    def arrays(self):
        return {k: getattr(self, k) for k in self.NAMES}


def scene_gbuffer(boxes, cam: abi.SceneCamera, W, H) -> HostGBuffer:
    g = HostGBuffer(H, W)
    load().oracle_scene_gbuffer(_p(boxes), boxes.shape[0], C.byref(cam), W, H, *[_p(getattr(g, k)) for k in g.NAMES])
    return g


def scene_csm(boxes, csm: abi.Csm, inv: np.ndarray, R) -> np.ndarray:
    out = np.zeros((4, R, R), np.float32)
    inv = np.ascontiguousarray(inv, dtype=np.float32)
    load().oracle_scene_csm(_p(boxes), boxes.shape[0], C.byref(csm), _p(inv), _p(out))
    return out


def scene_cubes(boxes, vpls, entries, face, fmt, layers=320):
    n = vpls.shape[0]
    na = max(1, (n + layers - 1) // layers)
    storage = np.zeros((na, layers, 6, face, face), np.float32 if fmt == abi.SGI_CUBE_F32 else np.uint16)
    at = abi.CubeAtlas()
    for a in range(na):
        at.atlas[a] = storage[a].ctypes.data
    at.num_atlases, at.layers_per_atlas, at.face_size, at.format = na, layers, face, fmt
    if n:
        v = np.ascontiguousarray(vpls, dtype=np.float32)
        e = np.ascontiguousarray(entries, dtype=np.int32)
        load().oracle_scene_cube_atlas(_p(boxes), boxes.shape[0], _p(v), _p(e), n, C.byref(at))
    return storage, at


def scene_diffuse(boxes, vpls, entries, face, layers=320):
    """Diffuse colour cubes (RGBA8 texels as uint32) of the CPU ray caster, and their sgi_diffuse_atlas."""
    n = vpls.shape[0]
    na = max(1, (n + layers - 1) // layers)
    storage = np.zeros((na, layers, 6, face, face), np.uint32)
    at = diffuse_struct(storage, layers)
    if n:
        v = np.ascontiguousarray(vpls, dtype=np.float32)
        e = np.ascontiguousarray(entries, dtype=np.int32)
        load().oracle_scene_diffuse_atlas(_p(boxes), boxes.shape[0], _p(v), _p(e), n, C.byref(at))
    return storage, at


def diffuse_struct(storage: np.ndarray, layers: int = 320) -> abi.DiffuseAtlas:
    at = abi.DiffuseAtlas()
    for a in range(storage.shape[0]):
        at.atlas[a] = storage[a].ctypes.data
    at.num_atlases, at.layers_per_atlas, at.face_size = storage.shape[0], layers, storage.shape[-1]
    return at


def color_vpls(prec, cvpls, centries, count, cubes: abi.CubeAtlas, diffuse: abi.DiffuseAtlas, csm: abi.Csm):
    """vpl_light_color.cs on the compacted VPLs (a recoloured copy)."""
    out = np.array(cvpls, dtype=np.float32, copy=True, order="C")
    e = np.ascontiguousarray(centries, dtype=np.int32)
    load().oracle_color_vpls(prec, _p(out), _p(e), count, C.byref(cubes), C.byref(diffuse), C.byref(csm))
    return out


def post_fx(prec, hdr, velocity, hist_in, taa=True):
    """taa.fs + gammaTonemap.fs on an RGBA16F frame (float16 [H, W, 4]): (ldr uint32 [H, W], TAA output float32
    [H, W, 4] holding binary16 values, or None)."""
    H, W = hdr.shape[:2]
    h = np.ascontiguousarray(hdr, dtype=np.float32)
    hi = None if hist_in is None else np.ascontiguousarray(hist_in, dtype=np.float32)
    ho = np.zeros((H, W, 4), np.float32)
    ldr = np.zeros((H, W), np.uint32)
    vel = np.ascontiguousarray(velocity, dtype=np.uint32)
    load().oracle_post_fx(prec, W, H, _p(h), _p(vel), _p(hi), _p(ho), _p(ldr), 1 if taa else 0)
    return ldr, (ho if taa else None)


def cube_struct(storage: np.ndarray, fmt: int, layers: int = 320) -> abi.CubeAtlas:
    at = abi.CubeAtlas()
    for a in range(storage.shape[0]):
        at.atlas[a] = storage[a].ctypes.data
    at.num_atlases, at.layers_per_atlas, at.face_size, at.format = storage.shape[0], layers, storage.shape[-1], fmt
    return at


def vis_cull(prec, vpls, csm: abi.Csm, cap):
    n = vpls.shape[0]
    idx = np.zeros(1 + max(n, 1), np.int32)
    v = np.ascontiguousarray(vpls, dtype=np.float32)
    load().oracle_vis_cull(prec, _p(v), n, C.byref(csm), cap, _p(idx))
    return idx


def tile_stage1(prec, cfg, g: HostGBuffer, cam: abi.Camera):
    T = ((cfg.width + cfg.tile_size - 1) // cfg.tile_size) * ((cfg.height + cfg.tile_size - 1) // cfg.tile_size)
    out = np.zeros((T, 8), _dt(prec))
    load().oracle_tile_stage1(prec, C.byref(cfg), C.byref(g.struct()), C.byref(cam), _p(out))
    return out


def tile_stage2(prec, cfg, stage1, cvpls, count):
    T = stage1.shape[0]
    lists = np.zeros((T, 1 + cfg.max_vpls_per_tile), np.int32)
    s1 = np.ascontiguousarray(stage1, dtype=_dt(prec))
    cv = np.ascontiguousarray(cvpls, dtype=np.float32)
    load().oracle_tile_stage2(prec, C.byref(cfg), _p(s1), _p(cv), count, _p(lists))
    return lists


def gather(prec, cfg, g: HostGBuffer, cam, cvpls, centries, count, lists, cubes: abi.CubeAtlas, time):
    res = np.zeros((cfg.height, cfg.width, 4), _dt(prec))
    lists_arr = None if lists is None else np.ascontiguousarray(lists, dtype=np.int32)
    cv = np.ascontiguousarray(cvpls, dtype=np.float32)
    ce = np.ascontiguousarray(centries, dtype=np.int32)
    load().oracle_gather(prec, C.byref(cfg), C.byref(g.struct()), C.byref(cam), _p(cv), _p(ce), count,
                         _p(lists_arr), C.byref(cubes), time, _p(res))
    return res


def gi_target(cfg, g: HostGBuffer, cam, cvpls, centries, count, lists, cubes: abi.CubeAtlas, time, batches):
    out = np.zeros((cfg.height, cfg.width, 4), np.float32)
    lists_arr = None if lists is None else np.ascontiguousarray(lists, dtype=np.int32)
    cv = np.ascontiguousarray(cvpls, dtype=np.float32)
    ce = np.ascontiguousarray(centries, dtype=np.int32)
    load().oracle_gi_target(C.byref(cfg), C.byref(g.struct()), C.byref(cam), _p(cv), _p(ce), count, _p(lists_arr),
                            C.byref(cubes), time, batches, _p(out))
    return out


def denoise(prec, cfg, cur: HostGBuffer, prev: HostGBuffer, reservoir, hdr_in, gi_prev, hist_prev, num_visible,
            time, fps, keep_passes=False, pass_flops=None):
    H, W = cfg.height, cfg.width
    dt = _dt(prec)
    comb = np.zeros((H, W, 4), dt)
    gi = np.zeros((H, W, 4), dt)
    hist = np.zeros((H, W), dt)
    passes = np.zeros((cfg.denoise_passes, H, W, 4), dt) if keep_passes else None
    keep = [np.ascontiguousarray(a, dtype=dt) for a in (reservoir, hdr_in, gi_prev, hist_prev)]
    fp = abi.FrameParams(time, fps)
    load().oracle_denoise(prec, C.byref(cfg), C.byref(cur.struct()), C.byref(prev.struct()),
                          *[_p(a) for a in keep], num_visible, C.byref(fp), _p(comb), _p(gi), _p(hist), _p(passes),
                          _p(pass_flops))
    return comb, gi, hist, passes


def count_reset():
    load().oracle_count_reset()


def count_read():
    """(flops, cmps) tallied by prec = 0 calls since the last count_reset."""
    out = np.zeros(2, np.uint64)
    load().oracle_count_read(_p(out))
    return int(out[0]), int(out[1])


def frame_flops(cfg, hs: "HostScene", k: int, gi_prev, hist_prev, time, fps):
    """Algorithmic FLOPs (and comparisons) of each pass of frame k, from the counting instantiation
    (the same values as the FP32 oracle). Keys follow the CUDA kernels: vpl_cull, tile_stage1,
    tile_stage2, gather (the sample loop), denoise_pass0 (the merge, fused into the gather kernel),
    atrous (passes 1 .. n-2 together), denoise_final, direct. Each entry is (flops, cmps)."""
    sc = hs.scene
    cam = hs.camera(k)
    csm = hs.csms[k]
    out = {}

    def run(name, fn):
        count_reset()
        r = fn()
        out[name] = count_read()
        return r

    idx = run("vpl_cull", lambda: vis_cull(0, sc.vpls, csm, cfg.max_visible))
    count = int(idx[0])
    order = idx[1:1 + count]
    cv = np.ascontiguousarray(sc.vpls[order])
    ce = np.ascontiguousarray(sc.entries[order])
    direct = run("direct", lambda: deferred(0, cfg, hs.gbuffers[k], cam, sc.points if len(sc.points) else None, csm))
    lists = None
    if cfg.gi_mode == abi.SGI_GI_TILED:
        s1 = run("tile_stage1", lambda: tile_stage1(0, cfg, hs.gbuffers[k], cam))
        lists = run("tile_stage2", lambda: tile_stage2(0, cfg, s1, cv, count))
    res = run("gather", lambda: gather(0, cfg, hs.gbuffers[k], cam, cv, ce, count, lists, hs.cubes, time))
    n = cfg.denoise_passes
    pf = np.zeros(n, np.uint64)
    count_reset()
    denoise(0, cfg, hs.gbuffers[k], hs.gbuffers[k - 1], res, direct, gi_prev, hist_prev, count, time, fps,
            pass_flops=pf)
    cum = [0] + [int(v) for v in pf]
    per = [cum[i + 1] - cum[i] for i in range(n)]
    out["denoise_pass0"] = (per[0], None)
    out["atrous"] = (sum(per[1:n - 1]), None)
    out["denoise_final"] = (per[n - 1], None)
    return out


def deferred(prec, cfg, g: HostGBuffer, cam, points, csm: abi.Csm, casters=None, caster_entries=None,
             caster_atlas: abi.CubeAtlas | None = None):
    """pbr.fs: point lights, optional shadow-casting point lights (records, atlas slots, host cube atlas)
    and the directional light with its CSM."""
    out = np.zeros((cfg.height, cfg.width, 4), _dt(prec))
    npts = 0 if points is None else points.shape[0]
    pts = None if points is None else np.ascontiguousarray(points, dtype=np.float32)
    nc = 0 if casters is None else casters.shape[0]
    cs = None if casters is None else np.ascontiguousarray(casters, dtype=np.float32)
    ce = None if caster_entries is None else np.ascontiguousarray(caster_entries, dtype=np.int32)
    at = C.byref(caster_atlas) if caster_atlas is not None else None
    load().oracle_deferred(prec, C.byref(cfg), C.byref(g.struct()), C.byref(cam), _p(pts), npts, C.byref(csm), _p(out),
                           _p(cs), _p(ce), nc, at)
    return out


class HostScene:
    """CPU-side inputs of a workload (oracle ray caster) with host-pointer structs."""

    def __init__(self, scene, w):
        from stratusgfx_gb300 import stage  # struct builders only
        self.scene, self.w = scene, w
        H, W = w.height, w.width
        self.gbuffers = [scene_gbuffer(scene.boxes, stage.scene_camera_struct(scene, k), W, H)
                         for k in range(len(scene.cameras))]
        R = w.csm_resolution
        self.csm_depth, self.csms = [], []
        for k in range(len(scene.cameras)):
            placeholder = stage.csm_struct(scene, k, 0, R)
            d = scene_csm(scene.boxes, placeholder, scene.csms[k].inv_cascade_proj_view, R)
            self.csm_depth.append(d)
            self.csms.append(stage.csm_struct(scene, k, d.ctypes.data, R))
        self.cube_storage, self.cubes = scene_cubes(scene.boxes, scene.vpls, scene.entries, w.cube_size,
                                                    w.cube_format, scene.layers_per_atlas)

    def camera(self, k):
        from stratusgfx_gb300 import stage
        return stage.camera_struct(self.scene, k)

    @classmethod
    def from_arrays(cls, scene, w, gbuffers, csm_depth, cube_storage):
        """A HostScene over inputs made elsewhere (e.g. copied back from the device generator, which is
        bit-identical to the CPU ray caster): gbuffers = dicts of G-buffer planes per frame, csm_depth =
        {frame: float32 [4, R, R]}, cube_storage = the cube atlas array (uint16 or float32)."""
        from stratusgfx_gb300 import stage
        hs = cls.__new__(cls)
        hs.scene, hs.w = scene, w
        hs.gbuffers = [None if g is None else HostGBuffer(w.height, w.width, g) for g in gbuffers]
        hs.csm_depth, hs.csms = {}, {}
        for k, d in csm_depth.items():
            hs.csm_depth[k] = np.ascontiguousarray(d, dtype=np.float32)
            hs.csms[k] = stage.csm_struct(scene, k, hs.csm_depth[k].ctypes.data, w.csm_resolution)
        hs.cube_storage = hs.cubes = None
        if cube_storage is not None:     # not needed by the culls
            storage = np.ascontiguousarray(cube_storage)
            if storage.dtype == np.int16:
                storage = storage.view(np.uint16)
            hs.cube_storage = storage
            hs.cubes = cube_struct(storage, w.cube_format, scene.layers_per_atlas)
        return hs


def frame(prec, cfg, hs: HostScene, k: int, gi_prev, hist_prev, time, fps, keep=False):
    """The whole stage for camera k (k >= 1; k - 1 is the previous frame), like sgi_render_frame.
    Returns a dict of every intermediate."""
    sc = hs.scene
    cam = hs.camera(k)
    csm = hs.csms[k]
    idx = vis_cull(prec, sc.vpls, csm, cfg.max_visible)
    count = int(idx[0])
    order = idx[1:1 + count]
    cv = np.ascontiguousarray(sc.vpls[order])
    ce = np.ascontiguousarray(sc.entries[order])
    direct = deferred(prec, cfg, hs.gbuffers[k], cam, sc.points if len(sc.points) else None, csm)
    direct_in = direct
    s1 = lists = None
    if cfg.gi_mode == abi.SGI_GI_TILED:
        s1 = tile_stage1(prec, cfg, hs.gbuffers[k], cam)
        lists = tile_stage2(prec, cfg, s1, cv, count)
    res = gather(prec, cfg, hs.gbuffers[k], cam, cv, ce, count, lists, hs.cubes, time)
    comb, gi, hist, passes = denoise(prec, cfg, hs.gbuffers[k], hs.gbuffers[k - 1], res, direct_in, gi_prev,
                                     hist_prev, count, time, fps, keep)
    return dict(visible_index=idx, count=count, direct=direct, stage1=s1, lists=lists, reservoir=res,
                combined=comb, gi=gi, hist=hist, passes=passes)
