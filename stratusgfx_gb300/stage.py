"""Python host mirror of StratusGFX RendererBackend's GI/lighting stage over the C ABI.

Method names follow the reference's (RendererBackend, StratusRendererBackend.cpp):
``cull_vpls`` = PerformVirtualPointLightCullingStage1_ (:1578-1661),
``cull_tiles`` = the tile culling of PerformVirtualPointLightCullingStage2_ (:1733-1783),
``direct_lighting`` = the deferred lighting block of RenderScene (:2011-2038),
``global_illumination`` = ComputeVirtualPointLightGlobalIllumination_ (:1816-1952),
``render_frame`` = the stage in RenderScene order. Errors raise ``SgiError`` with
the library's message, like the reference's exceptions / isValid_ flags.

Device memory and streams come from PyTorch; every compute step is a call into
libsgi.so. There is no other code path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import abi
from .scene import Scene, Workload


def _ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def _stream_ptr(stream) -> C.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


def default_config(width: int, height: int, **kw) -> abi.Config:
    """sgi_config_defaults (as abi.config_defaults states it) with overrides."""
    cfg = abi.config_defaults(width, height)
    for k, v in kw.items():
        if k == "fog_color":
            for i in range(3):
                cfg.fog_color[i] = v[i]
        else:
            setattr(cfg, k, v)
    return cfg


def workload_config(w: Workload, **kw) -> abi.Config:
    args = dict(max_vpls=max(w.num_vpls, 1), max_visible=max(w.num_vpls, 1), tile_size=w.tile_size,
                max_vpls_per_tile=w.max_per_tile, gi_mode=abi.SGI_GI_TILED, samples_per_pixel=w.samples,
                denoise_passes=w.denoise_passes)
    args.update(kw)
    return default_config(w.width, w.height, **args)


def gi_error_stats(g: "GBufferTensors", hdr: torch.Tensor, direct: torch.Tensor, target: torch.Tensor,
                   stream=None) -> dict:
    """sgi_gi_error_stats: FP64 error statistics (on the device) of the RGBA16F frame `hdr` against the
    converged frame direct + w * target, w = binary16(max(albedo, 0.01) + 1e-5); returns the PSNRs of the
    frame and of its GI term and the raw statistics."""
    import math
    H, W = hdr.shape[0], hdr.shape[1]
    st = abi.ErrorStats()
    lib = abi.load()
    gs = g.struct()
    abi.check(lib.sgi_gi_error_stats(C.byref(gs), hdr.data_ptr(), direct.data_ptr(), target.data_ptr(), W, H,
                                     C.byref(st), _stream_ptr(stream)))

    def psnr(peak, sse):
        return math.inf if sse == 0 else 10.0 * math.log10(peak * peak / (sse / st.values))
    return {"psnr_frame": psnr(st.peak_frame, st.sse_frame), "psnr_gi": psnr(st.peak_gi, st.sse_gi),
            "sse_frame": st.sse_frame, "sse_gi": st.sse_gi, "peak_frame": st.peak_frame, "peak_gi": st.peak_gi,
            "max_abs_frame": st.max_abs_frame, "max_abs_gi": st.max_abs_gi, "values": st.values}


class GBufferTensors:
    """One frame's G-buffer in the reference formats (row 0 = bottom)."""

    def __init__(self, H: int, W: int, device):
        self.depth = torch.empty((H, W), dtype=torch.float32, device=device)
        self.normal = torch.empty((H, W, 4), dtype=torch.uint8, device=device)
        self.albedo = torch.empty((H, W, 4), dtype=torch.uint8, device=device)
        self.base_reflectivity = torch.empty((H, W, 2), dtype=torch.uint8, device=device)
        self.rma = torch.empty((H, W, 4), dtype=torch.uint8, device=device)
        self.velocity = torch.empty((H, W, 2), dtype=torch.float16, device=device)
        self.id = torch.empty((H, W), dtype=torch.float32, device=device)
        self.ssao = torch.empty((H, W), dtype=torch.float16, device=device)

    def planes(self):
        return [self.depth, self.normal, self.albedo, self.base_reflectivity, self.rma, self.velocity, self.id,
                self.ssao]

    def struct(self) -> abi.GBuffer:
        return abi.GBuffer(*[_ptr(t) for t in self.planes()])

    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in self.planes())

    def copy_from(self, other: "GBufferTensors", non_blocking: bool = True) -> None:
        for a, b in zip(self.planes(), other.planes()):
            a.copy_(b, non_blocking=non_blocking)

    def pinned_clone(self) -> "GBufferTensors":
        g = GBufferTensors.__new__(GBufferTensors)
        for name in ("depth", "normal", "albedo", "base_reflectivity", "rma", "velocity", "id", "ssao"):
            setattr(g, name, getattr(self, name).cpu().pin_memory())
        return g

    def numpy(self) -> dict:
        return {name: getattr(self, name).cpu().numpy() for name in
                ("depth", "normal", "albedo", "base_reflectivity", "rma", "velocity", "id", "ssao")}


def camera_struct(scene: Scene, k: int) -> abi.Camera:
    cam = abi.Camera()
    c = scene.cameras[k]
    for i in range(16):
        cam.inv_proj_view[i] = float(c.inv_proj_view[i])
    for i in range(4):
        cam.view_position[i] = float(c.position[i])
    return cam


def scene_camera_struct(scene: Scene, k: int) -> abi.SceneCamera:
    sc = abi.SceneCamera()
    c = scene.cameras[k]
    for i in range(16):
        sc.proj_view[i] = float(c.proj_view[i])
        sc.inv_proj_view[i] = float(c.inv_proj_view[i])
        sc.prev_proj_view[i] = float(c.prev_proj_view[i])
    for i in range(4):
        sc.position[i] = float(c.position[i])
    return sc


def csm_struct(scene: Scene, k: int, depth_ptr: int, resolution: int) -> abi.Csm:
    cs = abi.Csm()
    f = scene.csms[k]
    cs.depth = depth_ptr
    cs.resolution = resolution
    cs.num_cascades = 4
    for c in range(4):
        for i in range(16):
            cs.cascade_proj_view[c][i] = float(f.cascade_proj_view[c, i])
    for c in range(3):
        for i in range(4):
            cs.cascade_planes[c][i] = float(f.cascade_planes[c, i])
    for i in range(4):
        cs.light_direction[i] = float(scene.light_direction[i])
        cs.light_color[i] = float(scene.light_color[i])
    cs.znear, cs.zfar, cs.depth_bias = f.znear, f.zfar, 0.0
    return cs


def inv_cascade_array(scene: Scene, k: int):
    arr = ((C.c_float * 16) * 4)()
    for c in range(4):
        for i in range(16):
            arr[c][i] = float(scene.csms[k].inv_cascade_proj_view[c, i])
    return arr


class DeviceScene:
    """All device-resident inputs of a workload, generated on the GPU by sgi_scene_*."""

    def __init__(self, scene: Scene, w: Workload, device="cuda", stream=None):
        lib = abi.load()
        self.scene, self.w, self.device = scene, w, device
        s = _stream_ptr(stream)
        H, W = w.height, w.width
        self.boxes = torch.from_numpy(scene.boxes).to(device)
        nb = scene.boxes.shape[0]
        self.vpls = torch.from_numpy(scene.vpls).to(device)
        self.entries = torch.from_numpy(scene.entries).to(device)
        self.points = torch.from_numpy(scene.points).to(device) if len(scene.points) else None
        nframes = len(scene.cameras)
        self.gbuffers = []
        for k in range(nframes):
            g = GBufferTensors(H, W, device)
            abi.check(lib.sgi_scene_gbuffer(C.c_void_p(_ptr(self.boxes)), nb, C.byref(scene_camera_struct(scene, k)),
                                            W, H, C.byref(g.struct()), s))
            self.gbuffers.append(g)
        R = w.csm_resolution
        self.csm_depth = [torch.empty((4, R, R), dtype=torch.float32, device=device) for _ in range(nframes)]
        self.csms = []
        for k in range(nframes):
            cs = csm_struct(scene, k, _ptr(self.csm_depth[k]), R)
            abi.check(lib.sgi_scene_csm(C.c_void_p(_ptr(self.boxes)), nb, C.byref(cs), C.byref(inv_cascade_array(scene, k)), s))
            self.csms.append(cs)
        n = scene.vpls.shape[0]
        layers = scene.layers_per_atlas
        num_atlases = max(1, (n + layers - 1) // layers)
        cube_dtype = torch.float32 if w.cube_format == abi.SGI_CUBE_F32 else torch.int16
        self.cube_storage = torch.empty((num_atlases, layers, 6, w.cube_size, w.cube_size), dtype=cube_dtype,
                                        device=device)
        self.cubes = abi.CubeAtlas()
        for a in range(num_atlases):
            self.cubes.atlas[a] = self.cube_storage[a].data_ptr()
        self.cubes.num_atlases = num_atlases
        self.cubes.layers_per_atlas = layers
        self.cubes.face_size = w.cube_size
        self.cubes.format = w.cube_format
        if n:
            abi.check(lib.sgi_scene_cube_atlas(C.c_void_p(_ptr(self.boxes)), nb, C.c_void_p(_ptr(self.vpls)),
                                               C.c_void_p(_ptr(self.entries)), n, C.byref(self.cubes), s))

    def camera(self, k: int) -> abi.Camera:
        return camera_struct(self.scene, k)


class ViewScene:
    """Another viewport of a room whose lights and shadow atlas a DeviceScene already holds: the
    view's own G-buffers (every camera of `scene`) and the CSM of its last frame, generated on the GPU;
    the VPLs, point lights and cube atlas are the room's."""

    def __init__(self, room: DeviceScene, scene: Scene, w: Workload, device="cuda", stream=None):
        lib = abi.load()
        self.scene, self.w, self.device = scene, w, device
        s = _stream_ptr(stream)
        H, W = w.height, w.width
        self.boxes, self.vpls, self.entries, self.points = room.boxes, room.vpls, room.entries, room.points
        self.cubes = room.cubes
        nb = scene.boxes.shape[0]
        nframes = len(scene.cameras)
        self.gbuffers = []
        for k in range(nframes):
            g = GBufferTensors(H, W, device)
            abi.check(lib.sgi_scene_gbuffer(C.c_void_p(_ptr(self.boxes)), nb, C.byref(scene_camera_struct(scene, k)),
                                            W, H, C.byref(g.struct()), s))
            self.gbuffers.append(g)
        R = w.csm_resolution
        k = nframes - 1
        self.csm_depth = {k: torch.empty((4, R, R), dtype=torch.float32, device=device)}
        cs = csm_struct(scene, k, _ptr(self.csm_depth[k]), R)
        abi.check(lib.sgi_scene_csm(C.c_void_p(_ptr(self.boxes)), nb, C.byref(cs), C.byref(inv_cascade_array(scene, k)), s))
        self.csms = {k: cs}

    def camera(self, k: int) -> abi.Camera:
        return camera_struct(self.scene, k)


class GiStage:
    def __init__(self, cfg: abi.Config):
        self.lib = abi.load()
        self.cfg = cfg
        h = C.c_void_p()
        abi.check(self.lib.sgi_create(C.byref(cfg), C.byref(h)))
        self.ctx = h
        self.H, self.W = cfg.height, cfg.width

    def close(self) -> None:
        if self.ctx:
            self.lib.sgi_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st: int) -> None:
        abi.check(st, self.ctx)

    def set_lights(self, vpls: torch.Tensor, entries: torch.Tensor, points: torch.Tensor | None, stream=None):
        n = 0 if vpls is None else vpls.shape[0]
        npts = 0 if points is None else points.shape[0]
        self._chk(self.lib.sgi_set_lights(self.ctx, C.c_void_p(_ptr(vpls)), C.c_void_p(_ptr(entries)), n,
                                          C.c_void_p(_ptr(points)), npts, _stream_ptr(stream)))

    def set_shadow_maps(self, csm: abi.Csm, cubes: abi.CubeAtlas):
        self._chk(self.lib.sgi_set_shadow_maps(self.ctx, C.byref(csm), C.byref(cubes)))

    def cull_vpls(self, stream=None):
        self._chk(self.lib.sgi_cull_vpls(self.ctx, _stream_ptr(stream)))

    def cull_tiles(self, g: GBufferTensors, cam: abi.Camera, stream=None):
        self._chk(self.lib.sgi_cull_tiles(self.ctx, C.byref(g.struct()), C.byref(cam), _stream_ptr(stream)))

    def direct_lighting(self, g: GBufferTensors, cam: abi.Camera, hdr_out: torch.Tensor, stream=None):
        self._chk(self.lib.sgi_direct_lighting(self.ctx, C.byref(g.struct()), C.byref(cam), C.c_void_p(_ptr(hdr_out)),
                                               _stream_ptr(stream)))

    def global_illumination(self, cur: GBufferTensors, prev: GBufferTensors, cam: abi.Camera, hdr_in, hdr_out,
                            time: float, fps: float, stream=None):
        fp = abi.FrameParams(time, fps)
        self._chk(self.lib.sgi_global_illumination(self.ctx, C.byref(cur.struct()), C.byref(prev.struct()),
                                                   C.byref(cam), C.c_void_p(_ptr(hdr_in)),
                                                   C.c_void_p(_ptr(hdr_out)), C.byref(fp), _stream_ptr(stream)))

    def render_frame(self, cur: GBufferTensors, prev: GBufferTensors, cam: abi.Camera, hdr_out, time: float,
                     fps: float, stream=None):
        fp = abi.FrameParams(time, fps)
        self._chk(self.lib.sgi_render_frame(self.ctx, C.byref(cur.struct()), C.byref(prev.struct()), C.byref(cam),
                                            C.byref(fp), C.c_void_p(_ptr(hdr_out)), _stream_ptr(stream)))

    def gi_target(self, g: GBufferTensors, cam: abi.Camera, time: float, batches: int, out: torch.Tensor,
                  stream=None):
        """Converged GI target (float32 [H, W, 4]) after this frame's culling."""
        self._chk(self.lib.sgi_gi_target(self.ctx, C.byref(g.struct()), C.byref(cam), time, batches,
                                         C.c_void_p(_ptr(out)), _stream_ptr(stream)))

    def reset_history(self, stream=None):
        self._chk(self.lib.sgi_reset_history(self.ctx, _stream_ptr(stream)))

    def read_debug(self, which: int, dtype) -> np.ndarray:
        need = C.c_size_t()
        self._chk(self.lib.sgi_read_debug(self.ctx, which, None, 0, C.byref(need)))
        buf = np.empty(need.value // np.dtype(dtype).itemsize, dtype=dtype)
        self._chk(self.lib.sgi_read_debug(self.ctx, which, buf.ctypes.data_as(C.c_void_p), need.value, None))
        return buf

    def set_timing(self, on: bool):
        self._chk(self.lib.sgi_set_timing(self.ctx, 1 if on else 0))

    def pass_times(self, split: bool = False) -> list[float]:
        """[vpl cull, direct, tile cull, gather, denoise] ms of the last timed frame; with split, also the
        denoise pass's a-trous passes and its final pass."""
        n = abi.SGI_NUM_PASS_TIMES_SPLIT if split else abi.SGI_NUM_PASS_TIMES
        arr = (C.c_float * n)()
        self._chk(self.lib.sgi_get_pass_times(self.ctx, arr, n))
        return list(arr)

    def launch_count(self) -> int:
        return int(self.lib.sgi_launch_count(self.ctx))
