"""ctypes mirror of include/sgi.h and include/sgi_scene.h, and the loader of libsgi.so.

The library is built in-tree by ``stratusgfx_gb300.build``; importing this
module never falls back to anything else: a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

SGI_OK = 0
SGI_ERR_ARG = -1
SGI_ERR_OOM = -2
SGI_ERR_CUDA = -3
SGI_ERR_TIMEOUT = -4
SGI_ERR_CAP = -5
SGI_ERR_STATE = -6

SGI_GI_REFERENCE = 0
SGI_GI_TILED = 1
SGI_CUBE_F32 = 0
SGI_CUBE_F16 = 1
SGI_CUBE_UNORM16 = 2
SGI_MAX_ATLASES = 14
SGI_MAX_CUBE_FACE = 16384
SGI_MAX_VPLS_BEFORE_CULL = 10000
SGI_MAX_VPLS_PER_FRAME = 4480
SGI_NUM_PASS_TIMES = 5
SGI_NUM_PASS_TIMES_SPLIT = 7
SGI_LOG_INFO = 0
SGI_LOG_ERROR = 1
LOG_FN = C.CFUNCTYPE(None, C.c_int32, C.c_char_p, C.c_void_p)
SGI_SHADING_EXACT = 0
SGI_SHADING_FAST = 1
SGI_ATROUS_DIRECT = 0
SGI_ATROUS_STAGED = 1
SGI_LANE_CHECKS = 12
SGI_NO_LIGHT = 0xFFFFFFFFFFFFFFFF

SGI_DEBUG_VISIBLE_INDEX = 0
SGI_DEBUG_COMPACT_VPLS = 1
SGI_DEBUG_COMPACT_ENTRIES = 2
SGI_DEBUG_TILE_STAGE1 = 3
SGI_DEBUG_TILE_LISTS = 4
SGI_DEBUG_RESERVOIR = 5
SGI_DEBUG_GI_HISTORY = 6
SGI_DEBUG_HISTORY_DEPTH = 7
SGI_DEBUG_DIRECT = 8
SGI_DEBUG_TAA_HISTORY = 9
SGI_DEBUG_PASS_BASE = 16


class Vpl(C.Structure):           # GpuVplData, 64 B
    _fields_ = [("position", C.c_float * 4), ("color", C.c_float * 4), ("specular_position", C.c_float * 4),
                ("radius", C.c_float), ("far_plane", C.c_float), ("intensity", C.c_float), ("pad_", C.c_float)]


class PointLight(C.Structure):    # GpuPointLight, 48 B
    _fields_ = [("position", C.c_float * 4), ("color", C.c_float * 4), ("radius", C.c_float),
                ("far_plane", C.c_float), ("pad_", C.c_float * 2)]


class AtlasEntry(C.Structure):    # GpuAtlasEntry, 8 B
    _fields_ = [("index", C.c_int32), ("layer", C.c_int32)]


class Config(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("max_vpls", C.c_int32), ("max_visible", C.c_int32),
                ("tile_size", C.c_int32), ("max_vpls_per_tile", C.c_int32), ("gi_mode", C.c_int32),
                ("samples_per_pixel", C.c_int32), ("denoise_passes", C.c_int32), ("debug_keep_passes", C.c_int32),
                ("min_roughness", C.c_float), ("use_perceptual_roughness", C.c_int32),
                ("min_gi_occlusion_factor", C.c_float), ("emission_strength", C.c_float),
                ("fog_density", C.c_float), ("fog_color", C.c_float * 3),
                ("point_light_ambient_intensity", C.c_float)]


def config_defaults(width: int, height: int) -> Config:
    """The values sgi_config_defaults writes (the reference's RendererSettings and
    shader constants), stated in Python so that code which must not load libsgi.so
    (the CPU reference arm of the benchmark) builds the same config; a test keeps
    the two equal field by field."""
    cfg = Config()
    cfg.width, cfg.height = width, height
    cfg.max_vpls = SGI_MAX_VPLS_BEFORE_CULL
    cfg.max_visible = SGI_MAX_VPLS_PER_FRAME
    cfg.tile_size = 5
    cfg.max_vpls_per_tile = 12
    cfg.gi_mode = SGI_GI_REFERENCE
    cfg.samples_per_pixel = 0
    cfg.denoise_passes = 4
    cfg.debug_keep_passes = 0
    cfg.min_roughness = 0.08
    cfg.use_perceptual_roughness = 1
    cfg.min_gi_occlusion_factor = 0.95
    cfg.emission_strength = 0.0
    cfg.fog_density = 0.0
    for i in range(3):
        cfg.fog_color[i] = 0.5
    cfg.point_light_ambient_intensity = 0.003
    return cfg


class GBuffer(C.Structure):
    _fields_ = [("depth", C.c_void_p), ("normal", C.c_void_p), ("albedo", C.c_void_p),
                ("base_reflectivity", C.c_void_p), ("roughness_metallic_ambient", C.c_void_p),
                ("velocity", C.c_void_p), ("id", C.c_void_p), ("ssao", C.c_void_p)]


class Camera(C.Structure):
    _fields_ = [("inv_proj_view", C.c_float * 16), ("view_position", C.c_float * 4)]


class Csm(C.Structure):
    _fields_ = [("depth", C.c_void_p), ("resolution", C.c_int32), ("num_cascades", C.c_int32),
                ("cascade_proj_view", (C.c_float * 16) * 4), ("cascade_planes", (C.c_float * 4) * 3),
                ("light_direction", C.c_float * 4), ("light_color", C.c_float * 4), ("znear", C.c_float),
                ("zfar", C.c_float), ("depth_bias", C.c_float), ("pad_", C.c_float)]


class CubeAtlas(C.Structure):
    _fields_ = [("atlas", C.c_void_p * SGI_MAX_ATLASES), ("num_atlases", C.c_int32),
                ("layers_per_atlas", C.c_int32), ("face_size", C.c_int32), ("format", C.c_int32)]


class DiffuseAtlas(C.Structure):  # sgi_diffuse_atlas
    _fields_ = [("atlas", C.c_void_p * 14), ("num_atlases", C.c_int32), ("layers_per_atlas", C.c_int32),
                ("face_size", C.c_int32), ("reserved", C.c_int32)]


class FrameParams(C.Structure):
    _fields_ = [("time", C.c_float), ("frames_per_second", C.c_float)]


class ErrorStats(C.Structure):    # sgi_error_stats
    _fields_ = [("sse_frame", C.c_double), ("sse_gi", C.c_double), ("peak_frame", C.c_double),
                ("peak_gi", C.c_double), ("max_abs_frame", C.c_double), ("max_abs_gi", C.c_double),
                ("values", C.c_int64)]


class Box(C.Structure):           # sgi_box, 64 B
    _fields_ = [("min", C.c_float * 4), ("max", C.c_float * 4), ("albedo", C.c_float * 4), ("roughness", C.c_float),
                ("metallic", C.c_float), ("reflectance", C.c_float), ("id", C.c_float)]


class NnConfig(C.Structure):
    _fields_ = [("max_batch", C.c_int32), ("max_height", C.c_int32), ("max_width", C.c_int32), ("seed", C.c_uint32)]


class SceneCamera(C.Structure):
    _fields_ = [("proj_view", C.c_float * 16), ("inv_proj_view", C.c_float * 16),
                ("prev_proj_view", C.c_float * 16), ("position", C.c_float * 4)]


class View(C.Structure):          # sgi_view (sgi_batch.h)
    _fields_ = [("ctx", C.c_void_p), ("cur", C.c_void_p), ("prev", C.c_void_p), ("cam", C.c_void_p),
                ("params", FrameParams), ("hdr_out", C.c_void_p)]


assert C.sizeof(Vpl) == 64 and C.sizeof(PointLight) == 48 and C.sizeof(AtlasEntry) == 8 and C.sizeof(Box) == 64

SGI_BLOCK_GATHER, SGI_BLOCK_ATROUS, SGI_BLOCK_DENOISE_FINAL, SGI_BLOCK_DIRECT = 0, 1, 2, 3

SGI_NN_CONV_WARP_MMA = 0
SGI_NN_CONV_TCGEN05 = 1
SGI_NN_BF16 = 0
SGI_NN_FP8 = 1

EXPORTS = {
    "sgi_abi_version": (C.c_int32, []),
    "sgi_status_string": (C.c_char_p, [C.c_int32]),
    "sgi_config_defaults": (None, [C.POINTER(Config), C.c_int32, C.c_int32]),
    "sgi_create": (C.c_int32, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "sgi_destroy": (C.c_int32, [C.c_void_p]),
    "sgi_last_error": (C.c_char_p, [C.c_void_p]),
    "sgi_set_lights": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]),
    "sgi_set_shadow_maps": (C.c_int32, [C.c_void_p, C.POINTER(Csm), C.POINTER(CubeAtlas)]),
    "sgi_cull_vpls": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "sgi_cull_tiles": (C.c_int32, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(Camera), C.c_void_p]),
    "sgi_direct_lighting": (C.c_int32, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(Camera), C.c_void_p, C.c_void_p]),
    "sgi_global_illumination": (C.c_int32, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(GBuffer), C.POINTER(Camera),
                                            C.c_void_p, C.c_void_p, C.POINTER(FrameParams), C.c_void_p]),
    "sgi_render_frame": (C.c_int32, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(GBuffer), C.POINTER(Camera),
                                     C.POINTER(FrameParams), C.c_void_p, C.c_void_p]),
    "sgi_reset_history": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "sgi_gi_error_stats": (C.c_int32, [C.POINTER(GBuffer), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                       C.POINTER(ErrorStats), C.c_void_p]),
    "sgi_gi_target": (C.c_int32, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(Camera), C.c_float, C.c_int32,
                                  C.c_void_p, C.c_void_p]),
    "sgi_read_debug": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "sgi_set_timing": (C.c_int32, [C.c_void_p, C.c_int32]),
    "sgi_get_pass_times": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float), C.c_int32]),
    "sgi_launch_count": (C.c_int64, [C.c_void_p]),
    "sgi_set_shading_precision": (C.c_int32, [C.c_void_p, C.c_int32]),
    "sgi_get_history": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int32), C.c_void_p]),
    "sgi_set_history": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "sgi_set_log_callback": (None, [C.c_void_p, C.c_void_p]),
    "sgi_log_message": (None, [C.c_int32, C.c_char_p]),
    "sgi_get_shading_precision": (C.c_int32, [C.c_void_p]),
    "sgi_set_atrous_staging": (C.c_int32, [C.c_void_p, C.c_int32]),
    "sgi_get_atrous_staging": (C.c_int32, [C.c_void_p]),
    "sgi_set_wait_test": (C.c_int32, [C.c_void_p, C.c_int64, C.c_int32]),
    "sgi_device_status": (C.c_int32, [C.c_void_p]),
    "sgi_lane_selftest": (C.c_int32, [C.c_int32, C.POINTER(C.c_uint32), C.POINTER(C.c_float)]),
    "sgi_slot_cache_create": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "sgi_slot_cache_destroy": (C.c_int32, [C.c_void_p]),
    "sgi_slot_cache_get": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(AtlasEntry), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_uint64)]),
    "sgi_slot_cache_remove": (C.c_int32, [C.c_void_p, C.c_uint64]),
    "sgi_slot_cache_find": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(AtlasEntry)]),
    "sgi_slot_cache_capacity": (C.c_int32, [C.c_void_p]),
    "sgi_slot_cache_free": (C.c_int32, [C.c_void_p]),
    "sgi_slot_cache_used": (C.c_int32, [C.c_void_p]),
    "sgi_prepare_vpls": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                     C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]),
    "sgi_nn_create": (C.c_int32, [C.POINTER(NnConfig), C.POINTER(C.c_void_p)]),
    "sgi_nn_destroy": (C.c_int32, [C.c_void_p]),
    "sgi_nn_last_error": (C.c_char_p, [C.c_void_p]),
    "sgi_nn_num_params": (C.c_int64, [C.c_void_p]),
    "sgi_nn_get_params": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64]),
    "sgi_nn_set_params": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64]),
    "sgi_nn_get_grads": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64]),
    "sgi_nn_get_optimizer_state": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                               C.POINTER(C.c_int64)]),
    "sgi_nn_set_optimizer_state": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64]),
    "sgi_nn_forward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                   C.c_void_p, C.c_void_p]),
    "sgi_nn_train_step": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                      C.c_int32, C.c_int32, C.c_float, C.c_int32, C.POINTER(C.c_float), C.c_void_p]),
    "sgi_nn_features": (C.c_int32, [C.c_void_p, C.POINTER(GBuffer), C.POINTER(Camera), C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p]),
    "sgi_cull_vpls_noalloc": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(Csm), C.c_int32, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p]),
    "sgi_nn_set_conv_path": (C.c_int32, [C.c_void_p, C.c_int32]),
    "sgi_nn_set_head_fusion": (C.c_int32, [C.c_void_p, C.c_int32]),
    "sgi_nn_set_precision": (C.c_int32, [C.c_void_p, C.c_int32]),
    "sgi_nn_calibrate_fp8": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "sgi_nn_device_status": (C.c_int32, [C.c_void_p]),
    "sgi_nn_set_wait_test": (C.c_int32, [C.c_void_p, C.c_int64, C.c_int32]),
    "sgi_nn_conv3x3": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                   C.c_void_p]),
    "sgi_render_frame_neural": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(GBuffer), C.POINTER(GBuffer),
                                            C.POINTER(Camera), C.POINTER(FrameParams), C.c_void_p, C.c_void_p]),
    "sgi_scene_gbuffer": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(SceneCamera), C.c_int32, C.c_int32,
                                      C.POINTER(GBuffer), C.c_void_p]),
    "sgi_scene_csm": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(Csm), C.POINTER((C.c_float * 16) * 4), C.c_void_p]),
    "sgi_scene_cube_atlas": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                         C.POINTER(CubeAtlas), C.c_void_p]),
    "sgi_set_block_shape": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "sgi_set_vpl_coloring": (C.c_int32, [C.c_void_p, C.POINTER(DiffuseAtlas)]),
    "sgi_post_fx": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(GBuffer), C.c_int32, C.c_void_p, C.c_void_p]),
    "sgi_set_shadow_point_lights": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(CubeAtlas),
                                                C.c_void_p]),
    "sgi_scene_diffuse_atlas": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                            C.POINTER(DiffuseAtlas), C.c_void_p]),
    "sgi_get_block_shape": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "sgi_batch_create": (C.c_int32, [C.POINTER(View), C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                     C.POINTER(C.c_void_p)]),
    "sgi_batch_launch": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "sgi_batch_create_persistent": (C.c_int32, [C.POINTER(View), C.c_int32, C.c_int32, C.c_void_p,
                                                C.POINTER(C.c_void_p)]),
    "sgi_batch_status": (C.c_int32, [C.c_void_p]),
    "sgi_batch_persistent_shape": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "sgi_batch_set_wait_limit": (C.c_int32, [C.c_void_p, C.c_int64]),
    "sgi_batch_skip_pass": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "sgi_batch_kernel_count": (C.c_int64, [C.c_void_p]),
    "sgi_batch_destroy": (C.c_int32, [C.c_void_p]),
    "sgi_batch_last_error": (C.c_char_p, [C.c_void_p]),
}

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Loads libsgi.so (declaring every exported signature). Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libsgi.so is not built ({path}); run python -m stratusgfx_gb300.build")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class SgiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"sgi status {status}: {msg}")
        self.status = status


def check(status: int, ctx=None) -> None:
    if status != SGI_OK:
        lib = load()
        msg = lib.sgi_last_error(ctx).decode() if ctx else lib.sgi_status_string(status).decode()
        raise SgiError(status, msg)
