"""The C-ABI library builds, loads without a GPU and exports every symbol include/*.h declares."""
import ctypes as C
import os
import re

from stratusgfx_gb300 import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(sgi_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_function():
    path = build.build()
    lib = C.CDLL(path)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(abi.EXPORTS), "ctypes mirror lacks declarations"


def test_struct_sizes_match_reference_std430_records():
    # StratusGpuCommon.h:297-307 static_asserts
    assert C.sizeof(abi.Vpl) == 64
    assert C.sizeof(abi.PointLight) == 48
    assert C.sizeof(abi.AtlasEntry) == 8


def test_config_defaults_are_the_reference_settings():
    lib = abi.load(build_if_missing=True)
    cfg = abi.Config()
    lib.sgi_config_defaults(C.byref(cfg), 1920, 1080)
    assert abs(cfg.min_roughness - 0.08) < 1e-7            # StratusRendererBackend.h:289
    assert abs(cfg.min_gi_occlusion_factor - 0.95) < 1e-7  # :293
    assert cfg.use_perceptual_roughness == 1               # :194
    assert cfg.denoise_passes == 4                         # StratusRendererBackend.cpp:1914
    assert cfg.max_visible == 4480 and cfg.max_vpls == 10000
    assert cfg.tile_size == 5 and cfg.max_vpls_per_tile == 12   # StratusRendererBackend.h:346-347, vpl_common.glsl:9
    assert lib.sgi_abi_version() == 1


def test_python_config_defaults_equal_the_library_defaults():
    """abi.config_defaults (used where libsgi.so must not be loaded) writes the same bytes."""
    lib = abi.load(build_if_missing=True)
    for W, H in ((1920, 1080), (17, 9)):
        cfg = abi.Config()
        lib.sgi_config_defaults(C.byref(cfg), W, H)
        assert bytes(cfg) == bytes(abi.config_defaults(W, H))


def test_create_rejects_bad_configs_before_touching_the_device():
    lib = abi.load(build_if_missing=True)
    h = C.c_void_p()
    for field, val in [("tile_size", 3), ("tile_size", 33), ("max_vpls_per_tile", 65), ("denoise_passes", 1), ("width", 0),
                       ("gi_mode", 3), ("max_vpls", 10001)]:
        cfg = abi.Config()
        lib.sgi_config_defaults(C.byref(cfg), 64, 48)
        setattr(cfg, field, val)
        assert lib.sgi_create(C.byref(cfg), C.byref(h)) == abi.SGI_ERR_ARG, field
    assert lib.sgi_create(None, C.byref(h)) == abi.SGI_ERR_ARG
    assert lib.sgi_status_string(abi.SGI_ERR_CAP) == b"capacity exceeded"


def test_log_callback_receives_failures():
    """sgi_set_log_callback: a rejected configuration is reported through the callback with its reason."""
    lib = abi.load(build_if_missing=True)
    got = []
    cb = abi.LOG_FN(lambda level, msg, user: got.append((level, msg.decode())))
    lib.sgi_set_log_callback(C.cast(cb, C.c_void_p), None)
    try:
        cfg = abi.config_defaults(64, 48)
        cfg.tile_size = 40
        h = C.c_void_p()
        assert lib.sgi_create(C.byref(cfg), C.byref(h)) == abi.SGI_ERR_ARG
        lib.sgi_log_message(abi.SGI_LOG_INFO, b"hello")
    finally:
        lib.sgi_set_log_callback(None, None)
    assert got[0][0] == abi.SGI_LOG_ERROR and "tile_size" in got[0][1]
    assert got[1] == (abi.SGI_LOG_INFO, "hello")
    lib.sgi_log_message(abi.SGI_LOG_INFO, b"nobody listens")   # no callback: nothing happens
    assert len(got) == 2
