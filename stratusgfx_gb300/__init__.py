"""GB300-native VPL global illumination + deferred lighting stage (StratusGFX GI/lighting drop-in).

The compute path is libsgi.so (hand-written CUDA for sm_103a behind the C ABI
declared in include/sgi.h); ``stage.GiStage`` is the Python host mirror of the
reference RendererBackend stage over that ABI.
"""
__all__ = ["abi", "build", "scene", "stage"]
