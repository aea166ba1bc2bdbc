"""Cache of the block-shape autotuner's choices (sgi_batch_create) in a JSON file.

The tuner of sgi_batch_create times every candidate thread-block shape of the
gather, the denoise passes and the direct lighting on each view, which costs a
few frames per view. The fastest shape depends on the viewport (and the kind of
frame: plain or neural), not on the scene, so the choices are kept per
"WIDTHxHEIGHT:kind" key: a batch whose views all have cached entries is built
with those shapes and without tuning; otherwise the tuner runs and its choices
are added to the file.
"""
from __future__ import annotations

import ctypes as C
import json
import os

from . import abi

PASSES = {"gather": abi.SGI_BLOCK_GATHER, "atrous": abi.SGI_BLOCK_ATROUS,
          "denoise_final": abi.SGI_BLOCK_DENOISE_FINAL, "direct": abi.SGI_BLOCK_DIRECT}


def _key(width: int, height: int, neural: bool) -> str:
    return f"{width}x{height}:{'neural' if neural else 'plain'}"


def load_cache(path: str) -> dict:
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def create_batch(views, sizes, net=None, cache: str | None = None, tune_frames: int = 2, stream=None):
    """sgi_batch_create over `views` (an abi.View array; sizes[i] = (width, height) of view i) with the block
    shapes of `cache` where every view has an entry, else tuned (tune_frames frames per shape) and recorded.
    Returns (batch handle, tuned: bool)."""
    lib = abi.load()
    n = len(sizes)
    neural = net is not None
    entries = load_cache(cache) if cache else {}
    keys = [_key(w, h, neural) for w, h in sizes]
    cached = all(k in entries for k in keys)
    if cached:
        for i in range(n):
            for name, p in PASSES.items():
                bx, by = entries[keys[i]][name]
                abi.check(lib.sgi_set_block_shape(C.c_void_p(views[i].ctx), p, bx, by))
    h = C.c_void_p()
    st = lib.sgi_batch_create(views, n, net.h if neural else None, 0 if cached else tune_frames, stream,
                              C.byref(h))
    if st != abi.SGI_OK:
        raise abi.SgiError(st, f"sgi_batch_create: {lib.sgi_batch_last_error(h)}")
    if cache and not cached:
        bx, by = C.c_int32(), C.c_int32()
        for i in range(n):
            e = {}
            for name, p in PASSES.items():
                abi.check(lib.sgi_get_block_shape(C.c_void_p(views[i].ctx), p, C.byref(bx), C.byref(by)))
                e[name] = [bx.value, by.value]
            entries[keys[i]] = e
        tmp = cache + ".tmp"
        with open(tmp, "w") as f:
            json.dump(entries, f, indent=1, sort_keys=True)
        os.replace(tmp, cache)
    return h, not cached
