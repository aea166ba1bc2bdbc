"""Shared test utilities: uploading oracle-side inputs to the device and comparing results."""
from __future__ import annotations

import numpy as np


def half_bits_equal(a16: np.ndarray, b16: np.ndarray) -> np.ndarray:
    """Elementwise equality of float16 arrays by value, NaN == NaN (any payload), +0 == -0."""
    a = a16.astype(np.float32)
    b = b16.astype(np.float32)
    return (a == b) | (np.isnan(a) & np.isnan(b))


def f32_equal(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a = np.asarray(a, dtype=np.float32)
    b = np.asarray(b, dtype=np.float32)
    return (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b)) | (a == b)


def rel_err(gpu: np.ndarray, ref: np.ndarray) -> float:
    g = np.asarray(gpu, dtype=np.float64)
    r = np.asarray(ref, dtype=np.float64)
    ok = np.isfinite(g) & np.isfinite(r)
    d = np.abs(g - r)[ok] / np.maximum(np.abs(r[ok]), 1e-6)
    return float(d.max()) if d.size else 0.0


def psnr(img: np.ndarray, ref: np.ndarray) -> float:
    x = np.asarray(img, dtype=np.float64)
    r = np.asarray(ref, dtype=np.float64)
    mse = float(np.mean((x - r) ** 2))
    peak = float(np.max(np.abs(r)))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def assert_bit_exact(gpu, ref, what: str, eq=None):
    eq = eq or f32_equal
    m = eq(gpu, ref)
    frac = float(m.mean())
    if frac < 1.0:
        bad = np.argwhere(~m)
        first = tuple(bad[0])
        raise AssertionError(f"{what}: {(~m).sum()} of {m.size} differ (exact fraction {frac:.6f}); "
                             f"first at {first}: gpu={gpu[first]!r} oracle={ref[first]!r}; "
                             f"max rel err {rel_err(gpu, ref):.3e}")


def upload_gbuffer(hg, device="cuda"):
    """oracle HostGBuffer -> stage.GBufferTensors holding the same bytes."""
    import torch
    from stratusgfx_gb300.stage import GBufferTensors
    H, W = hg.depth.shape
    g = GBufferTensors(H, W, device)
    for name in hg.NAMES:
        getattr(g, name).copy_(torch.from_numpy(np.ascontiguousarray(getattr(hg, name))))
    return g


def upload_cubes(storage: np.ndarray, fmt: int, layers: int = 320, device="cuda"):
    import torch
    from stratusgfx_gb300 import abi
    t = torch.from_numpy(storage.view(np.int16) if storage.dtype == np.uint16 else storage).to(device)
    at = abi.CubeAtlas()
    for a in range(storage.shape[0]):
        at.atlas[a] = t[a].data_ptr()
    at.num_atlases, at.layers_per_atlas, at.face_size, at.format = storage.shape[0], layers, storage.shape[-1], fmt
    return t, at


def half4_to_f32(buf: np.ndarray, H: int, W: int) -> np.ndarray:
    return buf.view(np.float16).reshape(H, W, 4).astype(np.float32)


def host_scene_from_device(ds, frames, cubes=True):
    """oracle HostScene over the device generator's inputs (bit-identical to the CPU ray caster) for
    the listed frames: their G-buffers and CSMs, and the cube atlas unless cubes=False."""
    from oracle import binding as O
    g = [None] * len(ds.gbuffers)
    for k in frames:
        g[k] = ds.gbuffers[k].numpy()
    csm = {k: ds.csm_depth[k].cpu().numpy() for k in frames}
    storage = ds.cube_storage.cpu().numpy() if cubes else None
    return O.HostScene.from_arrays(ds.scene, ds.w, g, csm, storage)


class GpuSetup:
    """A workload's inputs from the oracle's CPU ray caster, uploaded: G-buffers, CSMs, cube atlas, lights."""

    def __init__(self, w, seed: int, **cfgkw):
        import torch

        from oracle import binding as O
        from stratusgfx_gb300 import scene as S
        from stratusgfx_gb300 import stage
        self.w = w
        self.sc = S.workload_scene(w, seed)
        self.hs = O.HostScene(self.sc, w)
        self.cfg = stage.workload_config(w, **cfgkw)
        self.g = [upload_gbuffer(g) for g in self.hs.gbuffers]
        self.csm_t = [torch.from_numpy(d).cuda() for d in self.hs.csm_depth]
        self.csm = [stage.csm_struct(self.sc, k, self.csm_t[k].data_ptr(), w.csm_resolution)
                    for k in range(len(self.sc.cameras))]
        self.cube_t, self.cubes = upload_cubes(self.hs.cube_storage, w.cube_format, self.sc.layers_per_atlas)
        self.vpls = torch.from_numpy(self.sc.vpls).cuda()
        self.entries = torch.from_numpy(self.sc.entries).cuda()
        self.points = torch.from_numpy(self.sc.points).cuda() if len(self.sc.points) else None

    def stage(self, k=1, **cfgkw):
        from stratusgfx_gb300 import stage
        cfgkw.setdefault("debug_keep_passes", 1)
        cfg = stage.workload_config(self.w, **cfgkw)
        st = stage.GiStage(cfg)
        st.set_lights(self.vpls, self.entries, self.points)
        st.set_shadow_maps(self.csm[k], self.cubes)
        return st, cfg
