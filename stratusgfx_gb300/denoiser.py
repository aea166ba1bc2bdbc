"""The learned kernel-predicting denoiser (include/sgi_nn.h) from Python.

``KpcnDenoiser`` wraps an sgi_nn network; ``make_dataset`` renders training
pairs with the plain path (K-sample noisy GI + features vs the FP64-accumulated
converged GI of sgi_gi_target); ``train`` runs the library's own forward /
backward / Adam kernels on random crops. Weight files carry a versioned
header (magic, version, parameter count, layer shapes, dtype) and a CRC32.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import struct
import time
import zlib

import numpy as np
import torch

from . import abi, stage
from . import scene as S

CKPT_MAGIC = b"SGICKPT1"
MAGIC = b"SGIKPCN1"
LAYERS = [(16, 32), (32, 32), (32, 64), (64, 64), (64, 128), (128, 128), (192, 64), (64, 64), (96, 32), (32, 32),
          (32, 32)]
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "kpcn_bf16.bin")


def _p(t):
    return C.c_void_p(None if t is None else t.data_ptr())


class KpcnDenoiser:
    def __init__(self, max_batch: int, max_height: int, max_width: int, seed: int = 0):
        self.lib = abi.load()
        cfg = abi.NnConfig(max_batch, max_height, max_width, seed)
        h = C.c_void_p()
        abi.check(self.lib.sgi_nn_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.n = int(self.lib.sgi_nn_num_params(h))

    def close(self):
        if self.h:
            self.lib.sgi_nn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st):
        if st != abi.SGI_OK:
            raise abi.SgiError(st, self.lib.sgi_nn_last_error(self.h).decode())

    def params(self) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        self._chk(self.lib.sgi_nn_get_params(self.h, out.ctypes.data_as(C.c_void_p), self.n))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._chk(self.lib.sgi_nn_set_params(self.h, p.ctypes.data_as(C.c_void_p), self.n))

    def grads(self) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        self._chk(self.lib.sgi_nn_get_grads(self.h, out.ctypes.data_as(C.c_void_p), self.n))
        return out

    def train_step(self, feat, noisy, prev, target, lr: float, update: bool = True, want_loss: bool = True,
                   stream=None) -> float:
        B, H, W = feat.shape[:3]
        loss = C.c_float(0.0)
        self._chk(self.lib.sgi_nn_train_step(self.h, _p(feat), _p(noisy), _p(prev), _p(target), B, H, W, lr,
                                             1 if update else 0, C.byref(loss) if want_loss else None,
                                             stage._stream_ptr(stream)))
        return float(loss.value)

    def set_conv_path(self, path: int):
        """abi.SGI_NN_CONV_TCGEN05 (tcgen05.mma, TMEM accumulators) or abi.SGI_NN_CONV_WARP_MMA."""
        self._chk(self.lib.sgi_nn_set_conv_path(self.h, path))

    def set_head_fusion(self, enabled: bool):
        """The neural frame's kernel apply in the head convolution's epilogue (default) or as a separate pass."""
        self._chk(self.lib.sgi_nn_set_head_fusion(self.h, 1 if enabled else 0))

    def set_precision(self, precision: int):
        """abi.SGI_NN_BF16 or abi.SGI_NN_FP8 (after calibrate_fp8)."""
        self._chk(self.lib.sgi_nn_set_precision(self.h, precision))

    def calibrate_fp8(self, feat, stream=None):
        """Per-channel FP8 scales from the BF16 network's activations on `feat` [B, H, W, 16]."""
        B, H, W = feat.shape[:3]
        self._chk(self.lib.sgi_nn_calibrate_fp8(self.h, _p(feat), B, H, W, stage._stream_ptr(stream)))

    def set_wait_test(self, wait_ns: int = 0, skip_producer: bool = False):
        """Limit of the tensor-core kernels' waits (convolutions, weight gradients; 0: default) and the producer
        test switch."""
        self._chk(self.lib.sgi_nn_set_wait_test(self.h, int(wait_ns), 1 if skip_producer else 0))

    def device_status(self):
        """Synchronises; raises SgiError(SGI_ERR_TIMEOUT) if a tensor-core wait ran out."""
        self._chk(self.lib.sgi_nn_device_status(self.h))

    def forward(self, feat, noisy, prev, out, stream=None):
        B, H, W = feat.shape[:3]
        self._chk(self.lib.sgi_nn_forward(self.h, _p(feat), _p(noisy), _p(prev), B, H, W, _p(out),
                                          stage._stream_ptr(stream)))

    def save(self, path: str):
        p = self.params()
        shapes = b"".join(struct.pack("<ii", ci, co) for ci, co in LAYERS)
        body = p.tobytes()
        header = MAGIC + struct.pack("<IIqI", 1, len(LAYERS), self.n, 0) + shapes   # version 1, dtype 0 = fp32
        blob = header + body
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "wb") as f:
            f.write(blob + struct.pack("<I", zlib.crc32(blob) & 0xFFFFFFFF))

    def optimizer_state(self):
        """(m, v, step): the Adam moments and the number of updates taken."""
        m = np.empty(self.n, np.float32)
        v = np.empty(self.n, np.float32)
        step = C.c_int64()
        self._chk(self.lib.sgi_nn_get_optimizer_state(self.h, m.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p),
                                                      self.n, C.byref(step)))
        return m, v, step.value

    def set_optimizer_state(self, m, v, step: int):
        m = np.ascontiguousarray(m, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        self._chk(self.lib.sgi_nn_set_optimizer_state(self.h, m.ctypes.data_as(C.c_void_p),
                                                      v.ctypes.data_as(C.c_void_p), self.n, int(step)))

    def save_checkpoint(self, path: str):
        """Training checkpoint: parameters, Adam moments and step (magic, version 1, layer shapes, CRC32)."""
        m, v, step = self.optimizer_state()
        shapes = b"".join(struct.pack("<ii", ci, co) for ci, co in LAYERS)
        header = CKPT_MAGIC + struct.pack("<IIqq", 1, len(LAYERS), self.n, step) + shapes
        blob = header + self.params().tobytes() + m.tobytes() + v.tobytes()
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "wb") as f:
            f.write(blob + struct.pack("<I", zlib.crc32(blob) & 0xFFFFFFFF))

    def load_checkpoint(self, path: str):
        with open(path, "rb") as f:
            blob = f.read()
        data, crc = blob[:-4], struct.unpack("<I", blob[-4:])[0]
        if data[:8] != CKPT_MAGIC or zlib.crc32(data) & 0xFFFFFFFF != crc:
            raise ValueError(f"{path}: bad magic or CRC")
        version, nlayers, n, step = struct.unpack("<IIqq", data[8:32])
        shapes = [struct.unpack("<ii", data[32 + 8 * i:40 + 8 * i]) for i in range(nlayers)]
        if version != 1 or n != self.n or shapes != LAYERS:
            raise ValueError(f"{path}: incompatible checkpoint ({version}, {shapes})")
        off = 32 + 8 * nlayers
        arr = np.frombuffer(data[off:off + 12 * n], dtype=np.float32)
        self.set_params(arr[:n])
        self.set_optimizer_state(arr[n:2 * n], arr[2 * n:], step)

    def load(self, path: str):
        with open(path, "rb") as f:
            blob = f.read()
        data, crc = blob[:-4], struct.unpack("<I", blob[-4:])[0]
        if data[:8] != MAGIC or zlib.crc32(data) & 0xFFFFFFFF != crc:
            raise ValueError(f"{path}: bad magic or CRC")
        version, nlayers, n, dtype = struct.unpack("<IIqI", data[8:28])
        shapes = [struct.unpack("<ii", data[28 + 8 * i:36 + 8 * i]) for i in range(nlayers)]
        if version != 1 or dtype != 0 or n != self.n or shapes != LAYERS:
            raise ValueError(f"{path}: incompatible network ({version}, {shapes})")
        off = 28 + 8 * nlayers
        self.set_params(np.frombuffer(data[off:off + 4 * n], dtype=np.float32))


class Dataset:
    """Training pairs resident on the GPU: features BF16 [N, H, W, 16], noisy / prev / target float [N, H, W, 4]."""

    def __init__(self, n, H, W, device="cuda"):
        self.feat = torch.empty((n, H, W, 16), dtype=torch.bfloat16, device=device)
        self.noisy = torch.empty((n, H, W, 4), dtype=torch.float32, device=device)
        self.prev = torch.empty((n, H, W, 4), dtype=torch.float32, device=device)
        self.target = torch.empty((n, H, W, 4), dtype=torch.float32, device=device)
        self.n = 0


def make_dataset(num_frames: int, H: int = 256, W: int = 256, frames_per_room: int = 16, seed: int = 100,
                 samples=(2, 4, 8), batches: int = 64, num_boxes: int = 40, num_vpls: int = 2048,
                 log=print) -> Dataset:
    """Plain-path training pairs: each room (seeded generator) gets a camera path of frames_per_room
    frames, rendered with K samples per pixel (K cycles through `samples` room by room) through
    sgi_render_frame (a-trous history), then its features and the converged target (batches
    independent runs of 8 samples, FP64 sums: the same target for every K)."""
    ds = Dataset(num_frames, H, W)
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    t0 = time.time()
    room = 0
    while ds.n < num_frames:
        K = samples[room % len(samples)]
        w = S.Workload(f"train_room{num_boxes}_{W}x{H}", W, H, num_boxes, num_vpls, 4, 1024, 64, abi.SGI_CUBE_F16,
                       K, 5, frames_per_room)
        cfg = stage.workload_config(w)
        tcfg = stage.workload_config(w, samples_per_pixel=8)
        sc = S.workload_scene(w, seed + room)
        dsc = stage.DeviceScene(sc, w)
        st = stage.GiStage(cfg)
        tst = stage.GiStage(tcfg)
        tst.set_lights(dsc.vpls, dsc.entries, dsc.points)
        st.set_lights(dsc.vpls, dsc.entries, dsc.points)
        for k in range(1, len(sc.cameras)):
            if ds.n >= num_frames:
                break
            st.set_shadow_maps(dsc.csms[k], dsc.cubes)
            cam = dsc.camera(k)
            t = 1000.0 + 16.0 * k
            st.render_frame(dsc.gbuffers[k], dsc.gbuffers[k - 1], cam, out, t, 60.0)
            i = ds.n
            abi.check(st.lib.sgi_nn_features(st.ctx, C.byref(dsc.gbuffers[k].struct()), C.byref(cam),
                                             _p(ds.feat[i]), _p(ds.noisy[i]), _p(ds.prev[i]),
                                             stage._stream_ptr(None)), st.ctx)
            tst.set_shadow_maps(dsc.csms[k], dsc.cubes)
            tst.cull_vpls()
            tst.cull_tiles(dsc.gbuffers[k], cam)
            tst.gi_target(dsc.gbuffers[k], cam, t + 7.0e6, batches, ds.target[i])
            ds.n += 1
        torch.cuda.synchronize()
        st.close()
        tst.close()
        del dsc
        room += 1
    log(f"dataset: {ds.n} frames of {W}x{H} from {room} rooms in {time.time() - t0:.1f} s")
    return ds


def train(net: KpcnDenoiser, ds: Dataset, steps: int = 3000, batch: int = 16, crop: int = 128, lr: float = 2e-3,
          seed: int = 0, log=print, log_every: int = 250, checkpoint: str | None = None, checkpoint_every: int = 500,
          start: int = 0) -> list:
    """Adam on random crops; cosine learning-rate decay. Returns the logged losses. With `checkpoint`, the
    parameters, Adam moments and step are written there every checkpoint_every steps; `start` resumes a run
    at that step (after load_checkpoint): the crop sampler and the learning-rate schedule continue from it."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    H, W = ds.feat.shape[1:3]
    fb = torch.empty((batch, crop, crop, 16), dtype=torch.bfloat16, device="cuda")
    nb = torch.empty((batch, crop, crop, 4), dtype=torch.float32, device="cuda")
    pb = torch.empty_like(nb)
    tb = torch.empty_like(nb)
    losses = []
    t0 = time.time()
    for it in range(steps):
        idx = torch.randint(0, ds.n, (batch,), generator=g)
        ys = torch.randint(0, (H - crop) // 4 + 1, (batch,), generator=g) * 4
        xs = torch.randint(0, (W - crop) // 4 + 1, (batch,), generator=g) * 4
        if it < start:
            continue
        for b in range(batch):
            i, y, x = int(idx[b]), int(ys[b]), int(xs[b])
            fb[b].copy_(ds.feat[i, y:y + crop, x:x + crop])
            nb[b].copy_(ds.noisy[i, y:y + crop, x:x + crop])
            pb[b].copy_(ds.prev[i, y:y + crop, x:x + crop])
            tb[b].copy_(ds.target[i, y:y + crop, x:x + crop])
        cur_lr = lr * 0.5 * (1.0 + math.cos(math.pi * it / steps))
        want = (it % log_every == 0) or it == steps - 1
        loss = net.train_step(fb, nb, pb, tb, cur_lr, True, want)
        if want:
            losses.append((it, loss))
            log(f"step {it:5d} loss {loss:.5f} lr {cur_lr:.2e} ({time.time() - t0:.1f} s)")
        if checkpoint and (it + 1) % checkpoint_every == 0:
            net.save_checkpoint(checkpoint)
    torch.cuda.synchronize()
    return losses
