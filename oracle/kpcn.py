"""Float64 numpy oracle of the learned denoiser (TEST INFRASTRUCTURE ONLY).

The same U-Net, kernel apply and loss as include/sgi_nn.h, written directly
from the definitions: 3x3 convolutions with zero padding (weights
[cout][ky*3+kx][cin]), 2x2 average pooling, nearest 2x upsampling, ReLU, a
softmax 5x5 kernel with edge-clamped taps, a sigmoid temporal blend, and the
loss mean |log1p(out) - log1p(target)| over pixels and the three colour
channels. Used to check the GPU gradients (sgi_nn_train_step) and outputs
(sgi_nn_forward); its own backward is checked by finite differences.
"""
from __future__ import annotations

import numpy as np

LAYERS = [("e1a", 16, 32), ("e1b", 32, 32), ("e2a", 32, 64), ("e2b", 64, 64), ("b1", 64, 128), ("b2", 128, 128),
          ("d2a", 192, 64), ("d2b", 64, 64), ("d1a", 96, 32), ("d1b", 32, 32), ("head", 32, 32)]


def unpack(params: np.ndarray) -> dict:
    """Flat parameter vector (library layout) -> {name: (w [co, 9, ci], b [co])}."""
    out, off = {}, 0
    for name, ci, co in LAYERS:
        n = co * 9 * ci
        w = params[off:off + n].reshape(co, 9, ci)
        off += n
        b = params[off:off + co]
        off += co
        out[name] = (w, b)
    return out


def pack(grads: dict) -> np.ndarray:
    return np.concatenate([np.concatenate([grads[n][0].reshape(-1), grads[n][1]]) for n, _, _ in LAYERS])


def _cols(x):
    B, H, W, C = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    return np.stack([xp[:, ky:ky + H, kx:kx + W, :] for ky in range(3) for kx in range(3)], axis=3)


def conv(x, w, b):
    return np.einsum("bhwtc,otc->bhwo", _cols(x), w) + b


def conv_bwd(x, w, dz):
    cols = _cols(x)
    dw = np.einsum("bhwtc,bhwo->otc", cols, dz)
    db = dz.sum(axis=(0, 1, 2))
    dcols = np.einsum("bhwo,otc->bhwtc", dz, w)
    B, H, W, C = x.shape
    dxp = np.zeros((B, H + 2, W + 2, C))
    t = 0
    for ky in range(3):
        for kx in range(3):
            dxp[:, ky:ky + H, kx:kx + W, :] += dcols[:, :, :, t, :]
            t += 1
    return dxp[:, 1:H + 1, 1:W + 1, :], dw, db


def pool(x):
    B, H, W, C = x.shape
    return x.reshape(B, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def pool_bwd(d):
    return np.repeat(np.repeat(d, 2, axis=1), 2, axis=2) * 0.25


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_bwd(d):
    B, H, W, C = d.shape
    return d.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def forward(p: dict, feat: np.ndarray) -> dict:
    a = {}
    relu = lambda v: np.maximum(v, 0.0)  # noqa: E731
    a["e1a"] = relu(conv(feat, *p["e1a"]))
    a["e1b"] = relu(conv(a["e1a"], *p["e1b"]))
    a["p1"] = pool(a["e1b"])
    a["e2a"] = relu(conv(a["p1"], *p["e2a"]))
    a["e2b"] = relu(conv(a["e2a"], *p["e2b"]))
    a["p2"] = pool(a["e2b"])
    a["b1"] = relu(conv(a["p2"], *p["b1"]))
    a["b2"] = relu(conv(a["b1"], *p["b2"]))
    a["d2in"] = np.concatenate([up(a["b2"]), a["e2b"]], axis=3)
    a["d2a"] = relu(conv(a["d2in"], *p["d2a"]))
    a["d2b"] = relu(conv(a["d2a"], *p["d2b"]))
    a["d1in"] = np.concatenate([up(a["d2b"]), a["e1b"]], axis=3)
    a["d1a"] = relu(conv(a["d1in"], *p["d1a"]))
    a["d1b"] = relu(conv(a["d1a"], *p["d1b"]))
    a["head"] = conv(a["d1b"], *p["head"])
    return a


def apply(logits, noisy, prev, target=None):
    """Kernel apply (+ loss and dlogits when target is given). noisy/prev/target: [B, H, W, 3]."""
    B, H, W, _ = logits.shape
    l = logits[..., :25]
    l = l - l.max(axis=3, keepdims=True)
    e = np.exp(l)
    wk = e / e.sum(axis=3, keepdims=True)
    ys = np.clip(np.arange(H)[:, None] + (np.arange(25) // 5 - 2)[None, :], 0, H - 1)    # [H, 25]
    xs = np.clip(np.arange(W)[:, None] + (np.arange(25) % 5 - 2)[None, :], 0, W - 1)     # [W, 25]
    nb = noisy[:, ys[:, None, :], xs[None, :, :], :]                                      # [B, H, W, 25, 3]
    sp = np.einsum("bhwk,bhwkc->bhwc", wk, nb)
    alpha = 1.0 / (1.0 + np.exp(-logits[..., 25:26]))
    out = alpha * sp + (1.0 - alpha) * prev
    if target is None:
        return out
    oc = np.maximum(out, 0.0)
    d = np.log1p(oc) - np.log1p(np.maximum(target, 0.0))
    n = 3 * B * H * W
    loss = np.abs(d).sum() / n
    dout = np.where(out > 0.0, np.sign(d) / (1.0 + oc), 0.0) / n
    dalpha = (dout * (sp - prev)).sum(axis=3, keepdims=True)
    dw = alpha * np.einsum("bhwc,bhwkc->bhwk", dout, nb)
    dl = np.zeros_like(logits)
    dl[..., :25] = wk * (dw - (wk * dw).sum(axis=3, keepdims=True))
    dl[..., 25:26] = dalpha * alpha * (1.0 - alpha)
    return out, loss, dl


def backward(p: dict, feat: np.ndarray, a: dict, dlogits: np.ndarray) -> dict:
    g = {}
    dx, g["head"] = (lambda r: (r[0], r[1:]))(conv_bwd(a["d1b"], p["head"][0], dlogits))
    dz = dx * (a["d1b"] > 0)
    dx, *g["d1b"] = conv_bwd(a["d1a"], p["d1b"][0], dz)
    dz = dx * (a["d1a"] > 0)
    dd1in, *g["d1a"] = conv_bwd(a["d1in"], p["d1a"][0], dz)
    dd2b = up_bwd(dd1in[..., :64])
    dskip1 = dd1in[..., 64:]
    dz = dd2b * (a["d2b"] > 0)
    dx, *g["d2b"] = conv_bwd(a["d2a"], p["d2b"][0], dz)
    dz = dx * (a["d2a"] > 0)
    dd2in, *g["d2a"] = conv_bwd(a["d2in"], p["d2a"][0], dz)
    db2 = up_bwd(dd2in[..., :128])
    dskip2 = dd2in[..., 128:]
    dz = db2 * (a["b2"] > 0)
    dx, *g["b2"] = conv_bwd(a["b1"], p["b2"][0], dz)
    dz = dx * (a["b1"] > 0)
    dp2, *g["b1"] = conv_bwd(a["p2"], p["b1"][0], dz)
    de2b = dskip2 + pool_bwd(dp2)
    dz = de2b * (a["e2b"] > 0)
    dx, *g["e2b"] = conv_bwd(a["e2a"], p["e2b"][0], dz)
    dz = dx * (a["e2a"] > 0)
    dp1, *g["e2a"] = conv_bwd(a["p1"], p["e2a"][0], dz)
    de1b = dskip1 + pool_bwd(dp1)
    dz = de1b * (a["e1b"] > 0)
    dx, *g["e1b"] = conv_bwd(a["e1a"], p["e1b"][0], dz)
    dz = dx * (a["e1a"] > 0)
    _, *g["e1a"] = conv_bwd(feat, p["e1a"][0], dz)
    return {k: (v[0], v[1]) for k, v in g.items()}


def loss_and_grads(params: np.ndarray, feat, noisy, prev, target):
    p = unpack(params)
    a = forward(p, feat)
    out, loss, dl = apply(a["head"], noisy, prev, target)
    return loss, pack(backward(p, feat, a, dl)), out
