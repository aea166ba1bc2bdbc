"""Trains the learned denoiser on the GPU with the library's own kernels.

    python -m stratusgfx_gb300.train_denoiser --frames 4096 --steps 4000 --out PATH

Training pairs come from seeded random rooms (40 boxes, 2048 VPLs, 256 x 256
frames, K in {2, 4, 8} samples per pixel) rendered by the plain path; the
target is the converged GI of sgi_gi_target (64 batches of 8 samples, FP64
sums). The weights are written with a versioned header and CRC (denoiser.py).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=4096)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--crop", type=int, default=128)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=100)
    ap.add_argument("--out", default=None)
    ap.add_argument("--checkpoint", default=None, help="write parameters + Adam state here every 500 steps")
    ap.add_argument("--resume", action="store_true", help="continue from --checkpoint")
    args = ap.parse_args()
    import torch

    from stratusgfx_gb300 import build, denoiser
    build.build()
    torch.cuda.set_device(0)
    t0 = time.time()
    ds = denoiser.make_dataset(args.frames, args.size, args.size, seed=args.seed)
    t_data = time.time() - t0
    net = denoiser.KpcnDenoiser(args.batch, args.crop, args.crop, seed=args.seed)
    start = 0
    if args.resume and args.checkpoint and os.path.exists(args.checkpoint):
        net.load_checkpoint(args.checkpoint)
        start = net.optimizer_state()[2]
    t0 = time.time()
    losses = denoiser.train(net, ds, steps=args.steps, batch=args.batch, crop=args.crop, lr=args.lr, seed=args.seed,
                            checkpoint=args.checkpoint, start=start)
    t_train = time.time() - t0
    out = args.out or denoiser.WEIGHTS
    net.save(out)
    print(json.dumps({"weights": out, "frames": ds.n, "data_s": round(t_data, 1), "train_s": round(t_train, 1),
                      "steps": args.steps, "losses": losses}))


if __name__ == "__main__":
    main()
