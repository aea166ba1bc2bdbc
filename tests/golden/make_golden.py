"""Generates tests/golden/*.npz: the CPU oracle's outputs on tiny seeded scenes.

StratusGFX has no golden vectors for its shaders (its GLSL runs only inside an
OpenGL driver), so these fixtures record the oracle itself: they pin it
against regressions and give the GPU tests a second, committed reference.
Each fixture stores the scene description (boxes, lights, camera and cascade
matrices), so a machine with a different libm rebuilds bit-identical inputs
with the oracle's ray caster. Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import binding as O  # noqa: E402
from stratusgfx_gb300 import abi, stage  # noqa: E402
from stratusgfx_gb300 import scene as S  # noqa: E402

CASES = {
    # name: (workload, seed, config overrides)
    "tiled_64x40": (S.Workload("room12_64x40_vpl24", 64, 40, 12, 24, 2, 256, 8, abi.SGI_CUBE_F16, 4, 3, 2,
                               tile_size=16, max_per_tile=8), 11, {}),
    "reference_48x32": (S.Workload("room8_48x32_vpl16", 48, 32, 8, 16, 1, 256, 8, abi.SGI_CUBE_UNORM16, 0, 4, 2,
                                   tile_size=8, max_per_tile=4), 12, {"gi_mode": abi.SGI_GI_REFERENCE}),
}
TIME, FPS = 1000.0, 60.0


def run_case(w, sc, overrides):
    hs = O.HostScene(sc, w)
    cfg = stage.workload_config(w, **overrides)
    H, W = w.height, w.width
    out = {}
    for prec in (32, 64):
        gi = np.zeros((H, W, 4))
        hist = np.zeros((H, W))
        for k in (1, 2):
            r = O.frame(prec, cfg, hs, k, gi, hist, TIME + 16.0 * k, FPS)
            gi, hist = r["gi"], r["hist"]
            tag = f"f{prec}_k{k}_"
            out[tag + "combined"] = r["combined"]
            out[tag + "hist"] = r["hist"]
            if prec == 32:
                out[tag + "visible_index"] = r["visible_index"]
                out[tag + "reservoir"] = r["reservoir"]
                out[tag + "direct"] = r["direct"]
                if r["lists"] is not None:
                    out[tag + "lists"] = r["lists"]
    return out


def main():
    for name, (w, seed, overrides) in CASES.items():
        sc = S.workload_scene(w, seed)
        arrays = {"scene_" + k: v for k, v in S.scene_arrays(sc).items()}
        arrays.update(run_case(w, sc, overrides))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, sum(v.nbytes for v in arrays.values()), "bytes raw")


if __name__ == "__main__":
    main()
