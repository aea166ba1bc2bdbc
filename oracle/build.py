"""Builds the CPU oracle (TEST INFRASTRUCTURE ONLY) into oracle/_build/liboracle.so.

g++ with -ffp-contract=off so that binary32 expressions round operation by
operation (no fused multiply-add on any host), matching the CUDA kernels that
are built with -fmad=false. OpenMP parallelises over rows and tiles.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
SOURCES = ["oracle_api.cpp"]
DEPS = SOURCES + ["glsl.hpp", "counted.hpp", "passes.hpp", "../include/sgi.h", "../include/sgi_scene.h"]
# -fno-strict-aliasing: the operation-counting instantiation reads and writes float32
# buffers through its one-float wrapper type.
FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fno-strict-aliasing", "-fPIC",
         "-shared", "-Wall"]


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, d) for d in DEPS]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    cmd = ["g++"] + FLAGS + [os.path.join(HERE, s) for s in SOURCES] + ["-o", LIB]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + res.stdout)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
