"""Builds libsgi.so (CUDA kernels for sm_103a + the C++ host layer) in-tree.

Run as ``python -m stratusgfx_gb300.build``. Objects and the library land in
``stratusgfx_gb300/_build/``. nvcc cross-compiles, so this works on a machine
without a GPU.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsgi.so")
REPO = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: every binary32 product and sum rounds on its own, so kernel
# results are bit-reproducible against the CPU restatement of the shaders.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-Xcompiler", "-fPIC", "-I" + os.path.join(REPO, "include")]
CUDA_SOURCES = ["sgi_kernels.cu", "sgi_shade.cu", "sgi_shade_fast.cu", "sgi_scene.cu", "sgi_nn.cu", "sgi_nn_tc.cu",
                "sgi_selftest.cu", "sgi_stats.cu"]
HOST_SOURCES = ["sgi_api.cpp", "sgi_nn_api.cpp", "sgi_batch.cpp", "sgi_slots.cpp", "sgi_host.cpp"]
# The learned denoiser is checked against the oracle within a tolerance, not bit
# for bit, so its kernels keep the compiler's default multiply-add contraction.
FAST_MATH_OK = {"sgi_nn.cu", "sgi_nn_tc.cu"}
# The tolerance-mode shading kernels: contraction, approximate division and square
# root (subnormals are kept: the decision-side arithmetic must round as in the
# exact build).
FAST_SHADING = {"sgi_shade_fast.cu"}
FAST_SHADING_FLAGS = ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))), "include")


def _run(cmd: list[str]) -> str:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout)
    return res.stdout


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(CSRC, "sgi_shade.cu"))   # included by sgi_shade_fast.cu
    headers += [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            flags = [f for f in NVCC_FLAGS if not (src in FAST_MATH_OK and f == "-fmad=false")]
            if src in FAST_SHADING:
                flags = [f for f in flags if f not in ("-fmad=false", "-prec-div=true", "-prec-sqrt=true")]
                flags += FAST_SHADING_FLAGS
            jobs.append([nvcc] + flags + ["-Xptxas", "-v", "-c", s, "-o", o])
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cpp", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", "-I" + _cuda_include(),
                         "-I" + os.path.join(REPO, "include"), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for log in logs:
            sys.stdout.write(log)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
