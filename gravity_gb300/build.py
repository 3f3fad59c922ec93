"""Build recipe of libgbh.so (the C-ABI library) for sm_103a, in-tree.

Every .cu file under csrc/ is compiled in parallel by nvcc into
gravity_gb300/_build/ and linked into gravity_gb300/libgbh.so.  The library is
compiled with --fmad=false: the step's FP32 arithmetic rounds once per
operation, in source order, like the reference GLSL restated as IEEE FP32.
The group and learned walks (k_walk_group.cu) are new algorithms with no
bit-level counterpart in the reference, so their translation unit lets the
compiler contract multiply-adds.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbh.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                "-I", os.path.join(HERE, "..", "include")]
FMAD_CONTRACT = {"k_walk_group.cu"}


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    deps = [src] + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    deps.append(os.path.join(HERE, "..", "include", "gbh.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    fmad = "--fmad=true" if os.path.basename(src) in FMAD_CONTRACT else "--fmad=false"
    cmd = [NVCC] + FLAGS + [fmad, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
