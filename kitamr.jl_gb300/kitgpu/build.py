"""Build of libkitgpu.so (sm_103a) from csrc/: one nvcc process per translation unit, run in
parallel, then one link.  Output: kitgpu/_lib/libkitgpu.so (in-tree)."""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libkitgpu.so")
SOURCES = ["kg_api.cu", "kg_kernels.cu", "kg_flatten.cpp", "kg_devflat.cu", "kg_noalloc.cu"]
# the two builders of the gather form (host, device) must round every double expression alike:
# no FMA contraction in either
FILE_FLAGS = {"kg_flatten.cpp": ["-Xcompiler", "-ffp-contract=off"], "kg_devflat.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")


def _flags(extra=()):
    return ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", *ARCH, *extra]


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(CSRC, s) for s in SOURCES] + [
        os.path.join(CSRC, h) for h in ("kg_internal.h", "kg_device.cuh", "kg_devflat.h")] + [
        os.path.join(os.path.dirname(ROOT), "include", "kitgpu.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [NVCC, *_flags(FILE_FLAGS.get(src, ())), "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
