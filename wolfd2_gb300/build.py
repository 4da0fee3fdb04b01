"""In-tree build of the CUDA library (sm_103a) with plain nvcc.

``build_library()`` compiles ``csrc/w2_api.cu`` into ``_lib/libwolfd2gpu.so``.
The FP64 translation unit is compiled with ``--fmad=false`` so each reference
expression is evaluated operation by operation (no fused multiply-add), which
is what makes the device results bit-identical to the reference arithmetic.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libwolfd2gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the wolfd2 GPU library needs the CUDA toolkit")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cuh")))


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    inc = os.path.join(os.path.dirname(HERE), "include", "wolfd2_gpu.h")
    return any(os.path.getmtime(s) > t for s in sources() + [inc])


def build_library(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), "-O3", "-std=c++17", *ARCH, "-lineinfo", "--fmad=false", "-Xcompiler", "-ffp-contract=off",
           "-Xcompiler", "-fPIC", "-shared", "-o", tmp,
           os.path.join(CSRC, "w2_api.cu"), os.path.join(CSRC, "w2_noalloc.cu")]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB
