"""In-tree build of libdpg.so for sm_103a (nvcc, no cmake).

``python -m dynoplan_gb300.build`` or ``build_library()``.
"""
from __future__ import annotations

import os
import shutil
import subprocess

_HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(_HERE)
CSRC = os.path.join(_HERE, "csrc")
LIB = os.path.join(_HERE, "libdpg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = ["dpg.cu", "bench_util.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build_library(verbose: bool = False) -> str:
    """Compile every CUDA source into dynoplan_gb300/libdpg.so."""
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-o", LIB + ".tmp", *srcs, "-lcudart"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
