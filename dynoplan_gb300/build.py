"""In-tree build of libdpg.so for sm_103a (nvcc, no cmake).

``python -m dynoplan_gb300.build`` or ``build_library()``.  Translation units
compile in parallel, then link into dynoplan_gb300/libdpg.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile

_HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(_HERE)
CSRC = os.path.join(_HERE, "csrc")
LIB = os.path.join(_HERE, "libdpg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]

SOURCES = ["dpg.cu", "bench_util.cu", "mlp.cu", "search.cu", "prim_io.cu", "roadmap.cu", "tdb.cu", "lazy.cu", "tune.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build_library(verbose: bool = False) -> str:
    """Compile every CUDA source into dynoplan_gb300/libdpg.so."""
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    with tempfile.TemporaryDirectory(prefix="dpg_build_") as tmp:
        objs, procs = [], []
        for s in SOURCES:
            obj = os.path.join(tmp, s.replace(".cu", ".o"))
            cmd = [nvcc(), *ARCH, *FLAGS, *inc, "-c", os.path.join(CSRC, s), "-o", obj]
            if verbose:
                print(" ".join(cmd))
            procs.append(subprocess.Popen(cmd))
            objs.append(obj)
        for p in procs:
            if p.wait() != 0:
                raise subprocess.CalledProcessError(p.returncode, p.args)
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
