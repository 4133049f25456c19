"""Compiles the CUDA library libshdom_gb300.so in-tree (at3d_gb300/_build/).

Single translation unit pair, one -gencode for sm_103a, no CMake.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libshdom_gb300.so")
SOURCES = [os.path.join(HERE, "csrc", "shdom_gpu.cu"), os.path.join(HERE, "csrc", "shdom_plan.cpp"),
           os.path.join(HERE, "csrc", "shdom_paths.cpp"),
           os.path.join(HERE, "csrc", "shdom_mie.cpp"), os.path.join(HERE, "csrc", "shdom_mix.cpp")]
HEADERS = (sorted(glob.glob(os.path.join(HERE, "csrc", "*.h"))) + sorted(glob.glob(os.path.join(HERE, "csrc", "*.cuh")))
           + sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))))


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in SOURCES + HEADERS)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-O3", "-shared", "-diag-suppress", "550",
           "-o", tmp] + SOURCES + ["-lpthread"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
