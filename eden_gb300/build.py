"""Compile libeden_gpu.so in-tree for sm_103a with nvcc.

The library is the product's compute path; it is built next to this file
(eden_gb300/libeden_gpu.so) so the interpreter loads it from the source
tree.  Rebuilds only when a source is newer than the library.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libeden_gpu.so")
SOURCES = [os.path.join(HERE, "csrc", f) for f in ("eden_gpu.cu", "eden_kernels.cuh", "eden_math.cuh")]
HEADER = os.path.join(ROOT, "include", "eden_gpu.h")
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-shared"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in SOURCES + [HEADER])


def build(force: bool = False, verbose: bool = False) -> str:
    if force or needs_build():
        cmd = [nvcc(), *NVCC_FLAGS, os.path.join(HERE, "csrc", "eden_gpu.cu"), "-o", LIB + ".tmp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
