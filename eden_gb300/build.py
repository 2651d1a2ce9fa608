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
HEADER = os.path.join(ROOT, "include", "eden_gpu.h")
SOURCES = [os.path.join(HERE, "csrc", f) for f in ("eden_gpu.cu", "eden_grad.cu", "eden_codegen.cuh", "eden_window.cuh",
                                                   "eden_kernels.cuh", "eden_math.cuh")]
# translation units, compiled in parallel and linked into one library
UNITS = ["eden_gpu.cu", "eden_grad.cu"]
# the kernel sources the library compiles again at run time (NVRTC), in
# dependency order; build() embeds them as csrc/_rtc_src.inc
RTC_SOURCES = [HEADER] + [os.path.join(HERE, "csrc", f) for f in ("eden_math.cuh", "eden_kernels.cuh",
                                                                 "eden_window.cuh")]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
LINK_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-ldl"]


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


def embed_rtc_sources() -> str:
    """Writes csrc/_rtc_src.inc: the kernel headers as string literals, with
    their local #include lines and #pragma once removed (they are joined in
    dependency order)."""
    parts = []
    for path in RTC_SOURCES:
        text = []
        for line in open(path).read().splitlines():
            if line.startswith('#include "') or line.strip() == "#pragma once":
                continue
            text.append(line)
        body = "\n".join(text) + "\n"
        # raw-string chunks below the compilers' literal limits
        for k in range(0, len(body), 30000):
            parts.append(body[k:k + 30000])
    out = os.path.join(HERE, "csrc", "_rtc_src.inc")
    with open(out + ".tmp", "w") as f:
        f.write("// generated by eden_gb300/build.py from " + ", ".join(os.path.basename(p) for p in RTC_SOURCES) + "\n")
        f.write("static const char *const kRtcSourceParts[] = {\n")
        for chunk in parts:
            assert ")EDENRTC" not in chunk
            f.write('R"EDENRTC(' + chunk + ')EDENRTC",\n')
        f.write("};\n")
    os.replace(out + ".tmp", out)
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    if force or needs_build():
        embed_rtc_sources()
        objs, procs = [], []
        for unit in UNITS:
            obj = os.path.join(HERE, "csrc", "_" + unit.replace(".cu", ".o"))
            cmd = [nvcc(), *NVCC_FLAGS, "-c", os.path.join(HERE, "csrc", unit), "-o", obj]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((cmd, subprocess.Popen(cmd)))
            objs.append(obj)
        for cmd, p in procs:
            if p.wait() != 0:
                raise subprocess.CalledProcessError(p.returncode, cmd)
        cmd = [nvcc(), *LINK_FLAGS, *objs, "-o", LIB + ".tmp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    build_host(verbose)
    return LIB


HOST_SRC = os.path.join(HERE, "host", "eden_gpu_host.cpp")
HOST_BIN = os.path.join(HERE, "host", "eden_gpu_host")


def build_host(verbose: bool = False) -> str:
    """The C++ host program (eden_gb300/host/eden_gpu_host.cpp), linked
    against the library next to it."""
    if not os.path.exists(HOST_BIN) or any(os.path.getmtime(p) > os.path.getmtime(HOST_BIN)
                                           for p in (HOST_SRC, HEADER, LIB)):
        cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
               HOST_SRC, "-L", HERE, "-leden_gpu", "-Wl,-rpath,$ORIGIN/..", "-o", HOST_BIN + ".tmp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)
        os.replace(HOST_BIN + ".tmp", HOST_BIN)
    return HOST_BIN


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
