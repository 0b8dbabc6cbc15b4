"""Build libmsfec_cuda.so (sm_103a) in-tree with nvcc.

Every translation unit under csrc/ is compiled in parallel into _build/ and
linked into lib/libmsfec_cuda.so. Objects are rebuilt only when a source or
header is newer. No torch types cross the ABI, so no torch extension is used.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libmsfec_cuda.so")
HOSTLIB = os.path.join(LIBDIR, "libmsfec_host.so")
EXAMPLE = os.path.join(LIBDIR, "example_q1")
EXAMPLE_NR = os.path.join(LIBDIR, "example_nedrt")
EXAMPLE_PAIR = os.path.join(LIBDIR, "example_pairings")
EXAMPLE_STD = os.path.join(LIBDIR, "example_std")
HOST = os.path.join(HERE, "host")
CXX = os.environ.get("CXX", "g++")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    if not _stale(obj, src, _headers()):
        return obj, None
    cmd = [NVCC] + ARCH + FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, r.stderr + r.stdout
    return obj, None


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(_compile, srcs))
    errors = [(o, e) for o, e in results if e]
    if errors:
        msg = "\n".join(f"== {o}\n{e}" for o, e in errors)
        raise RuntimeError("nvcc failed:\n" + msg)
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr + r.stdout)
    build_host(objs)
    if verbose:
        print(LIB)
    return LIB


def build_host(objs=()):
    """QBasis/NedRTBasis/QNedBasis/RTDQBasis/QStd/NedRTStd shim + coarse solvers (g++, links the CUDA
    library) and the example drivers."""
    srcs = [os.path.join(HOST, f) for f in ("msfec_basis.cpp", "coarse_q1.cpp", "coarse_nedrt.cpp", "coarse_pairings.cpp")]
    deps = srcs + [os.path.join(HOST, "msfec_basis.hpp"), LIB] + glob.glob(os.path.join(INCLUDE, "*.h"))
    if not os.path.exists(HOSTLIB) or any(os.path.getmtime(d) > os.path.getmtime(HOSTLIB) for d in deps):
        cmd = [CXX, "-O2", "-std=c++17", "-fPIC", "-shared", "-I", INCLUDE, "-o", HOSTLIB] + srcs + \
              ["-L", LIBDIR, "-lmsfec_cuda", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host shim build failed:\n" + r.stderr)
    for src_name, out in (("example_q1.cpp", EXAMPLE), ("example_nedrt.cpp", EXAMPLE_NR),
                          ("example_pairings.cpp", EXAMPLE_PAIR), ("example_std.cpp", EXAMPLE_STD)):
        ex = os.path.join(HOST, src_name)
        if not os.path.exists(out) or os.path.getmtime(ex) > os.path.getmtime(out) or \
                os.path.getmtime(HOSTLIB) > os.path.getmtime(out):
            cmd = [CXX, "-O2", "-std=c++17", "-I", INCLUDE, "-o", out, ex, "-L", LIBDIR, "-lmsfec_host",
                   "-lmsfec_cuda", "-Wl,-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("example build failed:\n" + r.stderr)


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
