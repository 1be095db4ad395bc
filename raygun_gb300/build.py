"""Build the in-tree CUDA library ``librgcuda.so`` (sm_103a) from ``csrc/``.

Each translation unit is compiled in parallel with ``nvcc -c``, then linked with ``nvcc -shared``.
``-fmad=false`` keeps every floating-point operation separately rounded (fused multiply-adds are
written out where wanted), which the bit-exact ray-geometry contract relies on.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librgcuda.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["api.cu", "lbvh.cu", "trace.cu", "post.cu", "noalloc.cu", "filter.cu", "filter_api.cu", "measure.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _inputs():
    files = [os.path.join(CSRC, s) for s in SOURCES]
    files += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    files.append(os.path.join(INCLUDE, "rgcuda.h"))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _inputs())


FACADE_SRCS = [os.path.join(HERE, "host", "raygun.cpp"), os.path.join(HERE, "host", "collada.cpp")]
FACADE_LIB = os.path.join(HERE, "librgfacade.so")
FACADE_HDRS = [os.path.join(INCLUDE, "rg", "raygun.hpp"), os.path.join(INCLUDE, "rg", "collada.hpp")]


def build_facade(force: bool = False) -> str:
    """The C++ facade (include/rg/raygun.hpp) as librgfacade.so, linked to librgcuda.so."""
    deps = [*FACADE_SRCS, *FACADE_HDRS, os.path.join(INCLUDE, "rgcuda.h"), LIB]
    if not force and os.path.exists(FACADE_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(FACADE_LIB) for d in deps):
        return FACADE_LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I", INCLUDE, "-o", FACADE_LIB + ".tmp", *FACADE_SRCS,
           "-L", HERE, "-lrgcuda", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"facade build failed:\n{r.stderr}")
    os.replace(FACADE_LIB + ".tmp", FACADE_LIB)
    return FACADE_LIB


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    lib = _build_cuda(force, verbose, extra_flags)
    build_facade(force)
    return lib


def _build_cuda(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *ARCH, *FLAGS, *extra_flags, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
