"""The reference-compiled checker: Raygun's own shaders built as C++ (test infrastructure only).

Recipe (``build()``): read every file of ``resources/shaders`` from the reference tree, apply the
mechanical rewrites a C++ compiler needs, write them to ``oracle/_ref/src`` (git-ignored: reference
sources never enter this repository), then compile ``ref_shaders.cpp`` -- the GLSL shim plus the
glue that binds scene data to the shaders' globals -- into ``oracle/_ref/libref.so``.

The rewrites change no statement of the shaders' logic:
  * ``#version`` / ``#extension`` lines become blank (line numbers are kept);
  * ``inout T name`` parameters become ``T& name`` (GLSL copy-in/copy-out of an lvalue);
  * unsized ``T name[];`` buffer members become ``T* name;``;
  * the compute ``layout(local_size_...) in;`` declaration becomes blank.

The reference tree exists only where this package is built from it; elsewhere ``reference_present()``
is False and the committed golden fixtures (tests/golden) carry its outputs.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libref.so")
REFERENCE = os.environ.get("RAYGUN_REFERENCE", "/root/reference")
SHADERS = os.path.join(REFERENCE, "resources", "shaders")

_lib = None


def reference_present() -> bool:
    return os.path.isdir(SHADERS)


def staged_present() -> bool:
    """The rewritten shader copies of an earlier build (oracle/_ref/src) are there: the checker can be
    rebuilt from them where the reference tree itself is absent (the git-ignored folder travels with
    the working tree to the GPU host)."""
    src = os.path.join(OUT, "src")
    return os.path.isfile(os.path.join(src, "closesthit.rchit")) and os.path.isfile(os.path.join(src, "raygen.rgen"))


def _rewrite(text: str) -> str:
    out = []
    for line in text.split("\n"):
        s = line.strip()
        if s.startswith("#version") or s.startswith("#extension") or re.match(r"layout\s*\(\s*local_size", s):
            out.append("")
            continue
        line = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", line)
        line = re.sub(r"^(\s*)(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1\2* \3;", line)
        out.append(line)
    return "\n".join(out)


def build(force: bool = False) -> str:
    src = os.path.join(OUT, "src")
    if not reference_present():
        if not staged_present():
            raise RuntimeError(f"reference shaders not found under {SHADERS}")
        deps = [os.path.join(HERE, "ref_shaders.cpp"), os.path.join(HERE, "glsl_shim.hpp"), os.path.join(ORACLE, "rg_oracle.cpp")]
        deps += [os.path.join(src, n) for n in os.listdir(src)]
        return _compile(src, deps, force)
    os.makedirs(src, exist_ok=True)
    deps = [os.path.join(HERE, "ref_shaders.cpp"), os.path.join(HERE, "glsl_shim.hpp"), os.path.join(ORACLE, "rg_oracle.cpp")]
    for name in sorted(os.listdir(SHADERS)):
        p = os.path.join(SHADERS, name)
        if os.path.isfile(p):
            with open(p, encoding="utf-8") as f:
                text = _rewrite(f.read())
            dst = os.path.join(src, name)
            if not os.path.exists(dst) or open(dst, encoding="utf-8").read() != text:
                with open(dst, "w", encoding="utf-8") as f:
                    f.write(text)
            deps.append(dst)
    return _compile(src, deps, force)


def _compile(src, deps, force):
    if force or not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fsingle-precision-constant",
               "-fno-strict-aliasing", "-w", "-fPIC", "-shared", "-I", src, "-I", HERE,
               "-o", LIB, os.path.join(HERE, "ref_shaders.cpp"), "-lpthread"]
        subprocess.run(cmd, check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P, U32, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        L.ref_render.argtypes = [P, U32, P, U32, P, U32, P, U32, P, U32, P, U32, U32, P, P, P, P, I]
        L.ref_render.restype = I
        L.ref_post.argtypes = [P, U32, U32, P, P, P, P, P, I, I]
        L.ref_post.restype = I
        L.ref_scene_render.argtypes = [P, P, U32, U32, P, P, P, P, I, U32, U32]
        L.ref_scene_render.restype = I
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def render(scene, ubo=None, nthreads=None):
    """The reference raygen / closest-hit / miss programs over every pixel -> (base, normal, rough, rays)."""
    s = scene
    v, i, m, me, inst = (np.ascontiguousarray(x) for x in (s.vertices, s.indices, s.materials, s.meshes, s.instances))
    u = np.ascontiguousarray(s.ubo if ubo is None else ubo)
    imgs = [np.zeros((s.height, s.width, 4), np.float32) for _ in range(3)]
    rays = np.zeros(1, np.uint64)
    lib().ref_render(_p(v), len(v), _p(i), len(i), _p(m), len(m), _p(me), len(me), _p(inst), len(inst), _p(u),
                     s.width, s.height, _p(imgs[0]), _p(imgs[1]), _p(imgs[2]), _p(rays), nthreads or os.cpu_count())
    return imgs[0], imgs[1], imgs[2], int(rays[0])


def render_scene(oscene, ubo, width, height, nthreads=None, rows=(0, 1)):
    """The reference raygen over an oracle.OracleScene that persists across frames (refit and
    instance updates through the OracleScene) -> (base, normal, rough, rays); rows = (first, step)
    renders rows first, first + step, ... only."""
    u = np.ascontiguousarray(ubo)
    imgs = [np.zeros((height, width, 4), np.float32) for _ in range(3)]
    rays = np.zeros(1, np.uint64)
    lib().ref_scene_render(oscene.h, _p(u), width, height, _p(imgs[0]), _p(imgs[1]), _p(imgs[2]), _p(rays),
                           nthreads or os.cpu_count(), rows[0], rows[1])
    return imgs[0], imgs[1], imgs[2], int(rays[0])


def post(ubo, base, normal, rough, fxaa=True, debug=False, nthreads=1):
    """The reference compute passes -> final image [, debug images as in oracle.post]."""
    H, W = base.shape[:2]
    b, n, r = (np.ascontiguousarray(x, np.float32) for x in (base, normal, rough))
    fin = np.zeros((H, W, 4), np.float32)
    dbg = np.zeros((4, H, W, 4), np.float32) if debug else None
    u = np.ascontiguousarray(ubo)
    lib().ref_post(_p(u), W, H, _p(b), _p(n), _p(r), _p(fin), _p(dbg) if debug else None, 1 if fxaa else 0, nthreads)
    return (fin, dbg) if debug else fin
