"""CPU oracle for the ray-tracing path (test infrastructure only).

Only the tests, the smoke check and the benchmark's CPU-baseline leg use this package, and only as
the checker.  ``build()`` compiles ``rg_oracle.cpp`` into ``liborc.so`` next to this file; ``lib()``
loads it through ctypes.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
SRC = os.path.join(HERE, "rg_oracle.cpp")

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-o", LIB, SRC, "-lpthread"]
        subprocess.run(cmd, check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P, U32, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        L.orc_lbvh.argtypes = [P, U32, P, P, P, P, P]
        L.orc_lbvh.restype = U32
        L.orc_sah.argtypes = [P, U32, U32, P, P, P, P]
        L.orc_sah.restype = U32
        L.orc_scene_create.argtypes = [P, U32, P, U32, P, U32, P, U32, P, U32]
        L.orc_scene_create.restype = P
        L.orc_scene_destroy.argtypes = [P]
        L.orc_scene_refit.argtypes = [P, U32, P, U32, U32]
        L.orc_scene_refit.restype = I
        L.orc_scene_set_instances.argtypes = [P, P, U32]
        L.orc_scene_set_instances.restype = I
        L.orc_bvh_info.argtypes = [P, U32, P, P, P, P, P]
        L.orc_bvh_info.restype = I
        L.orc_instance_inverse.argtypes = [P, P]
        L.orc_instance_inverse.restype = I
        L.orc_trace.argtypes = [P, P, U32, P, P, I, I]
        L.orc_trace.restype = I
        L.orc_render.argtypes = [P, P, U32, U32, U32, U32, U32, P, P, P, P, I, I]
        L.orc_render.restype = I
        L.orc_post.argtypes = [P, U32, U32, P, P, P, P, P, I, I]
        L.orc_post.restype = I
        L.orc_round_half.argtypes = [P, P, ctypes.c_uint64]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def lbvh(boxes: np.ndarray):
    """boxes: (n, 6) float32 (lo xyz, hi xyz) -> dict(morton, order, left, right, nodeboxes)."""
    boxes = np.ascontiguousarray(boxes, np.float32)
    n = len(boxes)
    out = dict(morton=np.zeros(n, np.uint32), order=np.zeros(n, np.uint32),
               left=np.zeros(max(n - 1, 0), np.uint32), right=np.zeros(max(n - 1, 0), np.uint32),
               nodeboxes=np.zeros((max(n - 1, 0), 6), np.float32))
    lib().orc_lbvh(_p(boxes), n, _p(out["morton"]), _p(out["order"]), _p(out["left"]), _p(out["right"]),
                   _p(out["nodeboxes"]))
    return out


# level from which the binned-SAH builder halves ranges instead of binning (the CUDA library's
# kSahMedianLevel): it bounds the depth of every SAH tree by this + ceil(log2 n)
SAH_MEDIAN_LEVEL = 32


def sah(boxes: np.ndarray, median_level: int = SAH_MEDIAN_LEVEL):
    """Binned-SAH BVH2 over boxes (n, 6) -> dict(order, left, right, nodeboxes, levels); ranges are
    halved without binning from level median_level on."""
    boxes = np.ascontiguousarray(boxes, np.float32)
    n = len(boxes)
    out = dict(order=np.zeros(n, np.uint32), left=np.zeros(max(n - 1, 0), np.uint32),
               right=np.zeros(max(n - 1, 0), np.uint32), nodeboxes=np.zeros((max(n - 1, 0), 6), np.float32))
    levels = lib().orc_sah(_p(boxes), n, median_level, _p(out["order"]), _p(out["left"]), _p(out["right"]),
                           _p(out["nodeboxes"]))
    out["levels"] = int(levels)
    return out


def same_tree(a, b):
    """Two BVH2s in the LBVH layout are the same tree when their leaf order agrees and a walk from both
    roots meets the same structure and node boxes; internal node numbering may differ (the GPU
    numbers a level's nodes in the order its warps emit them)."""
    if not np.array_equal(a["order"], b["order"]):
        return False
    n = len(a["order"])
    if n <= 1:
        return True
    LEAF = 0x80000000
    st = [(0, 0)]
    while st:
        i, j = st.pop()
        if not np.array_equal(a["nodeboxes"][i], b["nodeboxes"][j]):
            return False
        for ca, cb in ((int(a["left"][i]), int(b["left"][j])), (int(a["right"][i]), int(b["right"][j]))):
            if (ca & LEAF) != (cb & LEAF):
                return False
            if ca & LEAF:
                if ca != cb:
                    return False
            else:
                st.append((ca, cb))
    return True


class OracleScene:
    """The oracle's view of a scene (BLAS per mesh, TLAS over the instances)."""

    def __init__(self, scene):
        self.scene = scene
        s = scene
        self._keep = [np.ascontiguousarray(s.vertices), np.ascontiguousarray(s.indices, np.uint32),
                      np.ascontiguousarray(s.materials), np.ascontiguousarray(s.meshes),
                      np.ascontiguousarray(s.instances)]
        v, i, m, me, inst = self._keep
        self.h = lib().orc_scene_create(_p(v), len(v), _p(i), len(i), _p(m), len(m), _p(me), len(me), _p(inst), len(inst))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_destroy(self.h)
            self.h = None

    def set_instances(self, instances):
        inst = np.ascontiguousarray(instances)
        lib().orc_scene_set_instances(self.h, _p(inst), len(inst))

    def refit(self, blas: int, vertices: np.ndarray, first: int):
        v = np.ascontiguousarray(vertices)
        assert lib().orc_scene_refit(self.h, blas, _p(v), first, len(v)) == 0

    def bvh(self, blas: int):
        """blas index, or -1 for the TLAS."""
        b = 0xFFFFFFFF if blas < 0 else blas
        n = lib().orc_bvh_info(self.h, b, None, None, None, None, None)
        out = dict(morton=np.zeros(n, np.uint32), order=np.zeros(n, np.uint32),
                   left=np.zeros(max(n - 1, 0), np.uint32), right=np.zeros(max(n - 1, 0), np.uint32),
                   nodeboxes=np.zeros((max(n - 1, 0), 6), np.float32))
        lib().orc_bvh_info(self.h, b, _p(out["morton"]), _p(out["order"]), _p(out["left"]), _p(out["right"]),
                           _p(out["nodeboxes"]))
        return out

    def instance_inverse(self):
        out = np.zeros((len(self.scene.instances), 12), np.float32)
        lib().orc_instance_inverse(self.h, _p(out))
        return out

    def trace(self, rays: np.ndarray, brute=False, nthreads=None):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        hf = np.zeros((n, 3), np.float32)
        hi = np.zeros((n, 2), np.uint32)
        lib().orc_trace(self.h, _p(rays), n, _p(hf), _p(hi), 1 if brute else 0, nthreads or os.cpu_count())
        return hf, hi

    def render(self, ubo=None, rows=None, nthreads=None, fp64=False, row_step=1):
        """-> (base, normal, rough) float32 (H, W, 4) images and stats dict; rows=(r0, r1) limits
        the raygen to rows r0, r0+row_step, ... < r1 (others stay zero)."""
        s = self.scene
        ubo = np.ascontiguousarray(s.ubo if ubo is None else ubo)
        W, H = s.width, s.height
        r0, r1 = rows if rows else (0, H)
        imgs = [np.zeros((H, W, 4), np.float32) for _ in range(3)]
        st = np.zeros(6, np.uint64)
        lib().orc_render(self.h, _p(ubo), W, H, r0, r1, row_step, _p(imgs[0]), _p(imgs[1]), _p(imgs[2]), _p(st),
                         nthreads or os.cpu_count(), 1 if fp64 else 0)
        keys = ("primary", "shadow", "secondary", "masked", "nodes", "tris")
        return imgs[0], imgs[1], imgs[2], {k: int(v) for k, v in zip(keys, st)}


def post(ubo, base, normal, rough, fxaa=True, debug=False, nthreads=1):
    """Post passes on G-buffers (H, W, 4).  Returns final (H, W, 4) [and the debug images:
    transitions, roughColorsA, roughColorsB, pre-FXAA final]."""
    H, W = base.shape[:2]
    b, n, r = (np.ascontiguousarray(x, np.float32).copy() for x in (base, normal, rough))
    fin = np.zeros((H, W, 4), np.float32)
    dbg = np.zeros((4, H, W, 4), np.float32) if debug else None
    u = np.ascontiguousarray(ubo)
    lib().orc_post(_p(u), W, H, _p(b), _p(n), _p(r), _p(fin), _p(dbg) if debug else None, 1 if fxaa else 0, nthreads)
    return (fin, dbg) if debug else fin


def round_half(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    lib().orc_round_half(_p(x), _p(out), x.size)
    return out
