"""ctypes bindings of the rgcuda C ABI (include/rgcuda.h) and a thin Python mirror of the
reference's render-facing interface (Raytracer / RenderSystem).

The library is built in-tree (``raygun_gb300/librgcuda.so``).  There is no fallback: when the
library is missing or no GPU is present every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librgcuda.so")

RG_OK = 0
ERRORS = {-1: "RG_ERR_INVALID_ARG", -2: "RG_ERR_CUDA", -3: "RG_ERR_OUT_OF_MEMORY", -4: "RG_ERR_NOT_READY",
          -5: "RG_ERR_STACK_OVERFLOW", -6: "RG_ERR_BUDGET", -7: "RG_ERR_NO_DEVICE", -8: "RG_ERR_TOO_LARGE"}
RG_FLAG_DEBUG_IMAGES = 1
RG_FLAG_COUNT_VISITS = 2
RG_FLAG_MEGAKERNEL = 4
RG_FLAG_KERNEL_TIMING = 8
RG_FLAG_HOST_LOOP = 16
RG_FLAG_TLAS_LBVH = 32
RG_FLAG_BLAS_LBVH = 64
IMAGES = {"final": 0, "base": 1, "normal": 2, "rough": 3, "rough_transition": 4, "rough_colors_a": 5,
          "rough_colors_b": 6, "pre_fxaa": 7, "filter_out": 8}

EXPORTS = [
    "rg_create", "rg_destroy", "rg_last_error", "rg_upload_geometry", "rg_update_vertices", "rg_update_materials",
    "rg_build_blas", "rg_refit_blas", "rg_build_tlas", "rg_build_tlas_device", "rg_set_resolution", "rg_render",
    "rg_download", "rg_framebuffer_device", "rg_download_image", "rg_synchronize", "rg_get_timings", "rg_get_stats",
    "rg_get_stream", "rg_bvh_info", "rg_instance_inverse", "rg_trace_rays", "rg_post_only", "rg_lbvh_build_host",
    "rg_update_vertices_device", "rg_get_total_stats", "rg_reset_total_stats", "rg_set_flags", "rg_launch_count",
    "rg_lbvh_build_device_noalloc", "rg_scene_create", "rg_scene_select", "rg_scene_destroy", "rg_scene_bytes",
    "rg_render_batch", "rg_batch_framebuffer", "rg_batch_download", "rg_batch_download_async", "rg_set_batch_tune", "rg_get_batch_tune",
    "rg_set_batch_slots", "rg_autotune_batch", "rg_get_memory", "rg_filter_create", "rg_filter_destroy",
    "rg_filter_last_error", "rg_filter_get_params", "rg_filter_set_params", "rg_filter_get_grads", "rg_filter_forward",
    "rg_filter_train_step", "rg_filter_input", "rg_filter_target", "rg_set_filter", "rg_set_glossy",
    "rg_bvh_records", "rg_download_async", "rg_trace_rays_device", "rg_measure_l2",
]
FILTER_PARAMS = 78243
# layer shapes of the learned filter: (out, in) real channel counts
FILTER_LAYERS = ((32, 12), (64, 32), (64, 64), (32, 64), (3, 32))

# one 4-wide traversal record (rg_bvh_records): planes lo_x, hi_x, lo_y, hi_y, lo_z, hi_z of 4 slots
WIDE_RECORD = np.dtype([("planes", "<f4", (6, 4)), ("ref", "<u4", 4)])
assert WIDE_RECORD.itemsize == 112

# rg_job (include/rgcuda.h): one render of a batch
JOB = np.dtype([("scene", "<u4"), ("width", "<u4"), ("height", "<u4"), ("options", "<i4"), ("ubo", scenes.UBO)])
RG_JOB_FXAA, RG_JOB_FILTER = 1, 2
SORT_KEYS = {"none": 0, "octant": 1, "morton": 2}
AUTOTUNE_CONFIGS = 36


def autotune_grid():
    """Configurations of rg_autotune_batch in its order: (threads, stack depth, sort key name)."""
    return [(t, d, k) for t in (64, 128, 256) for d in (16, 24, 32, 48) for k in ("none", "octant", "morton")]


class DeviceOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("flags", ctypes.c_uint32), ("hbm_budget_bytes", ctypes.c_uint64)]


class Timings(ctypes.Structure):
    _fields_ = ([(k, ctypes.c_float) for k in ("asBuild", "rtTotal", "rtOnly", "postproc", "rough", "refit")]
                + [("frames", ctypes.c_uint32)]
                + [(k, ctypes.c_float) for k in ("asBuildSum", "rtTotalSum", "rtOnlySum", "postprocSum", "roughSum",
                                                 "refitSum", "traceKernel", "traceKernelSum")]
                + [("traceLaunches", ctypes.c_uint32)])


class Stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("primary", "shadow", "secondary", "masked", "nodes", "tris",
                                               "stack_overflows", "iterations", "deep_overflows")]


class BatchTune(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32), ("stack_depth", ctypes.c_int32), ("sort_key", ctypes.c_int32)]


class RgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load librgcuda.so and declare its signatures (no GPU needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run `python -m raygun_gb300.build` (no CPU fallback exists)")
    L = ctypes.CDLL(path)
    P, U32, I32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32
    sig = {
        "rg_create": ([ctypes.POINTER(P), ctypes.POINTER(DeviceOpts)], I32),
        "rg_destroy": ([P], I32),
        "rg_last_error": ([P], ctypes.c_char_p),
        "rg_upload_geometry": ([P, P, U32, P, U32, P, U32], I32),
        "rg_update_vertices": ([P, U32, P, U32], I32),
        "rg_update_materials": ([P, U32, P, U32], I32),
        "rg_build_blas": ([P, U32, U32, U32, ctypes.POINTER(U32)], I32),
        "rg_refit_blas": ([P, U32], I32),
        "rg_build_tlas": ([P, P, U32], I32),
        "rg_build_tlas_device": ([P, P, U32], I32),
        "rg_set_resolution": ([P, U32, U32], I32),
        "rg_render": ([P, P, I32], I32),
        "rg_download": ([P, P], I32),
        "rg_framebuffer_device": ([P, ctypes.POINTER(P)], I32),
        "rg_download_image": ([P, I32, P], I32),
        "rg_synchronize": ([P], I32),
        "rg_get_timings": ([P, ctypes.POINTER(Timings)], I32),
        "rg_get_stats": ([P, ctypes.POINTER(Stats)], I32),
        "rg_get_stream": ([P, ctypes.POINTER(P)], I32),
        "rg_bvh_info": ([P, U32, ctypes.POINTER(U32), P, P, P, P, P], I32),
        "rg_instance_inverse": ([P, P], I32),
        "rg_bvh_records": ([P, U32, P, U32, ctypes.POINTER(U32)], I32),
        "rg_download_async": ([P, P], I32),
        "rg_trace_rays": ([P, P, U32, P, P], I32),
        "rg_trace_rays_device": ([P, P, U32, P, P], I32),
        "rg_measure_l2": ([I32, ctypes.c_uint64, I32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)], I32),
        "rg_post_only": ([P, P, P, P, P, I32], I32),
        "rg_lbvh_build_host": ([P, P, U32, P, P, P, P, P], I32),
        "rg_update_vertices_device": ([P, U32, P, U32], I32),
        "rg_get_total_stats": ([P, ctypes.POINTER(Stats)], I32),
        "rg_reset_total_stats": ([P], I32),
        "rg_set_flags": ([P, U32], I32),
        "rg_launch_count": ([ctypes.POINTER(ctypes.c_uint64)], I32),
        "rg_lbvh_build_device_noalloc": ([P, U32, P, P, P, P, P, P], I32),
        "rg_scene_create": ([P, ctypes.POINTER(U32)], I32),
        "rg_scene_select": ([P, U32], I32),
        "rg_scene_destroy": ([P, U32], I32),
        "rg_scene_bytes": ([P, U32, ctypes.POINTER(ctypes.c_uint64)], I32),
        "rg_render_batch": ([P, P, U32], I32),
        "rg_batch_framebuffer": ([P, U32, ctypes.POINTER(P)], I32),
        "rg_batch_download": ([P, U32, P], I32),
        "rg_batch_download_async": ([P, P], I32),
        "rg_set_batch_tune": ([P, ctypes.POINTER(BatchTune)], I32),
        "rg_get_batch_tune": ([P, ctypes.POINTER(BatchTune)], I32),
        "rg_set_batch_slots": ([P, U32], I32),
        "rg_autotune_batch": ([P, P, U32, U32, ctypes.POINTER(BatchTune), P], I32),
        "rg_get_memory": ([P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)], I32),
        "rg_filter_create": ([P, ctypes.c_uint64, ctypes.POINTER(P)], I32),
        "rg_filter_destroy": ([P], I32),
        "rg_filter_last_error": ([P], ctypes.c_char_p),
        "rg_filter_get_params": ([P, P, U32], I32),
        "rg_filter_set_params": ([P, P, U32], I32),
        "rg_filter_get_grads": ([P, P, U32], I32),
        "rg_filter_forward": ([P, P, U32, U32, U32, P], I32),
        "rg_filter_train_step": ([P, P, P, U32, U32, U32, ctypes.c_float, ctypes.POINTER(ctypes.c_float)], I32),
        "rg_filter_input": ([P, P], I32),
        "rg_filter_target": ([P, P], I32),
        "rg_set_filter": ([P, P], I32),
        "rg_set_glossy": ([P, U32], I32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def launch_count() -> int:
    """Kernels the library launched in this process."""
    v = ctypes.c_uint64()
    rc = load().rg_launch_count(ctypes.byref(v))
    if rc != RG_OK:
        raise RgError(rc, "rg_launch_count")
    return v.value


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """One rgcuda context (one device, one stream).  Methods follow the reference's Raytracer /
    RenderSystem calls they replace (see include/rgcuda.h)."""

    def __init__(self, device=0, flags=0, hbm_budget_bytes=0):
        self.L = load()
        self.h = ctypes.c_void_p()
        opts = DeviceOpts(device, flags, hbm_budget_bytes)
        rc = self.L.rg_create(ctypes.byref(self.h), ctypes.byref(opts))
        if rc != RG_OK:
            raise RgError(rc, "rg_create failed (no CUDA device?)")
        self.width = self.height = 0

    def _ck(self, rc):
        if rc != RG_OK:
            raise RgError(rc, self.L.rg_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.rg_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- RenderSystem::setupModelBuffers / updateModelBuffers
    def upload_geometry(self, vertices, indices, materials):
        v = np.ascontiguousarray(vertices, dtype=scenes.VERTEX)
        i = np.ascontiguousarray(indices, dtype=np.uint32)
        m = np.ascontiguousarray(materials, dtype=scenes.MATERIAL)
        self._ck(self.L.rg_upload_geometry(self.h, _p(v), len(v), _p(i), len(i), _p(m), len(m)))

    def update_vertices(self, first, vertices):
        v = np.ascontiguousarray(vertices, dtype=scenes.VERTEX)
        self._ck(self.L.rg_update_vertices(self.h, first, _p(v), len(v)))

    def update_vertices_device(self, first, dev_ptr: int, n: int):
        self._ck(self.L.rg_update_vertices_device(self.h, first, ctypes.c_void_p(dev_ptr), n))

    def update_materials(self, first, materials):
        m = np.ascontiguousarray(materials, dtype=scenes.MATERIAL)
        self._ck(self.L.rg_update_materials(self.h, first, _p(m), len(m)))

    # -- Raytracer::setupBottomLevelAS / setupTopLevelAS
    def build_blas(self, vertex_offset, index_offset, tri_count) -> int:
        out = ctypes.c_uint32()
        self._ck(self.L.rg_build_blas(self.h, vertex_offset, index_offset, tri_count, ctypes.byref(out)))
        return out.value

    def refit_blas(self, blas):
        self._ck(self.L.rg_refit_blas(self.h, blas))

    def build_tlas(self, instances):
        inst = np.ascontiguousarray(instances, dtype=scenes.INSTANCE)
        self._ck(self.L.rg_build_tlas(self.h, _p(inst), len(inst)))

    def build_tlas_device(self, dev_ptr: int, n: int):
        self._ck(self.L.rg_build_tlas_device(self.h, ctypes.c_void_p(dev_ptr), n))

    def set_resolution(self, w, h):
        self._ck(self.L.rg_set_resolution(self.h, w, h))
        self.width, self.height = w, h

    # -- RenderSystem::render -> Raytracer::doRaytracing
    def render(self, ubo, fxaa=True):
        u = np.ascontiguousarray(ubo, dtype=scenes.UBO)
        self._ck(self.L.rg_render(self.h, _p(u), 1 if fxaa else 0))

    def download(self, out=None):
        if out is None:
            out = np.empty((self.height, self.width, 4), np.float32)
        self._ck(self.L.rg_download(self.h, _p(out)))
        return out

    def download_to(self, host_ptr: int):
        self._ck(self.L.rg_download(self.h, ctypes.c_void_p(host_ptr)))

    def batch_download_async(self, host_ptr: int):
        """Queue the read-back of every image of the last batch (job order, contiguous RGBA32F) into
        host_ptr (valid until synchronize())."""
        self._ck(self.L.rg_batch_download_async(self.h, ctypes.c_void_p(host_ptr)))

    def download_async(self, host_ptr: int):
        """Queue the read-back of the last frame into host_ptr (valid until synchronize())."""
        self._ck(self.L.rg_download_async(self.h, ctypes.c_void_p(host_ptr)))

    def framebuffer_ptr(self) -> int:
        p = ctypes.c_void_p()
        self._ck(self.L.rg_framebuffer_device(self.h, ctypes.byref(p)))
        return p.value

    def download_image(self, which):
        out = np.empty((self.height, self.width, 4), np.float32)
        self._ck(self.L.rg_download_image(self.h, IMAGES[which] if isinstance(which, str) else which, _p(out)))
        return out

    def synchronize(self):
        self._ck(self.L.rg_synchronize(self.h))

    def timings(self) -> dict:
        t = Timings()
        self._ck(self.L.rg_get_timings(self.h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in Timings._fields_}

    def stats(self) -> dict:
        s = Stats()
        self._ck(self.L.rg_get_stats(self.h, ctypes.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in Stats._fields_}

    def total_stats(self) -> dict:
        s = Stats()
        self._ck(self.L.rg_get_total_stats(self.h, ctypes.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in Stats._fields_}

    def reset_total_stats(self):
        self._ck(self.L.rg_reset_total_stats(self.h))

    def set_flags(self, flags):
        self._ck(self.L.rg_set_flags(self.h, flags))

    def stream(self) -> int:
        p = ctypes.c_void_p()
        self._ck(self.L.rg_get_stream(self.h, ctypes.byref(p)))
        return p.value or 0

    # -- scene slots and batched rendering
    def scene_create(self) -> int:
        out = ctypes.c_uint32()
        self._ck(self.L.rg_scene_create(self.h, ctypes.byref(out)))
        return out.value

    def scene_select(self, scene: int):
        self._ck(self.L.rg_scene_select(self.h, scene))

    def scene_destroy(self, scene: int):
        self._ck(self.L.rg_scene_destroy(self.h, scene))

    def scene_bytes(self, scene: int) -> int:
        out = ctypes.c_uint64()
        self._ck(self.L.rg_scene_bytes(self.h, scene, ctypes.byref(out)))
        return out.value

    def render_batch(self, jobs):
        j = np.ascontiguousarray(jobs, dtype=JOB)
        self._ck(self.L.rg_render_batch(self.h, _p(j), len(j)))
        self._batch = [(int(x["width"]), int(x["height"])) for x in j]

    def batch_download(self, job: int, out=None):
        w, h = self._batch[job] if 0 <= job < len(getattr(self, "_batch", [])) else (0, 0)
        if out is None:
            out = np.empty((h, w, 4), np.float32)
        self._ck(self.L.rg_batch_download(self.h, job, _p(out)))
        return out

    def batch_framebuffer_ptr(self, job: int) -> int:
        p = ctypes.c_void_p()
        self._ck(self.L.rg_batch_framebuffer(self.h, job, ctypes.byref(p)))
        return p.value

    def set_batch_tune(self, threads=128, stack_depth=48, sort_key=0):
        key = SORT_KEYS[sort_key] if isinstance(sort_key, str) else sort_key
        t = BatchTune(threads, stack_depth, key)
        self._ck(self.L.rg_set_batch_tune(self.h, ctypes.byref(t)))

    def batch_tune(self) -> dict:
        t = BatchTune()
        self._ck(self.L.rg_get_batch_tune(self.h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in BatchTune._fields_}

    def autotune_batch(self, jobs, reps=1):
        """Selects the fastest traversal launch shape / ray-sort key for this batch; returns the
        chosen tune and the table {(threads, depth, sort): ms or None (stack overflow)}."""
        j = np.ascontiguousarray(jobs, dtype=JOB)
        best = BatchTune()
        ms = np.zeros(AUTOTUNE_CONFIGS, np.float32)
        self._ck(self.L.rg_autotune_batch(self.h, _p(j), len(j), reps, ctypes.byref(best), _p(ms)))
        self._batch = [(int(x["width"]), int(x["height"])) for x in j]
        table = {}
        for i, (t, d, k) in enumerate(autotune_grid()):
            table[(t, d, k)] = None if ms[i] < 0 else float(ms[i])
        return {k: getattr(best, k) for k, _ in BatchTune._fields_}, table

    def memory(self):
        """(allocated bytes, budget bytes) of this context."""
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._ck(self.L.rg_get_memory(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_filter(self, flt):
        self._filter = flt
        self._ck(self.L.rg_set_filter(self.h, flt.h if flt is not None else None))

    def set_glossy(self, seed: int):
        self._ck(self.L.rg_set_glossy(self.h, seed))

    def filter_input(self, dev_ptr: int):
        """The last frame's 16-channel BF16 filter input into device memory [H][W][16]."""
        self._ck(self.L.rg_filter_input(self.h, ctypes.c_void_p(dev_ptr)))

    def filter_target(self, dev_ptr: int):
        """The last frame's rough RGB as FP32 [H][W][4] into device memory."""
        self._ck(self.L.rg_filter_target(self.h, ctypes.c_void_p(dev_ptr)))

    def set_batch_slots(self, slots: int):
        self._ck(self.L.rg_set_batch_slots(self.h, slots))

    # -- parity / inspection
    def bvh(self, blas: int):
        b = 0xFFFFFFFF if blas < 0 else blas
        n = ctypes.c_uint32()
        self._ck(self.L.rg_bvh_info(self.h, b, ctypes.byref(n), None, None, None, None, None))
        n = n.value
        out = dict(morton=np.zeros(n, np.uint32), order=np.zeros(n, np.uint32),
                   left=np.zeros(max(n - 1, 0), np.uint32), right=np.zeros(max(n - 1, 0), np.uint32),
                   nodeboxes=np.zeros((max(n - 1, 0), 6), np.float32))
        self._ck(self.L.rg_bvh_info(self.h, b, None, _p(out["morton"]), _p(out["order"]), _p(out["left"]),
                                    _p(out["right"]), _p(out["nodeboxes"])))
        return out

    def bvh_records(self, blas: int):
        """The traversal's 4-wide records (WIDE_RECORD) of a BLAS, or of the TLAS for blas < 0."""
        b = 0xFFFFFFFF if blas < 0 else blas
        n = ctypes.c_uint32()
        self._ck(self.L.rg_bvh_records(self.h, b, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, WIDE_RECORD)
        if n.value:
            self._ck(self.L.rg_bvh_records(self.h, b, _p(out), n.value, ctypes.byref(n)))
        return out

    def instance_inverse(self, n):
        out = np.zeros((n, 12), np.float32)
        self._ck(self.L.rg_instance_inverse(self.h, _p(out)))
        return out

    def trace_rays(self, rays):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        tuv = np.zeros((n, 3), np.float32)
        ids = np.zeros((n, 2), np.uint32)
        self._ck(self.L.rg_trace_rays(self.h, _p(rays), n, _p(tuv), _p(ids)))
        return tuv, ids

    def trace_rays_device(self, d_rays: int, n: int, d_tuv: int, d_ids: int):
        """rg_trace_rays_device: device pointers (n x 8 floats in, n x 3 floats and n x 2 uint32 out),
        asynchronous on the context's stream."""
        self._ck(self.L.rg_trace_rays_device(self.h, ctypes.c_void_p(d_rays), n, ctypes.c_void_p(d_tuv), ctypes.c_void_p(d_ids)))

    def post_only(self, ubo, base, normal, rough, fxaa=True):
        u = np.ascontiguousarray(ubo, dtype=scenes.UBO)
        b, n, r = (np.ascontiguousarray(x, np.float32) for x in (base, normal, rough))
        self._ck(self.L.rg_post_only(self.h, _p(u), _p(b), _p(n), _p(r), 1 if fxaa else 0))

    def lbvh_build_host(self, boxes):
        boxes = np.ascontiguousarray(boxes, np.float32)
        n = len(boxes)
        out = dict(morton=np.zeros(n, np.uint32), order=np.zeros(n, np.uint32),
                   left=np.zeros(max(n - 1, 0), np.uint32), right=np.zeros(max(n - 1, 0), np.uint32),
                   nodeboxes=np.zeros((max(n - 1, 0), 6), np.float32))
        self._ck(self.L.rg_lbvh_build_host(self.h, _p(boxes), n, _p(out["morton"]), _p(out["order"]),
                                           _p(out["left"]), _p(out["right"]), _p(out["nodeboxes"])))
        return out


class Raytracer:
    """Drop-in shape of raygun::render::Raytracer + the RenderSystem calls around it
    (render/raytracer.hpp:36-46, render/render_system.hpp:52-63) over one Context."""

    def __init__(self, scene: scenes.Scene, device=0, flags=0, hbm_budget_bytes=0):
        self.ctx = Context(device, flags, hbm_budget_bytes)
        self.scene = scene
        self.blas_ids = []
        self.ctx.set_resolution(scene.width, scene.height)

    def setup_model_buffers(self):                # RenderSystem::setupModelBuffers
        s = self.scene
        self.ctx.upload_geometry(s.vertices, s.indices, s.materials)

    def setup_bottom_level_as(self):              # Raytracer::setupBottomLevelAS
        self.blas_ids = [self.ctx.build_blas(int(m["vertexOffset"]), int(m["indexOffset"]), int(m["triCount"]))
                         for m in self.scene.meshes]

    def setup_top_level_as(self, instances=None):  # Raytracer::setupTopLevelAS
        inst = self.scene.instances if instances is None else instances
        inst = inst.copy()
        inst["blas"] = np.asarray(self.blas_ids, np.uint32)[inst["blas"]]
        self.ctx.build_tlas(inst)

    def do_raytracing(self, ubo=None, fxaa=True):  # Raytracer::doRaytracing
        self.ctx.render(self.scene.ubo if ubo is None else ubo, fxaa)

    def prepare(self):
        self.setup_model_buffers()
        self.setup_bottom_level_as()
        self.setup_top_level_as()
        return self

    def render(self, ubo=None, fxaa=True):         # RenderSystem::render (headless)
        self.do_raytracing(ubo, fxaa)
        return self.ctx.download()


def load_scene(ctx: Context, scene: scenes.Scene):
    """setupModelBuffers + setupBottomLevelAS + setupTopLevelAS of `scene` into ctx's selected slot."""
    ctx.upload_geometry(scene.vertices, scene.indices, scene.materials)
    blas = [ctx.build_blas(int(m["vertexOffset"]), int(m["indexOffset"]), int(m["triCount"])) for m in scene.meshes]
    inst = scene.instances.copy()
    inst["blas"] = np.asarray(blas, np.uint32)[inst["blas"]]
    ctx.build_tlas(inst)
    return blas


class BatchRenderer:
    """Several scenes resident in one context, one scene slot each, rendered together by
    rg_render_batch: each job is RenderSystem::render of one scene with its own camera, size,
    samples and recursion depth."""

    def __init__(self, scene_list, device=0, flags=0, hbm_budget_bytes=0):
        self.ctx = Context(device, flags, hbm_budget_bytes)
        self.scenes = list(scene_list)
        self.slots = []
        for k, sc in enumerate(self.scenes):
            sid = 0 if k == 0 else self.ctx.scene_create()
            self.ctx.scene_select(sid)
            load_scene(self.ctx, sc)
            self.slots.append(sid)
        self.ctx.scene_select(0)

    def jobs(self, fxaa=True) -> np.ndarray:
        j = np.zeros(len(self.scenes), JOB)
        for k, sc in enumerate(self.scenes):
            j[k]["scene"] = self.slots[k]
            j[k]["width"], j[k]["height"] = sc.width, sc.height
            j[k]["options"] = RG_JOB_FXAA if fxaa else 0
            j[k]["ubo"] = sc.ubo[0] if sc.ubo.shape else sc.ubo
        return j

    def render(self, jobs=None, fxaa=True):
        jobs = self.jobs(fxaa) if jobs is None else jobs
        self.ctx.render_batch(jobs)
        return [self.ctx.batch_download(k) for k in range(len(jobs))]


class Filter:
    """The learned roughness filter (rg_filter_*): parameters, forward, Adam training step."""

    def __init__(self, ctx: Context, seed: int = 0):
        self.L = ctx.L
        self.h = ctypes.c_void_p()
        rc = self.L.rg_filter_create(ctx.h, seed, ctypes.byref(self.h))
        if rc != RG_OK:
            raise RgError(rc, "rg_filter_create failed")

    def _ck(self, rc):
        if rc != RG_OK:
            raise RgError(rc, self.L.rg_filter_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.rg_filter_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(FILTER_PARAMS, np.float32)
        self._ck(self.L.rg_filter_get_params(self.h, _p(out), FILTER_PARAMS))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self._ck(self.L.rg_filter_set_params(self.h, _p(p), len(p)))

    def grads(self) -> np.ndarray:
        out = np.zeros(FILTER_PARAMS, np.float32)
        self._ck(self.L.rg_filter_get_grads(self.h, _p(out), FILTER_PARAMS))
        return out

    def forward(self, d_in: int, batch: int, height: int, width: int, d_out: int):
        self._ck(self.L.rg_filter_forward(self.h, ctypes.c_void_p(d_in), batch, height, width, ctypes.c_void_p(d_out)))

    def train_step(self, d_in: int, d_target: int, batch: int, height: int, width: int, lr: float) -> float:
        loss = ctypes.c_float()
        self._ck(self.L.rg_filter_train_step(self.h, ctypes.c_void_p(d_in), ctypes.c_void_p(d_target), batch, height, width,
                                             ctypes.c_float(lr), ctypes.byref(loss)))
        return loss.value


def measure_l2(device=0, working_set_bytes=64 << 20, reps=64):
    """rg_measure_l2: (read GB/s, copy GB/s) of an L2-resident working set on `device`."""
    L = load()
    r, c = ctypes.c_double(), ctypes.c_double()
    rc = L.rg_measure_l2(device, working_set_bytes, reps, ctypes.byref(r), ctypes.byref(c))
    if rc != RG_OK:
        raise RgError(rc, "rg_measure_l2 failed")
    return r.value, c.value


def filter_layers(params: np.ndarray):
    """Split a parameter vector into [(W[out][in][3][3], b[out])] per layer."""
    out, off = [], 0
    for co, ci in FILTER_LAYERS:
        w = params[off:off + co * ci * 9].reshape(co, ci, 3, 3)
        off += co * ci * 9
        b = params[off:off + co]
        off += co
        out.append((w, b))
    return out
