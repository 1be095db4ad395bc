"""Render-request serving loop over the rgcuda C ABI.

Requests (a scene of a catalog, an image size, samples, recursion depth, an arrival time) queue up;
each scheduling step admits the waiting requests in arrival order as long as their scenes and the
batch's working memory fit the HBM budget, makes their scenes resident (scene slots, least recently
used scenes evicted first), renders them together with one ``rg_render_batch`` and reads every image
back.  ``run_open_loop`` replays a timed arrival sequence in real time and reports latency
percentiles, frames/s and Mrays/s.

The reference renders one scene per frame and has no request queue; every image a request gets is
the image ``RenderSystem::render`` (render/render_system.cpp:88-162) gives for its scene, size and
UBO.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time

import numpy as np

from . import scenes

# device bytes per path slot of the batch loop (payload, meta, 10 frames, two queue entries, hit)
PATH_SLOT_BYTES = 64 + 8 + 144 * 10 + 2 * 36 + 20
# per sample (payload sums), per output pixel (batch framebuffer), per pixel of the largest job
# (G-buffers, post scratch)
SAMPLE_BYTES, PIXEL_BYTES, SCRATCH_PIXEL_BYTES = 48, 16, 40
# per pixel of the largest filtered job: the learned filter's input, activations and prediction
FILTER_PIXEL_BYTES = 512
# device bytes per triangle of a resident BLAS (BVH2 nodes, 4-wide records, build scratch kept for
# refits, leaf-ordered triangles) and per instance of a TLAS; geometry buffers are counted as uploaded
BLAS_TRI_BYTES, TLAS_INSTANCE_BYTES = 236, 496


@dataclasses.dataclass
class Request:
    id: int
    scene: str
    width: int
    height: int
    spp: int
    depth: int
    arrival: float  # seconds from the start of the run
    fxaa: bool = True
    filter: bool = False  # the learned roughness filter in place of the roughness passes

    @property
    def samples(self) -> int:
        return self.width * self.height * self.spp


@dataclasses.dataclass
class Result:
    id: int
    arrival: float
    start: float
    finish: float
    ok: bool
    error: str = ""
    image: np.ndarray | None = None
    batch: int = -1

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


def scene_bytes_estimate(sc: scenes.Scene) -> int:
    """Device memory a scene takes once resident (model buffers, BLASes, TLAS)."""
    geo = sc.vertices.nbytes + sc.indices.nbytes + sc.materials.nbytes
    blas = int(sc.meshes["triCount"].astype(np.int64).sum()) * BLAS_TRI_BYTES
    return int(geo + blas + len(sc.instances) * TLAS_INSTANCE_BYTES + 4096 * len(sc.meshes))


def working_bytes(reqs, path_slots: int) -> int:
    """Device memory of one batch beyond its scenes: path state, sample sums, images, post scratch."""
    if not reqs:
        return 0
    samples = sum(r.samples for r in reqs)
    pixels = sum(r.width * r.height for r in reqs)
    filtered = [r.width * r.height for r in reqs if r.filter]
    return (min(samples, path_slots) * PATH_SLOT_BYTES + samples * SAMPLE_BYTES + pixels * PIXEL_BYTES
            + max(r.width * r.height for r in reqs) * SCRATCH_PIXEL_BYTES + max(filtered, default=0) * FILTER_PIXEL_BYTES)


class Residency:
    """Scenes resident in the context's scene slots, least recently used first.  Slot 0 stays empty
    and selected between uses, so any scene slot can be destroyed."""

    def __init__(self, ctx, catalog: dict):
        self.ctx = ctx
        self.catalog = catalog
        self.slots: collections.OrderedDict[str, int] = collections.OrderedDict()
        self.bytes: dict[str, int] = {}
        self.uploads = 0
        self.evictions = 0

    def resident_bytes(self) -> int:
        return sum(self.bytes.values())

    def footprint(self, key: str) -> int:
        return self.bytes[key] if key in self.bytes else scene_bytes_estimate(self.catalog[key])

    def evict_lru(self, keep) -> bool:
        for key in self.slots:
            if key not in keep:
                self.ctx.scene_select(0)
                self.ctx.scene_destroy(self.slots.pop(key))
                self.bytes.pop(key)
                self.evictions += 1
                return True
        return False

    def ensure(self, key: str) -> int:
        if key in self.slots:
            self.slots.move_to_end(key)
            return self.slots[key]
        from .rgcuda import load_scene
        slot = self.ctx.scene_create()
        self.ctx.scene_select(slot)
        try:
            load_scene(self.ctx, self.catalog[key])
        except Exception:
            self.ctx.scene_select(0)
            self.ctx.scene_destroy(slot)
            raise
        finally:
            self.ctx.scene_select(0)
        self.slots[key] = slot
        self.bytes[key] = self.ctx.scene_bytes(slot)
        self.uploads += 1
        return slot


class RenderServer:
    def __init__(self, ctx, catalog: dict, budget_bytes: int, max_batch: int = 64, path_slots: int = 1 << 23,
                 read_back: bool = True, keep_images: bool = False, learned_filter=None):
        """learned_filter: an rgcuda.Filter that requests asking for it (Request.filter) use in place
        of the roughness passes; without one such requests are turned away."""
        self.ctx = ctx
        self.filter = learned_filter
        if learned_filter is not None:
            ctx.set_filter(learned_filter)
        self.catalog = catalog
        self.budget = budget_bytes
        self.max_batch = max_batch
        self.path_slots = path_slots
        self.read_back = read_back
        self.keep_images = keep_images
        self.res = Residency(ctx, catalog)
        self.queue: collections.deque[Request] = collections.deque()
        self.batches = 0
        self.rays = 0
        self.batch_sizes = []
        ctx.set_batch_slots(path_slots)
        self._buf = None

    def submit(self, req: Request):
        self.queue.append(req)

    def _working_held(self) -> int:
        allocated, _ = self.ctx.memory()
        return max(0, allocated - self.res.resident_bytes())

    def admit(self):
        """Requests of the next batch (arrival order) and the ones that can never fit."""
        batch, rejected, keys = [], [], []
        held = self._working_held()
        for req in list(self.queue):
            if len(batch) >= self.max_batch:
                break
            if req.filter and self.filter is None:
                rejected.append(req)
                continue
            trial_keys = keys if req.scene in keys else keys + [req.scene]
            trial = batch + [req]
            need = sum(self.res.footprint(k) for k in trial_keys) + max(held, working_bytes(trial, self.path_slots))
            if need <= self.budget:
                batch, keys = trial, trial_keys
                continue
            alone = self.res.footprint(req.scene) + max(held, working_bytes([req], self.path_slots))
            if not batch and alone > self.budget:
                rejected.append(req)  # does not fit even on an otherwise empty device
                continue
            break
        return batch, rejected, keys

    def step(self, clock) -> list:
        """Render the next batch; returns the results of every request it finished or rejected."""
        batch, rejected, keys = self.admit()
        now = clock()
        out = [Result(r.id, r.arrival, now, now, False, "learned filter asked for, none loaded" if r.filter and self.filter is None
                      else "does not fit the HBM budget") for r in rejected]
        for r in rejected:
            self.queue.remove(r)
        if not batch:
            return out
        for r in batch:
            self.queue.remove(r)
        start = clock()
        from .rgcuda import JOB, RG_JOB_FILTER, RG_JOB_FXAA, RgError
        room = self.budget - max(self._working_held(), working_bytes(batch, self.path_slots))
        while self.res.resident_bytes() + sum(self.res.footprint(k) for k in keys if k not in self.res.slots) > room:
            if not self.res.evict_lru(set(keys)):
                break
        for attempt in range(2):
            try:
                slots = {k: self.res.ensure(k) for k in keys}
                jobs = np.zeros(len(batch), JOB)
                for j, r in enumerate(batch):
                    sc = self.catalog[r.scene]
                    jobs[j]["scene"] = slots[r.scene]
                    jobs[j]["width"], jobs[j]["height"] = r.width, r.height
                    jobs[j]["options"] = (RG_JOB_FXAA if r.fxaa else 0) | (RG_JOB_FILTER if r.filter else 0)
                    jobs[j]["ubo"] = scenes.reframe(sc, r.width, r.height, r.spp, r.depth)[0]
                self.ctx.render_batch(jobs)
                break
            except RgError as e:
                # over the context's hard budget after all (estimates are estimates): free every
                # scene this batch does not use and try once more; then fail the batch
                if e.code != -6 or attempt == 1:
                    t = clock()
                    return out + [Result(r.id, r.arrival, start, t, False, str(e)) for r in batch]
                while self.res.evict_lru(set(keys)):
                    pass
        images = []
        if self.read_back:
            total = sum(r.width * r.height * 4 for r in batch)
            if self._buf is None or self._buf.size < total:
                self._buf = np.empty(total, np.float32)
            off = 0
            for j, r in enumerate(batch):
                n = r.width * r.height * 4
                view = self._buf[off:off + n].reshape(r.height, r.width, 4)
                self.ctx.batch_download(j, view)
                images.append(view.copy() if self.keep_images else None)
                off += n
        else:
            self.ctx.synchronize()
            images = [None] * len(batch)
        st = self.ctx.stats()
        self.rays += st["primary"] + st["shadow"] + st["secondary"]
        finish = clock()
        self.batches += 1
        self.batch_sizes.append(len(batch))
        out += [Result(r.id, r.arrival, start, finish, True, image=img, batch=self.batches - 1) for r, img in zip(batch, images)]
        return out


def poisson_requests(n: int, rate: float, seed: int, pool_small, pool_large, large_fraction: float = 0.05,
                     filter_fraction: float = 0.0):
    """n requests with exponential inter-arrival gaps (mean 1/rate).  A request takes a scene of the
    batched-rendering distribution (its own size, samples and depth) or, with probability
    ``large_fraction``, a large terrain scene at a size drawn from 320x180 ... 3840x2160 with 1-8
    samples and depth 1-6.  Draw order per request: gap, large?, scene index, then for a large scene
    size index, samples, depth.  With probability ``filter_fraction`` a request asks for the learned
    filter (drawn from a stream of its own, seed ^ 0x5EED, so the other draws do not move)."""
    rng = scenes.Rng(seed)
    frng = scenes.Rng(seed ^ 0x5EED)
    t, out = 0.0, []
    for i in range(n):
        t += -math.log(1.0 - rng.uniform(1)[0]) / rate
        large = bool(pool_large) and rng.uniform(1)[0] < large_fraction
        pool = pool_large if large else pool_small
        key, sc = pool[min(int(rng.uniform(1, 0, len(pool))[0]), len(pool) - 1)]
        if large:
            w, h = scenes.SERVE_RESOLUTIONS[min(int(rng.uniform(1, 0, len(scenes.SERVE_RESOLUTIONS))[0]), len(scenes.SERVE_RESOLUTIONS) - 1)]
            spp = 1 + min(int(rng.uniform(1, 0, 8)[0]), 7)
            depth = 1 + min(int(rng.uniform(1, 0, 6)[0]), 5)
        else:
            w, h = sc.width, sc.height
            spp, depth = int(sc.ubo["numSamples"][0]), int(sc.ubo["maxRecursions"][0])
        filt = bool(frng.uniform(1)[0] < filter_fraction)
        out.append(Request(i, key, w, h, spp, depth, t, filter=filt))
    return out


def run_open_loop(server: RenderServer, requests, time_scale: float = 1.0):
    """Replay the arrivals in real time (arrival times divided by ``time_scale``); each step renders
    whatever has arrived and fits.  Returns the results in completion order and the wall time."""
    pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
    results = []
    t0 = time.perf_counter()
    clock = lambda: (time.perf_counter() - t0) * time_scale
    while pending or server.queue:
        now = clock()
        while pending and pending[0].arrival <= now:
            server.submit(pending.popleft())
        if server.queue:
            results += server.step(clock)
        elif pending:
            time.sleep(max(0.0, (pending[0].arrival - clock()) / time_scale))
    return results, clock()


def summarize(results, wall: float, rays: int) -> dict:
    ok = [r for r in results if r.ok]
    lat = np.array([r.latency for r in ok]) * 1e3
    first = min((r.arrival for r in results), default=0.0)
    span = max(wall - first, 1e-9)
    return {"requests": len(results), "completed": len(ok), "rejected": len(results) - len(ok),
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "mean_ms": float(lat.mean()) if len(lat) else None,
            "frames_per_s": len(ok) / span, "mrays_per_s": rays / span / 1e6, "seconds": span}
