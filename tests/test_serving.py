"""The render-request server (raygun_gb300/serving.py).

CPU: LRU residency and HBM-budget admission against a fake context that records what the server
asks of the C ABI; the Poisson arrival generator; the latency summary.
GPU: a small open-loop run whose budget forces evictions; every image it returns equals the single
render of the same scene, size and UBO.  Served images against the oracle's render of the same
request; requests that ask for the learned filter against rg_render with that filter, in a batch
that mixes them with plain requests.
"""
import math

import numpy as np
import pytest

from raygun_gb300 import scenes as S
from raygun_gb300 import serving as V


class FakeContext:
    """Scene slots and memory accounting of an rgcuda context, no GPU."""

    def __init__(self, working=0):
        self.slots = {0: 0}
        self.selected = 0
        self.working = working
        self.log = []
        self.batch_slots = None

    # scene slots
    def scene_create(self):
        k = next(i for i in range(1, 1000) if i not in self.slots)
        self.slots[k] = 0
        return k

    def scene_select(self, k):
        assert k in self.slots
        self.selected = k

    def scene_destroy(self, k):
        assert k != self.selected and k != 0
        self.log.append(("destroy", k))
        del self.slots[k]

    def scene_bytes(self, k):
        return self.slots[k]

    # what load_scene calls
    def upload_geometry(self, v, i, m):
        self.slots[self.selected] += v.nbytes + i.nbytes + m.nbytes

    def build_blas(self, vo, io, n):
        self.slots[self.selected] += n * V.BLAS_TRI_BYTES
        return 0

    def build_tlas(self, inst):
        self.slots[self.selected] += len(inst) * V.TLAS_INSTANCE_BYTES
        self.log.append(("load", self.selected))

    def memory(self):
        return sum(self.slots.values()) + self.working, 0

    def set_batch_slots(self, n):
        self.batch_slots = n

    def render_batch(self, jobs):
        self.log.append(("batch", [int(j["scene"]) for j in jobs]))

    def batch_download(self, j, out):
        out[...] = 0

    def synchronize(self):
        pass

    def stats(self):
        return {"primary": 1, "shadow": 0, "secondary": 0}


def small_catalog():
    scs = S.batch_scenes(n=3, seed=5, tri_range=(1e3, 3e3), resolutions=((32, 18),), samples=(1, 1), depths=(1, 2), hf_n=17)
    return {f"s{k}": sc for k, sc in enumerate(scs)}


def test_lru_residency_and_eviction():
    cat = small_catalog()
    foot = {k: V.scene_bytes_estimate(sc) for k, sc in cat.items()}
    req = lambda i, k: V.Request(i, k, 32, 18, 1, 1, 0.0)
    work = V.working_bytes([req(0, "s0")], 1 << 10)
    budget = foot["s0"] + foot["s1"] + work + 1024  # two scenes fit, three do not
    ctx = FakeContext()
    srv = V.RenderServer(ctx, cat, budget, path_slots=1 << 10, read_back=True)
    clock = lambda: 0.0
    for i, k in enumerate(["s0", "s1", "s0", "s2", "s1"]):
        srv.submit(req(i, k))
        res = srv.step(clock)
        assert len(res) == 1 and res[0].ok
    # s2 evicted s1 (least recently used: s0 was touched after s1); s1 then evicted s0
    assert srv.res.evictions == 2
    assert list(srv.res.slots) == ["s2", "s1"]
    loads = [e for e in ctx.log if e[0] == "load"]
    assert len(loads) == 4  # s0, s1, s2, s1 again
    assert ctx.batch_slots == 1 << 10


def test_admission_splits_batches_and_rejects_oversized():
    cat = small_catalog()
    foot = max(V.scene_bytes_estimate(sc) for sc in cat.values())
    small = lambda i, k: V.Request(i, k, 32, 18, 1, 1, 0.0)
    budget = 3 * foot + V.working_bytes([small(0, "s0")] * 2, 1 << 10) + 16
    ctx = FakeContext()
    srv = V.RenderServer(ctx, cat, budget, path_slots=1 << 10)
    huge = V.Request(9, "s1", 4096, 4096, 8, 1, 0.0)  # its working set alone exceeds the budget
    for r in (small(0, "s0"), small(1, "s1"), huge, small(2, "s2"), small(3, "s0")):
        srv.submit(r)
    clock = lambda: 0.0
    first = srv.step(clock)
    assert [r.id for r in first if r.ok] == [0, 1]  # the third request would exceed the budget
    second = srv.step(clock)  # the oversized request is turned away; the rest render in this step
    assert [(r.id, r.ok) for r in second] == [(9, False), (2, True), (3, True)]
    assert "budget" in second[0].error
    assert not srv.queue


def test_poisson_requests():
    cat = small_catalog()
    pool = list(cat.items())
    large = [("big", S.terrain_scene(S.Rng(1), "big", 3, 64, 36, 1, 2, hf_n=17, objects=4))]
    reqs = V.poisson_requests(4000, 400.0, 4, pool, large, large_fraction=0.1)
    gaps = np.diff([0.0] + [r.arrival for r in reqs])
    assert abs(gaps.mean() - 1 / 400) < 0.1 / 400
    frac = np.mean([r.scene == "big" for r in reqs])
    assert 0.08 < frac < 0.12
    big = [r for r in reqs if r.scene == "big"]
    assert {(r.width, r.height) for r in big} == set(S.SERVE_RESOLUTIONS)
    assert {r.spp for r in big} == set(range(1, 9))
    again = V.poisson_requests(4000, 400.0, 4, pool, large, large_fraction=0.1)
    assert [(r.scene, r.arrival) for r in reqs] == [(r.scene, r.arrival) for r in again]


def test_summary():
    res = [V.Result(i, 0.01 * i, 0.01 * i, 0.01 * i + 0.001 * (i + 1), True) for i in range(100)]
    s = V.summarize(res, 1.0, 1000)
    assert math.isclose(s["p50_ms"], 50.5, rel_tol=1e-6) and s["completed"] == 100
    assert s["frames_per_s"] == pytest.approx(100.0)


@pytest.mark.gpu
def test_gpu_open_loop_with_evictions(rg):
    cat = small_catalog()
    cat["big"] = S.terrain_scene(S.Rng(3), "big", 4, 48, 27, 1, 3, hf_n=33, objects=12)
    foot = sorted(V.scene_bytes_estimate(sc) for sc in cat.values())
    ctx = rg.Context()
    reqs = [V.Request(0, "s0", 32, 18, 1, 2, 0.0), V.Request(1, "big", 64, 36, 2, 3, 0.001),
            V.Request(2, "s1", 32, 18, 1, 1, 0.002), V.Request(3, "s2", 40, 24, 2, 2, 0.003),
            V.Request(4, "s0", 48, 27, 1, 4, 0.004), V.Request(5, "big", 33, 17, 3, 2, 0.005)]
    srv = V.RenderServer(ctx, cat, 1 << 40, max_batch=len(reqs), path_slots=1 << 16, keep_images=True)
    V.run_open_loop(srv, [V.Request(100 + r.id, r.scene, r.width, r.height, r.spp, r.depth, 0.0) for r in reqs])
    # every working buffer now has its final size; leave room for the two largest scenes only
    while srv.res.evict_lru(set()):
        pass
    srv.budget = srv._working_held() + foot[-1] + foot[-2] + 1024
    srv.max_batch = 2
    results, wall = V.run_open_loop(srv, reqs, time_scale=1e-3)
    assert all(r.ok for r in results), [r.error for r in results]
    assert srv.res.evictions > 0
    byid = {r.id: r for r in results}
    for q in reqs:
        sc = cat[q.scene]
        rt = rg.Raytracer(S.Scene(sc.name, sc.vertices, sc.indices, sc.materials, sc.meshes, sc.instances, sc.ubo,
                                  q.width, q.height)).prepare()
        ref = rt.render(S.reframe(sc, q.width, q.height, q.spp, q.depth))
        rt.ctx.close()
        assert np.array_equal(byid[q.id].image, ref), q
    s = V.summarize(results, wall, srv.rays)
    assert s["completed"] == len(reqs) and s["mrays_per_s"] > 0


def test_filter_requests_need_a_filter():
    cat = small_catalog()
    srv = V.RenderServer(FakeContext(), cat, 1 << 40, path_slots=1 << 10)
    srv.submit(V.Request(0, "s0", 32, 18, 1, 1, 0.0, filter=True))
    res = srv.step(lambda: 0.0)
    assert [(r.id, r.ok) for r in res] == [(0, False)] and "filter" in res[0].error
    reqs = V.poisson_requests(2000, 400.0, 4, list(cat.items()), [], filter_fraction=0.25)
    assert 0.2 < np.mean([r.filter for r in reqs]) < 0.3
    plain = V.poisson_requests(2000, 400.0, 4, list(cat.items()), [])
    assert [(r.scene, r.arrival) for r in reqs] == [(r.scene, r.arrival) for r in plain]


@pytest.mark.gpu
def test_gpu_served_images_vs_oracle_and_learned_filter(rg, orc):
    from raygun_gb300 import filter_train
    from test_gpu_parity import assert_image_close
    cat = small_catalog()
    ctx = rg.Context()
    flt = rg.Filter(ctx, seed=0)
    filter_train.load_weights(flt)  # the committed trained weights
    srv = V.RenderServer(ctx, cat, 1 << 40, max_batch=8, path_slots=1 << 16, keep_images=True, learned_filter=flt)
    reqs = [V.Request(0, "s0", 48, 27, 2, 3, 0.0), V.Request(1, "s1", 40, 24, 1, 4, 0.0),
            V.Request(2, "s0", 48, 27, 2, 3, 0.0, filter=True), V.Request(3, "s2", 64, 36, 2, 2, 0.0, filter=True)]
    results, _ = V.run_open_loop(srv, reqs)
    assert all(r.ok for r in results), [r.error for r in results]
    assert len({r.batch for r in results}) == 1  # one batch mixes plain and filtered jobs
    byid = {r.id: r for r in results}
    for q in reqs:
        sc = cat[q.scene]
        framed = S.Scene(sc.name, sc.vertices, sc.indices, sc.materials, sc.meshes, sc.instances,
                         S.reframe(sc, q.width, q.height, q.spp, q.depth), q.width, q.height)
        if not q.filter:  # the oracle's frame of the request
            o = orc.OracleScene(framed)
            b, n, r, _ = o.render()
            assert_image_close(byid[q.id].image, orc.post(framed.ubo, b, n, r), f"served request {q.id}")
        else:  # rg_render with the same filter weights, in a context of its own
            rt = rg.Raytracer(framed).prepare()
            f2 = rg.Filter(rt.ctx, seed=0)
            filter_train.load_weights(f2)
            rt.ctx.set_filter(f2)
            ref = rt.render()
            plain = None
            rt.ctx.set_filter(None)
            plain = rt.render()
            f2.close()
            rt.ctx.close()
            assert np.array_equal(byid[q.id].image, ref), q
            assert not np.array_equal(ref, plain)  # the filter changed the frame
    flt.close()
    ctx.close()
