"""Batched rendering (rg_render_batch): several scenes resident in one context (one scene slot
each), rendered by one wavefront loop in which finished path slots start the next job's work.

* every job's image equals the single-scene render of the same scene, bit for bit (the same
  kernels run on the same inputs; only the order rays are taken in changes), and so the oracle;
* ray counts of the batch are the sum of the single renders' counts;
* a small path pool (forced regeneration) and every traversal launch shape / ray-sort key of the
  autotuner's grid give the same images;
* the golden fixtures of the reference shaders, rendered as one batch, match their images;
* misuse returns status codes.
"""
import numpy as np
import pytest

from raygun_gb300 import scenes as S

pytestmark = pytest.mark.gpu

RAY_KEYS = ("primary", "shadow", "secondary", "masked")


def mini_batch(n=6, seed=7):
    return S.batch_scenes(n=n, seed=seed, tri_range=(1e3, 6e4), resolutions=((40, 24), (64, 36), (96, 54), (33, 17)),
                          samples=(1, 3), depths=(1, 6), hf_n=33)


@pytest.fixture(scope="module")
def batch(rg):
    scenes = mini_batch()
    singles, stats = [], []
    for sc in scenes:
        rt = rg.Raytracer(sc).prepare()
        singles.append(rt.render())
        stats.append(rt.ctx.stats())
        rt.ctx.close()
    return scenes, singles, stats


def test_batch_equals_single_renders(rg, batch):
    scenes, singles, stats = batch
    br = rg.BatchRenderer(scenes)
    imgs = br.render()
    st = br.ctx.stats()
    for k, (img, ref) in enumerate(zip(imgs, singles)):
        assert img.shape == ref.shape
        assert np.array_equal(img, ref), f"job {k}"
    for key in RAY_KEYS:
        assert st[key] == sum(s[key] for s in stats), key
    assert st["stack_overflows"] == 0


def test_batch_download_async(rg, batch):
    """rg_batch_download_async: every image of the last batch, in job order and contiguous, read back
    on the copy stream while the next batch renders; two batches in flight, each equal to the single
    renders (the second batch's cameras are the first's moved, so the two differ)."""
    import torch
    scenes, singles, _ = batch
    br = rg.BatchRenderer(scenes)
    jobs = br.jobs()
    moved = jobs.copy()
    for k, sc in enumerate(scenes):
        moved[k]["ubo"] = S.make_ubo((3.0 + k, 9.0, -30.0), (0, 2, 0), 55.0, sc.width, sc.height, (-0.4, -1.0, 0.3),
                                     int(sc.ubo["numSamples"][0]), int(sc.ubo["maxRecursions"][0]))[0]
    sizes = [sc.height * sc.width * 4 for sc in scenes]
    bufs = [torch.empty(sum(sizes), dtype=torch.float32).pin_memory() for _ in range(2)]
    br.ctx.render_batch(jobs)
    br.ctx.batch_download_async(bufs[0].data_ptr())
    br.ctx.render_batch(moved)
    br.ctx.batch_download_async(bufs[1].data_ptr())
    second = [br.ctx.batch_download(k) for k in range(len(moved))]
    br.ctx.synchronize()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    for k, sc in enumerate(scenes):
        a = bufs[0].numpy()[offs[k]:offs[k + 1]].reshape(sc.height, sc.width, 4)
        b = bufs[1].numpy()[offs[k]:offs[k + 1]].reshape(sc.height, sc.width, 4)
        assert np.array_equal(a, singles[k]), f"job {k}"
        assert np.array_equal(b, second[k]), f"job {k}, second batch"
    assert any(not np.array_equal(x, y) for x, y in zip(second, singles))
    br.ctx.close()


def test_host_loop_equals_graph(rg, batch):
    scenes, singles, stats = batch
    br = rg.BatchRenderer(scenes, flags=rg.RG_FLAG_HOST_LOOP)
    br.ctx.set_batch_slots(4096)
    for k, (img, ref) in enumerate(zip(br.render(), singles)):
        assert np.array_equal(img, ref), f"job {k}"
    st = br.ctx.stats()
    for key in RAY_KEYS:
        assert st[key] == sum(s[key] for s in stats), key
    assert st["iterations"] > 0


def test_graph_replay_reads_new_cameras(rg, batch):
    """The captured graph is replayed for a batch of the same shape: new cameras and scene contents
    come through the job table without a new capture."""
    scenes, singles, _ = batch
    br = rg.BatchRenderer(scenes)
    n0 = rg.launch_count()
    assert all(np.array_equal(a, b) for a, b in zip(br.render(), singles))
    n1 = rg.launch_count()
    assert n1 - n0 > 3 * len(scenes)  # raygen, rounds, tail, per-job resolve / post / FXAA
    jobs = br.jobs()
    moved = []
    for k, sc in enumerate(scenes):
        u = S.make_ubo((3.0 + k, 9.0, -30.0), (0, 2, 0), 55.0, sc.width, sc.height, (-0.4, -1.0, 0.3),
                       int(sc.ubo["numSamples"][0]), int(sc.ubo["maxRecursions"][0]))
        jobs[k]["ubo"] = u[0]
        moved.append(u)
    br.ctx.render_batch(jobs)
    for k, sc in enumerate(scenes):
        rt = rg.Raytracer(sc).prepare()
        assert np.array_equal(br.ctx.batch_download(k), rt.render(moved[k])), f"job {k}"
        rt.ctx.close()


def test_path_regeneration_small_pool(rg, batch):
    scenes, singles, _ = batch
    br = rg.BatchRenderer(scenes)
    br.ctx.set_batch_slots(1024)  # far fewer slots than samples: most slots run several paths
    for k, (img, ref) in enumerate(zip(br.render(), singles)):
        assert np.array_equal(img, ref), f"job {k}"


@pytest.mark.parametrize("threads", [64, 128, 256])
@pytest.mark.parametrize("depth", [16, 24, 32, 48])
def test_launch_shapes(rg, batch, threads, depth):
    scenes, singles, _ = batch
    br = rg.BatchRenderer(scenes)
    if threads == 256 and depth == 48:  # not built: beyond a block's static shared memory
        with pytest.raises(rg.RgError):
            br.ctx.set_batch_tune(threads, depth, "none")
        return
    br.ctx.set_batch_tune(threads, depth, "none")
    imgs = br.render()
    assert br.ctx.stats()["stack_overflows"] == 0
    for k, (img, ref) in enumerate(zip(imgs, singles)):
        assert np.array_equal(img, ref), f"job {k} threads {threads} depth {depth}"


@pytest.mark.parametrize("key", ["octant", "morton"])
def test_ray_sort_keys(rg, batch, key):
    scenes, singles, stats = batch
    br = rg.BatchRenderer(scenes)
    br.ctx.set_batch_tune(128, 32, key)
    br.ctx.set_batch_slots(2048)
    imgs = br.render()
    st = br.ctx.stats()
    for k, (img, ref) in enumerate(zip(imgs, singles)):
        assert np.array_equal(img, ref), f"job {k} sort {key}"
    for name in RAY_KEYS:
        assert st[name] == sum(s[name] for s in stats), name


def test_autotuner(rg, batch):
    scenes, singles, _ = batch
    br = rg.BatchRenderer(scenes)
    best, table = br.ctx.autotune_batch(br.jobs(), reps=1)
    assert len(table) == rg.AUTOTUNE_CONFIGS
    timed = {k: v for k, v in table.items() if v is not None}
    assert timed and all(v > 0 for v in timed.values())
    key = (best["threads"], best["stack_depth"], {v: k for k, v in rg.SORT_KEYS.items()}[best["sort_key"]])
    assert table[key] == min(timed.values())
    assert br.ctx.batch_tune() == best
    for k, (img, ref) in enumerate(zip(br.render(), singles)):
        assert np.array_equal(img, ref), f"job {k} after autotune"


def test_batch_vs_oracle(rg, orc):
    from test_gpu_parity import assert_image_close
    scenes = mini_batch(n=3, seed=11)
    br = rg.BatchRenderer(scenes)
    imgs = br.render()
    st = br.ctx.stats()
    total = {k: 0 for k in RAY_KEYS}
    for sc, img in zip(scenes, imgs):
        ob, on, orr, ost = orc.OracleScene(sc).render()
        for k in RAY_KEYS:
            total[k] += ost[k]
        assert_image_close(img, orc.post(sc.ubo, ob, on, orr), sc.name)
    for k in RAY_KEYS:
        assert st[k] == total[k], k


def test_golden_fixtures_as_one_batch(rg):
    from test_golden import FIXTURES, load
    from test_gpu_parity import assert_image_close
    pairs = [load(p) for p in FIXTURES]
    br = rg.BatchRenderer([sc for sc, _ in pairs])
    imgs = br.render()
    st = br.ctx.stats()
    assert st["primary"] + st["shadow"] + st["secondary"] == sum(int(g["rays"][0]) for _, g in pairs)
    for (sc, g), img in zip(pairs, imgs):
        assert_image_close(img, g["final"], f"{sc.name} final (batched)")


def test_same_scene_two_cameras(rg):
    sc = S.spheres_scene(n_spheres=12, width=48, height=27, num_samples=2, max_recursions=3, seed=13)
    moved = S.make_ubo((6, 4, -12), (0, 1, 0), 50.0, 40, 30, (-0.4, -1.0, 0.3), 1, 4)
    rt = rg.Raytracer(sc).prepare()
    ref_a = rt.render()
    rt.ctx.set_resolution(40, 30)
    ref_b = rt.render(moved)
    br = rg.BatchRenderer([sc])
    jobs = np.concatenate([br.jobs(), br.jobs()])
    jobs[1]["width"], jobs[1]["height"], jobs[1]["ubo"] = 40, 30, moved[0]
    br.ctx.render_batch(jobs)
    assert np.array_equal(br.ctx.batch_download(0), ref_a)
    assert np.array_equal(br.ctx.batch_download(1), ref_b)


def test_scene_slots_are_independent(rg):
    a = S.spheres_scene(n_spheres=8, width=32, height=18, num_samples=1, max_recursions=2, seed=21)
    b = S.spheres_scene(n_spheres=20, width=32, height=18, num_samples=1, max_recursions=2, seed=22)
    ctx = rg.Context()
    ctx.set_resolution(32, 18)
    rg.load_scene(ctx, a)
    ctx.render(a.ubo)
    first = ctx.download().copy()
    sb = ctx.scene_create()
    assert sb != 0
    ctx.scene_select(sb)
    rg.load_scene(ctx, b)
    ctx.render(b.ubo)
    img_b = ctx.download().copy()
    assert not np.array_equal(first, img_b)
    assert ctx.scene_bytes(sb) > 0
    ctx.scene_select(0)
    ctx.render(a.ubo)
    assert np.array_equal(ctx.download(), first)
    ctx.scene_destroy(sb)
    with pytest.raises(rg.RgError):
        ctx.scene_bytes(sb)
    again = ctx.scene_create()  # a freed slot id is reused
    assert again == sb


def test_batch_errors(rg):
    sc = S.spheres_scene(n_spheres=4, width=16, height=8, num_samples=1, max_recursions=1, seed=1)
    br = rg.BatchRenderer([sc])
    ctx = br.ctx
    jobs = br.jobs()
    bad = jobs.copy()
    bad[0]["scene"] = 7
    with pytest.raises(rg.RgError) as e:
        ctx.render_batch(bad)
    assert e.value.code == -1
    empty_slot = ctx.scene_create()
    bad = jobs.copy()
    bad[0]["scene"] = empty_slot
    with pytest.raises(rg.RgError) as e:
        ctx.render_batch(bad)
    assert e.value.code == -4  # no TLAS in that slot
    bad = jobs.copy()
    bad[0]["ubo"]["numSamples"] = 0
    with pytest.raises(rg.RgError):
        ctx.render_batch(bad)
    bad = jobs.copy()
    bad[0]["width"] = 0
    with pytest.raises(rg.RgError):
        ctx.render_batch(bad)
    with pytest.raises(rg.RgError):
        ctx.render_batch(jobs[:0])
    with pytest.raises(rg.RgError):
        ctx.set_batch_tune(96, 48, "none")
    with pytest.raises(rg.RgError):
        ctx.set_batch_tune(128, 20, "none")
    with pytest.raises(rg.RgError):
        ctx.scene_destroy(0)  # the selected slot
    fresh = rg.Context()
    with pytest.raises(rg.RgError) as e:
        fresh.batch_download_async(16)  # no batch rendered in this context
    assert e.value.code == -4
    fresh.close()
    ctx.render_batch(jobs)
    with pytest.raises(rg.RgError) as e:
        ctx.batch_download_async(0)  # null host buffer
    assert e.value.code == -1
    with pytest.raises(rg.RgError):
        ctx.batch_download(1)
    assert ctx.batch_download(0).shape == (8, 16, 4)


def test_batch_loop_limit_is_reported(rg, batch, monkeypatch):
    """The device-side round loop of the batch graph stops at an iteration limit and leaves a sticky
    flag, which the host reports as RG_ERR_CUDA at the next read-back.  Forced here with a limit of
    one body run (RG_BATCH_LOOP_LIMIT, read when the graph is captured): nothing faults or hangs,
    and a new context renders the batch correctly."""
    scenes, singles, _ = batch
    monkeypatch.setenv("RG_BATCH_LOOP_LIMIT", "1")
    br = rg.BatchRenderer(scenes)
    br.ctx.set_batch_slots(1024)  # a small pool: the batch needs many more than two rounds
    br.ctx.render_batch(br.jobs())
    with pytest.raises(rg.RgError) as e:
        br.ctx.batch_download(0)
    assert e.value.code == -2 and "iteration limit" in str(e.value), str(e.value)
    br.ctx.close()
    monkeypatch.delenv("RG_BATCH_LOOP_LIMIT")
    br = rg.BatchRenderer(scenes)
    assert all(np.array_equal(a, b) for a, b in zip(br.render(), singles))
    br.ctx.close()
