"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle on the same seeded
inputs.

Bars (written per test):
* LBVH: Morton codes, sorted order, topology, node boxes -- bit exact.
* closest hit: instance / primitive ids and t, u, v -- bit exact (both sides evaluate the same
  IEEE operations in the same order).
* G-buffers and the final image: per-channel |diff| <= 2/255 on >= 99.9 % of pixels and
  PSNR >= 50 dB against the oracle.  Ray geometry is bit exact; the residue comes from logf/powf
  (CUDA vs glibc), which only reach colours.
* post passes on identical G-buffers: bit exact.
* ray counts (primary / shadow / secondary / mask-0): exact.
"""
import numpy as np
import pytest

from raygun_gb300 import scenes as S
from test_oracle import camera_rays, random_boxes, random_rays

pytestmark = pytest.mark.gpu

TOL = 2.0 / 255.0


def psnr(a, b):
    mse = float(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
    return float("inf") if mse == 0 else 10 * np.log10(1.0 / mse)


def assert_image_close(gpu, ref, what, frac=0.999, min_psnr=50.0):
    assert np.isfinite(gpu).all(), f"{what}: non-finite values"
    err = np.abs(gpu - ref)
    ok = (err <= TOL).all(-1)
    p = psnr(np.clip(gpu, 0, 1), np.clip(ref, 0, 1))
    print(f"{what}: exact {np.mean(err.max(-1) == 0):.5f}, within 2/255 {ok.mean():.5f}, max {err.max():.4g}, psnr {p:.1f} dB")
    assert ok.mean() >= frac, f"{what}: only {ok.mean():.5f} of pixels within 2/255"
    assert p >= min_psnr, f"{what}: PSNR {p:.1f} dB < {min_psnr}"


def lbvh_equal(g, o):
    for k in ("morton", "order", "left", "right"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["nodeboxes"], o["nodeboxes"]), "nodeboxes"


@pytest.mark.parametrize("n,dup", [(1, False), (2, False), (3, False), (100, False), (2049, True), (70000, False),
                                   (300000, True), (1 << 20, False), ((1 << 20) + 1, True)])
def test_lbvh_build_bit_exact(rg, orc, n, dup):
    boxes = random_boxes(n, 7 + n, dup)
    ctx = rg.Context()
    lbvh_equal(ctx.lbvh_build_host(boxes), orc.lbvh(boxes))


def test_lbvh_sort_lookback_counts_unpublished_tiles(rg, orc, monkeypatch):
    """Onesweep passes in which every look-back that meets a tile not yet published counts that
    tile's keys itself (RG_SORT_SPIN_LIMIT=0) sort exactly as the published words do."""
    monkeypatch.setenv("RG_SORT_SPIN_LIMIT", "0")
    boxes = random_boxes(300000, 99, True)
    ctx = rg.Context()
    lbvh_equal(ctx.lbvh_build_host(boxes), orc.lbvh(boxes))


def test_lbvh_all_equal_keys(rg, orc):
    boxes = np.tile(np.array([[0, 0, 0, 1, 1, 1]], np.float32), (5000, 1))
    ctx = rg.Context()
    lbvh_equal(ctx.lbvh_build_host(boxes), orc.lbvh(boxes))


def small_two_level():
    return S.instanced_scene(width=96, height=54, counts=(6, 5, 3, 1, 4, 4, 1, 1), hf_n=32, ico_levels=(1, 2, 3, 3),
                             num_samples=2, max_recursions=5, name="mini-game-frame")


@pytest.fixture(scope="module")
def spheres_pair(rg, orc):
    sc = S.sphere_scene()
    # the LBVH BLAS, whose topology the oracle pins (the default binned-SAH BLAS is checked in
    # test_gpu_records.py)
    rt = rg.Raytracer(sc, flags=rg.RG_FLAG_DEBUG_IMAGES | rg.RG_FLAG_BLAS_LBVH).prepare()
    return sc, rt, orc.OracleScene(sc)


@pytest.fixture(scope="module")
def game_pair(rg, orc):
    # the LBVH TLAS and BLASes, whose topology the oracle pins (the default binned-SAH trees are
    # checked in test_gpu_records.py)
    sc = small_two_level()
    rt = rg.Raytracer(sc, flags=rg.RG_FLAG_DEBUG_IMAGES | rg.RG_FLAG_TLAS_LBVH | rg.RG_FLAG_BLAS_LBVH).prepare()
    return sc, rt, orc.OracleScene(sc)


def test_blas_tlas_spheres(spheres_pair):
    sc, rt, o = spheres_pair
    lbvh_equal(rt.ctx.bvh(0), o.bvh(0))
    g, r = rt.ctx.bvh(-1), o.bvh(-1)
    assert np.array_equal(g["morton"], r["morton"]) and np.array_equal(g["order"], r["order"])


def test_two_level_bvh(game_pair):
    sc, rt, o = game_pair
    for b in range(len(sc.meshes)):
        lbvh_equal(rt.ctx.bvh(b), o.bvh(b))
    lbvh_equal(rt.ctx.bvh(-1), o.bvh(-1))
    assert np.array_equal(rt.ctx.instance_inverse(len(sc.instances)), o.instance_inverse())


@pytest.mark.parametrize("which", ["spheres", "game-frame"])
def test_closest_hit_bit_exact(which, spheres_pair, game_pair):
    sc, rt, o = spheres_pair if which == "spheres" else game_pair
    if which == "spheres":
        rays = np.concatenate([camera_rays(sc, stride=2), random_rays(20000, 3)])
    else:
        rays = np.concatenate([camera_rays(sc), random_rays(20000, 4, lo=(-60, 0, -60), hi=(60, 14, 60))])
    rays = np.concatenate([rays, rays[:5] * np.array([1, 1, 1, 1, 0, 0, 0, 1], np.float32)])  # zero directions miss
    tg, ig = rt.ctx.trace_rays(rays)
    to, io = o.trace(rays)
    assert np.array_equal(ig, io)
    assert np.array_equal(tg, to)
    assert (ig[-5:, 0] == 0xFFFFFFFF).all()
    assert (ig[:, 0] != 0xFFFFFFFF).mean() > (0.2 if which == "spheres" else 0.03)


def _gbuffers(rt):
    return [rt.ctx.download_image(k) for k in ("base", "normal", "rough")]


@pytest.mark.parametrize("which", ["spheres", "game-frame"])
def test_gbuffer_and_frame_parity(which, spheres_pair, game_pair, orc):
    sc, rt, o = spheres_pair if which == "spheres" else game_pair
    rt.do_raytracing(fxaa=False)
    gb = _gbuffers(rt)
    st = rt.ctx.stats()
    ob, on, orr, ost = o.render()
    for k in ("primary", "shadow", "secondary", "masked"):
        assert st[k] == ost[k], (k, st[k], ost[k])
    assert st["stack_overflows"] == 0
    for name, g, r in zip(("base", "normal", "rough"), gb, (ob, on, orr)):
        assert_image_close(g, r, f"{which} {name}")
    rt.do_raytracing(fxaa=True)
    fin = rt.ctx.download()
    ref = orc.post(sc.ubo, ob, on, orr)
    assert_image_close(fin, ref, f"{which} final")


@pytest.mark.parametrize("show_alpha,fade", [(0, (0, 0, 0, 0)), (1, (0, 0, 0, 0)), (0, (0.2, 0.4, 0.6, 0.5))])
def test_post_passes_bit_exact(spheres_pair, orc, show_alpha, fade):
    sc, rt, o = spheres_pair
    ob, on, orr, _ = o.render()
    u = sc.ubo.copy()
    u["showAlpha"], u["fadeColor"] = show_alpha, fade
    for fx in (False, True):
        rt.ctx.post_only(u, ob, on, orr, fxaa=fx)
        fin = rt.ctx.download()
        ref, dbg = orc.post(u, ob, on, orr, fxaa=fx, debug=True)
        assert np.array_equal(fin, ref), f"fxaa={fx}: {np.mean(fin != ref)} differ"
    assert np.array_equal(rt.ctx.download_image("rough_transition")[..., 0], dbg[0][..., 0])
    assert np.array_equal(rt.ctx.download_image("rough_colors_a"), dbg[1])
    assert np.array_equal(rt.ctx.download_image("rough_colors_b"), dbg[2])
    assert np.array_equal(rt.ctx.download_image("pre_fxaa"), dbg[3])


@pytest.mark.parametrize("w,h", [(97, 55), (130, 33), (7, 90), (1, 1)])
def test_post_passes_odd_and_ragged_sizes(rg, orc, w, h):
    """The roughness pass stages its 64x32 tiles by TMA when the width is even and with plain loads
    when it is odd; tiles at the right and bottom edges are partial, and FXAA clamps at every edge.
    The composited frame stays bit-exact with the oracle's post passes."""
    sc = S.spheres_scene(n_spheres=8, width=w, height=h, num_samples=1, max_recursions=3, seed=21)
    ob, on, orr, _ = orc.OracleScene(sc).render()
    rt = rg.Raytracer(sc).prepare()
    for fx in (False, True):
        rt.ctx.post_only(sc.ubo, ob, on, orr, fxaa=fx)
        fin = rt.ctx.download()
        ref = orc.post(sc.ubo, ob, on, orr, fxaa=fx)
        assert np.array_equal(fin, ref), f"{w}x{h} fxaa={fx}: {np.mean(fin != ref)} differ"
    rt.ctx.close()


@pytest.mark.parametrize("w,h,spp", [(97, 55, 2), (31, 9, 3)])
def test_frame_at_odd_sizes(rg, orc, w, h, spp):
    """Frames whose sizes are not multiples of the 8x4 work-item tiles (partial tiles in both
    directions): G-buffers, final image and ray counts against the oracle."""
    sc = S.spheres_scene(n_spheres=10, width=w, height=h, num_samples=spp, max_recursions=4, seed=23)
    rt = rg.Raytracer(sc, flags=rg.RG_FLAG_DEBUG_IMAGES).prepare()
    rt.do_raytracing(fxaa=False)
    st = rt.ctx.stats()
    gb = [rt.ctx.download_image(k) for k in ("base", "normal", "rough")]
    fin = rt.render()
    ob, on, orr, ost = orc.OracleScene(sc).render()
    for k in ("primary", "shadow", "secondary", "masked"):
        assert st[k] == ost[k], (k, st[k], ost[k])
    for name, g, r in zip(("base", "normal", "rough"), gb, (ob, on, orr)):
        assert_image_close(g, r, f"{w}x{h} {name}")
    assert_image_close(fin, orc.post(sc.ubo, ob, on, orr), f"{w}x{h} final")
    rt.ctx.close()


def test_animation_refit_and_tlas_rebuild(rg, orc):
    sc = small_two_level()
    rt = rg.Raytracer(sc, flags=rg.RG_FLAG_TLAS_LBVH | rg.RG_FLAG_BLAS_LBVH).prepare()
    o = orc.OracleScene(sc)
    anim = S.FrameAnimator(sc, seed=7, refit_prob=0.5)
    for frame in range(3):
        refits = anim.step()
        for b, vo, nv in refits:
            rt.ctx.update_vertices(vo, sc.vertices[vo:vo + nv])
            rt.ctx.refit_blas(rt.blas_ids[b])
            o.refit(b, sc.vertices[vo:vo + nv], vo)
        rt.setup_top_level_as()
        o.set_instances(sc.instances)
        for b, _, _ in refits:
            lbvh_equal(rt.ctx.bvh(b), o.bvh(b))
        lbvh_equal(rt.ctx.bvh(-1), o.bvh(-1))
        fin = rt.render()
        ob, on, orr, _ = o.render()
        assert_image_close(fin, orc.post(sc.ubo, ob, on, orr), f"frame {frame}")


@pytest.mark.parametrize("spp,depth,mega", [(1, 0, False), (3, 1, False), (4, 7, False), (9, 2, False), (4, 7, True),
                                            (2, 3, True)])
def test_samples_and_depths(rg, orc, spp, depth, mega):
    sc = S.spheres_scene(n_spheres=16, width=80, height=45, num_samples=spp, max_recursions=depth, seed=5)
    rt = rg.Raytracer(sc, flags=rg.RG_FLAG_MEGAKERNEL if mega else 0).prepare()
    o = orc.OracleScene(sc)
    fin = rt.render()
    st = rt.ctx.stats()
    ob, on, orr, ost = o.render()
    for k in ("primary", "shadow", "secondary", "masked"):
        assert st[k] == ost[k], (k, st[k], ost[k])
    assert_image_close(fin, orc.post(sc.ubo, ob, on, orr), f"spp{spp} depth{depth} mega={mega}")


def test_download_async(rg):
    """Asynchronous read-backs through both staging slots deliver each frame's own pixels, equal to
    the synchronous read-back of the same frame."""
    torch = pytest.importorskip("torch")
    sc = small_two_level()
    rt = rg.Raytracer(sc).prepare()
    ubos = [sc.ubo.copy() for _ in range(3)]
    for k, u in enumerate(ubos):
        u["clearColor"] = np.array([0.1 * k, 0.2, 0.3], np.float32)
        u["lightDir"] = np.array([-0.4 + 0.2 * k, -1.0, 0.3], np.float32)
    want = []
    for u in ubos:
        rt.ctx.render(u, True)
        want.append(rt.ctx.download())
    bufs = [torch.empty(sc.height * sc.width * 4, dtype=torch.float32).pin_memory() for _ in ubos]
    for u, b in zip(ubos, bufs):
        rt.ctx.render(u, True)
        rt.ctx.download_async(b.data_ptr())
    rt.ctx.synchronize()
    for w, b in zip(want, bufs):
        assert np.array_equal(b.numpy().reshape(w.shape), w)
    assert not np.array_equal(want[0], want[2])
    rt.ctx.close()


def test_errors_are_status_codes(rg):
    ctx = rg.Context()
    sc = S.spheres_scene(n_spheres=2, width=16, height=16, slices=8, stacks=4)
    with pytest.raises(rg.RgError) as e:
        ctx.render(sc.ubo)
    assert e.value.code in (-4,)
    bad = sc.indices.copy()
    bad[0] = 10 ** 6
    with pytest.raises(rg.RgError) as e:
        ctx.upload_geometry(sc.vertices, bad, sc.materials)
    assert e.value.code == -1
    m = sc.materials.copy()
    m["rayConsumption"] = 0
    with pytest.raises(rg.RgError):
        ctx.upload_geometry(sc.vertices, sc.indices, m)
    ctx.upload_geometry(sc.vertices, sc.indices, sc.materials)
    with pytest.raises(rg.RgError):
        ctx.build_blas(0, 0, len(sc.indices))  # range beyond the index buffer
    u = sc.ubo.copy()
    u["numSamples"] = 0
    ctx.set_resolution(16, 16)
    b = ctx.build_blas(0, 0, len(sc.indices) // 3)
    inst = S.identity_instance(b)
    ctx.build_tlas(inst)
    with pytest.raises(rg.RgError):
        ctx.render(u)


def test_roughness_copy_wait_that_gives_up_is_reported(rg, monkeypatch):
    """The roughness pass's waits for its TMA-staged tiles are bounded.  With the first wait's bound
    at zero polls (RG_POST_WAIT_LIMIT=0) the pass gives up on its first tile, still waits (with the
    full bound) for that copy to land, and returns; rg_download then reports RG_ERR_CUDA naming the
    pass.  Nothing faults or hangs."""
    monkeypatch.setenv("RG_POST_WAIT_LIMIT", "0")
    sc = S.spheres_scene(n_spheres=6, width=96, height=54, num_samples=1, max_recursions=2, seed=2)  # even width: TMA
    rt = rg.Raytracer(sc).prepare()
    with pytest.raises(rg.RgError) as e:
        rt.render()
    assert e.value.code == -2 and "roughness" in str(e.value), str(e.value)
    rt.ctx.close()


def test_malformed_scene_rejected_on_host(rg, orc):
    """Index, vertex and material references that leave the uploaded buffers are rejected on the host
    with RG_ERR_INVALID_ARG before any kernel reads through them (the reference relied on Vulkan's
    robustBufferAccess instead, vulkan_context.cpp:256-257).  Indices are local to their mesh, so the
    checks are made per range: vertexOffset + index, and materialBufferOffset + vertex.matIndex."""
    sc = S.spheres_scene(n_spheres=2, width=16, height=16, slices=8, stacks=4)
    ctx = rg.Context()
    ctx.upload_geometry(sc.vertices, sc.indices, sc.materials)
    ctx.set_resolution(16, 16)
    nv, nt, nm = len(sc.vertices), len(sc.indices) // 3, len(sc.materials)
    maxi = int(sc.indices.max())
    for voff, ioff, n in ((nv - maxi, 0, nt),  # vertexOffset + index reaches nv
                          (0, 3, nt),  # one triangle past the index buffer
                          (1 << 31, 0, 1)):
        with pytest.raises(rg.RgError) as e:
            ctx.build_blas(voff, ioff, n)
        assert e.value.code == -1, (voff, ioff, n)
    b = ctx.build_blas(nv - maxi - 1, 0, nt)  # the last vertex is still inside
    b = ctx.build_blas(0, 0, nt)
    good = S.identity_instance(b)
    good["vertexBufferOffset"], good["indexBufferOffset"] = 0, 0
    ctx.build_tlas(good)
    maxm = int(sc.vertices["matIndex"].max())
    for field, value in (("indexBufferOffset", 3), ("vertexBufferOffset", nv - maxi),
                         ("materialBufferOffset", nm - maxm)):
        inst = np.concatenate([good, good])
        inst[1][field] = value
        with pytest.raises(rg.RgError) as e:
            ctx.build_tlas(inst)
        assert e.value.code == -1 and "instance 1" in str(e.value), field
    # instances that are never traversed (unknown BLAS, mask 0) are not checked
    skip = np.concatenate([good, good, good])
    skip[1]["blas"], skip[1]["indexBufferOffset"] = 99, 10 ** 6
    skip[2]["mask"], skip[2]["materialBufferOffset"] = 0, 10 ** 6
    ctx.build_tlas(skip)
    ctx.build_tlas(good)
    # a vertex update that points a referenced vertex past the materials is refused, and nothing changes
    v = sc.vertices[:1].copy()
    v["matIndex"] = nm
    with pytest.raises(rg.RgError) as e:
        ctx.update_vertices(0, v)
    assert e.value.code == -1
    ctx.render(sc.ubo)
    img = ctx.download()
    o = orc.OracleScene(sc)
    assert_image_close(img, orc.post(sc.ubo, *o.render()[:3]), "after refused updates")
    ctx.close()


def test_device_instances_with_foreign_offsets_are_skipped(rg, orc):
    """rg_build_tlas_device cannot check instances on the host: the TLAS build skips (never hits) an
    instance whose vertex/index offsets are not its BLAS's own or whose material offset takes the
    BLAS's materials past the buffer; the others trace as the oracle traces them."""
    import torch
    sc = S.spheres_scene(n_spheres=4, width=32, height=18, slices=8, stacks=4)
    ctx = rg.Context()
    ctx.upload_geometry(sc.vertices, sc.indices, sc.materials)
    b = ctx.build_blas(0, 0, len(sc.indices) // 3)
    inst = np.concatenate([S.identity_instance(b)] * 3)
    inst["transform"][1, :, 3] += (0, 50, 0)
    inst["transform"][2, :, 3] += (0, 100, 0)
    inst[1]["vertexBufferOffset"] = 1
    inst[2]["materialBufferOffset"] = len(sc.materials)
    d = torch.from_numpy(inst.view(np.uint8)).cuda()
    ctx.build_tlas_device(d.data_ptr(), len(inst))
    rays = np.zeros((3, 8), np.float32)
    rays[:, 0:3] = [(0, 5, -20), (0, 55, -20), (0, 105, -20)]
    rays[:, 3], rays[:, 7] = 1e-3, 1e4
    rays[:, 4:7] = (0, -0.25, 1)
    tuv, ids = ctx.trace_rays(rays)
    assert ids[0, 0] == 0 and ids[1, 0] == 0xFFFFFFFF and ids[2, 0] == 0xFFFFFFFF
    ctx.close()


def test_hbm_budget_rejects(rg):
    ctx = rg.Context(hbm_budget_bytes=1 << 20)
    with pytest.raises(rg.RgError) as e:
        ctx.set_resolution(1920, 1080)
    assert e.value.code == -6


def test_material_live_edit(rg, orc):
    """gpu/gpu_material.cpp:52-94 -> RenderSystem::updateModelBuffers: new material values reach the
    next frame without touching the BVHs."""
    sc = S.spheres_scene(n_spheres=10, width=80, height=45, num_samples=1, max_recursions=4, seed=11)
    rt = rg.Raytracer(sc).prepare()
    before = rt.render()
    mats = sc.materials.copy()
    mats["diffuse"][1:5] = [(1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), (1.0, 1.0, 0.0)]
    mats["reflectivity"][5] = 0.95
    mats["transparency"][6], mats["ior"][6] = 0.98, 1.33
    rt.ctx.update_materials(0, mats)
    after = rt.render()
    sc.materials = mats
    o = orc.OracleScene(sc)
    ob, on, orr, _ = o.render()
    assert_image_close(after, orc.post(sc.ubo, ob, on, orr), "after material edit")
    assert np.abs(after - before).max() > 0.1


def test_vertex_material_edit_without_refit(rg, orc):
    """The closest-hit shader reads v0's matIndex from the vertex buffer every frame
    (closesthit.rchit:100-109): a vertex update that only reassigns materials reaches the next
    frame without a refit (the traversal's triangle records carry the material index and are
    refreshed for the BLASes whose vertices changed)."""
    sc = S.spheres_scene(n_spheres=10, width=80, height=45, num_samples=1, max_recursions=4, seed=11)
    rt = rg.Raytracer(sc).prepare()
    before = rt.render()
    verts = sc.vertices.copy()
    nm = len(sc.materials)
    # reassign the material of every other sphere vertex (positions untouched)
    sel = np.arange(len(verts)) % 2 == 0
    verts["matIndex"][sel] = (verts["matIndex"][sel] + 3) % nm
    rt.ctx.update_vertices(0, verts)
    after = rt.render()
    sc.vertices = verts
    o = orc.OracleScene(sc)
    ob, on, orr, _ = o.render()
    assert_image_close(after, orc.post(sc.ubo, ob, on, orr), "after vertex material edit")
    assert np.abs(after - before).max() > 0.1


def test_contexts_on_two_host_threads(rg):
    """One context per host thread (the reference's single-threaded use, raygun.cpp:91-133, once per
    thread): two contexts rendering at the same time on two threads give the frames each gives
    alone, bit for bit."""
    import threading
    scs = [S.spheres_scene(n_spheres=8, width=96, height=54, num_samples=2, max_recursions=4, seed=21),
           S.instanced_scene(width=96, height=54, counts=(3, 2, 1, 1, 2, 2, 1, 1), hf_n=32, ico_levels=(1, 2, 3, 3),
                             num_samples=2, max_recursions=5, name="mini-game-frame-threads")]
    alone = []
    for sc in scs:
        rt = rg.Raytracer(sc).prepare()
        alone.append(rt.render())
        rt.ctx.close()
    rts = [rg.Raytracer(sc).prepare() for sc in scs]
    out = [[None] * 4 for _ in scs]
    errors = []

    def run(k):
        try:
            for i in range(4):
                out[k][i] = rts[k].render()
        except Exception as e:  # reported on the main thread
            errors.append(e)

    threads = [threading.Thread(target=run, args=(k,)) for k in range(len(scs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for k in range(len(scs)):
        for i in range(4):
            assert np.array_equal(out[k][i], alone[k]), (k, i)
    for rt in rts:
        rt.ctx.close()


def test_large_blas_is_lbvh(rg, orc):
    """BLASes of more than 2^18 triangles are built as LBVHs (the binned-SAH builder runs in one CTA
    and is kept for meshes up to that size): the oracle's LBVH, bit for bit."""
    g = 364  # 2 * 363^2 = 263,538 triangles
    ys, xs = np.meshgrid(np.arange(g, dtype=np.float32), np.arange(g, dtype=np.float32), indexing="ij")
    rng = np.random.RandomState(17)
    verts = np.zeros(g * g, S.VERTEX)
    verts["position"] = np.stack([xs.ravel(), rng.uniform(0, 0.5, g * g).astype(np.float32), ys.ravel()], 1)
    verts["normal"] = (0, 1, 0)
    q = (np.arange(g - 1)[:, None] * g + np.arange(g - 1)[None, :]).ravel().astype(np.uint32)
    idx = np.stack([q, q + g, q + 1, q + 1, q + g, q + g + 1], 1).astype(np.uint32).ravel()
    n = len(idx) // 3
    assert n > (1 << 18)
    sc = S.spheres_scene(n_spheres=1, width=8, height=8)
    ctx = rg.Context()
    ctx.upload_geometry(verts, idx, sc.materials)
    b = ctx.build_blas(0, 0, n)
    p = verts["position"][idx.astype(np.int64)].reshape(n, 3, 3)
    boxes = np.ascontiguousarray(np.concatenate([p.min(1), p.max(1)], 1), np.float32)
    lbvh_equal(ctx.bvh(b), orc.lbvh(boxes))
    ctx.close()


def deep_chain_scene(n_side=30, width=48, height=32):
    """Small triangles in the planes x = +-17^k (k < n_side), facing along x.  Every binned-SAH split
    peels the outermost triangles off, so the tree runs past the level from which the builder halves
    ranges (34 levels for 30 a side).  The camera at the origin looks down the +x chain: its rays
    descend the whole chain, pushing the far siblings of every record on the way."""
    xs = 17.0 ** np.arange(n_side)
    pos, nrm, idx = [], [], []
    for sign in (1.0, -1.0):
        for x in xs:
            b = len(pos)
            pos += [(sign * x, 0.0, 0.0), (sign * x, 0.0, 0.5), (sign * x, 0.5, 0.0)]
            nrm += [(-sign, 0.0, 0.0)] * 3
            idx.append((b, b + 1, b + 2))
    mesh = S.Mesh(np.array(pos), np.array(nrm), np.array(idx, np.uint32))
    assert np.isfinite(mesh.positions.astype(np.float32)).all()
    mats = S.random_materials(S.Rng(5), 1)
    ubo = S.make_ubo((0.0, 0.2, 0.2), (1.0, 0.2, 0.2), 60.0, width, height, (-0.4, -1.0, 0.3), 1, 3)
    return S._finish("deep-chain", [(mesh, np.zeros(len(pos), np.uint32))], mats, S.identity_instance(), ubo, width, height)


def test_deep_sah_blas_bounded_and_traced(rg, orc):
    """A BLAS whose surface-area splits peel one triangle at a time: the GPU builds the oracle's tree,
    whose ranges are halved from level 32 on (so no SAH tree is deeper than 32 + ceil(log2 n)
    levels), and rays through it hit what the oracle's rays hit."""
    sc = deep_chain_scene()
    n = int(sc.meshes["triCount"][0])
    p = sc.vertices["position"][sc.indices.astype(np.int64)].reshape(n, 3, 3)
    boxes = np.ascontiguousarray(np.concatenate([p.min(1), p.max(1)], 1), np.float32)
    ref = orc.sah(boxes)
    assert ref["levels"] == 34 and orc.sah(boxes, 1 << 20)["levels"] == 35  # the halving took over
    rt = rg.Raytracer(sc).prepare()
    assert orc.same_tree(rt.ctx.bvh(0), ref)
    o = orc.OracleScene(sc)
    rng = np.random.RandomState(3)
    k = 4000
    rays = np.zeros((k, 8), np.float32)
    rays[:, 0] = 0.0
    rays[:, 1:3] = rng.uniform(0.01, 0.2, (k, 2))
    rays[:, 3], rays[:, 7] = 1e-3, 3e38
    rays[:, 4] = np.where(np.arange(k) < k // 2, 1.0, -1.0)  # exactly along the chains: down the whole tree
    rays = np.concatenate([rays, camera_rays(sc)])
    to, io = o.trace(rays)
    assert (io[:, 0] != 0xFFFFFFFF).mean() > 0.3
    tg, ig = rt.ctx.trace_rays(rays)
    assert np.array_equal(ig, io) and np.array_equal(tg, to)
    assert rt.ctx.stats()["deep_overflows"] == 0
    rt.ctx.close()


def multi_chain_scene(chains=64, n_side=30, width=48, height=32):
    """`chains` copies of the deep chain side by side (chain j at z = 2j).  Each surface-area split
    peels the outermost triangles of every chain off at once, as a group that is then split along z,
    so a level holds 64 node tasks from level 6 on -- where the builder's task kernel takes over --
    while the chains still run past level 32, from which ranges are halved."""
    xs = 17.0 ** np.arange(n_side)
    pos, nrm, idx = [], [], []
    for j in range(chains):
        z = 2.0 * j
        for sign in (1.0, -1.0):
            for x in xs:
                b = len(pos)
                pos += [(sign * x, 0.0, z), (sign * x, 0.0, z + 0.5), (sign * x, 0.5, z)]
                nrm += [(-sign, 0.0, 0.0)] * 3
                idx.append((b, b + 1, b + 2))
    mesh = S.Mesh(np.array(pos), np.array(nrm), np.array(idx, np.uint32))
    mats = S.random_materials(S.Rng(8), 1)
    ubo = S.make_ubo((0.0, 0.2, 30.0), (1.0, 0.2, 30.0), 90.0, width, height, (-0.4, -1.0, 0.3), 1, 3)
    return S._finish("multi-chain", [(mesh, np.zeros(len(pos), np.uint32))], mats, S.identity_instance(), ubo, width, height)


def tasks_per_level(tree):
    """Internal nodes per level of a BVH2 in the LBVH layout."""
    counts, st = {}, [(0, 0)]
    while st:
        i, lv = st.pop()
        counts[lv] = counts.get(lv, 0) + 1
        for c in (int(tree["left"][i]), int(tree["right"][i])):
            if not c & 0x80000000:
                st.append((c, lv + 1))
    return counts


@pytest.mark.parametrize("chains", [64, 640])
def test_sah_task_kernel_past_the_median_level(rg, orc, chains):
    """The SAH builder's task kernel (a work queue over every SM, from the first level of 64 tasks
    on) builds the oracle's tree also where it halves ranges (level 32 on), and rays through it hit
    what the oracle's rays hit.  640 chains (38,400 triangles) also take the first levels' tasks
    over many CTAs each (builds of at least 32,768 primitives)."""
    sc = multi_chain_scene(chains=chains)
    n = int(sc.meshes["triCount"][0])
    p = sc.vertices["position"][sc.indices.astype(np.int64)].reshape(n, 3, 3)
    boxes = np.ascontiguousarray(np.concatenate([p.min(1), p.max(1)], 1), np.float32)
    ref = orc.sah(boxes)
    per = tasks_per_level(ref)
    handoff = min(lv for lv, k in per.items() if k >= 64)
    assert handoff < 32 and ref["levels"] > 33 and sum(k for lv, k in per.items() if lv >= 32) > 500, (handoff, ref["levels"])
    rt = rg.Raytracer(sc).prepare()
    assert orc.same_tree(rt.ctx.bvh(0), ref)
    o = orc.OracleScene(sc)
    rng = np.random.RandomState(4)
    k = 4000
    rays = np.zeros((k, 8), np.float32)
    rays[:, 1] = rng.uniform(0.01, 0.2, k)
    rays[:, 2] = 2.0 * rng.randint(0, 64, k) + rng.uniform(0.01, 0.2, k)  # inside one chain's triangles
    rays[:, 3], rays[:, 7] = 1e-3, 3e38
    rays[:, 4] = np.where(np.arange(k) < k // 2, 1.0, -1.0)
    rays = np.concatenate([rays, camera_rays(sc)])
    to, io = o.trace(rays)
    assert (io[:, 0] != 0xFFFFFFFF).mean() > 0.3
    tg, ig = rt.ctx.trace_rays(rays)
    assert np.array_equal(ig, io) and np.array_equal(tg, to)
    assert rt.ctx.stats()["deep_overflows"] == 0
    rt.ctx.close()


def stacked_scene(n=1 << 14, width=48, height=32):
    """n coincident triangles facing the camera.  Their centroids coincide, so the builder halves
    every range: a balanced tree of 14 levels whose boxes every camera ray enters, all at the same
    distance.  A ray then visits every record with all four children hit and pushes three of them at
    each of its 7 record levels: 21 entries plus the marker, beyond a 16-word stack (15 entries),
    within the default 48."""
    tri = np.array([(4.0, -3.0, -3.0), (4.0, 9.0, -3.0), (4.0, -3.0, 9.0)])
    pos = np.tile(tri, (n, 1))
    nrm = np.tile((-1.0, 0.0, 0.0), (3 * n, 1))
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    mesh = S.Mesh(pos, nrm, idx)
    mats = S.random_materials(S.Rng(6), 1)
    ubo = S.make_ubo((0.0, 0.0, 0.0), (1.0, 0.0, 0.0), 60.0, width, height, (-0.4, -1.0, 0.3), 1, 2)
    return S._finish("stacked", [(mesh, np.zeros(len(pos), np.uint32))], mats, S.identity_instance(), ubo, width, height)


def test_stack_overflow_is_retraced(rg, orc):
    """With a 16-word traversal stack (rg_set_batch_tune) every ray through the stacked scene
    overflows it; each is traced again with the deep stack, so the hits still equal the oracle's,
    from rg_trace_rays and from the wavefront trace kernel's query form (rg_trace_rays_device,
    re-traced by its last block), and the batch frame (the same kernel) equals rg_render's 48-word
    frame, which does not overflow, bit for bit."""
    import torch
    sc = stacked_scene()
    rt = rg.Raytracer(sc).prepare()
    # coincident centroids: every range is halved, on one CTA down to 64 tasks, then on every SM
    n = int(sc.meshes["triCount"][0])
    p = sc.vertices["position"][sc.indices.astype(np.int64)].reshape(n, 3, 3)
    assert orc.same_tree(rt.ctx.bvh(0), orc.sah(np.ascontiguousarray(np.concatenate([p.min(1), p.max(1)], 1), np.float32)))
    ref = rt.render()
    assert rt.ctx.stats()["stack_overflows"] == 0
    o = orc.OracleScene(sc)
    rays = camera_rays(sc)
    to, io = o.trace(rays)
    assert (io[:, 0] != 0xFFFFFFFF).mean() > 0.9
    d_rays = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    for depth in (48, 16):
        rt.ctx.set_batch_tune(128, depth, "none")
        tg, ig = rt.ctx.trace_rays(rays)
        st = rt.ctx.stats()
        assert np.array_equal(ig, io) and np.array_equal(tg, to), depth
        assert st["deep_overflows"] == 0
        assert (st["stack_overflows"] > 0) == (depth == 16), (depth, st)
        d_tuv = torch.full((len(rays), 3), -1.0, device="cuda")
        d_ids = torch.zeros((len(rays), 2), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rt.ctx.trace_rays_device(d_rays.data_ptr(), len(rays), d_tuv.data_ptr(), d_ids.data_ptr())
        rt.ctx.synchronize()
        st = rt.ctx.stats()
        assert np.array_equal(d_ids.cpu().numpy().view(np.uint32), io) and np.array_equal(d_tuv.cpu().numpy(), to), depth
        assert st["deep_overflows"] == 0
        assert (st["stack_overflows"] > 0) == (depth == 16), (depth, st)
    # the query form reads the rays as float4: a pointer off the 16-byte grid is turned away on the host
    with pytest.raises(rg.RgError, match="aligned"):
        rt.ctx.trace_rays_device(d_rays.data_ptr() + 4, len(rays) - 1, d_tuv.data_ptr(), d_ids.data_ptr())
    rt.ctx.close()
    for flags in (0, rg.RG_FLAG_HOST_LOOP):
        br = rg.BatchRenderer([sc], flags=flags)
        br.ctx.set_batch_tune(128, 16, "none")
        img = br.render()[0]
        st = br.ctx.stats()
        assert st["stack_overflows"] > 0 and st["deep_overflows"] == 0, st
        assert np.array_equal(img, ref), flags
        br.ctx.close()
