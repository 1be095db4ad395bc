"""Parity at the configurations the benchmark times, with the library's default trees.

* Game frame (1920x1080, 4x SSAA, depth 5, 1024 instances of 8 meshes, binned-SAH BLASes and TLAS),
  animated as the benchmark animates it (instances moved, BLASes refit):
  - every BLAS is the oracle's binned-SAH tree over the same triangle boxes (leaf order, structure,
    node boxes; the numbering of a level's nodes aside), and a refit BLAS keeps that topology with
    node boxes that are exactly the unions of its new triangle boxes;
  - closest hits of >= 200k camera and random rays: instance / primitive ids and t, u, v bit exact;
  - the whole frame: per-type ray counts exact, G-buffers and the final image within 2/255 on
    >= 99.9 % of pixels at PSNR >= 50 dB against the oracle.
* Sphere scene (640x360, 1 spp, depth 4, 61,442 triangles) with the default SAH BLAS: G-buffers,
  final image and ray counts against the oracle.
* Three scenes of the batched-rendering workload rendered as one batch: each image against the
  oracle's render of its scene.
"""
import numpy as np
import pytest

from raygun_gb300 import scenes as S
from test_gpu_parity import assert_image_close
from test_oracle import camera_rays, random_rays

pytestmark = pytest.mark.gpu

RAY_KEYS = ("primary", "shadow", "secondary", "masked")
LEAF = 0x80000000


def tri_boxes(sc, b):
    m = sc.meshes[b]
    n, io, vo = int(m["triCount"]), int(m["indexOffset"]), int(m["vertexOffset"])
    idx = sc.indices[io:io + 3 * n].astype(np.int64) + vo
    p = sc.vertices["position"][idx].reshape(n, 3, 3)
    return np.ascontiguousarray(np.concatenate([p.min(1), p.max(1)], 1), np.float32)


def refit_boxes(bvh, prim_boxes):
    """Node boxes of a BVH2 in the library's layout recomputed bottom-up, level by level, from
    primitive boxes."""
    n = len(bvh["order"])
    leaf = prim_boxes[bvh["order"]]
    kids = np.stack([bvh["left"], bvh["right"]], 1).astype(np.int64)
    is_leaf = (kids & LEAF) != 0
    level = np.full(n - 1, -1)
    level[0] = 0
    frontier = np.array([0])
    while len(frontier):
        c = kids[frontier][~is_leaf[frontier]]
        level[c] = level[frontier[0]] + 1  # a frontier is one level
        frontier = c
    assert (level >= 0).all()
    out = np.zeros((n - 1, 6), np.float32)
    for lv in range(level.max(), -1, -1):
        nodes = np.nonzero(level == lv)[0]
        bx = []
        for j in range(2):
            k = kids[nodes, j]
            lf = is_leaf[nodes, j]
            b = np.where(lf[:, None], leaf[k & ~LEAF], out[np.where(lf, 0, k)])
            bx.append(b)
        out[nodes, :3] = np.minimum(bx[0][:, :3], bx[1][:, :3])
        out[nodes, 3:] = np.maximum(bx[0][:, 3:], bx[1][:, 3:])
    return out


@pytest.fixture(scope="module")
def game(rg, orc):
    sc = S.game_frame_scene()
    rt = rg.Raytracer(sc, flags=rg.RG_FLAG_DEBUG_IMAGES).prepare()  # default flags: SAH BLASes and TLAS
    trees = [rt.ctx.bvh(rt.blas_ids[b]) for b in range(len(sc.meshes))]
    rest = [tri_boxes(sc, b) for b in range(len(sc.meshes))]
    o = orc.OracleScene(sc)
    # three frames of the benchmark's animation (its seed), with refits more frequent than its 5 % so
    # that refit BLASes are certain to be traced
    anim = S.FrameAnimator(sc, seed=101, refit_prob=0.5)
    refit = set()
    for _ in range(3):
        for b, vo, nv in anim.step():
            rt.ctx.update_vertices(vo, sc.vertices[vo:vo + nv])
            rt.ctx.refit_blas(rt.blas_ids[b])
            o.refit(b, sc.vertices[vo:vo + nv], vo)
            refit.add(b)
        rt.setup_top_level_as()
        o.set_instances(sc.instances)
    assert refit
    yield sc, rt, o, trees, rest, sorted(refit)
    rt.ctx.close()


def test_game_frame_blas_trees(orc, game):
    sc, rt, o, trees, rest, refit = game
    for b in range(len(sc.meshes)):
        ref = orc.sah(rest[b])
        assert orc.same_tree(trees[b], ref), f"BLAS {b} ({len(rest[b])} triangles)"
    for b in refit:  # the refit trees: same topology, boxes = unions of the jittered triangles' boxes
        g = rt.ctx.bvh(rt.blas_ids[b])
        for k in ("order", "left", "right"):
            assert np.array_equal(g[k], trees[b][k]), (b, k)
        assert np.array_equal(g["nodeboxes"], refit_boxes(g, tri_boxes(sc, b))), b


def test_game_frame_hits(game):
    sc, rt, o, *_ = game
    rays = np.concatenate([camera_rays(sc, stride=8),  # 32,400 camera rays spread over the frame
                           random_rays(100000, 11, lo=(-80, 0, -80), hi=(80, 16, 80)),
                           random_rays(100000, 12, lo=(-30, 20, -120), hi=(30, 40, -80))])
    assert len(rays) >= 200000
    tg, ig = rt.ctx.trace_rays(rays)
    to, io = o.trace(rays)
    assert np.array_equal(ig, io)
    assert np.array_equal(tg, to)
    assert rt.ctx.stats()["deep_overflows"] == 0
    assert (ig[:, 0] != 0xFFFFFFFF).mean() > 0.2
    # the same rays through the frame loop's traversal kernel (rg_trace_rays_device)
    import torch
    d_rays = torch.from_numpy(rays).cuda()
    d_tuv = torch.full((len(rays), 3), -1.0, device="cuda")
    d_ids = torch.zeros((len(rays), 2), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rt.ctx.trace_rays_device(d_rays.data_ptr(), len(rays), d_tuv.data_ptr(), d_ids.data_ptr())
    rt.ctx.synchronize()
    assert np.array_equal(d_ids.cpu().numpy().view(np.uint32), io)
    assert np.array_equal(d_tuv.cpu().numpy(), to)


def test_game_frame_image(orc, game):
    sc, rt, o, *_ = game
    assert (sc.width, sc.height, int(sc.ubo["numSamples"][0]), int(sc.ubo["maxRecursions"][0])) == (1920, 1080, 4, 5)
    rt.do_raytracing(fxaa=False)  # G-buffers as the trace left them (FXAA writes its output to base)
    st = rt.ctx.stats()
    gb = [rt.ctx.download_image(k) for k in ("base", "normal", "rough")]
    fin = rt.render()
    ob, on, orr, ost = o.render()
    for k in RAY_KEYS:
        assert st[k] == ost[k], (k, st[k], ost[k])
    assert st["deep_overflows"] == 0
    for name, g, r in zip(("base", "normal", "rough"), gb, (ob, on, orr)):
        assert_image_close(g, r, f"game frame {name}")
    assert_image_close(fin, orc.post(sc.ubo, ob, on, orr), "game frame final")


def test_sphere_scene_default_trees(rg, orc):
    sc = S.sphere_scene()
    rt = rg.Raytracer(sc, flags=rg.RG_FLAG_DEBUG_IMAGES).prepare()
    assert orc.same_tree(rt.ctx.bvh(rt.blas_ids[0]), orc.sah(tri_boxes(sc, 0)))
    rt.do_raytracing(fxaa=False)
    st = rt.ctx.stats()
    gb = [rt.ctx.download_image(k) for k in ("base", "normal", "rough")]
    fin = rt.render()
    o = orc.OracleScene(sc)
    ob, on, orr, ost = o.render()
    for k in RAY_KEYS:
        assert st[k] == ost[k], (k, st[k], ost[k])
    for name, g, r in zip(("base", "normal", "rough"), gb, (ob, on, orr)):
        assert_image_close(g, r, f"sphere scene {name}")
    assert_image_close(fin, orc.post(sc.ubo, ob, on, orr), "sphere scene final")
    rt.ctx.close()


def test_batch_workload_subset_vs_oracle(rg, orc):
    """Scenes 2, 7 and 22 of the batched-rendering workload (247k to 1.6M instanced triangles, 1 or
    2 spp, depths 2 to 6) as one batch with the default launch shape."""
    pick = [S.default_batch_scenes()[k] for k in (2, 7, 22)]
    br = rg.BatchRenderer(pick)
    imgs = br.render()
    st = br.ctx.stats()
    total = dict.fromkeys(RAY_KEYS, 0)
    for sc, img in zip(pick, imgs):
        o = orc.OracleScene(sc)
        ob, on, orr, ost = o.render()
        for k in RAY_KEYS:
            total[k] += ost[k]
        assert_image_close(img, orc.post(sc.ubo, ob, on, orr), f"batch {sc.name}")
    for k in RAY_KEYS:
        assert st[k] == total[k], (k, st[k], total[k])
    assert st["deep_overflows"] == 0
    br.ctx.close()
