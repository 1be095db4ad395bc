"""The traversal's 4-wide records (raygun_gb300/csrc/lbvh.cu k_wide_records) and its box tests.

Records are not compared with the oracle (its traversal walks the BVH2 itself); they are checked for
what the traversal relies on:
* structure: the record of BVH2 node i holds i's grandchildren (a leaf child stands in for its own
  slot), empty slots carry ref 0xFFFFFFFE and an inverted box;
* boxes: every slot's box is exactly its child's box (BLAS leaves: the triangle's box; internal
  children: the LBVH node box), for BLASes and the TLAS, also after BLAS refits.
The box tests accept at least what the exact test accepts, so hits equal the brute-force answer: rays
with zero, tiny and huge direction components (the clamped terms of the test), rays along the ground
plane and rays from vertices along an axis (origins on box planes) hit exactly what the oracle hits.
"""
import numpy as np
import pytest

from raygun_gb300 import scenes as S

from test_oracle import camera_rays, degenerate_rays, random_rays

pytestmark = pytest.mark.gpu

LEAF = 0x80000000
EMPTY = 0xFFFFFFFE


def small_two_level():
    return S.instanced_scene(width=96, height=54, counts=(6, 5, 3, 1, 4, 4, 1, 1), hf_n=32, ico_levels=(1, 2, 3, 3),
                             num_samples=2, max_recursions=5, name="mini-game-frame")


@pytest.fixture(scope="module", params=["spheres", "game-frame"])
def scene_pair(request, rg, orc):
    sc = S.sphere_scene() if request.param == "spheres" else small_two_level()
    rt = rg.Raytracer(sc).prepare()
    yield sc, rt, orc.OracleScene(sc)
    rt.ctx.close()


def tri_boxes(sc, b):
    m = sc.meshes[b]
    vo, io, nt = int(m["vertexOffset"]), int(m["indexOffset"]), int(m["triCount"])
    idx = sc.indices[io:io + 3 * nt].astype(np.int64).reshape(-1, 3) + vo
    p = sc.vertices["position"][idx]  # (nt, 3, 3) float32
    return np.concatenate([p.min(1), p.max(1)], 1)


def check_records(rec, bvh, leaf_boxes):
    """leaf_boxes: sorted position -> box (n x 6), or None (TLAS: instance boxes are not checked)."""
    left, right = bvh["left"].astype(np.int64), bvh["right"].astype(np.int64)
    m = len(left)
    assert len(rec) == m
    if m == 0:
        return 0
    # expected refs: grandchildren, leaves standing in for themselves
    exp = np.full((m, 4), EMPTY, np.int64)
    for i in range(m):
        k = 0
        for c in (left[i], right[i]):
            if c & LEAF:
                exp[i, k] = c
                k += 1
            else:
                exp[i, k], exp[i, k + 1] = left[c], right[c]
                k += 2
    got = rec["ref"].astype(np.int64)
    assert np.array_equal(got, exp)
    planes = rec["planes"]  # (m, 6, 4): lo_x, hi_x, lo_y, hi_y, lo_z, hi_z
    lo = planes[:, 0::2, :].transpose(0, 2, 1)  # (m, 4, 3)
    hi = planes[:, 1::2, :].transpose(0, 2, 1)
    empty = got == EMPTY
    assert (lo[empty] == np.inf).all() and (hi[empty] == -np.inf).all()
    internal = ~empty & ((got & LEAF) == 0)
    nb = bvh["nodeboxes"]
    assert np.array_equal(lo[internal], nb[got[internal], :3]) and np.array_equal(hi[internal], nb[got[internal], 3:])
    checked = int(internal.sum())
    if leaf_boxes is not None:
        leaf = ~empty & ((got & LEAF) != 0)
        lb = leaf_boxes[got[leaf] & ~LEAF]
        assert np.array_equal(lo[leaf], lb[:, :3]) and np.array_equal(hi[leaf], lb[:, 3:])
        checked += int(leaf.sum())
    return checked


def test_blas_records(rg, scene_pair):
    sc, rt, o = scene_pair
    checked = 0
    for b in range(len(sc.meshes)):
        bvh = rt.ctx.bvh(b)
        checked += check_records(rt.ctx.bvh_records(b), bvh, tri_boxes(sc, b)[bvh["order"]])
    assert checked > 1000


def half_area(b):
    d = np.maximum(b[..., 3:] - b[..., :3], 0).astype(np.float64)
    return d[..., 0] * d[..., 1] + d[..., 1] * d[..., 2] + d[..., 2] * d[..., 0]


def check_bvh2(bvh):
    """A BVH2 in the LBVH layout: every primitive in one leaf, every internal node reached once from
    the root, each internal node's box enclosing its internal children's boxes."""
    n = len(bvh["order"])
    assert sorted(bvh["order"].tolist()) == list(range(n))
    left, right, nb = bvh["left"].astype(np.int64), bvh["right"].astype(np.int64), bvh["nodeboxes"]
    seen_nodes, seen_leaves, st = set(), set(), [0]
    while st:
        i = st.pop()
        assert i not in seen_nodes
        seen_nodes.add(i)
        for c in (left[i], right[i]):
            if c & LEAF:
                assert (c & ~LEAF) not in seen_leaves
                seen_leaves.add(c & ~LEAF)
            else:
                assert (nb[i, :3] <= nb[c, :3]).all() and (nb[i, 3:] >= nb[c, 3:]).all()
                st.append(int(c))
    assert len(seen_nodes) == n - 1 and len(seen_leaves) == n


def test_sah_tlas(rg, orc):
    """The default TLAS (binned SAH) is a valid BVH2 over all instances with a lower surface-area cost
    than the LBVH over the same instances, and both trace the same hits."""
    sc = S.instanced_scene(width=96, height=54, num_samples=1, max_recursions=2, name="game-frame-instances")
    rt = rg.Raytracer(sc).prepare()
    rl = rg.Raytracer(sc, flags=rg.RG_FLAG_TLAS_LBVH).prepare()
    sah, lb = rt.ctx.bvh(-1), rl.ctx.bvh(-1)
    assert len(sah["order"]) == len(sc.instances) > 1000
    check_bvh2(sah)
    check_records(rt.ctx.bvh_records(-1), sah, None)
    cost = lambda b: half_area(b["nodeboxes"]).sum() / half_area(b["nodeboxes"][0])
    assert cost(sah) < 0.9 * cost(lb), (cost(sah), cost(lb))
    rays = np.concatenate([camera_rays(sc), random_rays(20000, 9, lo=(-60, 0, -60), hi=(60, 14, 60))])
    tg, ig = rt.ctx.trace_rays(rays)
    tl, il = rl.ctx.trace_rays(rays)
    to, io = orc.OracleScene(sc).trace(rays)
    assert np.array_equal(ig, io) and np.array_equal(tg, to)
    assert np.array_equal(il, io) and np.array_equal(tl, to)
    rt.ctx.close()
    rl.ctx.close()


def test_tlas_records(rg, scene_pair):
    sc, rt, o = scene_pair
    check_records(rt.ctx.bvh_records(-1), rt.ctx.bvh(-1), None)


def test_closest_hit_degenerate_directions(rg, scene_pair):
    sc, rt, o = scene_pair
    rays = np.concatenate([degenerate_rays(sc, 12000, 7), camera_rays(sc, stride=4)])
    tg, ig = rt.ctx.trace_rays(rays)
    to, io = o.trace(rays)
    assert np.array_equal(ig, io)
    assert np.array_equal(tg, to)
    assert (ig[:12000, 0] != 0xFFFFFFFF).sum() > 100


@pytest.mark.parametrize("n", [1, 33, None])
def test_device_query_degenerate_and_ragged(rg, scene_pair, n):
    """rg_trace_rays_device (the traversal kernel's query form: rays read and hits written in the
    caller's buffers) on degenerate directions, zero directions and ragged counts (one ray, a partial
    warp, every ray) gives the oracle's hits bit for bit, misses as zeros and 0xFFFFFFFF."""
    import torch
    sc, rt, o = scene_pair
    rays = np.concatenate([degenerate_rays(sc, 6000, 17), camera_rays(sc, stride=4)])
    rays = np.concatenate([rays, rays[:7] * np.array([1, 1, 1, 1, 0, 0, 0, 1], np.float32)])  # zero directions
    rays = np.ascontiguousarray(rays[::-1] if n is None else rays[-n:], np.float32)
    to, io = o.trace(rays)
    d_rays = torch.from_numpy(rays).cuda()
    d_tuv = torch.full((len(rays), 3), -1.0, device="cuda")
    d_ids = torch.zeros((len(rays), 2), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rt.ctx.trace_rays_device(d_rays.data_ptr(), len(rays), d_tuv.data_ptr(), d_ids.data_ptr())
    rt.ctx.synchronize()
    ig, tg = d_ids.cpu().numpy().view(np.uint32), d_tuv.cpu().numpy()
    assert np.array_equal(ig, io) and np.array_equal(tg, to)
    assert (ig[-1 if n else 0, 0] == 0xFFFFFFFF) and (tg[-1 if n else 0] == 0).all()  # a zero direction misses
    if n is None:
        assert (ig[:, 0] != 0xFFFFFFFF).sum() > 100


def test_records_follow_refit(rg, orc):
    """After BLAS refits and a TLAS rebuild the records carry the moved boxes, and hits still match
    the oracle."""
    sc = small_two_level()
    rt = rg.Raytracer(sc).prepare()
    o = orc.OracleScene(sc)
    anim = S.FrameAnimator(sc, seed=11, refit_prob=1.0)
    refits = anim.step()
    assert refits
    for b, vo, nv in refits:
        rt.ctx.update_vertices(vo, sc.vertices[vo:vo + nv])
        rt.ctx.refit_blas(rt.blas_ids[b])
        o.refit(b, sc.vertices[vo:vo + nv], vo)
    rt.setup_top_level_as()
    o.set_instances(sc.instances)
    for b, _, _ in refits:
        bvh = rt.ctx.bvh(b)
        check_records(rt.ctx.bvh_records(b), bvh, tri_boxes(sc, b)[bvh["order"]])
    rays = np.concatenate([camera_rays(sc), random_rays(5000, 8, lo=(-60, 0, -60), hi=(60, 14, 60))])
    tg, ig = rt.ctx.trace_rays(rays)
    to, io = o.trace(rays)
    assert np.array_equal(ig, io) and np.array_equal(tg, to)
    rt.ctx.close()


def test_sah_blas(rg, orc):
    """The default BLASes (binned SAH) are valid BVH2s with a lower surface-area cost than the LBVHs
    over the same triangles, their records hold the exact boxes, they follow refits, and they trace
    the oracle's hits."""
    sc = small_two_level()
    rt = rg.Raytracer(sc).prepare()
    rl = rg.Raytracer(sc, flags=rg.RG_FLAG_BLAS_LBVH).prepare()
    cost = lambda b: half_area(b["nodeboxes"]).sum() / half_area(b["nodeboxes"][0])
    tot_sah = tot_lbvh = 0.0
    for b in range(len(sc.meshes)):
        sah, lb = rt.ctx.bvh(b), rl.ctx.bvh(b)
        if len(sah["order"]) < 2:
            continue
        check_bvh2(sah)
        check_records(rt.ctx.bvh_records(b), sah, tri_boxes(sc, b)[sah["order"]])
        tot_sah += cost(sah)
        tot_lbvh += cost(lb)
    assert tot_sah < 0.97 * tot_lbvh, (tot_sah, tot_lbvh)
    o = orc.OracleScene(sc)
    rays = np.concatenate([camera_rays(sc), random_rays(20000, 12, lo=(-60, 0, -60), hi=(60, 14, 60)),
                           degenerate_rays(sc, 4000, 13)])
    tg, ig = rt.ctx.trace_rays(rays)
    to, io = o.trace(rays)
    assert np.array_equal(ig, io) and np.array_equal(tg, to)
    # refit of the SAH topology: records carry the moved boxes and hits still match
    anim = S.FrameAnimator(sc, seed=5, refit_prob=1.0)
    refits = anim.step()
    for b, vo, nv in refits:
        rt.ctx.update_vertices(vo, sc.vertices[vo:vo + nv])
        rt.ctx.refit_blas(rt.blas_ids[b])
        o.refit(b, sc.vertices[vo:vo + nv], vo)
    rt.setup_top_level_as()
    o.set_instances(sc.instances)
    for b, _, _ in refits:
        bvh = rt.ctx.bvh(b)
        if len(bvh["order"]) > 1:
            check_bvh2(bvh)
            check_records(rt.ctx.bvh_records(b), bvh, tri_boxes(sc, b)[bvh["order"]])
    tg, ig = rt.ctx.trace_rays(rays)
    to, io = o.trace(rays)
    assert np.array_equal(ig, io) and np.array_equal(tg, to)
    rt.ctx.close()
    rl.ctx.close()


def test_sah_blas_matches_oracle(rg, orc):
    """The default BLASes are the oracle's binned-SAH trees (oracle/rg_oracle.cpp sah_build): the same
    leaf order, structure and node boxes, up to the numbering of a level's nodes."""
    for sc in (small_two_level(), S.sphere_scene()):
        rt = rg.Raytracer(sc).prepare()
        compared = 0
        for b in range(len(sc.meshes)):
            boxes = tri_boxes(sc, b)
            if len(boxes) < 2:
                continue
            ref = orc.sah(boxes)
            assert orc.same_tree(rt.ctx.bvh(b), ref), b
            compared += 1
        assert compared >= 1
        rt.ctx.close()


def triangle_soup(n, seed):
    """n random triangles (side lengths up to ~2) scattered in a 100-unit cube, one mesh."""
    rng = np.random.RandomState(seed)
    c = rng.uniform(-50.0, 50.0, (n, 1, 3))
    pos = (c + rng.uniform(-1.0, 1.0, (n, 3, 3))).reshape(-1, 3)
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    mesh = S.Mesh(pos, np.tile((0.0, 1.0, 0.0), (3 * n, 1)), idx)
    mats = S.random_materials(S.Rng(seed), 1)
    ubo = S.make_ubo((0.0, 0.0, -120.0), (0.0, 0.0, 0.0), 60.0, 32, 18, (-0.4, -1.0, 0.3), 1, 2)
    return S._finish("soup", [(mesh, np.zeros(len(pos), np.uint32))], mats, S.identity_instance(), ubo, 32, 18)


@pytest.mark.parametrize("n", [32767, 32768, 100003])
def test_sah_blas_at_the_split_threshold(rg, orc, n):
    """Builds just below and at the size from which the first levels split each task over many CTAs
    (and a ragged larger one) give the oracle's binned-SAH tree."""
    sc = triangle_soup(n, 17 + n)
    rt = rg.Raytracer(sc).prepare()
    assert orc.same_tree(rt.ctx.bvh(0), orc.sah(tri_boxes(sc, 0)))
    rt.ctx.close()


def test_sah_task_wait_that_gives_up_is_reported(rg, monkeypatch):
    """Every wait of the SAH task kernel is bounded.  With the bound at zero polls
    (RG_SAH_WAIT_LIMIT=0) a warp that claims a slot whose task is not published yet gives up at
    once: that part of the tree stays as prepared (in-range refs only), and the context reports it
    at the next rg_synchronize as RG_ERR_CUDA naming the builder.  Nothing faults, and a refit of
    the unfinished tree stays in range."""
    monkeypatch.setenv("RG_SAH_WAIT_LIMIT", "0")
    sc = triangle_soup(100003, 5)
    rt = rg.Raytracer(sc)
    rt.setup_model_buffers()
    rt.setup_bottom_level_as()
    rt.ctx.refit_blas(rt.blas_ids[0])
    with pytest.raises(rg.RgError) as e:
        rt.ctx.synchronize()
    assert e.value.code == -2 and "SAH" in str(e.value), str(e.value)
    rt.ctx.close()
