"""CPU tests of the oracle itself: LBVH invariants, Morton codes against an independent numpy
evaluation, traversal against brute force, FP16 rounding, policies."""
import numpy as np
import pytest

from raygun_gb300 import scenes as S


def _expand10(v):
    v = v.astype(np.uint64)
    v = (v * 0x00010001) & 0xFF0000FF
    v = (v * 0x00000101) & 0x0F00F00F
    v = (v * 0x00000011) & 0xC30C30C3
    v = (v * 0x00000005) & 0x49249249
    return v.astype(np.uint32)


def numpy_morton(boxes):
    """Independent float32 evaluation of the Morton codes (same operation order)."""
    b = boxes.astype(np.float32)
    c = (b[:, :3] + b[:, 3:]) * np.float32(0.5)
    lo, hi = c.min(0), c.max(0)
    emax = np.float32((hi - lo).max())
    inv = np.float32(1.0) / emax if emax > 0 else np.float32(0.0)
    q = ((c - lo) * inv) * np.float32(1024.0)
    q = np.clip(q, np.float32(0), np.float32(1023)).astype(np.uint32)
    return (_expand10(q[:, 0]) << 2) | (_expand10(q[:, 1]) << 1) | _expand10(q[:, 2])


def random_boxes(n, seed, dup=False):
    rng = np.random.RandomState(seed)
    c = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    if dup:
        c[: n // 2] = c[0]
    e = rng.uniform(0.01, 0.5, (n, 3)).astype(np.float32)
    return np.concatenate([c - e, c + e], 1).astype(np.float32)


def check_topology(n, left, right, order):
    """Every leaf reached exactly once from the root; every internal node once."""
    if n == 1:
        return
    seen_leaf = np.zeros(n, int)
    seen_node = np.zeros(n - 1, int)
    stack = [0]
    while stack:
        i = stack.pop()
        seen_node[i] += 1
        for c in (left[i], right[i]):
            if c & 0x80000000:
                seen_leaf[c & 0x7FFFFFFF] += 1
            else:
                stack.append(int(c))
    assert (seen_leaf == 1).all() and (seen_node == 1).all()
    assert np.array_equal(np.sort(order), np.arange(n))


@pytest.mark.parametrize("n,dup", [(1, False), (2, False), (3, False), (17, False), (1000, False), (5000, True)])
def test_lbvh_oracle(orc, n, dup):
    boxes = random_boxes(n, n, dup)
    r = orc.lbvh(boxes)
    assert np.array_equal(r["morton"], numpy_morton(boxes))
    assert np.array_equal(r["order"], np.argsort(r["morton"], kind="stable"))
    check_topology(n, r["left"], r["right"], r["order"])
    if n > 1:
        nb = r["nodeboxes"]
        sorted_boxes = boxes[r["order"]]
        for i in range(n - 1):
            for c in (r["left"][i], r["right"][i]):
                cb = sorted_boxes[c & 0x7FFFFFFF] if c & 0x80000000 else nb[c]
                assert (nb[i, :3] <= cb[:3]).all() and (nb[i, 3:] >= cb[3:]).all()
        assert np.array_equal(nb[0, :3], boxes[:, :3].min(0)) and np.array_equal(nb[0, 3:], boxes[:, 3:].max(0))


def camera_rays(scene, stride=1):
    """Primary rays of the raygen (1 spp), float32, built in numpy."""
    u = scene.ubo[0]
    vi = u["viewInverse"].astype(np.float32)  # [col][row]
    pi = u["projInverse"].astype(np.float32)
    W, H = scene.width, scene.height
    ys, xs = np.mgrid[0:H:stride, 0:W:stride]
    px = (xs.astype(np.float32) + np.float32(0.5)) / np.float32(W)
    py = (ys.astype(np.float32) + np.float32(0.5)) / np.float32(H)
    d = np.stack([px * 2 - 1, py * 2 - 1, np.ones_like(px), np.ones_like(px)], -1).reshape(-1, 4).astype(np.float32)
    tg = d @ pi  # column-major: result_r = sum_c m[c][r] v_c
    t3 = tg[:, :3] / np.linalg.norm(tg[:, :3], axis=1, keepdims=True)
    dirs = t3 @ vi[:3, :3]
    o = np.broadcast_to(vi[3, :3], dirs.shape)
    rays = np.zeros((len(dirs), 8), np.float32)
    rays[:, :3], rays[:, 3], rays[:, 4:7], rays[:, 7] = o, 0.001, dirs, 10000.0
    return rays


def random_rays(n, seed, lo=(-12, 0.2, -12), hi=(12, 8, 12)):
    rng = np.random.RandomState(seed)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3], rays[:, 3], rays[:, 4:7], rays[:, 7] = o, 0.01, d, 1000.0
    return rays


def degenerate_rays(sc, n, seed):
    """Rays with zero, tiny (1e-30) and huge components, rays in the ground plane, rays from box planes."""
    rng = np.random.RandomState(seed)
    V = sc.vertices["position"]
    lo, hi = V.min(0), V.max(0)
    o = rng.uniform(lo - 2, hi + 2, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    kind = rng.randint(0, 6, n)
    for i in range(n):
        axes = rng.permutation(3)
        if kind[i] == 0:  # axis-parallel
            d[i, axes[1:]] = 0.0
        elif kind[i] == 1:  # in a coordinate plane
            d[i, axes[0]] = 0.0
        elif kind[i] == 2:  # tiny components
            d[i, axes[0]] = np.float32(1e-30) * np.sign(d[i, axes[0]] + 0.5)
            d[i, axes[1]] = np.float32(-3e-25)
        elif kind[i] == 3:  # huge direction (tiny 1/d)
            d[i] *= np.float32(1e25)
        elif kind[i] == 4:  # horizontal, starting on y = 0 (the ground plane of the scenes)
            o[i, 1] = 0.0
            d[i, 1] = 0.0
        else:  # from a vertex, along an axis
            o[i] = V[rng.randint(len(V))]
            d[i] = 0.0
            d[i, axes[0]] = 1.0 if rng.rand() < 0.5 else -1.0
    rays = np.zeros((n, 8), np.float32)
    rays[:, :3], rays[:, 3], rays[:, 4:7], rays[:, 7] = o, 0.0, d, 1e4
    rays[kind == 3, 7] = 1e-20  # t is scaled by |d|
    return rays


def test_traversal_matches_brute_force(orc):
    sc = S.spheres_scene(n_spheres=12, width=64, height=36, slices=16, stacks=8)
    o = orc.OracleScene(sc)
    rays = np.concatenate([camera_rays(sc), random_rays(3000, 1)])
    f1, i1 = o.trace(rays)
    f2, i2 = o.trace(rays, brute=True)
    assert np.array_equal(i1, i2)
    assert np.array_equal(f1, f2)
    assert (i1[:, 0] != 0xFFFFFFFF).mean() > 0.3


def test_traversal_two_level_matches_brute_force(orc):
    sc = S.instanced_scene(width=64, height=36, counts=(6, 5, 3, 0, 4, 4, 1, 1), hf_n=24, ico_levels=(1, 2, 2, 3))
    o = orc.OracleScene(sc)
    rays = random_rays(3000, 2, lo=(-60, 0, -60), hi=(60, 14, 60))
    f1, i1 = o.trace(rays)
    f2, i2 = o.trace(rays, brute=True)
    assert np.array_equal(i1, i2) and np.array_equal(f1, f2)
    assert (i1[:, 0] != 0xFFFFFFFF).sum() > 50


@pytest.mark.parametrize("which", ["spheres", "two-level"])
def test_traversal_degenerate_directions_match_brute_force(orc, which):
    """Zero, tiny and huge direction components, rays in the ground plane and rays from vertices along
    an axis (origins on box planes): the BVH walk finds what the brute force finds."""
    if which == "spheres":
        sc = S.spheres_scene(n_spheres=12, width=64, height=36, slices=16, stacks=8)
    else:
        sc = S.instanced_scene(width=64, height=36, counts=(6, 5, 3, 0, 4, 4, 1, 1), hf_n=24, ico_levels=(1, 2, 2, 3))
    o = orc.OracleScene(sc)
    rays = degenerate_rays(sc, 3000, 5)
    f1, i1 = o.trace(rays)
    f2, i2 = o.trace(rays, brute=True)
    assert np.array_equal(i1, i2) and np.array_equal(f1, f2)
    assert (i1[:, 0] != 0xFFFFFFFF).sum() > 100


def test_half_rounding(orc):
    x = np.concatenate([np.random.RandomState(0).randn(200000).astype(np.float32) * 30,
                        np.array([65504, 65520, 65519.9, 1e-8, -1e-8, 6e-5, 6.1e-5, 2.98e-8, np.inf, -np.inf], np.float32)])
    assert np.array_equal(orc.round_half(x), x.astype(np.float16).astype(np.float32))


def test_render_small_scene_finite(orc):
    sc = S.spheres_scene(n_spheres=8, width=48, height=27, slices=16, stacks=8)
    o = orc.OracleScene(sc)
    b, n, r, st = o.render(nthreads=2)
    assert np.isfinite(b).all() and np.isfinite(n).all() and np.isfinite(r).all()
    assert st["primary"] == 48 * 27
    fin = orc.post(sc.ubo, b, n, r)
    assert np.isfinite(fin).all() and (fin[..., :3] >= 0).all() and (fin[..., :3] <= 1).all()


def test_render_fp64_close_to_fp32(orc):
    sc = S.spheres_scene(n_spheres=8, width=48, height=27, slices=16, stacks=8)
    o = orc.OracleScene(sc)
    b32 = o.render(nthreads=2)[0]
    b64 = o.render(nthreads=2, fp64=True)[0]
    err = np.abs(b32[..., :3] - b64[..., :3])
    assert np.quantile(err, 0.99) < 2 / 255


def test_show_alpha_and_fade(orc):
    sc = S.spheres_scene(n_spheres=4, width=32, height=18, slices=12, stacks=6)
    o = orc.OracleScene(sc)
    b, n, r, _ = o.render(nthreads=1)
    u = sc.ubo.copy()
    u["showAlpha"] = 1
    fin = orc.post(u, b, n, r, fxaa=False)
    assert np.allclose(fin[..., 0], fin[..., 3]) and np.allclose(fin[..., 1], fin[..., 3])
    u = sc.ubo.copy()
    u["fadeColor"] = (1.0, 0.0, 0.0, 1.0)
    fin = orc.post(u, b, n, r, fxaa=False)
    assert np.allclose(fin[..., :3], [1.0, 0.0, 0.0])


def _check_bvh2(t, boxes):
    """A BVH2 in the LBVH layout: every primitive in one leaf, every internal node reached once, each
    node box the exact union of its children's boxes."""
    n = len(t["order"])
    assert sorted(t["order"].tolist()) == list(range(n))
    if n < 2:
        return
    L, R, nb = t["left"].astype(np.int64), t["right"].astype(np.int64), t["nodeboxes"]
    leaf_box = lambda c: boxes[t["order"][c & ~0x80000000]]
    seen, leaves, st = set(), set(), [0]
    while st:
        i = st.pop()
        assert i not in seen
        seen.add(i)
        kids = []
        for c in (L[i], R[i]):
            if c & 0x80000000:
                leaves.add(int(c & ~0x80000000))
                kids.append(leaf_box(c))
            else:
                st.append(int(c))
                kids.append(nb[c])
        u = np.concatenate([np.minimum(kids[0][:3], kids[1][:3]), np.maximum(kids[0][3:], kids[1][3:])])
        assert np.array_equal(nb[i], u)
    assert len(seen) == n - 1 and len(leaves) == n


def test_oracle_sah_tree(orc):
    """The oracle's binned-SAH builder (the CUDA library's default BLAS/TLAS builder restated): valid
    BVH2s with exact node boxes, a lower surface-area cost than the LBVH over the same boxes, and the
    depth bound of halving ranges from a fixed level on."""
    def half(b):
        d = np.maximum(b[..., 3:] - b[..., :3], 0).astype(np.float64)
        return d[..., 0] * d[..., 1] + d[..., 1] * d[..., 2] + d[..., 2] * d[..., 0]
    for n, dup in ((1, False), (2, False), (3, False), (257, False), (4000, True), (20000, False)):
        boxes = random_boxes(n, 100 + n, dup)
        t = orc.sah(boxes)
        _check_bvh2(t, boxes)
        assert orc.same_tree(t, orc.sah(boxes))  # deterministic
        if n >= 257:
            lb = orc.lbvh(boxes)
            cost = lambda b: half(b["nodeboxes"]).sum() / half(b["nodeboxes"][0])
            assert cost(t) < cost(lb), (n, cost(t), cost(lb))
    # small triangles at x = 17^k: every split takes one off the far end -> n - 1 levels, unless ranges
    # are halved from a lower level on: then at most that level + ceil(log2(what remains)) levels
    n = 30
    x = (17.0 ** np.arange(n)).astype(np.float32)
    boxes = np.zeros((n, 6), np.float32)
    boxes[:, 0], boxes[:, 3] = x, x
    boxes[:, 4], boxes[:, 5] = 0.5, 0.5
    assert orc.sah(boxes)["levels"] == n - 1
    for m in (0, 5, 10, 20):
        t = orc.sah(boxes, m)
        _check_bvh2(t, boxes)
        assert t["levels"] <= m + int(np.ceil(np.log2(n - m))), (m, t["levels"])
        assert orc.same_tree(t, orc.sah(boxes, m))
    assert orc.sah(boxes, 28)["levels"] == 29  # one more split peels the last two apart
