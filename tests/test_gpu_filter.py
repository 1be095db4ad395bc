"""The learned roughness filter (rg_filter_*, raygun_gb300/csrc/filter.cu) and the glossy reference
shading that makes its training targets.

The filter is a floating-point kernel chain, so its reference is a plain PyTorch FP32 evaluation of
the same network with the same BF16 roundings (weights, stored activations, the skip sum):
* forward: |GPU - reference| <= 2e-2 * max|reference| + 1e-3 on every output, on a batch whose
  image size is not a multiple of the kernel's 2 x 128 tile;
* gradients (lr = 0): per layer cosine >= 0.99 and relative norm error <= 5 % against autograd on the
  reference with straight-through roundings (the GPU also rounds gradients to BF16 between layers);
* training: the loss of a synthetic regression falls below a quarter of its start;
* in the frame: RG_IMAGE_FILTER_OUT equals the forward pass on the frame's own filter input;
* glossy shading: seed 0 renders bit-identical frames; a scene without roughness renders identically
  with any seed; rough materials change only where they are.
"""
import numpy as np
import pytest

from raygun_gb300 import scenes as S

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
F = torch.nn.functional


def bf(x):
    return x.to(torch.bfloat16).to(torch.float32)


def st_round(x):  # BF16 rounding in the forward pass, identity in the backward pass
    return x + (bf(x) - x).detach()


def ref_forward(rg, params, x16, rounding=bf):
    layers = [(torch.tensor(w), torch.tensor(b)) for w, b in rg.filter_layers(params)]
    x = x16[..., :12].permute(0, 3, 1, 2)
    conv = lambda t, wb: F.conv2d(t, bf(wb[0]), wb[1], padding=1)
    y1 = rounding(F.relu(conv(x, layers[0])))
    y2 = rounding(F.relu(conv(y1, layers[1])))
    y3 = rounding(F.relu(conv(y2, layers[2])))
    y4 = rounding(F.relu(conv(y3, layers[3])))
    x5 = rounding(y4 + y1)
    return conv(x5, layers[4]).permute(0, 2, 3, 1)


def random_input(B, H, W, seed):
    g = torch.Generator().manual_seed(seed)
    x = torch.zeros(B, H, W, 16)
    x[..., :12] = torch.rand(B, H, W, 12, generator=g) * 2 - 1
    return bf(x)


@pytest.fixture(scope="module")
def ctx(rg):
    return rg.Context()


def test_forward_matches_reference(rg, ctx):
    flt = rg.Filter(ctx, seed=3)
    params = flt.params()
    B, H, W = 2, 5, 150
    x = random_input(B, H, W, 1)
    d_in = x.to(torch.bfloat16).cuda()
    d_out = torch.zeros(B, H, W, 4, device="cuda")
    torch.cuda.synchronize()
    flt.forward(d_in.data_ptr(), B, H, W, d_out.data_ptr())
    got = d_out.cpu()[..., :3]
    ref = ref_forward(rg, params, x)
    err = (got - ref).abs()
    assert float(err.max()) <= 2e-2 * float(ref.abs().max()) + 1e-3, float(err.max())
    assert float(err.mean()) <= 2e-3 * float(ref.abs().mean()) + 1e-4


@pytest.mark.parametrize("B,H,W", [(1, 1080, 1920), (1, 1079, 1917), (2, 361, 643)])
def test_forward_matches_reference_full_size(rg, ctx, B, H, W):
    """Forward at the frame size the filter runs at (one 1080p frame), and at shapes whose row count
    is not a multiple of the kernel's 3-row groups and whose width leaves a partial 128-pixel strip,
    so every CTA walks several row segments and strips and crosses their seams.  Reference: the FP32
    PyTorch evaluation of the same network with the same BF16 roundings, run on the GPU with TF32
    off.  Bars: max |GPU - ref| <= 2e-2 * max|ref| + 1e-3 and mean <= 2e-3 * mean|ref| + 1e-4 (BF16
    activations can differ by one ulp where the FP32 sums round to different sides)."""
    flt = rg.Filter(ctx, seed=11)
    params = flt.params()
    x = random_input(B, H, W, 7)
    d_in = x.to(torch.bfloat16).cuda()
    d_out = torch.zeros(B, H, W, 4, device="cuda")
    torch.cuda.synchronize()
    flt.forward(d_in.data_ptr(), B, H, W, d_out.data_ptr())
    got = d_out[..., :3]
    tf32 = (torch.backends.cuda.matmul.allow_tf32, torch.backends.cudnn.allow_tf32)
    torch.backends.cuda.matmul.allow_tf32 = torch.backends.cudnn.allow_tf32 = False
    try:
        layers = [(torch.tensor(w).cuda(), torch.tensor(b).cuda()) for w, b in rg.filter_layers(params)]
        xx = x.cuda()[..., :12].permute(0, 3, 1, 2)
        conv = lambda t, wb: F.conv2d(t, bf(wb[0]), wb[1], padding=1)
        y1 = bf(F.relu(conv(xx, layers[0])))
        y2 = bf(F.relu(conv(y1, layers[1])))
        y3 = bf(F.relu(conv(y2, layers[2])))
        y4 = bf(F.relu(conv(y3, layers[3])))
        ref = conv(bf(y4 + y1), layers[4]).permute(0, 2, 3, 1)
    finally:
        torch.backends.cuda.matmul.allow_tf32, torch.backends.cudnn.allow_tf32 = tf32
    err = (got - ref).abs()
    emax, emean = float(err.max()), float(err.mean())
    rmax, rmean = float(ref.abs().max()), float(ref.abs().mean())
    print(f"{B}x{H}x{W}: max err {emax:.3g} (bar {2e-2 * rmax + 1e-3:.3g}), mean err {emean:.3g} "
          f"(bar {2e-3 * rmean + 1e-4:.3g}), exact {float((err == 0).float().mean()):.4f}")
    assert emax <= 2e-2 * rmax + 1e-3
    assert emean <= 2e-3 * rmean + 1e-4


def test_gradients_match_autograd(rg, ctx):
    flt = rg.Filter(ctx, seed=5)
    params = flt.params()
    B, H, W = 2, 6, 130
    x = random_input(B, H, W, 2)
    g = torch.Generator().manual_seed(9)
    target = torch.zeros(B, H, W, 4)
    target[..., :3] = torch.rand(B, H, W, 3, generator=g)
    d_in, d_t = x.to(torch.bfloat16).cuda(), target.cuda()
    torch.cuda.synchronize()
    loss_gpu = flt.train_step(d_in.data_ptr(), d_t.data_ptr(), B, H, W, 0.0)
    grads = flt.grads()
    p = torch.tensor(params, requires_grad=True)
    layers, off = [], 0
    for co, ci in rg.FILTER_LAYERS:
        w = p[off:off + co * ci * 9].view(co, ci, 3, 3)
        off += co * ci * 9
        b = p[off:off + co]
        off += co
        layers.append((w, b))
    xx = x[..., :12].permute(0, 3, 1, 2)
    conv = lambda t, wb: F.conv2d(t, st_round(wb[0]), wb[1], padding=1)
    y1 = st_round(F.relu(conv(xx, layers[0])))
    y2 = st_round(F.relu(conv(y1, layers[1])))
    y3 = st_round(F.relu(conv(y2, layers[2])))
    y4 = st_round(F.relu(conv(y3, layers[3])))
    out = conv(st_round(y4 + y1), layers[4]).permute(0, 2, 3, 1)
    loss = ((out - target[..., :3]) ** 2).mean()
    loss.backward()
    assert abs(loss_gpu - float(loss.detach())) <= 2e-2 * float(loss.detach())
    ref = p.grad.numpy()
    off = 0
    for k, (co, ci) in enumerate(rg.FILTER_LAYERS):
        n = co * ci * 9 + co
        a, r = grads[off:off + n].astype(np.float64), ref[off:off + n].astype(np.float64)
        off += n
        cos = a @ r / (np.linalg.norm(a) * np.linalg.norm(r) + 1e-30)
        rel = abs(np.linalg.norm(a) - np.linalg.norm(r)) / np.linalg.norm(r)
        assert cos >= 0.99 and rel <= 0.05, (k, cos, rel)


def test_training_reduces_loss(rg, ctx):
    flt = rg.Filter(ctx, seed=11)
    B, H, W = 4, 64, 64
    x = random_input(B, H, W, 4)
    # a smooth target the network can fit: a blurred mix of input channels
    mix = torch.tensor([[0.5, 0.1, 0.0], [0.0, 0.4, 0.2], [0.2, 0.0, 0.5]])
    t = torch.einsum("bhwc,cd->bhwd", x[..., :3], mix) + 0.3 * x[..., 8:11]
    t = F.avg_pool2d(t.permute(0, 3, 1, 2), 3, stride=1, padding=1).permute(0, 2, 3, 1)
    target = torch.zeros(B, H, W, 4)
    target[..., :3] = t
    d_in, d_t = x.to(torch.bfloat16).cuda(), target.cuda()
    torch.cuda.synchronize()
    first = flt.train_step(d_in.data_ptr(), d_t.data_ptr(), B, H, W, 1e-3)
    last = first
    for _ in range(300):
        last = flt.train_step(d_in.data_ptr(), d_t.data_ptr(), B, H, W, 1e-3)
    assert last < 0.25 * first, (first, last)


def test_filter_in_the_frame(rg):
    sc = S.spheres_scene(n_spheres=12, width=160, height=90, num_samples=2, max_recursions=3, seed=4)
    rt = rg.Raytracer(sc).prepare()
    ctx = rt.ctx
    flt = rg.Filter(ctx, seed=2)
    ctx.set_filter(flt)
    fin = rt.render()
    assert np.isfinite(fin).all()
    pred = ctx.download_image("filter_out")
    d_in = torch.zeros(sc.height, sc.width, 16, dtype=torch.bfloat16, device="cuda")
    ctx.filter_input(d_in.data_ptr())
    ctx.synchronize()
    d_out = torch.zeros(sc.height, sc.width, 4, device="cuda")
    flt.forward(d_in.data_ptr(), 1, sc.height, sc.width, d_out.data_ptr())
    assert np.array_equal(pred[..., :3], d_out.cpu().numpy()[..., :3])
    ctx.set_filter(None)
    plain = rt.render()
    assert not np.array_equal(plain, fin)


def test_glossy_shading(rg):
    base = S.spheres_scene(n_spheres=16, width=96, height=54, num_samples=2, max_recursions=3, seed=6)
    smooth = S.Scene(base.name, base.vertices, base.indices, base.materials.copy(), base.meshes, base.instances, base.ubo,
                     base.width, base.height)
    smooth.materials["roughness"] = 0.0
    for sc, rough in ((base, True), (smooth, False)):
        rt = rg.Raytracer(sc).prepare()
        rt.do_raytracing(fxaa=False)
        mirror = rt.ctx.download_image("rough")
        rt.ctx.set_glossy(0)
        rt.do_raytracing(fxaa=False)
        assert np.array_equal(rt.ctx.download_image("rough"), mirror)
        rt.ctx.set_glossy(1234)
        rt.do_raytracing(fxaa=False)
        glossy = rt.ctx.download_image("rough")
        assert np.isfinite(glossy).all()
        assert np.array_equal(glossy, mirror) != rough
        rt.ctx.close()


def test_trained_weights_beat_the_plain_passes(rg):
    """The committed weights (trained by bench.py --workload filter) on a scene they never saw: the
    prediction is closer to the 256-spp glossy reference than the plain roughness approximation."""
    import torch
    from raygun_gb300 import filter_train as FT
    W, H = 320, 180
    sc = FT.training_scene(123456, W, H)
    ctx = rg.Context(flags=rg.RG_FLAG_DEBUG_IMAGES)
    flt = rg.Filter(ctx)
    FT.load_weights(flt)
    d_in = torch.zeros(H, W, 16, dtype=torch.bfloat16, device="cuda")
    d_t = torch.zeros(H, W, 4, device="cuda")
    FT.render_pair(ctx, sc, d_in, d_t, seed=7)
    target = d_t.cpu().numpy()
    slot = ctx.scene_create()
    ctx.scene_select(slot)
    rg.load_scene(ctx, sc)
    ctx.render(sc.ubo, False)
    plain = ctx.download_image("rough_colors_a")
    ctx.set_filter(flt)
    ctx.render(sc.ubo, False)
    learned = ctx.download_image("filter_out")
    p_plain, p_learned = FT.psnr(plain[..., :3], target[..., :3]), FT.psnr(learned[..., :3], target[..., :3])
    assert p_learned > p_plain + 2.0, (p_plain, p_learned)
