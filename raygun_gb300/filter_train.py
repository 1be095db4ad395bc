"""Training and evaluation of the learned roughness filter (rg_filter_*).

Data, all rendered by the tracer itself:
  scenes   game-frame-type scenes (1024 instances of the eight procedural meshes, seeded) whose
           material roughness is redrawn uniform in [0, 1], each seen from a seeded camera;
  input    the 16-channel filter input of a 1-spp frame (rg_filter_input);
  target   the rough RGB of a 256-spp frame with glossy reference shading (rg_set_glossy): eight
           32-spp frames with different seeds, averaged (a frame takes at most 32 samples).
Training: random 128 x 128 crops, Adam (lr 1e-3), mean squared error on the RGB.
Evaluation: held-out scenes at 1920 x 1080; PSNR and SSIM against the 256-spp target of
  (a) the plain roughness approximation (roughColorsA after the 10 blur iterations) and
  (b) the filter's prediction, for the rough-reflection radiance and for the composited frame;
  and the post stage's time with either.
PyTorch only holds device buffers and cuts crops; every kernel is the library's.
"""
from __future__ import annotations

import math
import os
import time

import numpy as np

from . import scenes
from . import rgcuda as rg

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "filter_weights.bin")
CROP = 128


def training_scene(seed: int, width: int, height: int) -> scenes.Scene:
    """A game-frame-type scene (seed) with roughness U[0,1] (seed + 1) and a camera on a seeded orbit."""
    sc = scenes.instanced_scene(width=width, height=height, num_samples=1, max_recursions=5, seed=seed)
    rng = scenes.Rng(seed + 1)
    sc.materials["roughness"] = rng.uniform(len(sc.materials)).astype(np.float32)
    theta = rng.uniform(1, 0, 2 * math.pi)[0]
    radius = rng.uniform(1, 45, 110)[0]
    height_ = rng.uniform(1, 6, 40)[0]
    eye = (radius * math.sin(theta), height_, radius * math.cos(theta))
    sc.ubo = scenes.make_ubo(eye, (0.0, 2.0, 0.0), 60.0, width, height, (-0.4, -1.0, 0.3), 1, 5)
    return sc


def render_pair(ctx, sc, d_in, d_tgt, glossy_frames=8, glossy_spp=32, seed=1):
    """Input (1 spp) and 256-spp glossy target of one scene into the given device tensors."""
    import torch
    torch.cuda.synchronize()  # the destination tensors are ready before the library's stream writes them
    slot = ctx.scene_create()
    ctx.scene_select(slot)
    try:
        rg.load_scene(ctx, sc)
        ctx.set_resolution(sc.width, sc.height)
        ctx.render(sc.ubo, False)
        ctx.filter_input(d_in.data_ptr())
        ubo = sc.ubo.copy()
        ubo["numSamples"] = glossy_spp
        acc = torch.zeros_like(d_tgt)
        tmp = torch.empty_like(d_tgt)
        for k in range(glossy_frames):
            ctx.set_glossy(seed * 1000 + k + 1)
            ctx.render(ubo, False)
            ctx.filter_target(tmp.data_ptr())
            ctx.synchronize()
            acc += tmp
        ctx.set_glossy(0)
        d_tgt.copy_(acc / glossy_frames)
        torch.cuda.synchronize()
    finally:
        ctx.synchronize()
        ctx.scene_select(0)
        ctx.scene_destroy(slot)


def build_dataset(ctx, n_scenes: int, width: int, height: int, seed0: int = 3000, log=print):
    import torch
    X = torch.zeros(n_scenes, height, width, 16, dtype=torch.bfloat16, device="cuda")
    T = torch.zeros(n_scenes, height, width, 4, dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    for k in range(n_scenes):
        sc = training_scene(seed0 + k, width, height)
        render_pair(ctx, sc, X[k], T[k], seed=seed0 + k)
        if log and (k + 1) % 25 == 0:
            log(f"dataset {k + 1}/{n_scenes} scenes, {time.perf_counter() - t0:.1f} s")
    return X, T


def train(flt, X, T, crops: int, epochs: int, batch: int = 32, lr: float = 1e-3, seed: int = 5, log=print):
    """Adam over `crops` random 128 x 128 crops (fixed per run), `epochs` passes in shuffled order."""
    import torch
    n, H, W = X.shape[0], X.shape[1], X.shape[2]
    g = torch.Generator().manual_seed(seed)
    si = torch.randint(0, n, (crops,), generator=g)
    yi = torch.randint(0, H - CROP + 1, (crops,), generator=g)
    xi = torch.randint(0, W - CROP + 1, (crops,), generator=g)
    xb = torch.empty(batch, CROP, CROP, 16, dtype=torch.bfloat16, device="cuda")
    tb = torch.empty(batch, CROP, CROP, 4, dtype=torch.float32, device="cuda")
    losses, t0, steps = [], time.perf_counter(), 0
    for ep in range(epochs):
        order = torch.randperm(crops, generator=g)
        ep_loss = []
        for b0 in range(0, crops - batch + 1, batch):
            idx = order[b0:b0 + batch]
            for j, c in enumerate(idx.tolist()):
                s, y, x = int(si[c]), int(yi[c]), int(xi[c])
                xb[j].copy_(X[s, y:y + CROP, x:x + CROP])
                tb[j].copy_(T[s, y:y + CROP, x:x + CROP])
            torch.cuda.synchronize()
            ep_loss.append(flt.train_step(xb.data_ptr(), tb.data_ptr(), batch, CROP, CROP, lr))
            steps += 1
        losses.append(float(np.mean(ep_loss)))
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {losses[-1]:.5f} ({time.perf_counter() - t0:.1f} s)")
    return {"epochs": epochs, "crops": crops, "batch": batch, "steps": steps, "loss_per_epoch": losses,
            "seconds": time.perf_counter() - t0}


def psnr(a, b):
    mse = float(np.mean((np.clip(a, 0, 1) - np.clip(b, 0, 1)) ** 2))
    return float("inf") if mse == 0 else 10.0 * math.log10(1.0 / mse)


def ssim(a, b):
    """Mean SSIM (Wang et al. 2004; Gaussian window sigma 1.5, K1 0.01, K2 0.03, range 1) over the RGB
    channels of two images clamped to [0, 1]."""
    from scipy.ndimage import gaussian_filter
    a, b = np.clip(a, 0, 1).astype(np.float64), np.clip(b, 0, 1).astype(np.float64)
    c1, c2 = 0.01 ** 2, 0.03 ** 2
    vals = []
    for ch in range(3):
        x, y = a[..., ch], b[..., ch]
        mx, my = gaussian_filter(x, 1.5), gaussian_filter(y, 1.5)
        sxx = gaussian_filter(x * x, 1.5) - mx * mx
        syy = gaussian_filter(y * y, 1.5) - my * my
        sxy = gaussian_filter(x * y, 1.5) - mx * my
        m = ((2 * mx * my + c1) * (2 * sxy + c2)) / ((mx * mx + my * my + c1) * (sxx + syy + c2))
        vals.append(m.mean())
    return float(np.mean(vals))


def composite(base, rough_rgb):
    """postprocess.comp:28-50 without fade: clamp(mix(base.rgb, rough, base.a), 0, 1)."""
    a = base[..., 3:4]
    return np.clip(base[..., :3] * (1 - a) + rough_rgb[..., :3] * a, 0, 1)


def evaluate(flt, n_scenes: int = 4, width: int = 1920, height: int = 1080, seed0: int = 90000, log=print):
    import torch
    ctx = rg.Context(flags=rg.RG_FLAG_DEBUG_IMAGES)
    rows = []
    for k in range(n_scenes):
        sc = training_scene(seed0 + k, width, height)
        d_in = torch.zeros(height, width, 16, dtype=torch.bfloat16, device="cuda")
        d_t = torch.zeros(height, width, 4, device="cuda")
        render_pair(ctx, sc, d_in, d_t, seed=seed0 + k)
        target = d_t.cpu().numpy()
        slot = ctx.scene_create()
        ctx.scene_select(slot)
        rg.load_scene(ctx, sc)
        ctx.set_filter(None)
        ctx.render(sc.ubo, False)
        base = ctx.download_image("base")
        plain = ctx.download_image("rough_colors_a")
        ctx.set_filter(flt)
        ctx.render(sc.ubo, False)
        learned = ctx.download_image("filter_out")
        ctx.set_filter(None)
        ctx.synchronize()
        ctx.scene_select(0)
        ctx.scene_destroy(slot)
        ref_c, plain_c, learned_c = composite(base, target), composite(base, plain), composite(base, learned)
        rows.append({"scene": seed0 + k,
                     "rough_psnr_plain": psnr(plain[..., :3], target[..., :3]),
                     "rough_psnr_learned": psnr(learned[..., :3], target[..., :3]),
                     "rough_ssim_plain": ssim(plain, target), "rough_ssim_learned": ssim(learned, target),
                     "frame_psnr_plain": psnr(plain_c, ref_c), "frame_psnr_learned": psnr(learned_c, ref_c),
                     "frame_ssim_plain": ssim(plain_c, ref_c), "frame_ssim_learned": ssim(learned_c, ref_c)})
        if log:
            log(rows[-1])
    mean = {k: float(np.mean([r[k] for r in rows])) for k in rows[0] if k != "scene"}
    ctx.close()
    return mean, rows


def post_times(flt, frames: int = 20):
    """Post-stage and whole-frame times on the game frame (1080p, 4 spp) with the plain passes and
    with the filter (CUDA events of the library's profiler ranges)."""
    sc = scenes.game_frame_scene()
    rt = rg.Raytracer(sc).prepare()
    out = {}
    for name, f in (("plain", None), ("learned", flt)):
        rt.ctx.set_filter(f)
        for _ in range(3):
            rt.do_raytracing()
        rt.ctx.timings()
        for _ in range(frames):
            rt.do_raytracing()
        t = rt.ctx.timings()
        out[name] = {"rough_ms": t["roughSum"] / t["frames"], "post_ms": t["postprocSum"] / t["frames"],
                     "frame_ms": t["rtTotalSum"] / t["frames"]}
    rt.ctx.set_filter(None)
    rt.ctx.close()
    return out


def save_weights(flt, path: str = WEIGHTS):
    flt.params().astype("<f4").tofile(path)


def load_weights(flt, path: str = WEIGHTS):
    flt.set_params(np.fromfile(path, dtype="<f4"))


def main():
    """python -m raygun_gb300.filter_train --infer W H [--repeat N]: the committed weights on a
    seeded random 16-channel input of W x H (inference only); --train W H [--repeat N]: N Adam steps
    on a seeded random input and target of W x H (forward, backward, weight gradients).  Both are the
    workloads of the filter kernels' profiles."""
    import argparse
    import torch
    ap = argparse.ArgumentParser()
    mode = ap.add_mutually_exclusive_group(required=True)
    mode.add_argument("--infer", nargs=2, type=int, metavar=("W", "H"))
    mode.add_argument("--train", nargs=2, type=int, metavar=("W", "H"))
    ap.add_argument("--repeat", type=int, default=3)
    args = ap.parse_args()
    W, H = args.infer or args.train
    ctx = rg.Context()
    flt = rg.Filter(ctx)
    load_weights(flt)
    g = torch.Generator().manual_seed(1)
    x = torch.zeros(H, W, 16)
    x[..., :12] = torch.rand(H, W, 12, generator=g)
    d_in = x.to(torch.bfloat16).cuda()
    d_out = torch.empty(H, W, 4, device="cuda")
    torch.cuda.synchronize()
    if args.infer:
        for _ in range(args.repeat):
            flt.forward(d_in.data_ptr(), 1, H, W, d_out.data_ptr())
        print(f"filter forward {W}x{H} x{args.repeat}: mean prediction {float(d_out[..., :3].mean()):.5f}")
        return
    tgt = torch.zeros(H, W, 4)
    tgt[..., :3] = torch.rand(H, W, 3, generator=g)
    d_tgt = tgt.cuda()
    torch.cuda.synchronize()
    loss = 0.0
    for _ in range(args.repeat):
        loss = flt.train_step(d_in.data_ptr(), d_tgt.data_ptr(), 1, H, W, 1e-3)
    print(f"filter train {W}x{H} x{args.repeat}: last loss {loss:.5f}")


if __name__ == "__main__":
    main()
