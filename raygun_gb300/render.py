"""Headless render of the game-frame scene (1024 instances of the eight procedural meshes).

    python -m raygun_gb300.render [--res WxH] [--spp S] [--frames N] [--blas-lbvh] [--tlas-lbvh]
                                  [--learned-filter] [--out frame.npy]
    python -m raygun_gb300.render --lbvh-boxes N [--frames K]   (K LBVH builds over N seeded boxes)
    python -m raygun_gb300.render --secondary K [--res WxH]      (K closest-hit queries of the scene's
        first-bounce reflection / refraction rays at 2W x 2H pixel-centre camera rays)

Builds the scene, renders N frames through the library (RenderSystem::render without a window),
prints the rays of the last frame and optionally saves its RGBA32F framebuffer.  No timing: this is
the command profiling captures wrap, so that they see exactly the launches of N frames.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import rgcuda
from . import scenes as S


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--res", default="1920x1080")
    ap.add_argument("--spp", type=int, default=4)
    ap.add_argument("--frames", type=int, default=1)
    ap.add_argument("--blas-lbvh", action="store_true", help="BLASes as LBVHs (Morton sort, Karras) instead of binned SAH")
    ap.add_argument("--tlas-lbvh", action="store_true", help="the TLAS as an LBVH instead of binned SAH")
    ap.add_argument("--learned-filter", action="store_true", help="the learned roughness filter (committed weights)")
    ap.add_argument("--lbvh-boxes", type=int, default=0, help="instead of frames: LBVH builds over this many seeded boxes")
    ap.add_argument("--secondary", type=int, default=0,
                    help="instead of frames: this many rg_trace_rays_device queries of the first-bounce secondary rays")
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    if args.lbvh_boxes:
        rng = np.random.RandomState(7)
        c = rng.uniform(-100, 100, (args.lbvh_boxes, 3)).astype(np.float32)
        e = rng.uniform(0.01, 0.5, (args.lbvh_boxes, 3)).astype(np.float32)
        boxes = np.concatenate([c - e, c + e], 1)
        ctx = rgcuda.Context()
        for _ in range(args.frames):
            out = ctx.lbvh_build_host(boxes)
        print(json.dumps({"lbvh_boxes": args.lbvh_boxes, "builds": args.frames, "root_box": out["nodeboxes"][0].tolist()}))
        ctx.close()
        return
    w, h = (int(x) for x in args.res.split("x"))
    sc = S.instanced_scene(width=w, height=h, num_samples=args.spp)
    flags = (rgcuda.RG_FLAG_BLAS_LBVH if args.blas_lbvh else 0) | (rgcuda.RG_FLAG_TLAS_LBVH if args.tlas_lbvh else 0)
    rt = rgcuda.Raytracer(sc, flags=flags).prepare()
    if args.secondary:
        import torch
        from .rays import first_bounce_secondary
        dev = torch.device("cuda", 0)
        rays = first_bounce_secondary(rt.ctx, sc, sc.instances, dev, 2 * w, 2 * h)
        tuv = torch.empty(len(rays), 3, device=dev)
        ids = torch.empty(len(rays), 2, dtype=torch.int32, device=dev)
        torch.cuda.synchronize(dev)
        for _ in range(args.secondary):
            rt.ctx.trace_rays_device(rays.data_ptr(), len(rays), tuv.data_ptr(), ids.data_ptr())
        rt.ctx.synchronize()
        hits = int((ids[:, 0] != -1).sum())
        print(json.dumps({"width": 2 * w, "height": 2 * h, "secondary_rays": len(rays), "queries": args.secondary,
                          "hits": hits, "stack_overflows": rt.ctx.stats()["stack_overflows"]}))
        rt.ctx.close()
        return
    flt = None
    if args.learned_filter:
        from . import filter_train
        flt = rgcuda.Filter(rt.ctx, seed=0)
        filter_train.load_weights(flt)
        rt.ctx.set_filter(flt)
    fb = None
    for _ in range(args.frames):
        fb = rt.render()
    st = rt.ctx.stats()
    print(json.dumps({"width": w, "height": h, "spp": args.spp, "frames": args.frames,
                      "rays_last_frame": st["primary"] + st["shadow"] + st["secondary"],
                      "finite": bool(np.isfinite(fb).all())}))
    if args.out:
        np.save(args.out, fb)
    if flt is not None:
        rt.ctx.set_filter(None)
        flt.close()
    rt.ctx.close()


if __name__ == "__main__":
    main()
