"""Headless render of the game-frame scene (1024 instances of the eight procedural meshes).

    python -m raygun_gb300.render [--res WxH] [--spp S] [--frames N] [--out frame.npy]

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
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    w, h = (int(x) for x in args.res.split("x"))
    sc = S.instanced_scene(width=w, height=h, num_samples=args.spp)
    rt = rgcuda.Raytracer(sc).prepare()
    fb = None
    for _ in range(args.frames):
        fb = rt.render()
    st = rt.ctx.stats()
    print(json.dumps({"width": w, "height": h, "spp": args.spp, "frames": args.frames,
                      "rays_last_frame": st["primary"] + st["shadow"] + st["secondary"],
                      "finite": bool(np.isfinite(fb).all())}))
    if args.out:
        np.save(args.out, fb)
    rt.ctx.close()


if __name__ == "__main__":
    main()
