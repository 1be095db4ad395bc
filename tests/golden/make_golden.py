"""Generate the golden fixtures of the ray-tracing path from the REFERENCE's own shader code.

Run here, where the reference tree exists:  python tests/golden/make_golden.py
It builds the reference-compiled checker (oracle/ref: Raygun's GLSL compiled as C++ through a
GLSL shim, with the oracle's traversal standing in for the Vulkan driver) and, for each small
seeded scene, stores the scene's input arrays and the reference outputs:
  base / normal / rough  -- raygen.rgen's three RGBA16F images (stored as float16, exact)
  final, final_nofxaa    -- the presented image after FXAA and the postprocess output
  transitions            -- roughTransitions (R8_SNORM values, float32)
  rough_a, rough_b       -- roughColorsA / roughColorsB after the 10 blur iterations (float16)
  rays                   -- traced rays (traceRayEXT calls that traverse)
Inputs are stored too (not regenerated), so the fixtures do not depend on the host's libm.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from raygun_gb300 import scenes as S  # noqa: E402
from oracle import ref  # noqa: E402


def scenes():
    out = {
        "spheres16_96x54_s2_d4": S.spheres_scene(n_spheres=16, width=96, height=54, num_samples=2, max_recursions=4, seed=3),
        "instanced_96x54_s2_d5": S.instanced_scene(width=96, height=54, counts=(6, 5, 3, 1, 4, 4, 1, 1), hf_n=32,
                                                   ico_levels=(1, 2, 3, 3), num_samples=2, max_recursions=5, name="mini"),
        "spheres24_64x36_s4_d7": S.spheres_scene(n_spheres=24, width=64, height=36, num_samples=4, max_recursions=7, seed=9),
    }
    fade = S.spheres_scene(n_spheres=12, width=64, height=36, num_samples=1, max_recursions=3, seed=4)
    fade.ubo["fadeColor"] = (0.2, 0.4, 0.6, 0.5)
    out["spheres12_64x36_fade"] = fade
    alpha = S.spheres_scene(n_spheres=12, width=64, height=36, num_samples=1, max_recursions=3, seed=5)
    alpha.ubo["showAlpha"] = 1
    out["spheres12_64x36_showalpha"] = alpha
    return out


def main():
    ref.build()
    for name, sc in scenes().items():
        b, n, r, rays = ref.render(sc, nthreads=4)
        fin, dbg = ref.post(sc.ubo, b.copy(), n.copy(), r.copy(), fxaa=True, debug=True)
        nofx = ref.post(sc.ubo, b.copy(), n.copy(), r.copy(), fxaa=False)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(
            path, vertices=sc.vertices, indices=sc.indices, materials=sc.materials, meshes=sc.meshes,
            instances=sc.instances, ubo=sc.ubo, size=np.array([sc.width, sc.height]),
            base=b.astype(np.float16), normal=n.astype(np.float16), rough=r.astype(np.float16),
            final=fin.astype(np.float16), final_nofxaa=nofx.astype(np.float16), transitions=dbg[0][..., 0],
            rough_a=dbg[1].astype(np.float16), rough_b=dbg[2].astype(np.float16), rays=np.array([rays], np.uint64))
        for k, v in (("base", b), ("normal", n), ("rough", r), ("final", fin)):
            assert np.array_equal(v.astype(np.float16).astype(np.float32), v), (name, k)
        print(name, os.path.getsize(path), "bytes", rays, "rays")


if __name__ == "__main__":
    main()
