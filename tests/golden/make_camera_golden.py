"""Generate tests/golden/camera_glm.npz: camera matrices computed by the reference's own glm.

Run here, where the reference tree exists:  python tests/golden/make_camera_golden.py
It compiles glm_camera.cpp against the glm headers the reference vendors (vendor/glm/include, glm
0.9.9.5) with GLM_FORCE_DEPTH_ZERO_TO_ONE as the reference's pch.hpp sets it, feeds it seeded
camera cases (field of view, image size, near/far, position, look-at target or axis rotation,
scaling) and stores the cases with glm's viewInverse, projInverse and rotation quaternion.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref import REFERENCE  # noqa: E402

GLM = os.path.join(REFERENCE, "vendor", "glm", "include")


def cases(n=40, seed=21):
    rng = np.random.RandomState(seed)
    sizes = [(1920, 1080), (640, 360), (320, 180), (800, 800), (1280, 720), (97, 53)]
    c = np.zeros((n, 16), np.float32)
    for k in range(n):
        w, h = sizes[k % len(sizes)]
        fov = [45.0, 60.0, 30.0, 90.0, 72.5][k % 5]
        near, far = (0.1, 100.0) if k % 3 else (rng.uniform(0.01, 1.0), rng.uniform(50.0, 5000.0))
        pos = rng.uniform(-50, 50, 3)
        if k % 2 == 0:  # look at a target
            tgt = pos + rng.normal(size=3) * rng.uniform(1, 30)
            p = [0.0, *tgt, 0.0]
        else:  # rotate about an axis
            ax = rng.normal(size=3)
            ax /= np.linalg.norm(ax)
            p = [1.0, rng.uniform(-np.pi, np.pi), *ax]
        s = [1.0, 1.0, 1.0] if k % 4 < 2 else rng.uniform(0.3, 3.0, 3)
        c[k] = [fov, w, h, near, far, *pos, *p, *s]
    return c


def main():
    if not os.path.isdir(GLM):
        sys.exit(f"glm headers not found under {GLM}")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "glm_camera")
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", GLM, "-o", exe,
                        os.path.join(HERE, "glm_camera.cpp")], check=True)
        c = cases()
        r = subprocess.run([exe], input=c.tobytes(), capture_output=True, check=True)
    out = np.frombuffer(r.stdout, np.float32).reshape(len(c), 36)
    path = os.path.join(HERE, "camera_glm.npz")
    np.savez_compressed(path, cases=c, view_inverse=out[:, :16], proj_inverse=out[:, 16:32], rotation=out[:, 32:])
    print(path, len(c), "cases")


if __name__ == "__main__":
    main()
