"""The C++ facade (include/rg/raygun.hpp): Raygun's Scene / Entity / Camera / RenderSystem shape over
the C ABI, driven by tests/cpp/facade_demo.cpp.

CPU: the scene walk (DFS order, invisible and zero-volume subtrees skipped, model-less entities
descended), the global transforms, the packed buffers and the camera matrices.
GPU: the demo's frames (before and after a resize) against the oracle on the demo's own buffers.
"""
import math
import os
import subprocess

import numpy as np
import pytest

from raygun_gb300 import scenes as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "raygun_gb300")


@pytest.fixture(scope="module")
def demo(tmp_path_factory):
    from raygun_gb300 import build
    build.build()
    exe = os.path.join(PKG, "_build", "facade_demo")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "facade_demo.cpp")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-o", exe, src, "-L", PKG,
                    "-lrgfacade", "-lrgcuda", f"-Wl,-rpath,{PKG}"], check=True)
    return exe


def run(exe, out, walk_only):
    args = [exe, str(out)] + (["--walk-only"] if walk_only else [])
    subprocess.run(args, check=True, capture_output=True)
    rd = lambda n, dt: np.fromfile(os.path.join(out, n), dtype=dt)
    d = dict(vertices=rd("vertices.bin", S.VERTEX), indices=rd("indices.bin", np.uint32),
             materials=rd("materials.bin", S.MATERIAL), meshes=rd("meshes.bin", np.uint32).view(S.MESH),
             instances=rd("instances.bin", S.INSTANCE), ubo=rd("ubo.bin", S.UBO),
             names=open(os.path.join(out, "names.txt")).read().split())
    return d


def trs(t, deg=0.0, s=1.0):
    c, sn = math.cos(math.radians(deg)), math.sin(math.radians(deg))
    m = np.eye(4)
    m[:3, :3] = np.array([[c, 0, sn], [0, 1, 0], [-sn, 0, c]]) * s
    m[:3, 3] = t
    return m


def test_scene_walk_and_transforms(demo, tmp_path):
    d = run(demo, tmp_path, True)
    assert d["names"] == ["ground", "s0", "s0moon", "s1", "s2", "s3", "s4"]
    inst = d["instances"]
    assert len(inst) == 7 and set(inst["mask"]) == {0xFF}
    ring = trs((0, 1, 2), 30)
    expect = {"ground": np.eye(4), "s0": ring @ trs((-2, 0, 0), s=0.8),
              "s0moon": ring @ trs((-2, 0, 0), s=0.8) @ trs((0, 1.2, 0), s=0.4), "s1": ring, "s2": ring @ trs((2, 0, 0)),
              "s3": trs((3, 0, -1)) @ trs((0, 0.8, 0), s=0.8), "s4": trs((-3, 0.6, -2), s=0.6)}
    for k, name in enumerate(d["names"]):
        assert np.allclose(inst[k]["transform"], expect[name][:3], atol=1e-5), name
    # two meshes (quad, sphere) packed back to back; every model's materials in order
    assert len(d["meshes"]) == 2 and d["meshes"][0]["triCount"] == 2
    assert inst[0]["blas"] == 0 and set(inst["blas"][1:]) == {1}
    assert len(d["materials"]) == 11 and d["materials"][0]["effectId"] == 1
    # the hidden / flat subtrees' four models are packed but not drawn
    assert list(inst["materialBufferOffset"]) == [0, 1, 2, 3, 4, 9, 10]


def test_camera_matrices(demo, tmp_path):
    d = run(demo, tmp_path, True)
    u = d["ubo"][0]
    assert np.allclose(u["viewInverse"].T, S.look_at_view_inverse((0, 3, -9), (0, 1, 1)), atol=1e-5)
    assert np.allclose(u["projInverse"].T, S.perspective_inverse(60.0, 320 / 180), atol=1e-5)
    assert np.allclose(u["lightDir"], np.array([0.4, -0.6, -0.8]) / np.linalg.norm([0.4, -0.6, -0.8]), atol=1e-6)
    assert u["numSamples"] == 2 and u["maxRecursions"] == 4 and np.allclose(u["clearColor"], 0.2)


def test_camera_matches_glm():
    """The facade's Camera (viewInverse = T * R * S of its transform, projInverse = the inverse of
    glm's depth-[0,1] perspective with the Y flip, lookAt / axis rotations as quaternions) against the
    reference's own glm on 40 seeded cases (tests/golden/camera_glm.npz, made by
    tests/golden/make_camera_golden.py from the glm the reference vendors).  The facade inverts in
    double and rounds once, glm in float, so the bar is 1e-6 of each matrix's largest entry (measured:
    2e-7); the rotation quaternions agree to 5e-7 (up to sign, q and -q being one rotation)."""
    from raygun_gb300 import build
    build.build()
    exe = os.path.join(PKG, "_build", "camera_dump")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-o", exe,
                    os.path.join(ROOT, "tests", "cpp", "camera_dump.cpp"), "-L", PKG, "-lrgfacade", "-lrgcuda",
                    f"-Wl,-rpath,{PKG}"], check=True)
    g = np.load(os.path.join(ROOT, "tests", "golden", "camera_glm.npz"))
    r = subprocess.run([exe], input=g["cases"].astype(np.float32).tobytes(), capture_output=True, check=True)
    out = np.frombuffer(r.stdout, np.float32).reshape(len(g["cases"]), 36)
    for name, got, want in (("viewInverse", out[:, :16], g["view_inverse"]), ("projInverse", out[:, 16:32], g["proj_inverse"])):
        scale = np.abs(want).max(1, keepdims=True)
        err = np.abs(got - want) / scale
        assert err.max() <= 1e-6, (name, float(err.max()), int(err.max(1).argmax()))
    q, qw = out[:, 32:], g["rotation"]
    sign = np.where((q * qw).sum(1, keepdims=True) < 0, -1.0, 1.0)
    assert np.abs(q * sign - qw).max() <= 5e-7


@pytest.mark.gpu
def test_facade_frames_match_oracle(demo, tmp_path, orc):
    from test_gpu_parity import assert_image_close
    d = run(demo, tmp_path, False)
    for fb_name, ubo_name, (w, h) in (("framebuffer.bin", "ubo.bin", (320, 180)), ("framebuffer_small.bin", "ubo_small.bin", (160, 90))):
        ubo = np.fromfile(os.path.join(tmp_path, ubo_name), dtype=S.UBO)
        sc = S.Scene("facade", d["vertices"], d["indices"], d["materials"], d["meshes"], d["instances"], ubo, w, h)
        o = orc.OracleScene(sc)
        b, n, r, _ = o.render()
        ref = orc.post(ubo, b, n, r)
        fb = np.fromfile(os.path.join(tmp_path, fb_name), dtype=np.float32).reshape(h, w, 4)
        assert_image_close(fb, ref, f"facade {w}x{h}")
