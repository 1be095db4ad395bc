"""The ray sets of the closest-hit measurements (raygun_gb300/rays.py), on the CPU.

camera_rays_device built with torch on the CPU against the numpy camera rays the parity tests use
(raygen.h:84-90).  first_bounce_secondary against a stand-in context whose ray query answers with
the oracle's hits: one reflection ray per hit on a reflective material, one refraction ray per hit
on a transparent material unless it is totally reflected (closesthit.rchit:206-250), each from the
hit point with tmin 0.01 and tmax 1000.
"""
import numpy as np
import pytest

from raygun_gb300 import scenes as S
from test_oracle import camera_rays

torch = pytest.importorskip("torch")


def test_camera_rays_device_match_numpy():
    from raygun_gb300.rays import camera_rays_device
    sc = S.spheres_scene(n_spheres=8, width=48, height=27, seed=2)
    got = camera_rays_device(sc.ubo, sc.width, sc.height, torch.device("cpu")).numpy()
    ref = camera_rays(sc)
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-6)


class OracleQueries:
    """The one call first_bounce_secondary makes of a context, answered by the oracle."""

    def __init__(self, orc_scene):
        self.o = orc_scene

    def trace_rays_device(self, p_rays, n, p_tuv, p_ids):
        as_np = lambda p, shape, dt: np.ctypeslib.as_array((np.ctypeslib.ctypes.c_char * (int(np.prod(shape)) * np.dtype(dt).itemsize)).from_address(p)).view(dt).reshape(shape)
        rays = as_np(p_rays, (n, 8), np.float32).copy()
        tuv, ids = self.o.trace(rays)
        as_np(p_tuv, (n, 3), np.float32)[...] = tuv
        as_np(p_ids, (n, 2), np.int32)[...] = ids.view(np.int32)

    def synchronize(self):
        pass


def test_first_bounce_secondary_rays(orc):
    from raygun_gb300.rays import camera_rays_device, first_bounce_secondary
    sc = S.spheres_scene(n_spheres=16, width=64, height=36, seed=4)
    dev = torch.device("cpu")
    sec = first_bounce_secondary(OracleQueries(orc.OracleScene(sc)), sc, sc.instances, dev, sc.width, sc.height).numpy()
    cam = camera_rays_device(sc.ubo, sc.width, sc.height, dev).numpy()
    tuv, ids = orc.OracleScene(sc).trace(cam)
    hit = ids[:, 0] != 0xFFFFFFFF
    inst = sc.instances[ids[hit, 0].astype(np.int64)]
    prim = ids[hit, 1].astype(np.int64)
    i0 = sc.indices[inst["indexBufferOffset"].astype(np.int64) + 3 * prim].astype(np.int64) + inst["vertexBufferOffset"]
    mat = sc.materials[sc.vertices["matIndex"][i0].astype(np.int64) + inst["materialBufferOffset"]]
    n_refl = int((mat["reflectivity"] > 0).sum())
    n_trans = int((mat["transparency"] > 0).sum())
    assert n_refl > 0 and n_trans > 0
    # reflection rays first, then the refraction rays that are not totally reflected
    assert n_refl <= len(sec) <= n_refl + n_trans
    assert (sec[:, 3] == np.float32(0.01)).all() and (sec[:, 7] == np.float32(1000.0)).all()
    np.testing.assert_allclose(np.linalg.norm(sec[:, 4:7], axis=1), 1.0, atol=1e-5)
    # every origin is a hit point of a camera ray on such a material
    pts = cam[hit, :3] + cam[hit, 4:7] * tuv[hit, :1]
    refl_pts = pts[mat["reflectivity"] > 0]
    np.testing.assert_allclose(sec[:n_refl, :3], refl_pts, rtol=0, atol=1e-4)
