"""Golden fixtures made by the reference's own shader code (tests/golden/make_golden.py).

* oracle vs golden (CPU): bit exact -- this pins the oracle to the reference.
* CUDA path vs golden (GPU): the bars of test_gpu_parity (2/255 on >= 99.9 % of pixels, PSNR >= 50
  dB); ray counts exact.
* fixtures vs a fresh reference run (CPU, only where the reference tree exists).
"""
import glob
import os

import numpy as np
import pytest

from raygun_gb300 import scenes as S

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz")) if not p.endswith("camera_glm.npz"))
IDS = [os.path.basename(f)[:-4] for f in FIXTURES]


def load(path):
    d = np.load(path)
    w, h = (int(x) for x in d["size"])
    sc = S.Scene(os.path.basename(path)[:-4], d["vertices"], d["indices"], d["materials"], d["meshes"], d["instances"],
                 d["ubo"].copy(), w, h)
    return sc, {k: d[k].astype(np.float32) if d[k].dtype == np.float16 else d[k] for k in d.files}


def test_fixtures_present():
    assert len(FIXTURES) >= 5


@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_oracle_matches_reference_golden(orc, path):
    sc, g = load(path)
    o = orc.OracleScene(sc)
    b, n, r, st = o.render(nthreads=4)
    assert st["primary"] + st["shadow"] + st["secondary"] == int(g["rays"][0])
    for k, v in (("base", b), ("normal", n), ("rough", r)):
        assert np.array_equal(v, g[k]), k
    fin, dbg = orc.post(sc.ubo, b, n, r, fxaa=True, debug=True)
    assert np.array_equal(fin, g["final"])
    assert np.array_equal(orc.post(sc.ubo, g["base"], g["normal"], g["rough"], fxaa=False), g["final_nofxaa"])
    assert np.array_equal(dbg[0][..., 0], g["transitions"])
    assert np.array_equal(dbg[1], g["rough_a"]) and np.array_equal(dbg[2], g["rough_b"])


@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_fixture_is_current(path):
    ref = pytest.importorskip("oracle.ref")
    if not ref.reference_present():
        pytest.skip("reference tree not present")
    sc, g = load(path)
    b, n, r, rays = ref.render(sc, nthreads=4)
    assert rays == int(g["rays"][0])
    assert np.array_equal(b, g["base"]) and np.array_equal(n, g["normal"]) and np.array_equal(r, g["rough"])
    assert np.array_equal(ref.post(sc.ubo, b, n, r), g["final"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=IDS)
def test_gpu_matches_reference_golden(rg, path):
    from test_gpu_parity import assert_image_close
    sc, g = load(path)
    rt = rg.Raytracer(sc).prepare()
    rt.do_raytracing(fxaa=False)
    st = rt.ctx.stats()
    assert st["primary"] + st["shadow"] + st["secondary"] == int(g["rays"][0])
    if not int(sc.ubo["showAlpha"][0]):  # showAlpha rewrites the G-buffers in place
        for k in ("base", "normal", "rough"):
            assert_image_close(rt.ctx.download_image(k), g[k], f"{sc.name} {k}")
    assert_image_close(rt.ctx.download(), g["final_nofxaa"], f"{sc.name} final (no FXAA)")
    fin = rt.render()
    assert_image_close(fin, g["final"], f"{sc.name} final")
