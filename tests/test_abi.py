"""CPU tests of the C-ABI boundary: the library builds and loads, exports every entry point that
include/rgcuda.h declares, and its struct layouts match the reference layouts."""
import ctypes
import os
import re

import numpy as np

from raygun_gb300 import scenes as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "rgcuda.h")).read()
    return sorted(set(re.findall(r"^\s*(?:rg_status|const char\*)\s+(rg_\w+)\s*\(", src, re.M)))


def test_header_symbols_exported(rg):
    names = declared_functions()
    assert len(names) >= 20
    lib = ctypes.CDLL(rg.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(rg.EXPORTS) == names


def test_layouts():
    assert S.VERTEX.itemsize == 32 and S.MATERIAL.itemsize == 64 and S.UBO.itemsize == 192
    assert S.INSTANCE.itemsize == 72
    assert S.UBO.fields["numSamples"][1] == 140 and S.UBO.fields["maxRecursions"][1] == 156
    assert S.UBO.fields["fadeColor"][1] == 176
    assert S.MATERIAL.fields["effectId"][1] == 40 and S.MATERIAL.fields["emission"][1] == 48
    assert ctypes.sizeof(__import__("raygun_gb300.rgcuda", fromlist=["Stats"]).Stats) == 72


def test_no_device_is_an_error_not_a_fallback(rg):
    from conftest import HAVE_GPU
    if HAVE_GPU:
        return
    try:
        rg.Context()
    except rg.RgError as e:
        assert e.code == -7
    else:
        raise AssertionError("context created without a GPU")


def test_scene_generators_deterministic():
    a, b = S.sphere_scene(), S.sphere_scene()
    assert a.tri_count == 61442 and len(a.materials) == 65
    assert np.array_equal(a.vertices, b.vertices) and np.array_equal(a.materials, b.materials)
    c = S.instanced_scene(width=64, height=36, counts=(3, 2, 1, 0, 2, 2, 1, 1), hf_n=16, ico_levels=(1, 1, 2, 2))
    assert len(c.instances) == 12 and set(c.instances["mask"]) == {0xFF}


def test_game_frame_scene_sizes():
    s = S.game_frame_scene()
    assert len(s.instances) == 1024
    assert 11_000_000 < s.instanced_tri_count < 13_000_000
    assert s.meshes["triCount"].tolist() == [1280, 5120, 20480, 81920, 4096, 4096, 130050, 130050]


def test_batch_scene_generators():
    from test_gpu_batch import mini_batch
    scenes = mini_batch()
    assert len({(s.width, s.height) for s in scenes}) >= 3
    assert len({int(s.ubo["maxRecursions"][0]) for s in scenes}) >= 3
    assert all(1 <= int(s.ubo["numSamples"][0]) <= 3 for s in scenes)
    scs = S.default_batch_scenes()
    assert len(scs) == 64
    assert {(s.width, s.height) for s in scs} <= set(S.BATCH_RESOLUTIONS)
    assert {int(s.ubo["numSamples"][0]) for s in scs} == {1, 2, 3, 4}
    assert {int(s.ubo["maxRecursions"][0]) for s in scs} == {1, 2, 3, 4, 5, 6}
    tris = np.array([s.instanced_tri_count for s in scs])
    assert tris.min() >= 1000 and tris.max() <= 4_000_000
    assert np.median(np.log10(tris)) > 3.5  # log-uniform over [3, 6.6]
    again = S.default_batch_scenes()
    assert all(np.array_equal(a.instances, b.instances) for a, b in zip(scs, again))


def test_job_layout(rg):
    assert rg.JOB.itemsize == 208 and rg.JOB.fields["ubo"][1] == 16


def test_filter_weights_file():
    from raygun_gb300 import filter_train as FT, rgcuda
    w = np.fromfile(FT.WEIGHTS, dtype="<f4")
    assert len(w) == rgcuda.FILTER_PARAMS and np.isfinite(w).all()
    layers = rgcuda.filter_layers(w)
    assert [l[0].shape for l in layers] == [(32, 12, 3, 3), (64, 32, 3, 3), (64, 64, 3, 3), (32, 64, 3, 3), (3, 32, 3, 3)]
