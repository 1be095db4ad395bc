"""Collada (.dae) and .rgmat.json ingest of the C++ facade (include/rg/collada.hpp), driven by
tests/cpp/collada_dump.cpp.

CPU: the facade's import of tests/fixtures/pavilion.dae (a synthetic scene: <polylist>, <polygons>
and multi-material <triangles>, normals inside <vertices>, translate/rotate/scale and <matrix>
nodes, a mirrored node, child nodes merged into their root child, a material based on another, a
material without a file) equals an independent reading of the same files written here with
xml.etree; the node transforms survive the decompose / recompose round trip; where the reference
tree is present, the same holds for its room.dae + ball.dae example scene.
GPU: the facade renders the imported fixture like the oracle renders the same buffers.
"""
import json
import math
import os
import subprocess
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from raygun_gb300 import scenes as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "raygun_gb300")
FIX = os.path.join(ROOT, "tests", "fixtures")
from oracle.ref import REFERENCE  # noqa: E402  (where the reference tree is, if anywhere)


@pytest.fixture(scope="module")
def dump_exe():
    from raygun_gb300 import build
    build.build()
    exe = os.path.join(PKG, "_build", "collada_dump")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "collada_dump.cpp")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-o", exe, src, "-L", PKG,
                    "-lrgfacade", "-lrgcuda", f"-Wl,-rpath,{PKG}"], check=True)
    return exe


def run_dump(exe, out, dae, matdir, ball=None, render=None):
    args = [exe, dae, matdir or "-", str(out)]
    if ball:
        args += ["--ball", ball]
    if render:
        args += ["--render", str(render[0]), str(render[1])]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rd = lambda n, dt: np.fromfile(os.path.join(out, n), dtype=dt)
    d = dict(vertices=rd("vertices.bin", S.VERTEX), indices=rd("indices.bin", np.uint32),
             materials=rd("materials.bin", S.MATERIAL), meshes=rd("meshes.bin", np.uint32).view(S.MESH),
             instances=rd("instances.bin", S.INSTANCE), ubo=rd("ubo.bin", S.UBO),
             info=json.load(open(os.path.join(out, "info.json"))))
    if render:
        d["framebuffer"] = rd("framebuffer.bin", np.float32).reshape(render[1], render[0], 4)
        d["stats"] = [int(x) for x in open(os.path.join(out, "stats.txt")).read().split()]
    return d


# ---- independent reading of the same files ---------------------------------------------------------
def _tag(e):
    return e.tag.split("}")[-1]


def _kids(e, name):
    return [k for k in e if _tag(k) == name]


def _kid(e, name):
    k = _kids(e, name)
    return k[0] if k else None


def _floats(t):
    return np.array([float(x) for x in (t or "").split()], np.float32)


def _ints(t):
    return [int(x) for x in (t or "").split()]


def read_material(path):
    m = S._material((1.0, 0.0, 1.0))[0]  # gpu_material.def defaults
    if not os.path.exists(path):
        return m
    d = json.load(open(path))
    if d.get("type") != "Material":
        return m
    if "basedOn" in d:
        base = os.path.join(os.path.dirname(path), d["basedOn"] + ".rgmat.json")
        if os.path.exists(base):
            m = read_material(base)
    for k, v in d.items():
        if k in ("diffuse", "specular"):
            m[k] = v
        elif k in ("transparency", "reflectivity", "roughness", "ior", "emission", "effectId", "rayConsumption"):
            m[k] = v
    return m


def node_matrix(n):
    m = np.eye(4)
    for e in n:
        t = _tag(e)
        v = _floats(e.text).astype(np.float64)
        if t == "matrix":
            m = m @ v.reshape(4, 4)
        elif t == "translate":
            x = np.eye(4)
            x[:3, 3] = v
            m = m @ x
        elif t == "scale":
            m = m @ np.diag([v[0], v[1], v[2], 1.0])
        elif t == "rotate":
            ax = v[:3] / np.linalg.norm(v[:3])
            a = math.radians(v[3])
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            r = np.eye(4)
            r[:3, :3] = np.eye(3) * math.cos(a) + math.sin(a) * K + (1 - math.cos(a)) * np.outer(ax, ax)
            m = m @ r
    return m


def read_collada(path, matdir):
    """Per root child of the visual scene: (name, 4x4 matrix, positions, normals, matIndex, indices),
    plus the material ids / names in import order and their records."""
    root = ET.parse(path).getroot()
    lm = _kid(root, "library_materials")
    mats = sorted(((m.get("id"), m.get("name") or m.get("id")) for m in _kids(lm, "material")) if lm is not None else [])
    if not mats:
        mats = [("", "DefaultMaterial")]
    index = {mid: k for k, (mid, _) in enumerate(mats)}
    geos = {g.get("id"): g for g in _kids(_kid(root, "library_geometries"), "geometry")}
    vss = _kids(_kid(root, "library_visual_scenes"), "visual_scene")
    scene = _kid(root, "scene")
    vs = vss[0]
    if scene is not None and _kid(scene, "instance_visual_scene") is not None:
        want = _kid(scene, "instance_visual_scene").get("url").lstrip("#")
        vs = next(v for v in vss if v.get("id") == want)

    def prim_corners(mesh, prim):
        srcs = {}
        for s in _kids(mesh, "source"):
            acc = _kid(_kid(s, "technique_common"), "accessor")
            srcs[s.get("id")] = (_floats(_kid(s, "float_array").text), int(acc.get("stride", "1")))
        verts = {v.get("id"): [(i.get("semantic"), i.get("source").lstrip("#")) for i in _kids(v, "input")] for v in _kids(mesh, "vertices")}
        inputs = [(i.get("semantic"), i.get("source").lstrip("#"), int(i.get("offset", "0"))) for i in _kids(prim, "input")]
        stride = max(o for _, _, o in inputs) + 1
        pos = nrm = None
        for sem, src, off in inputs:
            if sem == "VERTEX":
                for vs_, vsrc in verts[src]:
                    if vs_ == "POSITION":
                        pos = (srcs[vsrc], off)
                    elif vs_ == "NORMAL":
                        nrm = (srcs[vsrc], off)
            elif sem == "NORMAL":
                nrm = (srcs[src], off)
        if _tag(prim) == "polygons":
            ps = [_ints(p.text) for p in _kids(prim, "p")]
            counts = [len(p) // stride for p in ps]
            flat = [x for p in ps for x in p]
        else:
            flat = _ints(_kid(prim, "p").text)
            counts = _ints(_kid(prim, "vcount").text) if _tag(prim) == "polylist" else [3] * (len(flat) // stride // 3)
        def get(s, c):
            (data, st), off = s
            i = flat[c * stride + off]
            return data[i * st:i * st + 3]
        tris, c0 = [], 0
        for n in counts:
            for k in range(1, n - 1):
                tris += [c0, c0 + k, c0 + k + 1]
            c0 += n
        P = np.array([get(pos, c) for c in tris], np.float32).reshape(-1, 3)
        N = np.array([get(nrm, c) for c in tris], np.float32).reshape(-1, 3)
        return P, N

    def collapse(node, acc):
        for ig in _kids(node, "instance_geometry"):
            geo = geos[ig.get("url").lstrip("#")]
            bind = {}
            bm = _kid(ig, "bind_material")
            if bm is not None:
                for im in _kids(_kid(bm, "technique_common"), "instance_material"):
                    bind[im.get("symbol")] = im.get("target").lstrip("#")
            mesh = _kid(geo, "mesh")
            for prim in mesh:
                if _tag(prim) not in ("triangles", "polylist", "polygons"):
                    continue
                sym = prim.get("material", "")
                mi = index.get(bind.get(sym, sym), 0)
                P, N = prim_corners(mesh, prim)
                acc.append((P, N, np.full(len(P), mi, np.uint32)))
        for c in _kids(node, "node"):
            collapse(c, acc)

    children = []
    for n in _kids(vs, "node"):
        acc = []
        collapse(n, acc)
        P = np.concatenate([a[0] for a in acc])
        N = np.concatenate([a[1] for a in acc])
        M = np.concatenate([a[2] for a in acc])
        children.append((n.get("name") or n.get("id"), node_matrix(n), P, N, M, np.arange(len(P), dtype=np.uint32)))
    records = [read_material(os.path.join(matdir, name + ".rgmat.json")) for _, name in mats] if matdir else []
    return children, mats, records


def check_against_reader(d, children, mats, records, extra_models=0):
    info = d["info"]
    assert info["materialIds"] == [m for m, _ in mats]
    assert info["materialNames"] == [n for _, n in mats]
    assert [c["name"] for c in info["children"]] == [c[0] for c in children]
    meshes = d["meshes"]
    nmat = len(records)
    for k, (name, M, P, N, MI, I) in enumerate(children):
        vo, io, nt = (int(x) for x in meshes[k])
        v = d["vertices"][vo:vo + len(P)]
        assert nt * 3 == len(I), name
        assert np.array_equal(v["position"], P), name
        assert np.array_equal(v["normal"], N), name
        assert np.array_equal(v["matIndex"], MI), name
        assert np.array_equal(d["indices"][io:io + len(I)], I), name
        if nmat:
            for field in S.MATERIAL.names:
                got = d["materials"][k * nmat:(k + 1) * nmat][field]
                want = np.array([r[field] for r in records])
                assert np.allclose(got, want, rtol=0, atol=0), (name, field)
        inst = d["instances"][k]
        assert int(inst["materialBufferOffset"]) == k * nmat
        # decompose (facade Transform) / recompose (toMat4) round trip of the node matrix
        assert np.allclose(inst["transform"], M[:3, :4], rtol=1e-5, atol=1e-5), name
    assert len(d["instances"]) == len(children) + extra_models


# ---- tests ------------------------------------------------------------------------------------------
def test_fixture_import(dump_exe, tmp_path):
    dae, matdir = os.path.join(FIX, "pavilion.dae"), os.path.join(FIX, "materials")
    d = run_dump(dump_exe, tmp_path, dae, matdir)
    children, mats, records = read_collada(dae, matdir)
    info = d["info"]
    assert info["upAxis"] == "Y_UP"
    assert info["materialIds"] == ["brass-mat", "clear-mat", "ghost-mat", "ground-mat", "stone-mat"]
    assert [(c["name"], c["vertices"]) for c in info["children"]] == [("Ground", 6), ("Pillars", 96), ("Orb", 24), ("Mirror", 36)]
    orb = info["children"][2]
    assert np.allclose(orb["scaling"], [1.5, 1.5, 1.5], atol=1e-6)
    q = math.radians(45) / 2
    assert np.allclose(np.abs(orb["rotation"]), [math.cos(q), 0, math.sin(q), 0], atol=1e-6)
    assert np.allclose(info["children"][3]["scaling"], [-0.8, -0.8, -0.8], atol=1e-6)  # mirrored basis
    brass, ghost = records[0], records[2]
    assert np.allclose(brass["roughness"], 0.3) and np.allclose(brass["reflectivity"], 0.7)  # basedOn stone
    assert np.allclose(ghost["diffuse"], [1, 0, 1])  # no file: the default material
    check_against_reader(d, children, mats, records)


def test_fixture_without_materials(dump_exe, tmp_path):
    dae = os.path.join(FIX, "pavilion.dae")
    d = run_dump(dump_exe, tmp_path, dae, None)
    assert len(d["materials"]) == 0
    children, mats, _ = read_collada(dae, None)
    check_against_reader(d, children, mats, [])


def test_bad_files_are_errors(dump_exe, tmp_path):
    bad = tmp_path / "bad.dae"
    bad.write_text("<COLLADA><library_visual_scenes><visual_scene id='s'><node name='a'><matrix>1 2 3</matrix>"
                   "</node></visual_scene></library_visual_scenes></COLLADA>")
    r = subprocess.run([dump_exe, str(bad), "-", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 1 and "16 numbers" in r.stderr
    trunc = tmp_path / "trunc.dae"
    trunc.write_text(open(os.path.join(FIX, "pavilion.dae")).read()[:3000])
    r = subprocess.run([dump_exe, str(trunc), "-", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 1 and "XML" in r.stderr


def test_oracle_renders_fixture(dump_exe, tmp_path, orc):
    d = run_dump(dump_exe, tmp_path, os.path.join(FIX, "pavilion.dae"), os.path.join(FIX, "materials"))
    ubo = d["ubo"].copy()
    ubo["numSamples"], ubo["maxRecursions"] = 1, 4
    sc = S.Scene("pavilion", d["vertices"], d["indices"], d["materials"], d["meshes"], d["instances"], ubo, 160, 90)
    b, n, r, st = orc.OracleScene(sc).render(nthreads=4)
    assert st["primary"] == 160 * 90
    assert st["shadow"] > 0 and st["secondary"] > 0  # glass orbs and reflective materials were hit
    assert (n[..., 3] < math.log(10000.0) * 0.25 - 1e-3).mean() > 0.3  # most pixels see geometry


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "resources", "models")), reason="reference tree not present")
def test_reference_example_scene(dump_exe, tmp_path):
    models = os.path.join(REFERENCE, "resources", "models")
    matdir = os.path.join(REFERENCE, "resources", "materials")
    d = run_dump(dump_exe, tmp_path, os.path.join(models, "room.dae"), matdir, ball=os.path.join(models, "ball.dae"))
    children, mats, records = read_collada(os.path.join(models, "room.dae"), matdir)
    assert [n for _, n in mats] == ["floor", "ph3_black", "ph3_red", "raygun", "wall"]
    assert [c[0] for c in children] == ["Raygun", "ph3_games", "room"]
    assert [len(c[2]) // 3 for c in children] == [6658, 4686 + 5742, 396 + 152]
    check_against_reader(d, children, mats, records, extra_models=1)
    ball = d["instances"][-1]
    assert np.allclose(ball["transform"][:, 3], [3, 0, -3])
    bchildren, _, _ = read_collada(os.path.join(models, "ball.dae"), matdir)
    vo = int(d["meshes"][len(children)]["vertexOffset"])
    assert np.array_equal(d["vertices"]["position"][vo:vo + len(bchildren[0][2])], bchildren[0][2])


@pytest.mark.gpu
def test_gpu_renders_fixture_like_oracle(dump_exe, tmp_path, orc):
    from test_gpu_parity import assert_image_close
    W, H = 192, 108
    d = run_dump(dump_exe, tmp_path, os.path.join(FIX, "pavilion.dae"), os.path.join(FIX, "materials"), render=(W, H))
    sc = S.Scene("pavilion", d["vertices"], d["indices"], d["materials"], d["meshes"], d["instances"], d["ubo"], W, H)
    ob, on, orr, ost = orc.OracleScene(sc).render(nthreads=4)
    assert d["stats"] == [ost["primary"], ost["shadow"], ost["secondary"]]
    assert_image_close(d["framebuffer"], orc.post(sc.ubo, ob, on, orr), "pavilion (Collada import)")
