"""Seeded procedural scenes for the ray-tracing path.

Every array here uses the byte layouts of Raygun's shared GLSL/C++ structs:

* ``VERTEX`` (32 B)   -- resources/shaders/vertex.def:3-7, render/vertex.hpp:27-29
* ``MATERIAL`` (64 B) -- resources/shaders/gpu_material.def:11-26, gpu/gpu_material.hpp:27-31
* ``UBO`` (192 B)     -- resources/shaders/uniform_buffer_object.def:3-17 (std140; mat4 column-major
                         as glm stores it, ``showAlpha`` widened to a 32-bit word as std140 does)
* ``INSTANCE`` (72 B) -- the 3x4 row-major transform of VkAccelerationStructureInstanceKHR
                         (render/acceleration_structure.cpp:43-45) plus the BLAS handle and the
                         InstanceOffsetTableEntry (resources/shaders/instance_offset_table.def:1-3)

Indices are mesh-local (0..nv_mesh-1) exactly as Raygun packs them: the BLAS adds
``firstVertex`` (acceleration_structure.cpp:188-191) and the closest-hit shader adds
``vertexBufferOffset`` (closesthit.rchit:98-106).

Random numbers come from an in-repo counter-based splitmix64 stream so that the same seed
gives the same scene on every machine (numpy's Generator streams are not version-stable).
Draw order is documented at each generator.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

VERTEX = np.dtype([("position", "<f4", 3), ("matIndex", "<u4"), ("normal", "<f4", 3), ("pad1", "<f4")])
MATERIAL = np.dtype([
    ("diffuse", "<f4", 3), ("transparency", "<f4"),
    ("specular", "<f4", 3), ("reflectivity", "<f4"),
    ("roughness", "<f4"), ("ior", "<f4"), ("effectId", "<u4"), ("rayConsumption", "<u4"),
    ("emission", "<f4"), ("pad0", "<f4"), ("pad1", "<f4"), ("pad2", "<f4"),
])
UBO = np.dtype([
    ("viewInverse", "<f4", (4, 4)), ("projInverse", "<f4", (4, 4)),
    ("clearColor", "<f4", 3), ("numSamples", "<i4"),
    ("lightDir", "<f4", 3), ("maxRecursions", "<i4"),
    ("time", "<f4"), ("showAlpha", "<u4"), ("pad0", "<f4"), ("pad1", "<f4"),
    ("fadeColor", "<f4", 4),
])
INSTANCE = np.dtype([
    ("transform", "<f4", (3, 4)), ("blas", "<u4"), ("mask", "<u4"),
    ("vertexBufferOffset", "<u4"), ("indexBufferOffset", "<u4"), ("materialBufferOffset", "<u4"),
    ("pad", "<u4"),
])
MESH = np.dtype([("vertexOffset", "<u4"), ("indexOffset", "<u4"), ("triCount", "<u4")])

assert VERTEX.itemsize == 32 and MATERIAL.itemsize == 64 and UBO.itemsize == 192
assert INSTANCE.itemsize == 72 and MESH.itemsize == 12

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class Rng:
    """Counter-based splitmix64: output k of seed s is mix(s + (k+1) * golden)."""

    def __init__(self, seed: int):
        self.seed = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.counter = 0

    def u64(self, n: int) -> np.ndarray:
        k = np.arange(self.counter + 1, self.counter + 1 + n, dtype=np.uint64)
        self.counter += n
        with np.errstate(over="ignore"):
            z = self.seed + k * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))

    def uniform(self, n: int, lo=0.0, hi=1.0) -> np.ndarray:
        u = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
        return lo + (hi - lo) * u

    def normal(self, n: int, sigma=1.0) -> np.ndarray:
        """Box-Muller, one output per pair of uniforms (u1 in (0,1], u2 in [0,1))."""
        u1 = 1.0 - self.uniform(n)
        u2 = self.uniform(n)
        return sigma * np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)


@dataclasses.dataclass
class Mesh:
    positions: np.ndarray  # (nv, 3) float64
    normals: np.ndarray    # (nv, 3) float64
    indices: np.ndarray    # (nt, 3) uint32, mesh-local


@dataclasses.dataclass
class Scene:
    name: str
    vertices: np.ndarray   # VERTEX
    indices: np.ndarray    # uint32, mesh-local triples
    materials: np.ndarray  # MATERIAL
    meshes: np.ndarray     # MESH, one entry per BLAS
    instances: np.ndarray  # INSTANCE, in scene-walk order (customIndex = position)
    ubo: np.ndarray        # UBO, shape (1,)
    width: int
    height: int

    @property
    def tri_count(self) -> int:
        return int(self.meshes["triCount"].sum())

    @property
    def instanced_tri_count(self) -> int:
        return int(self.meshes["triCount"][self.instances["blas"]].sum())


# ----------------------------------------------------------------------------- meshes

def uv_sphere(slices=32, stacks=16) -> Mesh:
    """Unit UV sphere: (stacks+1) rings of ``slices`` vertices, pole rings collapsed.

    Triangles = slices*2 (pole fans) + slices*(stacks-2)*2 = 960 for 32x16.
    """
    th = np.arange(stacks + 1) * (math.pi / stacks)
    ph = np.arange(slices) * (2.0 * math.pi / slices)
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    pos = np.stack([st * np.cos(ph)[None, :], np.broadcast_to(ct, (stacks + 1, slices)),
                    st * np.sin(ph)[None, :]], axis=-1).reshape(-1, 3)
    tris = []
    for s in range(stacks):
        for j in range(slices):
            a = s * slices + j
            b = s * slices + (j + 1) % slices
            c = (s + 1) * slices + (j + 1) % slices
            d = (s + 1) * slices + j
            if s != 0:
                tris.append((a, b, c))
            if s != stacks - 1:
                tris.append((a, c, d))
    idx = np.asarray(tris, dtype=np.uint32)
    return Mesh(pos, pos.copy(), idx)


def quad(half: float) -> Mesh:
    pos = np.array([[-half, 0, -half], [half, 0, -half], [half, 0, half], [-half, 0, half]], dtype=np.float64)
    nrm = np.tile([0.0, 1.0, 0.0], (4, 1))
    return Mesh(pos, nrm, np.array([[0, 2, 1], [0, 3, 2]], dtype=np.uint32))


def icosphere(subdiv: int) -> Mesh:
    """Unit icosphere with 20*4^subdiv triangles (shared midpoint vertices)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        m = inv.reshape(3, -1).T + base  # midpoints of edges (01, 12, 20)
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1),
                            np.stack([c, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return Mesh(v, v.copy(), f.astype(np.uint32))


def torus(major_segments=64, minor_segments=32, R=1.0, r=0.35) -> Mesh:
    u = np.arange(major_segments) * (2 * math.pi / major_segments)
    w = np.arange(minor_segments) * (2 * math.pi / minor_segments)
    cu, su = np.cos(u)[:, None], np.sin(u)[:, None]
    cw, sw = np.cos(w)[None, :], np.sin(w)[None, :]
    pos = np.stack([(R + r * cw) * cu, np.broadcast_to(r * sw, (major_segments, minor_segments)),
                    (R + r * cw) * su], -1).reshape(-1, 3)
    nrm = np.stack([cw * cu, np.broadcast_to(sw, (major_segments, minor_segments)), cw * su], -1).reshape(-1, 3)
    i = np.arange(major_segments)[:, None]
    j = np.arange(minor_segments)[None, :]
    a = i * minor_segments + j
    b = ((i + 1) % major_segments) * minor_segments + j
    c = ((i + 1) % major_segments) * minor_segments + (j + 1) % minor_segments
    d = i * minor_segments + (j + 1) % minor_segments
    idx = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return Mesh(pos, nrm, idx.astype(np.uint32))


def heightfield(rng: Rng, n=256, disp=0.5) -> Mesh:
    """n x n grid with unit cell spacing (x, z in [-(n-1)/2, (n-1)/2]) and heights y ~ U[0, disp];
    (n-1)^2*2 triangles.  Draws n*n uniforms (row-major) for the heights."""
    xs = np.arange(n, dtype=np.float64) - (n - 1) / 2.0
    gx, gz = np.meshgrid(xs, xs, indexing="xy")
    gy = rng.uniform(n * n, 0.0, disp).reshape(n, n)
    pos = np.stack([gx, gy, gz], -1).reshape(-1, 3)
    # normals from central differences of the height grid
    dyx = np.gradient(gy, 1.0, axis=1)
    dyz = np.gradient(gy, 1.0, axis=0)
    nrm = np.stack([-dyx, np.ones_like(gy), -dyz], -1).reshape(-1, 3)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    i = np.arange(n - 1)[:, None]
    j = np.arange(n - 1)[None, :]
    a = i * n + j
    b = i * n + j + 1
    c = (i + 1) * n + j + 1
    d = (i + 1) * n + j
    idx = np.concatenate([np.stack([a, c, b], -1).reshape(-1, 3), np.stack([a, d, c], -1).reshape(-1, 3)])
    return Mesh(pos, nrm, idx.astype(np.uint32))


# ----------------------------------------------------------------------------- camera / ubo

def look_at_view_inverse(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Camera-to-world matrix T*R with R = glm::quatLookAt(dir, up) (camera looks down -Z).

    Mirrors Transform::lookAt + Transform::toMat4 (transform.hpp:38-46,82-86) used by
    Camera::viewInverse (camera.hpp:34).
    """
    eye = np.asarray(eye, np.float64)
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    c2 = -f
    c0 = np.cross(np.asarray(up, np.float64), c2)
    c0 /= np.linalg.norm(c0)
    c1 = np.cross(c2, c0)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = c0, c1, c2, eye
    return m


def perspective_inverse(fovy_deg: float, aspect: float, near=0.1, far=100.0) -> np.ndarray:
    """inverse(glm::perspectiveRH_ZO(...)) with the Y flip of Camera::updateProjection (camera.cpp:34-47)."""
    th = math.tan(math.radians(fovy_deg) / 2.0)
    p = np.zeros((4, 4))
    p[0, 0] = 1.0 / (aspect * th)
    p[1, 1] = -1.0 / th
    p[2, 2] = far / (near - far)
    p[3, 2] = -1.0
    p[2, 3] = -(far * near) / (far - near)
    return np.linalg.inv(p)


def make_ubo(eye, target, fovy_deg, width, height, light_dir, num_samples, max_recursions,
             fade=(0.0, 0.0, 0.0, 0.0), show_alpha=False, time=0.0) -> np.ndarray:
    """UBO with the defaults of RenderSystem::resetUniformBuffer/updateUniformBuffer
    (render_system.cpp:235-268): clearColor 0.2, fade off."""
    u = np.zeros(1, dtype=UBO)
    u["viewInverse"][0] = look_at_view_inverse(eye, target).T.astype(np.float32)   # column-major
    u["projInverse"][0] = perspective_inverse(fovy_deg, width / height).T.astype(np.float32)
    u["clearColor"][0] = (0.2, 0.2, 0.2)
    u["numSamples"][0] = num_samples
    ld = np.asarray(light_dir, np.float64)
    u["lightDir"][0] = (ld / np.linalg.norm(ld)).astype(np.float32)
    u["maxRecursions"][0] = max_recursions
    u["time"][0] = time
    u["showAlpha"][0] = 1 if show_alpha else 0
    u["fadeColor"][0] = fade
    return u


# ----------------------------------------------------------------------------- assembly

def _material(diffuse, transparency=0.0, specular=(1, 1, 1), reflectivity=0.0, roughness=0.0,
              ior=1.0, effect_id=0, ray_consumption=1, emission=0.0):
    m = np.zeros(1, dtype=MATERIAL)
    m["diffuse"], m["transparency"], m["specular"] = diffuse, transparency, specular
    m["reflectivity"], m["roughness"], m["ior"] = reflectivity, roughness, ior
    m["effectId"], m["rayConsumption"], m["emission"] = effect_id, ray_consumption, emission
    return m


def random_materials(rng: Rng, n: int) -> np.ndarray:
    """The sphere material distribution (per material, in this draw order):
    albedo U[0,1]^3, class u (<0.5 diffuse, <0.75 reflective, else refractive),
    reflectivity U[0.2,1] (used by reflective), roughness U[0,0.5].
    Refractive materials take glass.rgmat.json's transparency 0.98 / reflectivity 0.9 / IOR 1.5."""
    out = np.zeros(n, dtype=MATERIAL)
    for k in range(n):
        alb = rng.uniform(3)
        cls = rng.uniform(1)[0]
        refl = rng.uniform(1, 0.2, 1.0)[0]
        rough = rng.uniform(1, 0.0, 0.5)[0]
        if cls < 0.5:
            out[k] = _material(alb, roughness=rough)
        elif cls < 0.75:
            out[k] = _material(alb, reflectivity=refl, roughness=rough)
        else:
            out[k] = _material(alb, transparency=0.98, reflectivity=0.9, ior=1.5, roughness=rough)
    return out


def floor_material() -> np.ndarray:
    """resources/materials/floor.rgmat.json: white, reflectivity 0.3, grid effect (effectId 1)."""
    return _material((1.0, 1.0, 1.0), reflectivity=0.3, effect_id=1)


def _pack_vertices(positions, normals, mat_index) -> np.ndarray:
    v = np.zeros(len(positions), dtype=VERTEX)
    v["position"] = positions.astype(np.float32)
    v["normal"] = normals.astype(np.float32)
    v["matIndex"] = mat_index
    return v


def _finish(name, parts, materials, instances, ubo, width, height) -> Scene:
    """parts: list of (Mesh, matIndex array) -> one BLAS each, packed back to back
    like RenderSystem::updateVertexAndIndexBuffer (render_system.cpp:270-304)."""
    verts, idxs, meshes = [], [], np.zeros(len(parts), dtype=MESH)
    vo = io = 0
    for k, (mesh, mi) in enumerate(parts):
        verts.append(_pack_vertices(mesh.positions, mesh.normals, mi))
        idxs.append(mesh.indices.reshape(-1))
        meshes[k] = (vo, io, len(mesh.indices))
        vo += len(mesh.positions)
        io += mesh.indices.size
    inst = instances
    inst["vertexBufferOffset"] = meshes["vertexOffset"][inst["blas"]]
    inst["indexBufferOffset"] = meshes["indexOffset"][inst["blas"]]
    return Scene(name, np.concatenate(verts), np.concatenate(idxs).astype(np.uint32), materials,
                 meshes, inst, ubo, width, height)


def identity_instance(blas=0, material_offset=0) -> np.ndarray:
    i = np.zeros(1, dtype=INSTANCE)
    i["transform"][0] = np.eye(4)[:3]
    i["blas"], i["mask"], i["materialBufferOffset"] = blas, 0xFF, material_offset
    return i


def spheres_scene(n_spheres=64, width=640, height=360, num_samples=1, max_recursions=4,
                  slices=32, stacks=16, seed=0, ground_half=30.0, name=None) -> Scene:
    """The single-level sphere scene: ground quad (2 tris, floor material, grid effect) plus
    ``n_spheres`` UV spheres merged into ONE mesh / ONE BLAS under an identity instance.

    Draw order per sphere: centre (x,y,z) in [-10,10]x[0.5,6]x[-10,10], radius U[0.3,1.5],
    then its material (random_materials order). Camera (0,5,-20) -> origin, vFOV 60 deg,
    light dir normalize(-0.4,-1,0.3).  Defaults = 640x360, 1 spp, depth 4, 61,442 triangles.
    """
    rng = Rng(seed)
    unit = uv_sphere(slices, stacks)
    pos = [quad(ground_half).positions]
    nrm = [quad(ground_half).normals]
    idx = [quad(ground_half).indices]
    mat_idx = [np.zeros(4, np.uint32)]
    mats = [floor_material()]
    base = 4
    for k in range(n_spheres):
        c = np.array([rng.uniform(1, -10, 10)[0], rng.uniform(1, 0.5, 6)[0], rng.uniform(1, -10, 10)[0]])
        r = rng.uniform(1, 0.3, 1.5)[0]
        mats.append(random_materials(rng, 1))
        pos.append(unit.positions * r + c)
        nrm.append(unit.normals)
        idx.append(unit.indices + base)
        mat_idx.append(np.full(len(unit.positions), k + 1, np.uint32))
        base += len(unit.positions)
    mesh = Mesh(np.concatenate(pos), np.concatenate(nrm), np.concatenate(idx))
    ubo = make_ubo((0, 5, -20), (0, 0, 0), 60.0, width, height, (-0.4, -1.0, 0.3), num_samples, max_recursions)
    return _finish(name or f"spheres{n_spheres}_{width}x{height}", [(mesh, np.concatenate(mat_idx))],
                   np.concatenate(mats), identity_instance(), ubo, width, height)


def sphere_scene() -> Scene:
    """640x360, 1 spp, depth 4, 64 spheres + ground = 61,442 triangles, single-level BVH."""
    return spheres_scene(name="spheres")


# ----------------------------------------------------------------------------- two-level scene

def _rot_axis_angle(axis, angle):
    axis = np.asarray(axis, np.float64)
    axis = axis / np.linalg.norm(axis)
    x, y, z = axis
    c, s = math.cos(angle), math.sin(angle)
    C = 1 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


def _random_axis(rng: Rng):
    z = rng.uniform(1, -1, 1)[0]
    a = rng.uniform(1, 0, 2 * math.pi)[0]
    s = math.sqrt(max(0.0, 1 - z * z))
    return np.array([s * math.cos(a), s * math.sin(a), z])


GAME_FRAME_MESH_COUNTS = (300, 250, 150, 50, 130, 130, 7, 7)
"""Instances per mesh for the game-frame scene, in mesh order
(ico3, ico4, ico5, ico6, torusA, torusB, heightA, heightB): 1024 instances, ~11.7M triangles."""


def instanced_scene(width=1920, height=1080, num_samples=4, max_recursions=5, seed=1,
                    counts=GAME_FRAME_MESH_COUNTS, hf_n=256, ico_levels=(3, 4, 5, 6), name="game-frame") -> Scene:
    """The two-level game-frame scene: 8 meshes (icospheres subdiv 3..6, two 64x32 tori,
    two 256x256 unit-spaced heightfields with U[0,0.5] displacement), instanced ``sum(counts)`` times.

    Draw order: heightfield A heights, heightfield B heights, then per instance (mesh order,
    then instance order): axis (2 draws), angle U[0,2pi), scale U[0.5,2.0], position (3 draws),
    material (random_materials order). Heightfield instances are terrain tiles laid on a 4x4 grid
    instead (uniform scale to 48 x 48 world units, no rotation), still drawing the same values.
    """
    rng = Rng(seed)
    meshes = [icosphere(s) for s in ico_levels]
    meshes += [torus(64, 32, 1.0, 0.35), torus(64, 32, 1.0, 0.18)]
    meshes += [heightfield(rng, hf_n), heightfield(rng, hf_n)]
    parts = [(m, np.zeros(len(m.positions), np.uint32)) for m in meshes]
    n_inst = int(sum(counts))
    inst = np.zeros(n_inst, dtype=INSTANCE)
    mats = np.zeros(n_inst, dtype=MATERIAL)
    k = 0
    hf_k = 0
    for mesh_id, cnt in enumerate(counts):
        for _ in range(cnt):
            axis = _random_axis(rng)
            angle = rng.uniform(1, 0, 2 * math.pi)[0]
            scale = rng.uniform(1, 0.5, 2.0)[0]
            p = np.array([rng.uniform(1, -60, 60)[0], rng.uniform(1, 0.5, 14)[0], rng.uniform(1, -60, 60)[0]])
            mats[k] = random_materials(rng, 1)[0]
            if mesh_id >= 6:  # terrain tile: uniform scale to a 48 x 48 tile
                gx, gz = hf_k % 4, hf_k // 4
                m3 = np.eye(3) * (48.0 / (hf_n - 1))
                p = np.array([-72.0 + 48.0 * gx, -0.5, -72.0 + 48.0 * gz])
                hf_k += 1
                mats[k] = _material(mats[k]["diffuse"], roughness=float(mats[k]["roughness"]),
                                    reflectivity=0.3, effect_id=1)
            else:
                m3 = _rot_axis_angle(axis, angle) * scale
            t = np.zeros((3, 4))
            t[:, :3], t[:, 3] = m3, p
            inst[k]["transform"] = t.astype(np.float32)
            inst[k]["blas"], inst[k]["mask"], inst[k]["materialBufferOffset"] = mesh_id, 0xFF, k
            k += 1
    ubo = make_ubo((0, 30, -100), (0, 2, 0), 60.0, width, height, (-0.4, -1.0, 0.3), num_samples, max_recursions)
    return _finish(name, parts, mats, inst, ubo, width, height)


def game_frame_scene() -> Scene:
    return instanced_scene()


class FrameAnimator:
    """Per-frame updates of the game-frame path.

    Each frame: 10% of instances (chosen without replacement) get a rigid move composed onto their
    transform -- translation N(0,0.2) per axis, rotation by U[0,10] deg about a random axis through
    the instance origin; each BLAS is independently chosen for a refit with probability 0.05 and
    then gets per-vertex position jitter N(0,0.01) around its rest pose.
    """

    def __init__(self, scene: Scene, seed=101, move_frac=0.10, refit_prob=0.05, jitter=0.01):
        self.scene = scene
        self.rng = Rng(seed)
        self.move_frac, self.refit_prob, self.jitter = move_frac, refit_prob, jitter
        self.rest = scene.vertices["position"].copy()

    def step(self):
        """Mutate scene.instances in place; return list of (blas, new VERTEX slice) to refit."""
        s = self.scene
        n = len(s.instances)
        m = max(1, int(round(self.move_frac * n)))
        keys = self.rng.u64(n)
        chosen = np.argsort(keys, kind="stable")[:m]
        for i in chosen:
            d = self.rng.normal(3, 0.2)
            axis = _random_axis(self.rng)
            ang = math.radians(self.rng.uniform(1, 0, 10)[0])
            t = s.instances[i]["transform"].astype(np.float64)
            r = _rot_axis_angle(axis, ang)
            t[:, :3] = r @ t[:, :3]
            t[:, 3] += d
            s.instances[i]["transform"] = t.astype(np.float32)
        refits = []
        picks = self.rng.uniform(len(s.meshes))
        for b in np.nonzero(picks < self.refit_prob)[0]:
            vo = int(s.meshes[b]["vertexOffset"])
            nv = _mesh_vertex_count(s, b)
            jit = self.rng.normal(nv * 3, self.jitter).reshape(nv, 3)
            s.vertices["position"][vo:vo + nv] = (self.rest[vo:vo + nv] + jit).astype(np.float32)
            refits.append((int(b), vo, nv))
        return refits


def _mesh_vertex_count(scene: Scene, b: int) -> int:
    vo = int(scene.meshes[b]["vertexOffset"])
    if b + 1 < len(scene.meshes):
        return int(scene.meshes[b + 1]["vertexOffset"]) - vo
    return len(scene.vertices) - vo


def mesh_vertex_count(scene: Scene, b: int) -> int:
    return _mesh_vertex_count(scene, b)


# ----------------------------------------------------------------------------- batched scenes

BATCH_RESOLUTIONS = ((320, 180), (640, 360), (1280, 720), (1920, 1080))
_MESH_CACHE: dict = {}


def _catalog_mesh(kind: str) -> Mesh:
    """The seed-free meshes of the game-frame set, built once per process."""
    if kind not in _MESH_CACHE:
        if kind.startswith("ico"):
            _MESH_CACHE[kind] = icosphere(int(kind[3:]))
        elif kind == "torus_a":
            _MESH_CACHE[kind] = torus(64, 32, 1.0, 0.35)
        else:
            _MESH_CACHE[kind] = torus(64, 32, 1.0, 0.18)
    return _MESH_CACHE[kind]


BATCH_KINDS = ("ico3", "ico4", "ico5", "ico6", "torus_a", "torus_b", "heightfield")
BATCH_KIND_TRIS = (1280, 5120, 20480, 81920, 4096, 4096, 130050)


def batch_scene(rng: Rng, name: str, target_tris: float, width: int, height: int, num_samples: int,
                max_recursions: int, hf_n: int = 256) -> Scene:
    """One scene of the batched workload, built from the game-frame meshes (icospheres subdiv 3-6,
    the two 64x32 tori, 256x256 heightfields): instances are added until the instanced triangle
    count reaches ``target_tris`` (to within the smallest mesh), over a ground quad (2 triangles,
    floor material) so that every scene has a horizon.

    Draw order: per instance, the mesh kind (uniform over the kinds that still fit the remaining
    budget; the smallest kind when none fits and the scene is still empty), then for a heightfield its
    heights, then axis (2 draws), angle U[0,2pi), scale U[0.5,2], position (3 draws), material.
    Objects spread over a square of half-size R = 3 sqrt(instances) + 6 at heights U[0.5,6];
    heightfields are terrain tiles (48 x 48 world units) laid on a grid around the origin.  The
    camera looks at the centre from (0, 0.5R + 6, -1.6R - 8) with a 60 degree vertical field of view.
    """
    kinds_tris = dict(zip(BATCH_KINDS, BATCH_KIND_TRIS))
    if hf_n != 256:
        kinds_tris["heightfield"] = 2 * (hf_n - 1) ** 2
    chosen = []
    remaining = float(target_tris)
    while True:
        fits = [k for k in BATCH_KINDS if kinds_tris[k] <= remaining]
        if not fits:
            if chosen:
                break
            fits = [min(BATCH_KINDS, key=lambda k: kinds_tris[k])]
        kind = fits[min(int(rng.uniform(1, 0, len(fits))[0]), len(fits) - 1)]
        chosen.append(kind)
        remaining -= kinds_tris[kind]
    # one BLAS per distinct seed-free kind, one per heightfield instance (each has its own heights)
    half = 3.0 * math.sqrt(len(chosen)) + 6.0
    parts, blas_of = [(quad(1.6 * half + 30.0), None)], {}
    n = len(chosen) + 1
    inst = np.zeros(n, dtype=INSTANCE)
    mats = np.zeros(n, dtype=MATERIAL)
    inst[0] = identity_instance(0, 0)[0]
    mats[0] = floor_material()[0]
    hf_k = 0
    grid = max(1, int(math.ceil(math.sqrt(sum(1 for k in chosen if k == "heightfield")))))
    for i, kind in enumerate(chosen, start=1):
        if kind == "heightfield":
            parts.append((heightfield(rng, hf_n), None))
            b = len(parts) - 1
        else:
            if kind not in blas_of:
                parts.append((_catalog_mesh(kind), None))
                blas_of[kind] = len(parts) - 1
            b = blas_of[kind]
        axis = _random_axis(rng)
        angle = rng.uniform(1, 0, 2 * math.pi)[0]
        scale = rng.uniform(1, 0.5, 2.0)[0]
        p = np.array([rng.uniform(1, -half, half)[0], rng.uniform(1, 0.5, 6.0)[0], rng.uniform(1, -half, half)[0]])
        mats[i] = random_materials(rng, 1)[0]
        if kind == "heightfield":
            gx, gz = hf_k % grid, hf_k // grid
            m3 = np.eye(3) * (48.0 / (hf_n - 1))
            p = np.array([-24.0 * grid + 48.0 * gx, -0.5, -24.0 * grid + 48.0 * gz])
            hf_k += 1
            mats[i] = _material(mats[i]["diffuse"], roughness=float(mats[i]["roughness"]), reflectivity=0.3, effect_id=1)
        else:
            m3 = _rot_axis_angle(axis, angle) * scale
        t = np.zeros((3, 4))
        t[:, :3], t[:, 3] = m3, p
        inst[i]["transform"] = t.astype(np.float32)
        inst[i]["blas"], inst[i]["mask"], inst[i]["materialBufferOffset"] = b, 0xFF, i
    parts = [(m, np.zeros(len(m.positions), np.uint32)) for m, _ in parts]
    eye = (0.0, 0.5 * half + 6.0, -1.6 * half - 8.0)
    ubo = make_ubo(eye, (0, 1, 0), 60.0, width, height, (-0.4, -1.0, 0.3), num_samples, max_recursions)
    return _finish(name, parts, mats, inst, ubo, width, height)


def batch_scenes(n=64, seed=2, tri_range=(1e3, 4e6), resolutions=BATCH_RESOLUTIONS, samples=(1, 4), depths=(1, 6),
                 hf_n=256) -> list:
    """The batched-rendering workload: ``n`` independent scenes with triangle counts log-uniform in
    ``tri_range``, resolution uniform over ``resolutions``, samples uniform in ``samples`` and
    recursion depth uniform in ``depths`` (both inclusive).

    Draw order per scene: log10(triangles), resolution index, samples, depth, then the scene's own
    draws (batch_scene)."""
    rng = Rng(seed)
    lo, hi = math.log10(tri_range[0]), math.log10(tri_range[1])
    out = []
    for k in range(n):
        target = 10.0 ** rng.uniform(1, lo, hi)[0]
        w, h = resolutions[min(int(rng.uniform(1, 0, len(resolutions))[0]), len(resolutions) - 1)]
        spp = samples[0] + min(int(rng.uniform(1, 0, samples[1] - samples[0] + 1)[0]), samples[1] - samples[0])
        depth = depths[0] + min(int(rng.uniform(1, 0, depths[1] - depths[0] + 1)[0]), depths[1] - depths[0])
        out.append(batch_scene(rng, f"batch{k:02d}", target, w, h, spp, depth, hf_n))
    return out


def default_batch_scenes() -> list:
    return batch_scenes()


# ----------------------------------------------------------------------------- large terrain scenes

SERVE_RESOLUTIONS = BATCH_RESOLUTIONS + ((3840, 2160),)
_FIELD_CACHE: dict = {}


def _terrain_field(k: int, hf_n: int) -> Mesh:
    """Distinct base heightfield k (seed 4000 + k), built once per process."""
    key = (k, hf_n)
    if key not in _FIELD_CACHE:
        _FIELD_CACHE[key] = heightfield(Rng(4000 + k), hf_n)
    return _FIELD_CACHE[key]


def terrain_scene(rng: Rng, name: str, fields: int, width: int, height: int, num_samples: int, max_recursions: int,
                  hf_n: int = 708, distinct: int = 4, objects: int = 256) -> Scene:
    """A large scene: ``fields`` tessellated heightfield tiles of 2(hf_n-1)^2 triangles each (~1M at
    hf_n = 708), each its own BLAS, laid on a square grid of 48 x 48 world-unit tiles, plus
    ``objects`` instances of the game-frame meshes above them.  The tiles' vertex data comes from
    ``distinct`` base heightfields (tile k uses base k mod distinct): BLASes are built per tile, so
    device memory grows with ``fields`` while host memory does not.

    Draw order: per tile, diffuse (3 draws) and roughness; then per object the kind index, axis
    (2 draws), angle, scale U[0.5,2], position (3 draws), material (random_materials)."""
    base = [_terrain_field(k, hf_n) for k in range(min(distinct, fields))]
    kinds = [_catalog_mesh(k) for k in ("ico3", "ico4", "ico5", "ico6", "torus_a", "torus_b")]
    parts = [(m, np.zeros(len(m.positions), np.uint32)) for m in base + kinds]
    proto = _finish(name, parts, np.zeros(1, dtype=MATERIAL), np.zeros(0, dtype=INSTANCE), None, width, height)
    meshes = list(proto.meshes)
    tile_mesh = []
    for f in range(fields):
        if f < len(base):
            tile_mesh.append(f)
        else:
            meshes.append(proto.meshes[f % len(base)])
            tile_mesh.append(len(meshes) - 1)
    meshes = np.array(meshes, dtype=MESH)
    grid = max(1, int(math.ceil(math.sqrt(fields))))
    half = 24.0 * grid
    n = fields + objects
    inst = np.zeros(n, dtype=INSTANCE)
    mats = np.zeros(n, dtype=MATERIAL)
    scale = 48.0 / (hf_n - 1)
    for f in range(fields):
        diffuse = rng.uniform(3, 0.4, 1.0)
        rough = rng.uniform(1, 0.0, 0.5)[0]
        t = np.zeros((3, 4))
        t[:, :3] = np.eye(3) * scale
        t[:, 3] = (-half + 24.0 + 48.0 * (f % grid), -0.5, -half + 24.0 + 48.0 * (f // grid))
        inst[f]["transform"] = t.astype(np.float32)
        inst[f]["blas"], inst[f]["mask"], inst[f]["materialBufferOffset"] = tile_mesh[f], 0xFF, f
        mats[f] = _material(diffuse, roughness=float(rough), reflectivity=0.3, effect_id=1)[0]
    for i in range(fields, n):
        kind = min(int(rng.uniform(1, 0, len(kinds))[0]), len(kinds) - 1)
        axis = _random_axis(rng)
        angle = rng.uniform(1, 0, 2 * math.pi)[0]
        sc_ = rng.uniform(1, 0.5, 2.0)[0]
        p = np.array([rng.uniform(1, -half, half)[0], rng.uniform(1, 0.5, 6.0)[0], rng.uniform(1, -half, half)[0]])
        mats[i] = random_materials(rng, 1)[0]
        t = np.zeros((3, 4))
        t[:, :3], t[:, 3] = _rot_axis_angle(axis, angle) * sc_, p
        inst[i]["transform"] = t.astype(np.float32)
        inst[i]["blas"], inst[i]["mask"], inst[i]["materialBufferOffset"] = len(base) + kind, 0xFF, i
    inst["vertexBufferOffset"] = meshes["vertexOffset"][inst["blas"]]
    inst["indexBufferOffset"] = meshes["indexOffset"][inst["blas"]]
    eye = (0.0, 0.35 * half + 10.0, -0.9 * half - 10.0)
    ubo = make_ubo(eye, (0, 0, 0), 60.0, width, height, (-0.4, -1.0, 0.3), num_samples, max_recursions)
    return Scene(name, proto.vertices, proto.indices, mats, meshes, inst, ubo, width, height)


def reframe(scene: Scene, width: int, height: int, num_samples: int, max_recursions: int) -> np.ndarray:
    """The scene's camera at another image size / sample count / depth: same view, projection of the
    new aspect ratio."""
    u = scene.ubo.copy()
    vi = u["viewInverse"][0]
    fov = 60.0
    ubo = make_ubo((0, 0, 0), (0, 0, 1), fov, width, height, tuple(u["lightDir"][0]), num_samples, max_recursions)
    ubo["viewInverse"] = vi
    for k in ("clearColor", "time", "showAlpha", "fadeColor"):
        ubo[k] = u[k]
    return ubo
