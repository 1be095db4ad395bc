// raygun.cpp -- the C++ facade (include/rg/raygun.hpp) over the rgcuda C ABI.
#include "../../include/rg/raygun.hpp"

#include <cstring>
#include <unordered_map>

namespace rg {

mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r;
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            float s = 0.0f;
            for (int k = 0; k < 4; ++k) s += a.m[k][row] * b.m[c][k];
            r.m[c][row] = s;
        }
    return r;
}

// inverse through the adjugate, evaluated in double and rounded once
mat4 inverse(const mat4& a) {
    double m[16], inv[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) m[4 * c + r] = a.m[c][r];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (det == 0.0) throw std::runtime_error("singular matrix");
    mat4 r;
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) r.m[c][row] = (float)(inv[4 * c + row] / det);
    return r;
}

mat4 perspective(float fovy, float aspect, float zNear, float zFar) {
    const float th = std::tan(fovy / 2.0f);
    mat4 r;
    std::memset(r.m, 0, sizeof r.m);
    r.m[0][0] = 1.0f / (aspect * th);
    r.m[1][1] = 1.0f / th;
    r.m[2][2] = zFar / (zNear - zFar);
    r.m[2][3] = -1.0f;
    r.m[3][2] = -(zFar * zNear) / (zFar - zNear);
    return r;
}

quat operator*(const quat& a, const quat& b) {
    return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
            a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z, a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x};
}

quat angleAxis(float angle, vec3 axis) {
    vec3 n = normalize(axis);
    float s = std::sin(angle * 0.5f);
    return {std::cos(angle * 0.5f), n.x * s, n.y * s, n.z * s};
}

// rotation taking the camera's -Z to `direction` with `up` as the vertical reference
quat quatLookAt(vec3 direction, vec3 up) {
    vec3 c2 = -direction;
    vec3 c0 = normalize(cross(up, c2));
    vec3 c1 = cross(c2, c0);
    // rotation matrix (columns c0, c1, c2) -> unit quaternion, largest-component method
    float m00 = c0.x, m11 = c1.y, m22 = c2.z;
    float tr = m00 + m11 + m22;
    quat q;
    if (tr > 0.0f) {
        float s = std::sqrt(tr + 1.0f) * 2.0f;
        q = {0.25f * s, (c1.z - c2.y) / s, (c2.x - c0.z) / s, (c0.y - c1.x) / s};
    } else if (m00 > m11 && m00 > m22) {
        float s = std::sqrt(1.0f + m00 - m11 - m22) * 2.0f;
        q = {(c1.z - c2.y) / s, 0.25f * s, (c1.x + c0.y) / s, (c2.x + c0.z) / s};
    } else if (m11 > m22) {
        float s = std::sqrt(1.0f + m11 - m00 - m22) * 2.0f;
        q = {(c2.x - c0.z) / s, (c1.x + c0.y) / s, 0.25f * s, (c2.y + c1.z) / s};
    } else {
        float s = std::sqrt(1.0f + m22 - m00 - m11) * 2.0f;
        q = {(c0.y - c1.x) / s, (c2.x + c0.z) / s, (c2.y + c1.z) / s, 0.25f * s};
    }
    return q;
}

mat4 toMat4(const quat& q) {
    const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z, xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    mat4 r;
    r.m[0][0] = 1 - 2 * (yy + zz); r.m[0][1] = 2 * (xy + wz);     r.m[0][2] = 2 * (xz - wy);
    r.m[1][0] = 2 * (xy - wz);     r.m[1][1] = 1 - 2 * (xx + zz); r.m[1][2] = 2 * (yz + wx);
    r.m[2][0] = 2 * (xz + wy);     r.m[2][1] = 2 * (yz - wx);     r.m[2][2] = 1 - 2 * (xx + yy);
    return r;
}

vec3 rotate(const quat& q, vec3 v) {
    quat p{0, v.x, v.y, v.z}, c{q.w, -q.x, -q.y, -q.z};
    quat r = q * p * c;
    return {r.x, r.y, r.z};
}

mat4 Transform::toMat4() const {
    mat4 t, s;
    t.m[3][0] = position.x;
    t.m[3][1] = position.y;
    t.m[3][2] = position.z;
    s.m[0][0] = scaling.x;
    s.m[1][1] = scaling.y;
    s.m[2][2] = scaling.z;
    return t * rg::toMat4(rotation) * s;
}

Transform operator*(const Transform& x, const Transform& y) {
    Transform r;
    r.position = rotate(x.rotation, x.scaling * y.position) + x.position;
    r.rotation = x.rotation * y.rotation;
    r.scaling = x.scaling * y.scaling;
    return r;
}

Material::Material() {
    std::memset(&gpu, 0, sizeof gpu);
    gpu.diffuse[0] = 1.0f;  // gpu_material.def defaults
    gpu.diffuse[2] = 1.0f;
    gpu.specular[0] = gpu.specular[1] = gpu.specular[2] = 1.0f;
    gpu.ior = 1.0f;
    gpu.rayConsumption = 1;
}

Transform Entity::globalTransform() const { return m_parent ? m_parent->globalTransform() * m_transform : m_transform; }

void Entity::addChild(std::shared_ptr<Entity> child) {
    child->m_parent = this;
    m_children.push_back(std::move(child));
}

std::shared_ptr<Entity> Entity::emplaceChild(const std::string& childName) {
    auto e = std::make_shared<Entity>(childName);
    addChild(e);
    return e;
}

void Entity::forEachEntity(const std::function<bool(const Entity&)>& f) const {
    if (!f(*this)) return;
    for (const auto& c : m_children) c->forEachEntity(f);
}

void Camera::updateProjection(uint32_t width, uint32_t height) {
    float aspect = (float)width / (float)height;
    if (!std::isfinite(aspect)) aspect = 16.0f / 9.0f;
    m_projection = perspective(fovDegrees * 3.14159265358979f / 180.0f, aspect, zNear, zFar);
    m_projection.m[1][1] *= -1.0f;  // glm's flipped Y (camera.cpp:45-46)
}

PackedModels packModels(const std::vector<std::shared_ptr<Model>>& models) {
    PackedModels p;
    std::unordered_map<const Mesh*, bool> seen;
    for (const auto& m : models)
        if (m && m->mesh && !seen[m->mesh.get()]) {
            seen[m->mesh.get()] = true;
            p.meshes.push_back(m->mesh);
        }
    for (const auto& mesh : p.meshes) {
        mesh->vertexOffset = (uint32_t)p.vertices.size();
        mesh->indexOffset = (uint32_t)p.indices.size();
        p.vertices.insert(p.vertices.end(), mesh->vertices.begin(), mesh->vertices.end());
        p.indices.insert(p.indices.end(), mesh->indices.begin(), mesh->indices.end());
    }
    for (const auto& m : models) {
        if (!m) continue;
        m->materialOffset = (uint32_t)p.materials.size();
        for (const auto& mat : m->materials) p.materials.push_back(mat->gpu);
    }
    return p;
}

std::vector<rg_instance> sceneInstances(const Scene& scene) {
    std::vector<rg_instance> out;
    scene.root->forEachEntity([&](const Entity& e) {
        if (!e.isVisible()) return false;                // do not descend into invisible subtrees
        if (e.transform().isZeroVolume()) return false;  // nor zero-volume ones
        if (!e.model) return true;                        // no model: its children may still render
        rg_instance i;
        std::memset(&i, 0, sizeof i);
        const mat4 m = e.globalTransform().toMat4();
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) i.transform[r][c] = m.m[c][r];  // transpose: 3x4 row-major
        i.blas = e.model->mesh->blas;
        i.mask = 0xFF;
        i.vertexBufferOffset = e.model->mesh->vertexOffset;
        i.indexBufferOffset = e.model->mesh->indexOffset;
        i.materialBufferOffset = e.model->materialOffset;
        out.push_back(i);
        return true;
    });
    return out;
}

rg_ubo defaultUbo() {
    rg_ubo u;
    std::memset(&u, 0, sizeof u);
    vec3 l = normalize(vec3(0.4f, -0.6f, -0.8f));
    u.lightDir[0] = l.x;
    u.lightDir[1] = l.y;
    u.lightDir[2] = l.z;
    u.numSamples = 1;
    u.maxRecursions = 5;
    return u;
}

void setCamera(rg_ubo& u, const Camera& camera, uint32_t width, uint32_t height) {
    Camera c = camera;
    c.updateProjection(width, height);
    const mat4 vi = c.viewInverse(), pi = c.projInverse();
    std::memcpy(u.viewInverse, vi.m, sizeof u.viewInverse);
    std::memcpy(u.projInverse, pi.m, sizeof u.projInverse);
    u.clearColor[0] = u.clearColor[1] = u.clearColor[2] = 0.2f;
}

RenderSystem::RenderSystem(uint32_t width, uint32_t height, int device, uint32_t flags, uint64_t hbmBudget) : m_w(width), m_h(height) {
    rg_device_opts o{device, flags, hbmBudget};
    rg_status s = rg_create(&m_ctx, &o);
    if (s != RG_OK) throw std::runtime_error("rg_create failed: " + std::to_string(s));
    check(rg_set_resolution(m_ctx, width, height), "rg_set_resolution");
    m_framebuffer.assign(4ull * width * height, 0.0f);
    resetUniformBuffer();
}

RenderSystem::~RenderSystem() {
    if (m_ctx) rg_destroy(m_ctx);
}

void RenderSystem::check(rg_status s, const char* what) const {
    if (s != RG_OK) throw std::runtime_error(std::string(what) + ": " + rg_last_error(m_ctx));
}

void RenderSystem::setupModelBuffers(const std::vector<std::shared_ptr<Model>>& models) {
    m_models = models;
    PackedModels p = packModels(models);
    m_meshes = p.meshes;
    check(rg_upload_geometry(m_ctx, p.vertices.data(), (uint32_t)p.vertices.size(), p.indices.data(), (uint32_t)p.indices.size(),
                             p.materials.data(), (uint32_t)p.materials.size()),
          "rg_upload_geometry");
    for (const auto& mesh : m_meshes)
        check(rg_build_blas(m_ctx, mesh->vertexOffset, mesh->indexOffset, (uint32_t)mesh->numFaces(), &mesh->blas), "rg_build_blas");
}

void RenderSystem::updateModelBuffers() {
    PackedModels p = packModels(m_models);
    check(rg_update_vertices(m_ctx, 0, p.vertices.data(), (uint32_t)p.vertices.size()), "rg_update_vertices");
    check(rg_update_materials(m_ctx, 0, p.materials.data(), (uint32_t)p.materials.size()), "rg_update_materials");
    for (const auto& mesh : m_meshes) check(rg_refit_blas(m_ctx, mesh->blas), "rg_refit_blas");
}

void RenderSystem::resetUniformBuffer() { m_ubo = defaultUbo(); }

void RenderSystem::updateUniformBuffer(const Camera& camera) { setCamera(m_ubo, camera, m_w, m_h); }

std::vector<rg_instance> RenderSystem::instancesOf(const Scene& scene) const { return sceneInstances(scene); }

const std::vector<float>& RenderSystem::render(const Scene& scene) {
    updateUniformBuffer(*scene.camera);
    std::vector<rg_instance> inst = instancesOf(scene);
    check(rg_build_tlas(m_ctx, inst.data(), (uint32_t)inst.size()), "rg_build_tlas");
    check(rg_render(m_ctx, &m_ubo, useFXAA ? 1 : 0), "rg_render");
    check(rg_download(m_ctx, m_framebuffer.data()), "rg_download");
    return m_framebuffer;
}

void RenderSystem::resize(uint32_t width, uint32_t height) {
    check(rg_set_resolution(m_ctx, width, height), "rg_set_resolution");
    m_w = width;
    m_h = height;
    m_framebuffer.assign(4ull * width * height, 0.0f);
}

rg_timings RenderSystem::timings() {
    rg_timings t;
    check(rg_get_timings(m_ctx, &t), "rg_get_timings");
    return t;
}

rg_stats RenderSystem::stats() {
    rg_stats s;
    check(rg_get_stats(m_ctx, &s), "rg_get_stats");
    return s;
}

}  // namespace rg
