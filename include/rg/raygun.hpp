// raygun.hpp -- C++ facade with Raygun's render-facing shape over the rgcuda C ABI.
//
// A Scene of Entities (transform hierarchy, visibility, Models of Meshes + Materials) and a Camera
// go in; RenderSystem::render(Scene&) walks the scene exactly as TopLevelAS does
// (render/acceleration_structure.cpp:63-85), rebuilds the TLAS, ray traces and post-processes the
// frame on the GPU and returns the RGBA32F framebuffer.  Names and semantics follow:
//   Transform   raygun/transform.hpp:27-106        Entity  raygun/entity.hpp:32-131, entity.cpp:180-199
//   Camera      raygun/camera.hpp:30-46, camera.cpp:34-47
//   Mesh/Model  raygun/render/mesh.hpp:30-52, model.hpp:33-42
//   Material    resources/shaders/gpu_material.def:11-26 (defaults included)
//   RenderSystem raygun/render/render_system.cpp:88-330 (setupModelBuffers, resetUniformBuffer,
//               updateUniformBuffer, render) + Raytracer::setupBottomLevelAS / setupTopLevelAS
// The glm math the reference uses (quaternions, perspective with depth [0,1], inverse) is restated
// here from its mathematical definitions.
#pragma once

#include <cmath>
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../rgcuda.h"

namespace rg {

struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
inline vec3 operator+(vec3 a, vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(vec3 a, vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(vec3 a, vec3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator*(vec3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator-(vec3 a) { return {-a.x, -a.y, -a.z}; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline vec3 normalize(vec3 a) { return a * (1.0f / std::sqrt(dot(a, a))); }

// column-major 4x4 (m[col][row]), as glm stores it
struct mat4 {
    float m[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
};
mat4 operator*(const mat4& a, const mat4& b);
mat4 inverse(const mat4& a);
mat4 perspective(float fovyRadians, float aspect, float zNear, float zFar);  // right-handed, depth [0,1]

struct quat {  // w + xi + yj + zk
    float w = 1, x = 0, y = 0, z = 0;
};
quat operator*(const quat& a, const quat& b);
quat angleAxis(float angle, vec3 axis);
quat quatLookAt(vec3 direction, vec3 up);
vec3 rotate(const quat& q, vec3 v);
mat4 toMat4(const quat& q);

// raygun/transform.hpp:27-106
struct Transform {
    vec3 position{0, 0, 0};
    quat rotation{};
    vec3 scaling{1, 1, 1};
    mat4 toMat4() const;  // T * R * S
    bool isZeroVolume() const { return scaling.x * scaling.y * scaling.z == 0.0f; }
    void move(vec3 t) { position = position + t; }
    void rotate(float angle, vec3 axis) { rotation = rotation * angleAxis(angle, axis); }
    void lookAt(vec3 target) { rotation = quatLookAt(normalize(target - position), vec3(0, 1, 0)); }
    void scale(float f) { scaling = scaling * f; }
    void scale(vec3 f) { scaling = scaling * f; }
};
Transform operator*(const Transform& x, const Transform& y);  // transform.hpp:99-106

// resources/shaders/gpu_material.def:11-26 with its defaults
struct Material {
    rg_material gpu;
    Material();
};

struct Mesh {  // render/mesh.hpp:30-52
    std::vector<rg_vertex> vertices;
    std::vector<uint32_t> indices;  // mesh-local
    // filled by RenderSystem::setupModelBuffers / setupBottomLevelAS (the BufferRefs + BLAS)
    uint32_t vertexOffset = 0, indexOffset = 0, blas = 0xFFFFFFFFu;
    size_t numFaces() const { return indices.size() / 3; }
};

struct Model {  // render/model.hpp:33-42
    std::shared_ptr<Mesh> mesh;
    std::vector<std::shared_ptr<Material>> materials;
    uint32_t materialOffset = 0;  // materialBufferRef
};

class Entity {  // raygun/entity.hpp:32-131
  public:
    explicit Entity(std::string name) : name(std::move(name)) {}
    virtual ~Entity() = default;
    const Transform& transform() const { return m_transform; }
    void setTransform(const Transform& t) { m_transform = t; }
    Transform& mutableTransform() { return m_transform; }
    Transform globalTransform() const;  // parents' transforms * own (entity.cpp:187-199)
    bool isVisible() const { return m_visible; }
    void setVisible(bool v) { m_visible = v; }
    const std::vector<std::shared_ptr<Entity>>& children() const { return m_children; }
    void addChild(std::shared_ptr<Entity> child);
    std::shared_ptr<Entity> emplaceChild(const std::string& childName = "");
    // depth first; f returns false to skip the entity's children (entity.hpp:67-84)
    void forEachEntity(const std::function<bool(const Entity&)>& f) const;

    std::string name;
    std::shared_ptr<Model> model;

  private:
    Transform m_transform;
    bool m_visible = true;
    const Entity* m_parent = nullptr;
    std::vector<std::shared_ptr<Entity>> m_children;
};

class Camera : public Entity {  // raygun/camera.hpp, camera.cpp:34-47
  public:
    Camera() : Entity("camera") {}
    mat4 viewInverse() const { return globalTransform().toMat4(); }
    mat4 projInverse() const { return inverse(m_projection); }
    void updateProjection(uint32_t width, uint32_t height);
    float fovDegrees = 45.0f, zNear = 0.1f, zFar = 100.0f;

  private:
    mat4 m_projection;
};

struct Scene {  // raygun/scene.hpp:36-52
    std::shared_ptr<Camera> camera = std::make_shared<Camera>();
    std::shared_ptr<Entity> root = std::make_shared<Entity>("root");
};

// host-side parts of setupModelBuffers / TopLevelAS / updateUniformBuffer, usable without a GPU
struct PackedModels {
    std::vector<rg_vertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<rg_material> materials;
    std::vector<std::shared_ptr<Mesh>> meshes;  // distinct meshes, first-seen order
};
// packs distinct meshes back to back and each model's materials (render_system.cpp:270-330);
// fills Mesh::vertexOffset/indexOffset and Model::materialOffset
PackedModels packModels(const std::vector<std::shared_ptr<Model>>& models);
// the scene walk of TopLevelAS (acceleration_structure.cpp:63-85): customIndex = position
std::vector<rg_instance> sceneInstances(const Scene& scene);
rg_ubo defaultUbo();  // RenderSystem::resetUniformBuffer (render_system.cpp:235-244)
void setCamera(rg_ubo& ubo, const Camera& camera, uint32_t width, uint32_t height);  // :246-255

class RenderSystem {
  public:
    RenderSystem(uint32_t width, uint32_t height, int device = 0, uint32_t flags = 0, uint64_t hbmBudget = 0);
    ~RenderSystem();
    RenderSystem(const RenderSystem&) = delete;
    RenderSystem& operator=(const RenderSystem&) = delete;

    // render_system.cpp:192-223: packs the distinct meshes and every model's materials into the
    // device buffers (meshes in first-seen order) and builds one BLAS per distinct mesh
    // (raytracer.cpp:54-74)
    void setupModelBuffers(const std::vector<std::shared_ptr<Model>>& models);
    // render_system.cpp:225-233: re-uploads vertices (refitting every BLAS) and materials
    void updateModelBuffers();
    void resetUniformBuffer();                       // render_system.cpp:235-244
    void updateUniformBuffer(const Camera& camera);  // render_system.cpp:246-268
    // acceleration_structure.cpp:63-85: the instances of the scene walk
    std::vector<rg_instance> instancesOf(const Scene& scene) const;
    // render_system.cpp:88-162 without presentation: TLAS, trace, post, FXAA; framebuffer RGBA32F
    const std::vector<float>& render(const Scene& scene);
    void resize(uint32_t width, uint32_t height);   // render_system.cpp:66-81

    rg_ubo& ubo() { return m_ubo; }
    bool useFXAA = true;  // raytracer.cpp:136
    rg_timings timings();
    rg_stats stats();
    rg_ctx* context() { return m_ctx; }
    uint32_t width() const { return m_w; }
    uint32_t height() const { return m_h; }

  private:
    void check(rg_status s, const char* what) const;
    rg_ctx* m_ctx = nullptr;
    uint32_t m_w, m_h;
    rg_ubo m_ubo{};
    std::vector<std::shared_ptr<Model>> m_models;
    std::vector<std::shared_ptr<Mesh>> m_meshes;
    std::vector<float> m_framebuffer;
};

}  // namespace rg
