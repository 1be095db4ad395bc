// facade_demo.cpp -- drives the C++ facade (include/rg/raygun.hpp) the way Raygun's game code does:
// builds a scene graph (nested transforms, an invisible subtree, a zero-volume subtree, a model-less
// pivot entity), renders it, resizes, renders again.  Writes the packed buffers, the instances of
// the scene walk, the UBO and the framebuffers to <out_dir> for the Python tests.
//   facade_demo <out_dir> [--walk-only]     (--walk-only: no GPU, walk + packing only)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>

#include "rg/raygun.hpp"

using namespace rg;

static std::shared_ptr<Mesh> uv_sphere(int slices, int stacks) {
    auto m = std::make_shared<Mesh>();
    for (int s = 0; s <= stacks; ++s)
        for (int j = 0; j < slices; ++j) {
            double th = M_PI * s / stacks, ph = 2 * M_PI * j / slices;
            rg_vertex v;
            std::memset(&v, 0, sizeof v);
            v.position[0] = (float)(std::sin(th) * std::cos(ph));
            v.position[1] = (float)std::cos(th);
            v.position[2] = (float)(std::sin(th) * std::sin(ph));
            std::memcpy(v.normal, v.position, sizeof v.normal);
            m->vertices.push_back(v);
        }
    for (int s = 0; s < stacks; ++s)
        for (int j = 0; j < slices; ++j) {
            uint32_t a = s * slices + j, b = s * slices + (j + 1) % slices, c = (s + 1) * slices + (j + 1) % slices,
                     d = (s + 1) * slices + j;
            if (s != 0) m->indices.insert(m->indices.end(), {a, b, c});
            if (s != stacks - 1) m->indices.insert(m->indices.end(), {a, c, d});
        }
    return m;
}

static std::shared_ptr<Mesh> quad(float h) {
    auto m = std::make_shared<Mesh>();
    float p[4][3] = {{-h, 0, -h}, {h, 0, -h}, {h, 0, h}, {-h, 0, h}};
    for (auto& q : p) {
        rg_vertex v;
        std::memset(&v, 0, sizeof v);
        std::memcpy(v.position, q, sizeof v.position);
        v.normal[1] = 1.0f;
        m->vertices.push_back(v);
    }
    m->indices = {0, 2, 1, 0, 3, 2};
    return m;
}

static std::shared_ptr<Material> material(float r, float g, float b, float refl, float transp, float ior, uint32_t effect) {
    auto m = std::make_shared<Material>();
    m->gpu.diffuse[0] = r;
    m->gpu.diffuse[1] = g;
    m->gpu.diffuse[2] = b;
    m->gpu.reflectivity = refl;
    m->gpu.transparency = transp;
    m->gpu.ior = ior;
    m->gpu.effectId = effect;
    m->gpu.roughness = 0.2f;
    return m;
}

template <class T>
static void dump(const std::string& path, const std::vector<T>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: facade_demo <out_dir> [--walk-only]\n");
        return 2;
    }
    const std::string out = argv[1];
    const bool walkOnly = argc > 2 && std::string(argv[2]) == "--walk-only";
    auto sphere = uv_sphere(16, 8);
    auto ground = quad(20.0f);
    std::vector<std::shared_ptr<Model>> models;
    auto model = [&](std::shared_ptr<Mesh> mesh, std::shared_ptr<Material> mat) {
        auto m = std::make_shared<Model>();
        m->mesh = mesh;
        m->materials = {mat};
        models.push_back(m);
        return m;
    };
    Scene scene;
    auto addEntity = [](std::shared_ptr<Entity> parent, const char* name, vec3 pos, float scale, std::shared_ptr<Model> m) {
        auto e = parent->emplaceChild(name);
        e->mutableTransform().position = pos;
        e->mutableTransform().scale(scale);
        e->model = m;
        return e;
    };
    addEntity(scene.root, "ground", {0, 0, 0}, 1.0f, model(ground, material(1, 1, 1, 0.3f, 0, 1, 1)));
    auto ring = addEntity(scene.root, "ring", {0, 1, 2}, 1.0f, nullptr);
    ring->mutableTransform().rotate(0.5235988f, {0, 1, 0});
    auto s0 = addEntity(ring, "s0", {-2, 0, 0}, 0.8f, model(sphere, material(0.9f, 0.1f, 0.1f, 0, 0, 1, 0)));
    addEntity(s0, "s0moon", {0, 1.2f, 0}, 0.4f, model(sphere, material(1, 1, 1, 0.9f, 0.98f, 1.5f, 0)));
    addEntity(ring, "s1", {0, 0, 0}, 1.0f, model(sphere, material(0.8f, 0.8f, 0.9f, 0.8f, 0, 1, 0)));
    addEntity(ring, "s2", {2, 0, 0}, 1.0f, model(sphere, material(1, 1, 1, 0.9f, 0.98f, 1.5f, 0)));
    auto hidden = addEntity(ring, "hidden", {0, 2, 0}, 1.0f, model(sphere, material(0, 0, 1, 0, 0, 1, 0)));
    hidden->setVisible(false);
    addEntity(hidden, "hiddenChild", {0, 1, 0}, 0.5f, model(sphere, material(0, 0, 1, 0, 0, 1, 0)));
    auto flat = addEntity(ring, "flat", {0, -1, 0}, 1.0f, model(sphere, material(0, 1, 1, 0, 0, 1, 0)));
    flat->mutableTransform().scaling = {1, 0, 1};
    addEntity(flat, "flatChild", {0, 1, 0}, 0.5f, model(sphere, material(0, 1, 1, 0, 0, 1, 0)));
    auto pivot = addEntity(scene.root, "pivot", {3, 0, -1}, 1.0f, nullptr);
    addEntity(pivot, "s3", {0, 0.8f, 0}, 0.8f, model(sphere, material(0.1f, 0.8f, 0.2f, 0, 0, 1, 0)));
    addEntity(scene.root, "s4", {-3, 0.6f, -2}, 0.6f, model(sphere, material(0.2f, 0.6f, 0.2f, 0.5f, 0, 1, 0)));
    scene.camera->mutableTransform().position = {0, 3, -9};
    scene.camera->mutableTransform().lookAt({0, 1, 1});
    scene.camera->fovDegrees = 60.0f;

    // names of the instanced entities in walk order
    {
        std::ofstream f(out + "/names.txt");
        scene.root->forEachEntity([&](const Entity& e) {
            if (!e.isVisible() || e.transform().isZeroVolume()) return false;
            if (e.model) f << e.name << "\n";
            return true;
        });
    }
    const uint32_t W = 320, H = 180;
    std::vector<rg_instance> inst;
    rg_ubo ubo = defaultUbo();
    ubo.numSamples = 2;
    ubo.maxRecursions = 4;
    PackedModels packed;
    if (walkOnly) {
        packed = packModels(models);
        for (size_t k = 0; k < packed.meshes.size(); ++k) packed.meshes[k]->blas = (uint32_t)k;
        inst = sceneInstances(scene);
        setCamera(ubo, *scene.camera, W, H);
    } else {
        RenderSystem rs(W, H);
        rs.setupModelBuffers(models);
        rs.ubo().numSamples = 2;
        rs.ubo().maxRecursions = 4;
        const std::vector<float>& fb = rs.render(scene);
        dump(out + "/framebuffer.bin", fb);
        ubo = rs.ubo();
        inst = rs.instancesOf(scene);
        rg_stats st = rs.stats();
        std::ofstream(out + "/stats.txt") << st.primary << " " << st.shadow << " " << st.secondary << "\n";
        rs.resize(W / 2, H / 2);  // render_system.cpp:66-81
        const std::vector<float>& small = rs.render(scene);
        dump(out + "/framebuffer_small.bin", small);
        std::vector<rg_ubo> u2{rs.ubo()};
        dump(out + "/ubo_small.bin", u2);
        packed = packModels(models);  // same packing as setupModelBuffers did
    }
    dump(out + "/vertices.bin", packed.vertices);
    dump(out + "/indices.bin", packed.indices);
    dump(out + "/materials.bin", packed.materials);
    std::vector<uint32_t> meshes;
    for (const auto& m : packed.meshes) meshes.insert(meshes.end(), {m->vertexOffset, m->indexOffset, (uint32_t)m->numFaces()});
    dump(out + "/meshes.bin", meshes);
    dump(out + "/instances.bin", inst);
    std::vector<rg_ubo> u{ubo};
    dump(out + "/ubo.bin", u);
    std::printf("instances %zu\n", inst.size());
    return 0;
}
