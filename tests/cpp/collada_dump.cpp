// collada_dump.cpp -- loads a Collada scene through the C++ facade's ingest (include/rg/collada.hpp)
// the way Raygun's example scene does (the level entity, optionally a ball entity whose model is its
// file's first node moved to (3, 0, -3), a camera at ball + (5, 10, 10) looking at it), then writes
// the packed buffers, the instances of the scene walk, the UBO and a summary for the Python tests.
//   collada_dump <level.dae> <materials dir | -> <out_dir> [--ball ball.dae] [--render W H]
// Without --render no GPU is used.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>

#include "rg/collada.hpp"
#include "rg/raygun.hpp"

using namespace rg;

template <class T>
static void dump(const std::string& path, const std::vector<T>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: collada_dump <level.dae> <materials dir | -> <out_dir> [--ball ball.dae] [--render W H]\n");
        return 2;
    }
    const std::string dae = argv[1], matDir = std::string(argv[2]) == "-" ? "" : argv[2], out = argv[3];
    std::string ballPath;
    uint32_t W = 0, H = 0;
    for (int a = 4; a < argc; ++a) {
        const std::string s = argv[a];
        if (s == "--ball" && a + 1 < argc) ballPath = argv[++a];
        else if (s == "--render" && a + 2 < argc) {
            W = (uint32_t)std::stoul(argv[++a]);
            H = (uint32_t)std::stoul(argv[++a]);
        }
    }
    try {
        Scene scene;
        ColladaInfo info;
        auto level = loadColladaEntity("level", dae, matDir, &info);
        scene.root->addChild(level);
        vec3 target(0, 0, 0);
        if (!ballPath.empty()) {
            auto loaded = loadColladaEntity("Ball", ballPath, matDir);
            auto ball = std::make_shared<Entity>("Ball");
            ball->model = loaded->children().at(0)->model;
            ball->mutableTransform().position = vec3(3.0f, 0.0f, -3.0f);
            scene.root->addChild(ball);
            target = ball->transform().position;
        }
        scene.camera->mutableTransform().position = target + vec3(5.0f, 10.0f, 10.0f);
        scene.camera->mutableTransform().lookAt(target);

        std::vector<std::shared_ptr<Model>> models;
        scene.root->forEachEntity([&](const Entity& e) {
            if (e.model) models.push_back(e.model);
            return true;
        });
        // summary
        {
            std::ofstream f(out + "/info.json");
            f << "{\"upAxis\": \"" << info.upAxis << "\", \"materialIds\": [";
            for (size_t k = 0; k < info.materialIds.size(); ++k) f << (k ? ", " : "") << "\"" << info.materialIds[k] << "\"";
            f << "], \"materialNames\": [";
            for (size_t k = 0; k < info.materialNames.size(); ++k) f << (k ? ", " : "") << "\"" << info.materialNames[k] << "\"";
            f << "], \"children\": [";
            bool first = true;
            for (const auto& c : level->children()) {
                const Transform& t = c->transform();
                f << (first ? "" : ", ") << "{\"name\": \"" << c->name << "\", \"vertices\": " << c->model->mesh->vertices.size()
                  << ", \"indices\": " << c->model->mesh->indices.size() << ", \"position\": [" << t.position.x << ", "
                  << t.position.y << ", " << t.position.z << "], \"rotation\": [" << t.rotation.w << ", " << t.rotation.x << ", "
                  << t.rotation.y << ", " << t.rotation.z << "], \"scaling\": [" << t.scaling.x << ", " << t.scaling.y << ", "
                  << t.scaling.z << "]}";
                first = false;
            }
            f << "]}\n";
        }
        std::vector<rg_instance> inst;
        rg_ubo ubo = defaultUbo();
        PackedModels packed;
        if (W == 0) {
            packed = packModels(models);
            for (size_t k = 0; k < packed.meshes.size(); ++k) packed.meshes[k]->blas = (uint32_t)k;
            inst = sceneInstances(scene);
            setCamera(ubo, *scene.camera, 640, 360);
        } else {
            RenderSystem rs(W, H);
            rs.setupModelBuffers(models);
            const std::vector<float>& fb = rs.render(scene);
            dump(out + "/framebuffer.bin", fb);
            ubo = rs.ubo();
            inst = rs.instancesOf(scene);
            rg_stats st = rs.stats();
            std::ofstream(out + "/stats.txt") << st.primary << " " << st.shadow << " " << st.secondary << "\n";
            packed = packModels(models);
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
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
