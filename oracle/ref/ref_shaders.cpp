// ref_shaders.cpp -- Raygun's own GLSL shaders compiled as C++ (the reference-compiled checker).
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref/build.py from the reference tree into the ignored
// oracle/_ref/ folder; used to pin the oracle (rg_oracle.cpp) to the reference's shader code and to
// generate the golden fixtures under tests/golden/.
//
// What is the reference's: every line of raygen.rgen/raygen.h, closesthit.rchit, miss.rmiss,
// shadowMiss.rmiss, rough_prepare.comp, rough_blur*.comp, postprocess.comp, fxaa.comp/fxaa.h.
// What is not (it lives in the Vulkan driver): BVH traversal and the triangle test, which come
// from the oracle (closest hit, ties to the smaller instance/primitive), and the image / sampler
// access rules of glsl_shim.hpp.
#include "../rg_oracle.cpp"  // oracle internals: Scene, closest_hit, rh (FP16 rounding)

#include <thread>
#include <vector>

#include "glsl_shim.hpp"

namespace rgsl {
thread_local Invocation* g_inv = nullptr;
float round_half(float f) { return rh(f); }
}  // namespace rgsl

// ---- the shaders ---------------------------------------------------------------------------------
namespace sh_raygen {
RGSL_IMPORT;
#include "raygen.rgen"
}  // namespace sh_raygen
namespace sh_chit {
RGSL_IMPORT;
#include "closesthit.rchit"
}  // namespace sh_chit
namespace sh_miss {
RGSL_IMPORT;
#include "miss.rmiss"
}  // namespace sh_miss
namespace sh_smiss {
RGSL_IMPORT;
#include "shadowMiss.rmiss"
}  // namespace sh_smiss
namespace sh_prepare {
RGSL_IMPORT;
#include "rough_prepare.comp"
}  // namespace sh_prepare
namespace sh_blur_h {
RGSL_IMPORT;
#include "rough_blur_h.comp"
}  // namespace sh_blur_h
namespace sh_blur_v {
RGSL_IMPORT;
#include "rough_blur_v.comp"
}  // namespace sh_blur_v
namespace sh_post {
RGSL_IMPORT;
#include "postprocess.comp"
}  // namespace sh_post
namespace sh_fxaa {
RGSL_IMPORT;
#include "fxaa.comp"
}  // namespace sh_fxaa

#undef payload

// ---- glue ------------------------------------------------------------------------------------------
namespace rgref {

using rgsl::vec3;
using rgsl::vec4;

const Scene* g_scene = nullptr;
thread_local uint64_t g_rays = 0;
alignas(16) thread_local unsigned char g_payload[256];

template <class U>
void fill_ubo(U& ubo, const Ubo& u) {
    for (int c = 0; c < 4; ++c) {
        ubo.viewInverse.c[c] = vec4(u.viewInverse[4 * c], u.viewInverse[4 * c + 1], u.viewInverse[4 * c + 2], u.viewInverse[4 * c + 3]);
        ubo.projInverse.c[c] = vec4(u.projInverse[4 * c], u.projInverse[4 * c + 1], u.projInverse[4 * c + 2], u.projInverse[4 * c + 3]);
    }
    ubo.clearColor = vec3(u.clearColor[0], u.clearColor[1], u.clearColor[2]);
    ubo.numSamples = u.numSamples;
    ubo.lightDir = vec3(u.lightDir[0], u.lightDir[1], u.lightDir[2]);
    ubo.maxRecursions = u.maxRecursions;
    ubo.time = u.time;
    ubo.showAlpha = u.showAlpha != 0;
    ubo.fadeColor = vec4(u.fadeColor[0], u.fadeColor[1], u.fadeColor[2], u.fadeColor[3]);
}

// one shared payload behind every shader's `payload`
void bind_payload_this_thread() {
    sh_raygen::rgref_payload = reinterpret_cast<decltype(sh_raygen::rgref_payload)>(g_payload);
    sh_chit::rgref_payload = reinterpret_cast<decltype(sh_chit::rgref_payload)>(g_payload);
    sh_miss::rgref_payload = reinterpret_cast<decltype(sh_miss::rgref_payload)>(g_payload);
    sh_smiss::rgref_payload = reinterpret_cast<decltype(sh_smiss::rgref_payload)>(g_payload);
}

struct ChitData {
    std::vector<sh_chit::Vertex> v;
    std::vector<rgsl::uint> i;
    std::vector<sh_chit::Material> m;
    std::vector<sh_chit::InstanceOffsetTableEntry> e;
} g_chit;

void bind_scene(const Scene& s, const Ubo& u) {
    g_scene = &s;
    fill_ubo(sh_raygen::ubo, u);
    fill_ubo(sh_chit::ubo, u);
    fill_ubo(sh_miss::ubo, u);
    g_chit.v.resize(s.vertices.size());
    for (size_t k = 0; k < s.vertices.size(); ++k) {
        const Vertex& a = s.vertices[k];
        g_chit.v[k].position = vec3(a.position[0], a.position[1], a.position[2]);
        g_chit.v[k].matIndex = a.matIndex;
        g_chit.v[k].normal = vec3(a.normal[0], a.normal[1], a.normal[2]);
        g_chit.v[k].pad1 = a.pad1;
    }
    g_chit.i.assign(s.indices.begin(), s.indices.end());
    g_chit.m.resize(s.materials.size());
    for (size_t k = 0; k < s.materials.size(); ++k) {
        const Material& a = s.materials[k];
        sh_chit::Material& b = g_chit.m[k];
        b.diffuse = vec3(a.diffuse[0], a.diffuse[1], a.diffuse[2]);
        b.transparency = a.transparency;
        b.specular = vec3(a.specular[0], a.specular[1], a.specular[2]);
        b.reflectivity = a.reflectivity;
        b.roughness = a.roughness;
        b.ior = a.ior;
        b.effectId = a.effectId;
        b.rayConsumption = a.rayConsumption;
        b.emission = a.emission;
        b.pad0 = a.pad0;
        b.pad1 = a.pad1;
        b.pad2 = a.pad2;
    }
    g_chit.e.resize(s.inst.size());
    for (size_t k = 0; k < s.inst.size(); ++k) {
        g_chit.e[k].vertexBufferOffset = s.inst[k].vOff;
        g_chit.e[k].indexBufferOffset = s.inst[k].iOff;
        g_chit.e[k].materialBufferOffset = s.inst[k].mOff;
    }
    sh_chit::vertices.v = g_chit.v.data();
    sh_chit::indices.i = g_chit.i.data();
    sh_chit::materials.m = g_chit.m.data();
    sh_chit::instanceOffsetTable.e = g_chit.e.data();
}

}  // namespace rgref

namespace rgsl {
// traceRayEXT: traversal by the oracle, then the reference's closest-hit or miss program
void trace_ray(uint cullMask, int missIndex, const vec3& o, float tmin, const vec3& d, float tmax) {
    Invocation* parent = g_inv;
    Invocation inv;
    inv.worldO = o;
    inv.worldD = d;
    Hit h{};
    h.hit = false;
    const bool zero = d.x == 0.0f && d.y == 0.0f && d.z == 0.0f;  // P3
    if (cullMask != 0u && !zero) {
        float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
        TraceStats st;
        h = closest_hit(*rgref::g_scene, of, df, tmin, tmax, st);
        rgref::g_rays++;
    }
    g_inv = &inv;
    if (h.hit) {
        const Inst& in = rgref::g_scene->inst[h.inst];
        inv.hitT = h.t;
        inv.customIndex = (int)h.inst;
        inv.primitiveID = (int)h.prim;
        for (int c = 0; c < 4; ++c) inv.objectToWorld.c[c] = vec3(in.m[c], in.m[4 + c], in.m[8 + c]);
        sh_chit::attribs = vec3(h.u, h.v, 0.0f);
        sh_chit::main();
    } else if (missIndex == 0) {
        sh_miss::main();
    } else {
        sh_smiss::main();
    }
    g_inv = parent;
}
}  // namespace rgsl

namespace rgref {

struct Images {
    int W, H;
    std::vector<float> base, normal, rough, fin, trans, A, B;
    rgsl::image2D img[7];
    Images(int w, int h) : W(w), H(h) {
        size_t n = 4 * (size_t)w * h;
        for (auto* v : {&base, &normal, &rough, &fin, &trans, &A, &B}) v->assign(n, 0.0f);
        std::vector<float>* all[7] = {&fin, &base, &normal, &rough, &trans, &A, &B};
        for (int k = 0; k < 7; ++k) {
            img[k].px = all[k]->data();
            img[k].W = w;
            img[k].H = h;
            img[k].fmt = k == 4 ? rgsl::FMT_R8_SNORM : rgsl::FMT_RGBA16F;
        }
    }
};

// compute.h bindings: finalImage, baseImage, normalImage, roughImage, roughTransitions, roughColorsA/B
#define RG_BIND_COMPUTE(ns, I, u)                       \
    rgref::fill_ubo(ns::ubo, u);                        \
    ns::finalImage = (I).img[0];                        \
    ns::baseImage = (I).img[1];                         \
    ns::normalImage = (I).img[2];                       \
    ns::roughImage = (I).img[3];                        \
    ns::roughTransitions = (I).img[4];                  \
    ns::roughColorsA = (I).img[5];                      \
    ns::roughColorsB = (I).img[6];                      \
    ns::finalSampler.img = &ns::finalImage;             \
    ns::baseSampler.img = &ns::baseImage;               \
    ns::normalSampler.img = &ns::normalImage;           \
    ns::roughSampler.img = &ns::roughImage;             \
    ns::roughTransitionsSampler.img = &ns::roughTransitions; \
    ns::roughColorsASampler.img = &ns::roughColorsA;    \
    ns::roughColorsBSampler.img = &ns::roughColorsB

// one compute dispatch over W x H invocations, rows spread over nthreads threads (the invocations of
// a dispatch write distinct pixels and read only the previous dispatch's images)
template <class F>
void dispatch(int W, int H, F main, int nthreads = 1) {
    auto rows = [&](std::atomic<int>& next) {
        rgsl::Invocation inv;
        rgsl::g_inv = &inv;
        for (;;) {
            const int y = next.fetch_add(1);
            if (y >= H) break;
            for (int x = 0; x < W; ++x) {
                inv.globalID = rgsl::uvec3((rgsl::uint)x, (rgsl::uint)y, 0u);
                main();
            }
        }
        rgsl::g_inv = nullptr;
    };
    std::atomic<int> next{0};
    if (nthreads <= 1) {
        rows(next);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back([&] { rows(next); });
    for (auto& x : th) x.join();
}

// raygen over every pixel of an already bound scene
void raygen_all(uint32_t W, uint32_t H, float* base, float* normal, float* rough, uint64_t* rays, int nthreads, uint32_t row0 = 0,
                uint32_t rowStep = 1) {
    Images I((int)W, (int)H);
    sh_raygen::image = I.img[1];
    sh_raygen::normalImage = I.img[2];
    sh_raygen::roughImage = I.img[3];
    if (nthreads < 1) nthreads = 1;
    std::vector<uint64_t> counts(nthreads, 0);
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t] {
            bind_payload_this_thread();
            g_rays = 0;
            rgsl::Invocation inv;
            inv.launchSize = rgsl::uvec3(W, H, 1u);
            for (;;) {
                const uint32_t y = row0 + next.fetch_add(1) * rowStep;
                if (y >= H) break;
                for (uint32_t x = 0; x < W; ++x) {
                    inv.launchID = rgsl::uvec3(x, y, 0u);
                    rgsl::g_inv = &inv;
                    sh_raygen::main();
                }
            }
            counts[t] = g_rays;
        });
    for (auto& x : th) x.join();
    std::memcpy(base, I.base.data(), 16 * (size_t)W * H);
    std::memcpy(normal, I.normal.data(), 16 * (size_t)W * H);
    std::memcpy(rough, I.rough.data(), 16 * (size_t)W * H);
    if (rays) {
        uint64_t tot = 0;
        for (auto c : counts) tot += c;
        *rays = tot;
    }
}

}  // namespace rgref

extern "C" {

// the reference raygen for every pixel: base / normal / rough images (W*H*4 floats each)
int ref_render(const void* vertices, uint32_t nv, const uint32_t* indices, uint32_t ni, const void* materials, uint32_t nm,
               const uint32_t* meshes, uint32_t nmesh, const void* instances, uint32_t ninst, const void* ubo, uint32_t W,
               uint32_t H, float* base, float* normal, float* rough, uint64_t* rays, int nthreads) {
    orc_scene* sc = orc_scene_create(vertices, nv, indices, ni, materials, nm, meshes, nmesh, instances, ninst);
    rgref::bind_scene(*(const Scene*)sc, *(const Ubo*)ubo);
    rgref::raygen_all(W, H, base, normal, rough, rays, nthreads);
    orc_scene_destroy(sc);
    return 0;
}

// the same on an oracle scene that persists across frames (orc_scene_refit / orc_scene_set_instances
// between calls move its instances and refit its BLASes, as a frame loop does);
// rows row0, row0 + rowStep, ... only (the others stay zero)
int ref_scene_render(orc_scene* sc, const void* ubo, uint32_t W, uint32_t H, float* base, float* normal, float* rough, uint64_t* rays,
                     int nthreads, uint32_t row0, uint32_t rowStep) {
    rgref::bind_scene(*(const Scene*)sc, *(const Ubo*)ubo);
    rgref::raygen_all(W, H, base, normal, rough, rays, nthreads, row0, rowStep < 1 ? 1 : rowStep);
    return 0;
}

// the reference compute passes of Raytracer::doRaytracing (raytracer.cpp:106-142) on the G-buffers;
// final_out = the image the reference presents (FXAA output after the swap, or finalImage);
// debug (nullable): roughTransitions, roughColorsA, roughColorsB, finalImage before FXAA
int ref_post(const void* ubo_, uint32_t W, uint32_t H, const float* base, const float* normal, const float* rough, float* final_out,
             float* debug, int fxaa, int nthreads) {
    const Ubo& u = *(const Ubo*)ubo_;
    rgref::Images I((int)W, (int)H);
    std::memcpy(I.base.data(), base, 16 * (size_t)W * H);
    std::memcpy(I.normal.data(), normal, 16 * (size_t)W * H);
    std::memcpy(I.rough.data(), rough, 16 * (size_t)W * H);
    RG_BIND_COMPUTE(sh_prepare, I, u);
    RG_BIND_COMPUTE(sh_blur_h, I, u);
    RG_BIND_COMPUTE(sh_blur_v, I, u);
    RG_BIND_COMPUTE(sh_post, I, u);
    RG_BIND_COMPUTE(sh_fxaa, I, u);
    rgref::dispatch((int)W, (int)H, sh_prepare::main, nthreads);
    for (int i = 0; i < 10; ++i) {  // raytracer.cpp:116-121
        rgref::dispatch((int)W, (int)H, sh_blur_h::main, nthreads);
        rgref::dispatch((int)W, (int)H, sh_blur_v::main, nthreads);
    }
    rgref::dispatch((int)W, (int)H, sh_post::main, nthreads);
    size_t n = 4 * (size_t)W * H;
    if (debug) {
        std::memcpy(debug, I.trans.data(), 4 * n);
        std::memcpy(debug + n, I.A.data(), 4 * n);
        std::memcpy(debug + 2 * n, I.B.data(), 4 * n);
        std::memcpy(debug + 3 * n, I.fin.data(), 4 * n);
    }
    if (fxaa) {
        rgref::dispatch((int)W, (int)H, sh_fxaa::main, nthreads);  // writes baseImage, then swap (raytracer.cpp:137-140)
        std::memcpy(final_out, I.base.data(), 4 * n);
    } else {
        std::memcpy(final_out, I.fin.data(), 4 * n);
    }
    return 0;
}

}  // extern "C"
