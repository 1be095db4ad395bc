// api.cu -- the rgcuda C ABI: context, device memory, BLAS/TLAS management, frame pipeline.
//
// Replaces the Vulkan objects the reference's renderer owns (render/raytracer.cpp,
// render/render_system.cpp, render/acceleration_structure.cpp): buffers become device
// allocations, the pipeline and descriptor sets become kernel parameters, image barriers become
// stream order, and the profiler's timestamp queries (raygun/profiler.cpp:55-105) become CUDA
// events around the same five ranges.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "rg_internal.cuh"

using namespace rg;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    template <class T> T* as() const { return static_cast<T*>(p); }
};

struct BvhSet {  // buffers of one LBVH (BLAS or TLAS)
    uint32_t n = 0;
    DevBuf primBoxes, morton, order, left, right, nodeBoxes, parents, flags, wide;
};

struct BlasRec {
    uint32_t vOff = 0, iOff = 0, triCount = 0;
    uint32_t maxMat = 0;  // largest matIndex its triangles' vertices carry, as of geometry generation gen
    uint64_t gen = 0;
    BvhSet bvh;
    DevBuf tris;
};

// CUDA events of one frame's profiler ranges (raygun/profiler.def:6-10)
enum { EV_AS0, EV_AS1, EV_REFIT0, EV_REFIT1, EV_RT0, EV_POST0, EV_ROUGH1, EV_POST1, EV_COUNT };
struct FrameEvents {
    cudaEvent_t ev[EV_COUNT] = {};
    bool hasAs = false, hasRefit = false, hasFrame = false;
    std::vector<cudaEvent_t> kernel;  // (start, end) pairs around traversal launches
    size_t kernelUsed = 0;
};

// hands out the next (start, end) pair of a frame's traversal-launch events, creating them lazily
bool next_kernel_events(void* user, cudaEvent_t* a, cudaEvent_t* b) {
    FrameEvents* f = static_cast<FrameEvents*>(user);
    while (f->kernel.size() < f->kernelUsed + 2) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return false;
        f->kernel.push_back(e);
    }
    *a = f->kernel[f->kernelUsed];
    *b = f->kernel[f->kernelUsed + 1];
    f->kernelUsed += 2;
    return true;
}

}  // namespace

namespace rg {
std::atomic<uint64_t> g_launches{0};
}

// one scene slot: model buffers, BLASes and TLAS (render_system.cpp:192-223, raytracer.cpp:54-85)
struct SceneState {
    DevBuf vertices, indices, materials;
    uint32_t nv = 0, ni = 0, nm = 0;
    // Host copies the range checks read (the reference relied on Vulkan's robustBufferAccess,
    // vulkan_context.cpp:256-257; here every index, vertex and material reference is checked before
    // a kernel reads through it): the index buffer, each vertex's matIndex, and per range the
    // largest local index (iOff, triCount) and the largest matIndex of the vertices it references
    // (vOff, iOff, triCount).
    std::vector<uint32_t> hostIdx, hostMat;
    uint64_t gen = 1;  // geometry generation: every rg_upload_geometry starts a new one
    std::vector<rg_instance> hostInst;  // instances of the last host-built TLAS (empty after a device build)
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> maxIdx;
    std::map<std::tuple<uint32_t, uint32_t, uint32_t>, uint32_t> maxMat;
    std::vector<BlasRec> blas;
    DevBuf blasTable;
    DevBuf instIn, instDev, tlasLeaves;
    BvhSet tlas;
    uint32_t nInst = 0;
    bool tlasReady = false;
};

struct rg_ctx {
    int device = 0;
    uint32_t flags = 0;
    uint64_t budget = 0, allocated = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    // scene slots; sc = the selected one (geometry / BLAS / TLAS calls act on it)
    std::vector<SceneState*> scenes;
    SceneState* sc = nullptr;
    uint32_t scId = 0;
    // shared sort scratch
    DevBuf keysA, keysB, valsA, valsB, sortState, bounds, sahQueue;
    // images (raytracer.cpp:173-195)
    uint32_t W = 0, H = 0;
    DevBuf base, normal, rough, finalImg, fxaaOut, fb, dbgT, dbgA, dbgB;
    bool lastFxaa = true;
    // misc
    DevBuf counters, tmpA, tmpB, tmpC, tmpD;  // counters: 8 per-frame + 8 cumulative
    DevBuf samples, workCounter;               // per-sample payload sums, persistent-kernel work counter
    // wavefront path state
    DevBuf wfPayload, wfMeta, wfFrames, wfQO0, wfQO1, wfQD0, wfQD1, wfQP0, wfQP1, wfHitTUV, wfHitInst, wfCounts, wfOverflow;
    uint32_t* hostCount = nullptr;             // pinned words for polling the queue length and work counter
    int lastIterations = 0;
    // batch rendering: job table, per-slot job / sample index, ray-sort scratch, per-job images
    DevBuf jobTable, slotJob, slotSample, sortKeys, sortPerm, sortHist;
    DevBuf bBase, bNormal, bRough, bFinal, bFxaa, batchFb;
    std::vector<size_t> batchOffset;           // per job: first pixel in batchFb
    std::vector<uint32_t> batchW, batchH;
    uint32_t batchSlots = 1u << 25;            // path slots of the batch loop (path state ~1.6 KB each: 54 GB at most)
    TraceTune tune;
    // graph form of the batch: second stream (loop body capture), instantiated graph and what it
    // was captured for, loop words (device), launch accounting
    cudaStream_t stream2 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    std::vector<uint8_t> graphKey;
    DevBuf loopWords;
    uint64_t graphFixedKernels = 0;
    int graphBodyKernels = 0;
    uint32_t bodyRunsSeen = 0;
    bool graphPending = false;
    // learned roughness filter used by the frames (nullable), glossy reference shading seed (0 = off),
    // samples of the last frame
    rg_filter* filter = nullptr;
    uint32_t glossySeed = 0;
    uint32_t lastSamples = 1;
    std::vector<FrameEvents*> evPool, evPending;
    FrameEvents* evCur = nullptr;  // ranges recorded since the last frame
    rg_timings lastTimings{};
    bool haveFrame = false;
    // asynchronous read-back (rg_download_async): two device staging slots, copied to the host on
    // their own stream while the next frame renders; a slot is reused once its last copy finished
    cudaStream_t copyStream = nullptr;
    DevBuf readback[2];
    cudaEvent_t staged[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    bool copyIssued[2] = {false, false};
    int readbackSlot = 0;
};

namespace {

rg_status fail(rg_ctx* c, rg_status code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            return fail(c, e_ == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                            \
        }                                                                                               \
    } while (0)

#define TRY(expr)                    \
    do {                             \
        rg_status s_ = (expr);       \
        if (s_ != RG_OK) return s_;  \
    } while (0)

// largest mesh-local index of triangles [iOff/3, iOff/3 + n) of the index buffer (cached per range)
uint32_t range_max_index(SceneState& st, uint32_t iOff, uint32_t n) {
    const auto key = std::make_pair(iOff, n);
    auto it = st.maxIdx.find(key);
    if (it != st.maxIdx.end()) return it->second;
    uint32_t m = 0;
    for (size_t k = iOff, e = (size_t)iOff + 3ull * n; k < e; ++k) m = std::max(m, st.hostIdx[k]);
    st.maxIdx.emplace(key, m);
    return m;
}

// largest matIndex of the vertices vOff + index referenced by that range (the range's vertex
// references must already be known to lie inside the vertex buffer)
uint32_t range_max_material(SceneState& st, uint32_t vOff, uint32_t iOff, uint32_t n) {
    const auto key = std::make_tuple(vOff, iOff, n);
    auto it = st.maxMat.find(key);
    if (it != st.maxMat.end()) return it->second;
    uint32_t m = 0;
    for (size_t k = iOff, e = (size_t)iOff + 3ull * n; k < e; ++k) m = std::max(m, st.hostMat[(size_t)vOff + st.hostIdx[k]]);
    st.maxMat.emplace(key, m);
    return m;
}

bool range_ok(SceneState& st, uint32_t vOff, uint32_t iOff, uint32_t n, uint32_t mOff, std::string* why);

// an instance the TLAS traverses (known BLAS, non-zero mask) reaches only uploaded indices, vertices
// and materials through its offset table entry (closesthit.rchit:98-109)
bool instance_ok(SceneState& st, const rg_instance& in, std::string* why) {
    if (in.blas >= st.blas.size() || !(in.mask & 0xFFu)) return true;  // never traversed
    const BlasRec& r = st.blas[in.blas];
    if (r.gen == st.gen && in.vertexBufferOffset == r.vOff && in.indexBufferOffset == r.iOff) {
        // the BLAS's own ranges, checked when it was built: only the material offset is new
        if (r.triCount == 0 || (uint64_t)in.materialBufferOffset + r.maxMat < st.nm) return true;
        *why = "material offset + vertex matIndex outside the material buffer";
        return false;
    }
    return range_ok(st, in.vertexBufferOffset, in.indexBufferOffset, r.triCount, in.materialBufferOffset, why);
}

// the triangle range [iOff/3, iOff/3 + n) with vertex offset vOff stays inside the index and vertex
// buffers; with a material offset (mOff != ~0u) its vertices' materials stay inside the material buffer
bool range_ok(SceneState& st, uint32_t vOff, uint32_t iOff, uint32_t n, uint32_t mOff, std::string* why) {
    if (n == 0) return true;
    if ((uint64_t)iOff + 3ull * n > st.ni) {
        *why = "triangle range outside the index buffer";
        return false;
    }
    if ((uint64_t)vOff + range_max_index(st, iOff, n) >= st.nv) {
        *why = "vertex offset + index outside the vertex buffer";
        return false;
    }
    if (mOff != ~0u && (uint64_t)mOff + range_max_material(st, vOff, iOff, n) >= st.nm) {
        *why = "material offset + vertex matIndex outside the material buffer";
        return false;
    }
    return true;
}

// status word of the device-side waits: 1 when a staged tile copy of the roughness pass never
// landed, 2 when a task wait of the SAH builder gave up, 3 when a wait of the learned filter did
int* wait_status(rg_ctx* c) { return reinterpret_cast<int*>(c->counters.as<unsigned long long>() + 16); }
// polls of a staged tile copy before the roughness pass gives up (RG_POST_WAIT_LIMIT overrides; 0
// makes the pass give up on its first copy, which tests use to check the reported status -- the
// pass still waits, with the full bound, for that copy to land before it returns)
uint32_t post_wait_limit() {
    const char* env = getenv("RG_POST_WAIT_LIMIT");
    return env ? (uint32_t)strtoul(env, nullptr, 10) : (1u << 24);
}
const char* wait_failure(uint32_t code) {
    if (code == 2) return "BVH build: a task of the SAH builder was never published";
    if (code == 3) return "learned filter: a copy or tensor-core completion wait gave up";
    return "roughness pass: a staged tile copy did not complete";
}

rg_status ensure(rg_ctx* c, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return RG_OK;
    size_t grow = bytes;
    if (c->budget && c->allocated - b.cap + grow > c->budget)
        return fail(c, RG_ERR_BUDGET, "device memory budget exceeded (" + std::to_string(c->allocated - b.cap + grow) + " > " +
                                          std::to_string(c->budget) + " bytes)");
    if (b.p) {
        cudaFree(b.p);
        c->allocated -= b.cap;
        b.p = nullptr;
        b.cap = 0;
    }
    cudaError_t e = cudaMalloc(&b.p, grow);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return fail(c, RG_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b.cap = grow;
    c->allocated += grow;
    return RG_OK;
}

// bookkeeping of finished batch-graph launches (call after the stream was synchronized): launch
// accounting of the loop body runs, iteration count, the loop's iteration-limit flag
rg_status settle_graph(rg_ctx* c) {
    if (!c->graphPending) return RG_OK;
    c->graphPending = false;
    const uint32_t runs = c->hostCount[6];
    count_launch((uint64_t)(runs - c->bodyRunsSeen) * (uint64_t)c->graphBodyKernels);
    c->bodyRunsSeen = runs;
    c->lastIterations = 2 * (int)c->hostCount[4];
    if (c->hostCount[5]) {
        CK(cudaMemsetAsync(c->loopWords.as<uint32_t>() + 1, 0, sizeof(uint32_t), c->stream));
        return fail(c, RG_ERR_CUDA, "batch round loop stopped at its iteration limit");
    }
    return RG_OK;
}

void release(rg_ctx* c, DevBuf& b) {
    if (b.p) {
        cudaFree(b.p);
        c->allocated -= b.cap;
    }
    b.p = nullptr;
    b.cap = 0;
}

rg_status ensure_sort_scratch(rg_ctx* c, uint32_t n) {
    TRY(ensure(c, c->keysA, 4ull * n));
    TRY(ensure(c, c->keysB, 4ull * n));
    TRY(ensure(c, c->valsA, 4ull * n));
    TRY(ensure(c, c->valsB, 4ull * n));
    TRY(ensure(c, c->sortState, 4ull * sort_state_words(n)));
    TRY(ensure(c, c->sahQueue, sah_queue_bytes(std::min(n, kSahBlasMaxPrims))));
    TRY(ensure(c, c->bounds, 64));
    return RG_OK;
}

rg_status ensure_bvh(rg_ctx* c, BvhSet& s, uint32_t n) {
    s.n = n;
    uint64_t m = n > 1 ? n - 1 : 1;
    TRY(ensure(c, s.primBoxes, 24ull * n));
    TRY(ensure(c, s.morton, 4ull * n));
    TRY(ensure(c, s.order, 4ull * n));
    TRY(ensure(c, s.left, 4ull * m));
    TRY(ensure(c, s.right, 4ull * m));
    TRY(ensure(c, s.nodeBoxes, 24ull * m));
    TRY(ensure(c, s.parents, 8ull * n));
    TRY(ensure(c, s.flags, 4ull * m));
    TRY(ensure(c, s.wide, sizeof(WideNode) * m));
    return ensure_sort_scratch(c, n);
}

LbvhBuffers buffers(rg_ctx* c, const BvhSet& s) {
    LbvhBuffers b;
    b.n = s.n;
    b.primBoxes = s.primBoxes.as<float>();
    b.morton = s.morton.as<uint32_t>();
    b.order = s.order.as<uint32_t>();
    b.left = s.left.as<uint32_t>();
    b.right = s.right.as<uint32_t>();
    b.nodeBoxes = s.nodeBoxes.as<float>();
    b.keysA = c->keysA.as<uint32_t>();
    b.keysB = c->keysB.as<uint32_t>();
    b.valsA = c->valsA.as<uint32_t>();
    b.valsB = c->valsB.as<uint32_t>();
    b.sortState = c->sortState.as<uint32_t>();
    b.parents = s.parents.as<uint32_t>();
    b.flags = s.flags.as<uint32_t>();
    b.bounds = c->bounds.as<uint32_t>();
    b.sahQueue = c->sahQueue.as<unsigned char>();
    b.status = wait_status(c);
    return b;
}

// root box of an LBVH: internal node 0, or the single primitive's box
const float* root_box(const BvhSet& s) { return s.n > 1 ? s.nodeBoxes.as<float>() : s.primBoxes.as<float>(); }

rg_status upload_blas_entry(rg_ctx* c, uint32_t b) {
    BlasRec& r = c->sc->blas[b];
    DevBlas e;
    std::memset(&e, 0, sizeof(e));
    e.wide = r.bvh.wide.as<WideNode>();
    e.tris = r.tris.as<float4>();
    e.n = r.bvh.n;
    e.maxMat = r.maxMat;
    e.vOff = r.vOff;
    e.iOff = r.iOff;
    DevBlas* d = c->sc->blasTable.as<DevBlas>() + b;
    CK(cudaMemcpyAsync(d, &e, sizeof(DevBlas), cudaMemcpyHostToDevice, c->stream));
    if (r.bvh.n > 0) CK(cudaMemcpyAsync(d->root, root_box(r.bvh), 24, cudaMemcpyDeviceToDevice, c->stream));
    return RG_OK;
}

rg_status set_device(rg_ctx* c) {
    CK(cudaSetDevice(c->device));
    return RG_OK;
}

// event set collecting the ranges of the frame being assembled
rg_status cur_events(rg_ctx* c, FrameEvents** out) {
    if (!c->evCur) {
        if (!c->evPool.empty()) {
            c->evCur = c->evPool.back();
            c->evPool.pop_back();
        } else {
            FrameEvents* f = new FrameEvents();
            for (auto& e : f->ev) {
                cudaError_t r = cudaEventCreate(&e);
                if (r != cudaSuccess) {
                    delete f;
                    CK(r);
                }
            }
            c->evCur = f;
        }
        c->evCur->hasAs = c->evCur->hasRefit = c->evCur->hasFrame = false;
        c->evCur->kernelUsed = 0;
    }
    *out = c->evCur;
    return RG_OK;
}

DevScene scene_of(const SceneState& st) {
    DevScene s;
    s.blas = st.blasTable.as<DevBlas>();
    s.inst = st.instDev.as<DevInstance>();
    s.tlasWide = st.tlas.wide.as<WideNode>();
    s.tlasLeaves = st.tlasLeaves.as<InstRec>();
    s.tlasN = st.nInst;
    s.pad = 0;
    s.tlasRoot = root_box(st.tlas);
    s.vertices = st.vertices.as<rg_vertex>();
    s.indices = st.indices.as<uint32_t>();
    s.materials = st.materials.as<rg_material>();
    return s;
}

rg_status build_tlas_from_device_instances(rg_ctx* c, uint32_t n, bool checkOffsets) {
    c->sc->nInst = n;
    c->sc->tlasReady = false;
    TRY(ensure(c, c->sc->instDev, sizeof(DevInstance) * (size_t)(n ? n : 1)));
    TRY(ensure(c, c->sc->tlasLeaves, sizeof(InstRec) * (size_t)(n ? n : 1)));
    TRY(ensure_bvh(c, c->sc->tlas, n));
    FrameEvents* fe;
    TRY(cur_events(c, &fe));
    CK(cudaEventRecord(fe->ev[EV_AS0], c->stream));
    CK(setup_instances(c->sc->instIn.as<rg_instance>(), n, c->sc->blasTable.as<DevBlas>(), (uint32_t)c->sc->blas.size(),
                       c->sc->instDev.as<DevInstance>(), c->sc->tlas.primBoxes.as<float>(), checkOffsets, c->sc->nm, c->stream));
    if (!(c->flags & RG_FLAG_TLAS_LBVH) && n > 1 && n <= kSahMaxPrims)
        CK(sah_build(buffers(c, c->sc->tlas), false, nullptr, c->stream));
    else CK(lbvh_build(buffers(c, c->sc->tlas), c->stream));
    CK(wide_records(buffers(c, c->sc->tlas), c->sc->tlas.wide.as<WideNode>(), c->stream));
    CK(inst_records(c->sc->tlas.order.as<uint32_t>(), n, c->sc->instDev.as<DevInstance>(), c->sc->blasTable.as<DevBlas>(),
                    c->sc->tlasLeaves.as<InstRec>(), c->stream));
    CK(cudaEventRecord(fe->ev[EV_AS1], c->stream));
    fe->hasAs = true;
    c->sc->tlasReady = true;
    return RG_OK;
}

void release_bvh(rg_ctx* c, BvhSet& s) {
    DevBuf* bb[] = {&s.primBoxes, &s.morton, &s.order, &s.left, &s.right, &s.nodeBoxes, &s.parents, &s.flags, &s.wide};
    for (DevBuf* b : bb) release(c, *b);
}

void release_scene(rg_ctx* c, SceneState& st) {
    DevBuf* bufs[] = {&st.vertices, &st.indices, &st.materials, &st.blasTable, &st.instIn, &st.instDev, &st.tlasLeaves};
    for (DevBuf* b : bufs) release(c, *b);
    release_bvh(c, st.tlas);
    for (auto& r : st.blas) {
        release_bvh(c, r.bvh);
        release(c, r.tris);
    }
    st.blas.clear();
}

uint64_t scene_bytes(const SceneState& st) {
    auto bvh = [](const BvhSet& s) {
        return s.primBoxes.cap + s.morton.cap + s.order.cap + s.left.cap + s.right.cap + s.nodeBoxes.cap +
               s.parents.cap + s.flags.cap + s.wide.cap;
    };
    uint64_t b = st.vertices.cap + st.indices.cap + st.materials.cap + st.blasTable.cap + st.instIn.cap + st.instDev.cap +
                 st.tlasLeaves.cap + bvh(st.tlas);
    for (const auto& r : st.blas) b += bvh(r.bvh) + r.tris.cap;
    return b;
}

// path state of the wavefront loop for `paths` path slots
// path state for `paths` paths; queues and hit records for max(paths, hitSlots) entries
rg_status ensure_wavefront(rg_ctx* c, size_t paths, WavefrontBuffers& w, size_t hitSlots = 0) {
    const size_t P = paths ? paths : 1, Q = std::max(P, hitSlots);
    TRY(ensure(c, c->wfPayload, 64 * P));
    TRY(ensure(c, c->wfMeta, 8 * P));
    TRY(ensure(c, c->wfFrames, 144ull * kMaxFrames * P));
    TRY(ensure(c, c->wfQO0, 16 * Q));
    TRY(ensure(c, c->wfQO1, 16 * Q));
    TRY(ensure(c, c->wfQD0, 16 * Q));
    TRY(ensure(c, c->wfQD1, 16 * Q));
    TRY(ensure(c, c->wfQP0, 4 * Q));
    TRY(ensure(c, c->wfQP1, 4 * Q));
    TRY(ensure(c, c->wfHitTUV, 16 * Q));
    TRY(ensure(c, c->wfHitInst, 4 * Q));
    TRY(ensure(c, c->wfOverflow, 4 * Q));
    if (!c->wfCounts.p) {  // the overflow list length and the finished-block count start at zero
        TRY(ensure(c, c->wfCounts, 32));
        CK(cudaMemsetAsync(c->wfCounts.p, 0, 32, c->stream));
    }
    w.payload = c->wfPayload.as<float4>();
    w.meta = c->wfMeta.as<int2>();
    w.frames = c->wfFrames.p;
    w.qO[0] = c->wfQO0.as<float4>();
    w.qO[1] = c->wfQO1.as<float4>();
    w.qD[0] = c->wfQD0.as<float4>();
    w.qD[1] = c->wfQD1.as<float4>();
    w.qPath[0] = c->wfQP0.as<uint32_t>();
    w.qPath[1] = c->wfQP1.as<uint32_t>();
    w.hitTUV = c->wfHitTUV.as<float4>();
    w.hitInst = c->wfHitInst.as<uint32_t>();
    w.counts = c->wfCounts.as<uint32_t>();
    w.overflow = c->wfOverflow.as<uint32_t>();
    return RG_OK;
}

}  // namespace

extern "C" {

rg_status rg_create(rg_ctx** out, const rg_device_opts* opts) {
    if (!out) return RG_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return RG_ERR_NO_DEVICE;
    rg_ctx* c = new rg_ctx();
    if (opts) {
        c->device = opts->device;
        c->flags = opts->flags;
        c->budget = opts->hbm_budget_bytes;
    }
    if (c->device < 0 || c->device >= count) {
        delete c;
        return RG_ERR_INVALID_ARG;
    }
    if (cudaSetDevice(c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return RG_ERR_CUDA;
    }
    c->scenes.push_back(new SceneState());
    c->sc = c->scenes[0];
    // counters: 8 per frame, 8 cumulative, then one status word of the roughness pass
    if (ensure(c, c->counters, 18 * sizeof(unsigned long long)) != RG_OK) {
        delete c;
        return RG_ERR_OUT_OF_MEMORY;
    }
    cudaMemsetAsync(c->counters.p, 0, 18 * sizeof(unsigned long long), c->stream);
    if (cudaHostAlloc(&c->hostCount, 8 * sizeof(uint32_t), cudaHostAllocDefault) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copyStream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->staged[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->staged[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->copied[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->copied[1], cudaEventDisableTiming) != cudaSuccess) {
        rg_destroy(c);
        return RG_ERR_OUT_OF_MEMORY;
    }
    *out = c;
    return RG_OK;
}

rg_status rg_destroy(rg_ctx* c) {
    if (!c) return RG_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->copyStream) cudaStreamSynchronize(c->copyStream);
    release(c, c->readback[0]);
    release(c, c->readback[1]);
    for (int k = 0; k < 2; ++k) {
        if (c->staged[k]) cudaEventDestroy(c->staged[k]);
        if (c->copied[k]) cudaEventDestroy(c->copied[k]);
    }
    if (c->copyStream) cudaStreamDestroy(c->copyStream);
    DevBuf* bufs[] = {&c->keysA, &c->keysB, &c->valsA, &c->valsB, &c->sortState, &c->bounds, &c->sahQueue, &c->base, &c->normal, &c->rough,
                      &c->finalImg, &c->fxaaOut, &c->fb, &c->dbgT, &c->dbgA, &c->dbgB, &c->counters, &c->tmpA, &c->tmpB, &c->tmpC,
                      &c->tmpD, &c->samples, &c->workCounter, &c->wfPayload, &c->wfMeta, &c->wfFrames, &c->wfQO0, &c->wfQO1,
                      &c->wfQD0, &c->wfQD1, &c->wfQP0, &c->wfQP1, &c->wfHitTUV, &c->wfHitInst, &c->wfCounts, &c->wfOverflow, &c->jobTable,
                      &c->slotJob, &c->slotSample, &c->sortKeys, &c->sortPerm, &c->sortHist, &c->bBase, &c->bNormal, &c->bRough,
                      &c->bFinal, &c->bFxaa, &c->batchFb};
    for (DevBuf* b : bufs) release(c, *b);
    for (SceneState* st : c->scenes)
        if (st) {
            release_scene(c, *st);
            delete st;
        }
    std::vector<FrameEvents*> all = c->evPool;
    all.insert(all.end(), c->evPending.begin(), c->evPending.end());
    if (c->evCur) all.push_back(c->evCur);
    for (FrameEvents* f : all) {
        for (auto& e : f->ev)
            if (e) cudaEventDestroy(e);
        for (auto& e : f->kernel) cudaEventDestroy(e);
        delete f;
    }
    if (c->graphExec) cudaGraphExecDestroy(c->graphExec);
    if (c->graph) cudaGraphDestroy(c->graph);
    release(c, c->loopWords);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->hostCount) cudaFreeHost(c->hostCount);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return RG_OK;
}

const char* rg_last_error(const rg_ctx* c) { return c ? c->err.c_str() : "null context"; }

rg_status rg_upload_geometry(rg_ctx* c, const rg_vertex* v, uint32_t nv, const uint32_t* idx, uint32_t ni, const rg_material* m,
                             uint32_t nm) {
    if (!c) return RG_ERR_INVALID_ARG;
    if ((nv && !v) || (ni && !idx) || (nm && !m) || ni % 3 != 0) return fail(c, RG_ERR_INVALID_ARG, "bad geometry arrays");
    for (uint32_t k = 0; k < nm; ++k)
        if (m[k].rayConsumption < 1 || m[k].rayConsumption > 5)
            return fail(c, RG_ERR_INVALID_ARG, "material rayConsumption outside 1..5 (gpu_material.def:21)");
    for (uint32_t k = 0; k < ni; ++k)
        if (idx[k] >= nv) return fail(c, RG_ERR_INVALID_ARG, "index " + std::to_string(k) + " out of range");
    TRY(set_device(c));
    TRY(ensure(c, c->sc->vertices, sizeof(rg_vertex) * (size_t)nv));
    TRY(ensure(c, c->sc->indices, 4ull * ni));
    TRY(ensure(c, c->sc->materials, sizeof(rg_material) * (size_t)nm));
    if (nv) CK(cudaMemcpyAsync(c->sc->vertices.p, v, sizeof(rg_vertex) * (size_t)nv, cudaMemcpyHostToDevice, c->stream));
    if (ni) CK(cudaMemcpyAsync(c->sc->indices.p, idx, 4ull * ni, cudaMemcpyHostToDevice, c->stream));
    if (nm) CK(cudaMemcpyAsync(c->sc->materials.p, m, sizeof(rg_material) * (size_t)nm, cudaMemcpyHostToDevice, c->stream));
    c->sc->nv = nv;
    c->sc->ni = ni;
    c->sc->nm = nm;
    c->sc->hostIdx.assign(idx, idx + ni);
    c->sc->hostMat.resize(nv);
    for (uint32_t k = 0; k < nv; ++k) c->sc->hostMat[k] = v[k].matIndex;
    c->sc->maxIdx.clear();
    c->sc->maxMat.clear();
    ++c->sc->gen;
    return RG_OK;
}

rg_status rg_update_vertices(rg_ctx* c, uint32_t first, const rg_vertex* v, uint32_t n) {
    if (!c || (n && !v) || (uint64_t)first + n > c->sc->nv) return fail(c, RG_ERR_INVALID_ARG, "vertex range outside the uploaded buffer");
    TRY(set_device(c));
    std::vector<uint32_t> before(c->sc->hostMat.begin() + first, c->sc->hostMat.begin() + first + n);
    bool matChanged = false;
    for (uint32_t k = 0; k < n; ++k) {
        matChanged |= before[k] != v[k].matIndex;
        c->sc->hostMat[first + k] = v[k].matIndex;
    }
    if (matChanged) {  // the instances of the current TLAS must still reach only uploaded materials
        SceneState& st = *c->sc;
        st.maxMat.clear();
        std::vector<uint32_t> oldMax(st.blas.size());
        for (uint32_t b = 0; b < st.blas.size(); ++b) {  // the BLASes' material bounds
            BlasRec& r = st.blas[b];
            oldMax[b] = r.maxMat;
            if (r.gen == st.gen && r.triCount) r.maxMat = range_max_material(st, r.vOff, r.iOff, r.triCount);
        }
        std::string why;
        for (const rg_instance& in : st.hostInst)
            if (!instance_ok(st, in, &why)) {  // refused: nothing was copied, nothing changes
                std::copy(before.begin(), before.end(), st.hostMat.begin() + first);
                for (uint32_t b = 0; b < st.blas.size(); ++b) st.blas[b].maxMat = oldMax[b];
                st.maxMat.clear();
                return fail(c, RG_ERR_INVALID_ARG, "vertex update: " + why);
            }
        for (uint32_t b = 0; b < st.blas.size(); ++b)
            if (st.blas[b].maxMat != oldMax[b]) TRY(upload_blas_entry(c, b));
    }
    if (n) CK(cudaMemcpyAsync(c->sc->vertices.as<rg_vertex>() + first, v, sizeof(rg_vertex) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    return RG_OK;
}

rg_status rg_update_vertices_device(rg_ctx* c, uint32_t first, const rg_vertex* v, uint32_t n) {
    if (!c || (n && !v) || (uint64_t)first + n > c->sc->nv) return fail(c, RG_ERR_INVALID_ARG, "vertex range outside the uploaded buffer");
    TRY(set_device(c));
    if (n) CK(cudaMemcpyAsync(c->sc->vertices.as<rg_vertex>() + first, v, sizeof(rg_vertex) * (size_t)n, cudaMemcpyDeviceToDevice, c->stream));
    return RG_OK;
}

rg_status rg_update_materials(rg_ctx* c, uint32_t first, const rg_material* m, uint32_t n) {
    if (!c || (n && !m) || (uint64_t)first + n > c->sc->nm) return fail(c, RG_ERR_INVALID_ARG, "material range outside the uploaded buffer");
    for (uint32_t k = 0; k < n; ++k)
        if (m[k].rayConsumption < 1 || m[k].rayConsumption > 5) return fail(c, RG_ERR_INVALID_ARG, "material rayConsumption outside 1..5");
    TRY(set_device(c));
    if (n) CK(cudaMemcpyAsync(c->sc->materials.as<rg_material>() + first, m, sizeof(rg_material) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    return RG_OK;
}

rg_status rg_build_blas(rg_ctx* c, uint32_t vOff, uint32_t iOff, uint32_t triCount, uint32_t* out) {
    if (!c || !out) return RG_ERR_INVALID_ARG;
    if (triCount >= 0x7FFFFFFFu) return fail(c, RG_ERR_INVALID_ARG, "too many triangles");
    std::string why;
    if (!range_ok(*c->sc, vOff, iOff, triCount, ~0u, &why)) return fail(c, RG_ERR_INVALID_ARG, why);
    TRY(set_device(c));
    uint32_t b = (uint32_t)c->sc->blas.size();
    c->sc->blas.emplace_back();
    BlasRec& r = c->sc->blas.back();
    r.vOff = vOff;
    r.iOff = iOff;
    r.triCount = triCount;
    r.maxMat = triCount ? range_max_material(*c->sc, vOff, iOff, triCount) : 0u;
    r.gen = c->sc->gen;
    TRY(ensure_bvh(c, r.bvh, triCount));
    TRY(ensure(c, r.tris, 48ull * (triCount ? triCount : 1)));
    if (triCount) {
        CK(tri_boxes(c->sc->vertices.as<rg_vertex>(), c->sc->indices.as<uint32_t>(), vOff, iOff, triCount, r.bvh.primBoxes.as<float>(), c->stream));
        // binned SAH where it fits (once per scene load; refits keep its topology), else the LBVH
        const bool sah = !(c->flags & RG_FLAG_BLAS_LBVH) && triCount > 1 && triCount <= kSahBlasMaxPrims;
        if (sah) {
            CK(sah_build(buffers(c, r.bvh), true, nullptr, c->stream));
            CK(cudaMemsetAsync(r.bvh.morton.p, 0, 4ull * triCount, c->stream));  // no Morton order in an SAH tree
        } else {
            CK(lbvh_build(buffers(c, r.bvh), c->stream));
        }
        CK(wide_records(buffers(c, r.bvh), r.bvh.wide.as<WideNode>(), c->stream));
        CK(tri_records(c->sc->vertices.as<rg_vertex>(), c->sc->indices.as<uint32_t>(), vOff, iOff, r.bvh.order.as<uint32_t>(), triCount,
                       r.tris.as<float4>(), c->stream));
    }
    // the BLAS table grows; copy the existing entries over
    DevBuf old = c->sc->blasTable;
    c->sc->blasTable = DevBuf{};
    TRY(ensure(c, c->sc->blasTable, sizeof(DevBlas) * c->sc->blas.size()));
    if (old.p) {
        CK(cudaMemcpyAsync(c->sc->blasTable.p, old.p, sizeof(DevBlas) * b, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        release(c, old);
    }
    TRY(upload_blas_entry(c, b));
    *out = b;
    c->sc->tlasReady = false;  // instances point at the BLAS table, which moved
    return RG_OK;
}

rg_status rg_refit_blas(rg_ctx* c, uint32_t b) {
    if (!c || b >= c->sc->blas.size()) return fail(c, RG_ERR_INVALID_ARG, "unknown BLAS");
    TRY(set_device(c));
    BlasRec& r = c->sc->blas[b];
    uint32_t n = r.bvh.n;
    if (!n) return RG_OK;
    std::string why;  // geometry uploaded since the build must still hold the BLAS's triangles
    if (!range_ok(*c->sc, r.vOff, r.iOff, n, ~0u, &why)) return fail(c, RG_ERR_INVALID_ARG, "refit: " + why);
    FrameEvents* fe;
    TRY(cur_events(c, &fe));
    if (!fe->hasRefit) CK(cudaEventRecord(fe->ev[EV_REFIT0], c->stream));
    CK(tri_boxes(c->sc->vertices.as<rg_vertex>(), c->sc->indices.as<uint32_t>(), r.vOff, r.iOff, n, r.bvh.primBoxes.as<float>(), c->stream));
    CK(lbvh_refit(buffers(c, r.bvh), c->stream));
    CK(wide_records(buffers(c, r.bvh), r.bvh.wide.as<WideNode>(), c->stream));
    CK(tri_records(c->sc->vertices.as<rg_vertex>(), c->sc->indices.as<uint32_t>(), r.vOff, r.iOff, r.bvh.order.as<uint32_t>(), n,
                   r.tris.as<float4>(), c->stream));
    CK(cudaMemcpyAsync(c->sc->blasTable.as<DevBlas>()[b].root, root_box(r.bvh), 24, cudaMemcpyDeviceToDevice, c->stream));
    if (c->sc->tlasReady)  // the TLAS leaf records carry copies of the BLAS root boxes
        CK(inst_records(c->sc->tlas.order.as<uint32_t>(), c->sc->nInst, c->sc->instDev.as<DevInstance>(),
                        c->sc->blasTable.as<DevBlas>(), c->sc->tlasLeaves.as<InstRec>(), c->stream));
    CK(cudaEventRecord(fe->ev[EV_REFIT1], c->stream));
    fe->hasRefit = true;
    return RG_OK;
}

rg_status rg_build_tlas(rg_ctx* c, const rg_instance* inst, uint32_t n) {
    if (!c || (n && !inst)) return RG_ERR_INVALID_ARG;
    std::string why;
    for (uint32_t i = 0; i < n; ++i)
        if (!instance_ok(*c->sc, inst[i], &why)) return fail(c, RG_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": " + why);
    TRY(set_device(c));
    TRY(ensure(c, c->sc->instIn, sizeof(rg_instance) * (size_t)(n ? n : 1)));
    if (n) CK(cudaMemcpyAsync(c->sc->instIn.p, inst, sizeof(rg_instance) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    c->sc->hostInst.assign(inst, inst + n);
    return build_tlas_from_device_instances(c, n, false);
}

rg_status rg_build_tlas_device(rg_ctx* c, const rg_instance* d_inst, uint32_t n) {
    if (!c || (n && !d_inst)) return RG_ERR_INVALID_ARG;
    TRY(set_device(c));
    TRY(ensure(c, c->sc->instIn, sizeof(rg_instance) * (size_t)(n ? n : 1)));
    if (n) CK(cudaMemcpyAsync(c->sc->instIn.p, d_inst, sizeof(rg_instance) * (size_t)n, cudaMemcpyDeviceToDevice, c->stream));
    c->sc->hostInst.clear();
    return build_tlas_from_device_instances(c, n, true);
}

rg_status rg_set_resolution(rg_ctx* c, uint32_t w, uint32_t h) {
    if (!c || w == 0 || h == 0 || w > 16384 || h > 16384) return fail(c, RG_ERR_INVALID_ARG, "resolution must be 1..16384");
    TRY(set_device(c));
    size_t px = (size_t)w * h;
    TRY(ensure(c, c->base, 8 * px));
    TRY(ensure(c, c->normal, 8 * px));
    TRY(ensure(c, c->rough, 8 * px));
    TRY(ensure(c, c->finalImg, 8 * px));
    TRY(ensure(c, c->fxaaOut, 8 * px));
    TRY(ensure(c, c->fb, 16 * px));
    if (c->flags & RG_FLAG_DEBUG_IMAGES) {
        TRY(ensure(c, c->dbgT, 4 * px));
        TRY(ensure(c, c->dbgA, 8 * px));
        TRY(ensure(c, c->dbgB, 8 * px));
    }
    c->W = w;
    c->H = h;
    c->haveFrame = false;
    return RG_OK;
}

static rg_status run_post(rg_ctx* c, const rg_ubo* ubo, int32_t fxaa) {
    PostParams pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.status = wait_status(c);
    pp.waitLimit = post_wait_limit();
    pp.W = c->W;
    pp.H = c->H;
    pp.base = c->base.as<uint2>();
    pp.normal = c->normal.as<uint2>();
    pp.rough = c->rough.as<uint2>();
    pp.finalImg = c->finalImg.as<uint2>();
    pp.fxaaOut = c->fxaaOut.as<uint2>();
    pp.framebuffer = c->fb.as<float4>();
    if (c->flags & RG_FLAG_DEBUG_IMAGES) {
        pp.dbgTransition = c->dbgT.as<float>();
        pp.dbgA = c->dbgA.as<uint2>();
        pp.dbgB = c->dbgB.as<uint2>();
    }
    for (int k = 0; k < 4; ++k) pp.fade[k] = ubo->fadeColor[k];
    pp.showAlpha = ubo->showAlpha ? 1 : 0;
    pp.fxaa = fxaa ? 1 : 0;
    FrameEvents* fe;
    TRY(cur_events(c, &fe));
    CK(cudaEventRecord(fe->ev[EV_POST0], c->stream));
    if (c->filter)  // the learned filter in place of the roughness passes, then the same FXAA
        CK(filter_frame(c->filter, pp.base, pp.normal, pp.rough, c->W, c->H, (float)c->lastSamples, pp.fade, pp.showAlpha, pp.finalImg, wait_status(c),
                        c->stream));
    else
        CK(launch_rough_post(pp, c->stream));
    CK(cudaEventRecord(fe->ev[EV_ROUGH1], c->stream));
    CK(launch_fxaa(pp, c->stream));
    CK(cudaEventRecord(fe->ev[EV_POST1], c->stream));
    fe->hasFrame = true;
    c->evPending.push_back(fe);
    c->evCur = nullptr;
    c->lastFxaa = fxaa != 0;
    c->haveFrame = true;
    return RG_OK;
}

static rg_status check_ubo(rg_ctx* c, const rg_ubo* ubo) {
    if (!ubo) return fail(c, RG_ERR_INVALID_ARG, "null ubo");
    if (ubo->numSamples < 1 || ubo->numSamples > 32) return fail(c, RG_ERR_INVALID_ARG, "numSamples outside 1..32 (render_system.cpp:263)");
    if (ubo->maxRecursions < 0 || ubo->maxRecursions > 8) return fail(c, RG_ERR_INVALID_ARG, "maxRecursions outside 0..8");
    return RG_OK;
}

rg_status rg_render(rg_ctx* c, const rg_ubo* ubo, int32_t fxaa) {
    if (!c) return RG_ERR_INVALID_ARG;
    TRY(check_ubo(c, ubo));
    if (!c->W) return fail(c, RG_ERR_NOT_READY, "rg_set_resolution was not called");
    if (!c->sc->tlasReady) return fail(c, RG_ERR_NOT_READY, "no TLAS (call rg_build_tlas after the last rg_build_blas)");
    TRY(set_device(c));
    TRY(ensure(c, c->samples, 48ull * c->W * c->H * (uint32_t)ubo->numSamples));
    TRY(ensure(c, c->workCounter, 16));
    TraceParams tp;
    std::memset(&tp, 0, sizeof(tp));
    tp.scene = scene_of(*c->sc);
    tp.ubo = *ubo;
    tp.W = c->W;
    tp.H = c->H;
    tp.base = c->base.as<uint2>();
    tp.normal = c->normal.as<uint2>();
    tp.rough = c->rough.as<uint2>();
    tp.counters = c->counters.as<unsigned long long>();
    tp.countVisits = (c->flags & RG_FLAG_COUNT_VISITS) ? 1 : 0;
    tp.samples = c->samples.as<float4>();
    tp.workCounter = c->workCounter.as<uint32_t>();
    tp.glossySeed = c->glossySeed;
    c->lastSamples = (uint32_t)ubo->numSamples;
    const bool mega = (c->flags & RG_FLAG_MEGAKERNEL) != 0;
    if (!mega)
        TRY(ensure_wavefront(c, (size_t)c->W * c->H * (uint32_t)ubo->numSamples, tp.wf,
                             frame_work_items(c->W, c->H, (uint32_t)ubo->numSamples)));
    CK(cudaMemsetAsync(c->counters.p, 0, 64, c->stream));
    FrameEvents* fe;
    TRY(cur_events(c, &fe));
    CK(cudaEventRecord(fe->ev[EV_RT0], c->stream));
    if (mega) {
        c->lastIterations = 0;
        CK(launch_trace(tp, c->stream));
    }
    else if (c->flags & RG_FLAG_KERNEL_TIMING)
        CK(launch_trace_wavefront(tp, c->stream, c->hostCount, &c->lastIterations, next_kernel_events, fe));
    else
        CK(launch_trace_wavefront(tp, c->stream, c->hostCount, &c->lastIterations));
    return run_post(c, ubo, fxaa);
}

rg_status rg_post_only(rg_ctx* c, const rg_ubo* ubo, const float* base, const float* normal, const float* rough, int32_t fxaa) {
    if (!c || !base || !normal || !rough) return RG_ERR_INVALID_ARG;
    if (!ubo) return fail(c, RG_ERR_INVALID_ARG, "null ubo");
    if (!c->W) return fail(c, RG_ERR_NOT_READY, "rg_set_resolution was not called");
    TRY(set_device(c));
    size_t px = (size_t)c->W * c->H;
    TRY(ensure(c, c->tmpA, 16 * px));
    const float* src[3] = {base, normal, rough};
    DevBuf* dst[3] = {&c->base, &c->normal, &c->rough};
    for (int k = 0; k < 3; ++k) {
        CK(cudaMemcpyAsync(c->tmpA.p, src[k], 16 * px, cudaMemcpyHostToDevice, c->stream));
        CK(f32_to_h16(c->tmpA.as<float4>(), dst[k]->as<uint2>(), px, c->stream));
    }
    FrameEvents* fe;
    TRY(cur_events(c, &fe));
    CK(cudaEventRecord(fe->ev[EV_RT0], c->stream));
    return run_post(c, ubo, fxaa);
}

rg_status rg_download(rg_ctx* c, float* host) {
    if (!c || !host) return RG_ERR_INVALID_ARG;
    if (!c->haveFrame) return fail(c, RG_ERR_NOT_READY, "no frame rendered");
    TRY(set_device(c));
    CK(cudaMemcpyAsync(host, c->fb.p, 16ull * c->W * c->H, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&c->hostCount[7], wait_status(c), 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    TRY(settle_graph(c));
    if (c->hostCount[7]) return fail(c, RG_ERR_CUDA, wait_failure(c->hostCount[7]));
    return RG_OK;
}

rg_status rg_download_async(rg_ctx* c, float* host) {
    if (!c || !host) return RG_ERR_INVALID_ARG;
    if (!c->haveFrame) return fail(c, RG_ERR_NOT_READY, "no frame rendered");
    TRY(set_device(c));
    const size_t bytes = 16ull * c->W * c->H;
    const int k = c->readbackSlot;
    TRY(ensure(c, c->readback[k], bytes));
    if (c->copyIssued[k]) CK(cudaStreamWaitEvent(c->stream, c->copied[k], 0));  // the slot's previous copy left
    CK(cudaMemcpyAsync(c->readback[k].p, c->fb.p, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaEventRecord(c->staged[k], c->stream));
    CK(cudaStreamWaitEvent(c->copyStream, c->staged[k], 0));
    CK(cudaMemcpyAsync(host, c->readback[k].p, bytes, cudaMemcpyDeviceToHost, c->copyStream));
    CK(cudaEventRecord(c->copied[k], c->copyStream));
    c->copyIssued[k] = true;
    c->readbackSlot = k ^ 1;
    return RG_OK;
}

rg_status rg_framebuffer_device(rg_ctx* c, float** d) {
    if (!c || !d) return RG_ERR_INVALID_ARG;
    if (!c->W) return fail(c, RG_ERR_NOT_READY, "rg_set_resolution was not called");
    *d = c->fb.as<float>();
    return RG_OK;
}

rg_status rg_download_image(rg_ctx* c, int32_t which, float* host) {
    if (!c || !host) return RG_ERR_INVALID_ARG;
    if (!c->haveFrame) return fail(c, RG_ERR_NOT_READY, "no frame rendered");
    TRY(set_device(c));
    size_t px = (size_t)c->W * c->H;
    TRY(ensure(c, c->tmpB, 16 * px));
    const uint2* h16 = nullptr;
    switch (which) {
        case RG_IMAGE_FINAL: h16 = c->lastFxaa ? c->fxaaOut.as<uint2>() : c->finalImg.as<uint2>(); break;
        case RG_IMAGE_BASE: h16 = c->lastFxaa ? c->finalImg.as<uint2>() : c->base.as<uint2>(); break;  // swapped by FXAA (raytracer.cpp:139)
        case RG_IMAGE_NORMAL: h16 = c->normal.as<uint2>(); break;
        case RG_IMAGE_ROUGH: h16 = c->rough.as<uint2>(); break;
        case RG_IMAGE_PRE_FXAA: h16 = c->finalImg.as<uint2>(); break;
        case RG_IMAGE_FILTER_OUT:
            if (!c->filter) return fail(c, RG_ERR_NOT_READY, "no learned filter set (rg_set_filter)");
            CK(cudaMemcpyAsync(c->tmpB.p, filter_prediction(c->filter), 16 * px, cudaMemcpyDeviceToDevice, c->stream));
            break;
        case RG_IMAGE_ROUGH_COLORS_A:
        case RG_IMAGE_ROUGH_COLORS_B:
        case RG_IMAGE_ROUGH_TRANSITION:
            if (!(c->flags & RG_FLAG_DEBUG_IMAGES)) return fail(c, RG_ERR_NOT_READY, "context created without RG_FLAG_DEBUG_IMAGES");
            if (which == RG_IMAGE_ROUGH_TRANSITION) {
                CK(r32_to_rgba(c->dbgT.as<float>(), c->tmpB.as<float4>(), px, c->stream));
            } else {
                h16 = which == RG_IMAGE_ROUGH_COLORS_A ? c->dbgA.as<uint2>() : c->dbgB.as<uint2>();
            }
            break;
        default: return fail(c, RG_ERR_INVALID_ARG, "unknown image");
    }
    if (h16) CK(h16_to_f32(h16, c->tmpB.as<float4>(), px, c->stream));
    CK(cudaMemcpyAsync(host, c->tmpB.p, 16 * px, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    TRY(settle_graph(c));
    return RG_OK;
}

rg_status rg_synchronize(rg_ctx* c) {
    if (!c) return RG_ERR_INVALID_ARG;
    TRY(set_device(c));
    CK(cudaMemcpyAsync(&c->hostCount[7], wait_status(c), 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaStreamSynchronize(c->copyStream));
    TRY(settle_graph(c));
    if (c->hostCount[7]) return fail(c, RG_ERR_CUDA, wait_failure(c->hostCount[7]));
    return RG_OK;
}

rg_status rg_get_timings(rg_ctx* c, rg_timings* t) {
    if (!c || !t) return RG_ERR_INVALID_ARG;
    TRY(set_device(c));
    CK(cudaStreamSynchronize(c->stream));
    TRY(settle_graph(c));
    auto el = [&](cudaEvent_t a, cudaEvent_t b) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
            cudaGetLastError();
            ms = 0.0f;
        }
        return ms;
    };
    rg_timings r = c->lastTimings;
    r.frames = 0;
    r.asBuildSum = r.rtTotalSum = r.rtOnlySum = r.postprocSum = r.roughSum = r.refitSum = 0.0f;
    r.traceKernelSum = 0.0f;
    r.traceLaunches = 0;
    for (FrameEvents* f : c->evPending) {
        float as = f->hasAs ? el(f->ev[EV_AS0], f->ev[EV_AS1]) : 0.0f;
        float rf = f->hasRefit ? el(f->ev[EV_REFIT0], f->ev[EV_REFIT1]) : 0.0f;
        float rt = el(f->ev[EV_RT0], f->ev[EV_POST0]);
        float ro = el(f->ev[EV_POST0], f->ev[EV_ROUGH1]);
        float po = el(f->ev[EV_POST0], f->ev[EV_POST1]);
        float tk = 0.0f;
        for (size_t k = 0; k + 1 < f->kernelUsed; k += 2) tk += el(f->kernel[k], f->kernel[k + 1]);
        r.traceLaunches += (uint32_t)(f->kernelUsed / 2);
        r.traceKernel = tk;
        r.traceKernelSum += tk;
        r.asBuild = as; r.refit = rf; r.rtOnly = rt; r.rough = ro; r.postproc = po; r.rtTotal = rt + po;
        r.asBuildSum += as; r.refitSum += rf; r.rtOnlySum += rt; r.roughSum += ro; r.postprocSum += po; r.rtTotalSum += rt + po;
        r.frames++;
        c->evPool.push_back(f);
    }
    c->evPending.clear();
    c->lastTimings = r;
    *t = r;
    return RG_OK;
}

static rg_status read_stats(rg_ctx* c, rg_stats* s, int base);
rg_status rg_get_stats(rg_ctx* c, rg_stats* s) { return read_stats(c, s, 0); }

static rg_status read_stats(rg_ctx* c, rg_stats* s, int base) {
    if (!c || !s) return RG_ERR_INVALID_ARG;
    TRY(set_device(c));
    unsigned long long v[16];
    CK(cudaMemcpyAsync(v, c->counters.p, 128, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    TRY(settle_graph(c));
    s->primary = v[base + 0];
    s->shadow = v[base + 1];
    s->secondary = v[base + 2];
    s->masked = v[base + 3];
    s->nodes = v[base + 4];
    s->tris = v[base + 5];
    s->stack_overflows = v[base + 6];
    s->iterations = base == 0 ? (uint64_t)c->lastIterations : 0;
    s->deep_overflows = v[base + 7];
    return RG_OK;
}

rg_status rg_get_total_stats(rg_ctx* c, rg_stats* s) { return read_stats(c, s, 8); }

rg_status rg_reset_total_stats(rg_ctx* c) {
    if (!c) return RG_ERR_INVALID_ARG;
    TRY(set_device(c));
    CK(cudaMemsetAsync(c->counters.as<unsigned long long>() + 8, 0, 64, c->stream));
    return RG_OK;
}

rg_status rg_set_flags(rg_ctx* c, uint32_t flags) {
    if (!c) return RG_ERR_INVALID_ARG;
    TRY(set_device(c));
    c->flags = flags;
    if ((flags & RG_FLAG_DEBUG_IMAGES) && c->W) TRY(rg_set_resolution(c, c->W, c->H));
    return RG_OK;
}

rg_status rg_launch_count(uint64_t* out) {
    if (!out) return RG_ERR_INVALID_ARG;
    *out = rg::g_launches.load();
    return RG_OK;
}

rg_status rg_get_stream(rg_ctx* c, void** s) {
    if (!c || !s) return RG_ERR_INVALID_ARG;
    *s = (void*)c->stream;
    return RG_OK;
}

static rg_status download_bvh(rg_ctx* c, const BvhSet& s, uint32_t* morton, uint32_t* order, uint32_t* left, uint32_t* right,
                              float* nodeboxes) {
    uint32_t n = s.n;
    if (morton && n) CK(cudaMemcpyAsync(morton, s.morton.p, 4ull * n, cudaMemcpyDeviceToHost, c->stream));
    if (order && n) CK(cudaMemcpyAsync(order, s.order.p, 4ull * n, cudaMemcpyDeviceToHost, c->stream));
    if (n > 1) {
        if (left) CK(cudaMemcpyAsync(left, s.left.p, 4ull * (n - 1), cudaMemcpyDeviceToHost, c->stream));
        if (right) CK(cudaMemcpyAsync(right, s.right.p, 4ull * (n - 1), cudaMemcpyDeviceToHost, c->stream));
        if (nodeboxes) CK(cudaMemcpyAsync(nodeboxes, s.nodeBoxes.p, 24ull * (n - 1), cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return RG_OK;
}

rg_status rg_bvh_info(rg_ctx* c, uint32_t b, uint32_t* n_out, uint32_t* morton, uint32_t* order, uint32_t* left, uint32_t* right,
                      float* nodeboxes) {
    if (!c) return RG_ERR_INVALID_ARG;
    const BvhSet* s = nullptr;
    if (b == 0xFFFFFFFFu) {
        if (!c->sc->tlasReady) return fail(c, RG_ERR_NOT_READY, "no TLAS");
        s = &c->sc->tlas;
    } else if (b < c->sc->blas.size()) {
        s = &c->sc->blas[b].bvh;
    } else {
        return fail(c, RG_ERR_INVALID_ARG, "unknown BLAS");
    }
    if (n_out) *n_out = s->n;
    TRY(set_device(c));
    return download_bvh(c, *s, morton, order, left, right, nodeboxes);
}

rg_status rg_bvh_records(rg_ctx* c, uint32_t b, void* out, uint32_t capacity, uint32_t* n_out) {
    if (!c) return RG_ERR_INVALID_ARG;
    const BvhSet* s = nullptr;
    if (b == 0xFFFFFFFFu) {
        if (!c->sc->tlasReady) return fail(c, RG_ERR_NOT_READY, "no TLAS");
        s = &c->sc->tlas;
    } else if (b < c->sc->blas.size()) {
        s = &c->sc->blas[b].bvh;
    } else {
        return fail(c, RG_ERR_INVALID_ARG, "unknown BLAS");
    }
    const uint32_t m = s->n > 1 ? s->n - 1 : 0;
    if (n_out) *n_out = m;
    if (!out || !m || !capacity) return RG_OK;
    TRY(set_device(c));
    CK(cudaMemcpyAsync(out, s->wide.p, sizeof(WideNode) * (size_t)std::min(m, capacity), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return RG_OK;
}

rg_status rg_instance_inverse(rg_ctx* c, float* out) {
    if (!c || !out) return RG_ERR_INVALID_ARG;
    if (!c->sc->tlasReady) return fail(c, RG_ERR_NOT_READY, "no TLAS");
    TRY(set_device(c));
    std::vector<DevInstance> h(c->sc->nInst);
    if (c->sc->nInst) CK(cudaMemcpyAsync(h.data(), c->sc->instDev.p, sizeof(DevInstance) * c->sc->nInst, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (uint32_t i = 0; i < c->sc->nInst; ++i)
        for (int r = 0; r < 3; ++r) {
            out[12 * i + 4 * r + 0] = h[i].inv[r].x;
            out[12 * i + 4 * r + 1] = h[i].inv[r].y;
            out[12 * i + 4 * r + 2] = h[i].inv[r].z;
            out[12 * i + 4 * r + 3] = h[i].inv[r].w;
        }
    return RG_OK;
}

rg_status rg_trace_rays(rg_ctx* c, const float* rays, uint32_t n, float* tuv, uint32_t* ids) {
    if (!c || (n && (!rays || !tuv || !ids))) return RG_ERR_INVALID_ARG;
    if (!c->sc->tlasReady) return fail(c, RG_ERR_NOT_READY, "no TLAS");
    if (!n) return RG_OK;
    TRY(set_device(c));
    TRY(ensure(c, c->tmpA, 32ull * n));
    TRY(ensure(c, c->tmpC, 12ull * n));
    TRY(ensure(c, c->tmpD, 8ull * n));
    CK(cudaMemcpyAsync(c->tmpA.p, rays, 32ull * n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->counters.p, 0, 64, c->stream));  // rg_get_stats then reports this call's overflows
    CK(launch_trace_rays(scene_of(*c->sc), c->tmpA.as<float>(), n, c->tmpC.as<float>(), c->tmpD.as<uint32_t>(),
                         c->counters.as<unsigned long long>(), c->tune.depth, c->stream));
    CK(cudaMemcpyAsync(tuv, c->tmpC.p, 12ull * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(ids, c->tmpD.p, 8ull * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return RG_OK;
}

rg_status rg_trace_rays_device(rg_ctx* c, const float* d_rays, uint32_t n, float* d_tuv, uint32_t* d_ids) {
    if (!c || (n && (!d_rays || !d_tuv || !d_ids))) return RG_ERR_INVALID_ARG;
    if (reinterpret_cast<uintptr_t>(d_rays) & 15u) return fail(c, RG_ERR_INVALID_ARG, "trace_rays_device: rays must be 16-byte aligned");
    if (!c->sc->tlasReady) return fail(c, RG_ERR_NOT_READY, "no TLAS");
    if (!n) return RG_OK;
    TRY(set_device(c));
    // the traversal kernel reads the rays and writes the hits in the caller's buffers; of the frame
    // loop's state it uses the counters and the overflow list (rays re-traced with the deep stack)
    TRY(ensure(c, c->wfOverflow, 4ull * n));
    if (!c->wfCounts.p) {
        TRY(ensure(c, c->wfCounts, 32));
        CK(cudaMemsetAsync(c->wfCounts.p, 0, 32, c->stream));
    }
    TraceParams tp;
    std::memset(&tp, 0, sizeof(tp));
    tp.scene = scene_of(*c->sc);
    tp.counters = c->counters.as<unsigned long long>();
    tp.countVisits = (c->flags & RG_FLAG_COUNT_VISITS) ? 1 : 0;
    tp.wf.counts = c->wfCounts.as<uint32_t>();
    tp.wf.overflow = c->wfOverflow.as<uint32_t>();
    CK(cudaMemsetAsync(c->counters.p, 0, 64, c->stream));
    CK(launch_trace_queue(tp, d_rays, n, d_tuv, d_ids, c->tune.depth, c->stream));
    return RG_OK;
}

rg_status rg_lbvh_build_host(rg_ctx* c, const float* boxes, uint32_t n, uint32_t* morton, uint32_t* order, uint32_t* left,
                             uint32_t* right, float* nodeboxes) {
    if (!c || (n && !boxes)) return RG_ERR_INVALID_ARG;
    TRY(set_device(c));
    BvhSet s;
    rg_status st = ensure_bvh(c, s, n);
    if (st == RG_OK && n) {
        cudaError_t e = cudaMemcpyAsync(s.primBoxes.p, boxes, 24ull * n, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = lbvh_build(buffers(c, s), c->stream);
        if (e != cudaSuccess) st = fail(c, RG_ERR_CUDA, cudaGetErrorString(e));
        if (st == RG_OK) st = download_bvh(c, s, morton, order, left, right, nodeboxes);
    }
    DevBuf* bb[] = {&s.primBoxes, &s.morton, &s.order, &s.left, &s.right, &s.nodeBoxes, &s.parents, &s.flags, &s.wide};
    cudaStreamSynchronize(c->stream);
    for (DevBuf* b : bb) release(c, *b);
    return st;
}

}  // extern "C"


// ---- batch helpers ----------------------------------------------------------------------------------
namespace {

// per job: resolve of its samples, roughness + postprocess + FXAA into its slice of batchFb
cudaError_t enqueue_batch_posts(rg_ctx* c, const JobDesc* jd, const rg_job* jobs, uint32_t n) {
    for (uint32_t j = 0; j < n; ++j) {
        const JobDesc& d = jd[j];
        cudaError_t e = launch_resolve_job(c->samples.as<float4>(), d, c->bBase.as<uint2>(), c->bNormal.as<uint2>(),
                                           c->bRough.as<uint2>(), c->stream);
        if (e != cudaSuccess) return e;
        PostParams pp;
        std::memset(&pp, 0, sizeof(pp));
        pp.status = wait_status(c);
        pp.waitLimit = post_wait_limit();
        pp.W = d.W;
        pp.H = d.H;
        pp.base = c->bBase.as<uint2>();
        pp.normal = c->bNormal.as<uint2>();
        pp.rough = c->bRough.as<uint2>();
        pp.finalImg = c->bFinal.as<uint2>();
        pp.fxaaOut = c->bFxaa.as<uint2>();
        pp.framebuffer = c->batchFb.as<float4>() + c->batchOffset[j];
        for (int k = 0; k < 4; ++k) pp.fade[k] = d.ubo.fadeColor[k];
        pp.showAlpha = d.ubo.showAlpha ? 1 : 0;
        pp.fxaa = (jobs[j].options & RG_JOB_FXAA) ? 1 : 0;
        if (jobs[j].options & RG_JOB_FILTER)  // the learned filter in place of the roughness passes
            e = filter_frame(c->filter, pp.base, pp.normal, pp.rough, d.W, d.H, (float)d.S, pp.fade, pp.showAlpha, pp.finalImg, wait_status(c),
                             c->stream);
        else
            e = launch_rough_post(pp, c->stream);
        if (e != cudaSuccess) return e;
        if ((e = launch_fxaa(pp, c->stream)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <class T>
void key_put(std::vector<uint8_t>& k, const T& v) {
    const uint8_t* b = reinterpret_cast<const uint8_t*>(&v);
    k.insert(k.end(), b, b + sizeof(T));
}

// what a captured batch graph depends on besides the job table's contents (scenes, cameras)
std::vector<uint8_t> batch_graph_key(rg_ctx* c, const TraceParams& tp, const SortScratch& sort, const JobDesc* jd,
                                     const rg_job* jobs, uint32_t n) {
    std::vector<uint8_t> k;
    key_put(k, tp);
    key_put(k, c->tune);
    key_put(k, sort);
    const void* ptrs[] = {c->bBase.p, c->bNormal.p, c->bRough.p, c->bFinal.p, c->bFxaa.p, c->batchFb.p, c->loopWords.p,
                          c->hostCount};
    key_put(k, ptrs);
    for (uint32_t j = 0; j < n; ++j) {
        key_put(k, jd[j].W);
        key_put(k, jd[j].H);
        key_put(k, jd[j].S);
        key_put(k, jd[j].sampleBase);
        key_put(k, jd[j].ubo.fadeColor);
        key_put(k, jd[j].ubo.showAlpha);
        key_put(k, jobs[j].options);
        key_put(k, c->batchOffset[j]);
    }
    return k;
}

rg_status launch_batch_graph(rg_ctx* c, const TraceParams& tp, const SortScratch& sort, const JobDesc* jd, const rg_job* jobs,
                             uint32_t n) {
    if (!c->loopWords.p) {
        TRY(ensure(c, c->loopWords, 16));
        CK(cudaMemsetAsync(c->loopWords.p, 0, 16, c->stream));
        c->bodyRunsSeen = 0;
    }
    std::vector<uint8_t> key = batch_graph_key(c, tp, sort, jd, jobs, n);
    if (!c->graphExec || key != c->graphKey) {
        if (c->graphExec) cudaGraphExecDestroy(c->graphExec);
        if (c->graph) cudaGraphDestroy(c->graph);
        c->graphExec = nullptr;
        c->graph = nullptr;
        c->graphKey.clear();
        const uint64_t before = g_launches.load();
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
        cudaError_t e = capture_trace_batch(tp, c->tune, sort, c->stream, c->stream2, c->loopWords.as<uint32_t>());
        const uint64_t postsBefore = g_launches.load();
        if (e == cudaSuccess) e = enqueue_batch_posts(c, jd, jobs, n);
        const uint64_t posts = g_launches.load() - postsBefore;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->hostCount + 4, c->loopWords.p, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
        g_launches.store(before);  // captured launches are counted when the graph runs
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return fail(c, RG_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        cudaError_t e3 = cudaGraphInstantiate(&c->graphExec, g, 0);
        if (e3 != cudaSuccess) {
            cudaGraphDestroy(g);
            c->graphExec = nullptr;
            return fail(c, RG_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(e3));
        }
        c->graph = g;
        c->graphKey = std::move(key);
        c->graphFixedKernels = (uint64_t)batch_graph_kernels(c->tune, &c->graphBodyKernels) + posts;
    }
    CK(cudaGraphLaunch(c->graphExec, c->stream));
    count_launch(c->graphFixedKernels);
    c->graphPending = true;
    return RG_OK;
}

}  // namespace

// ---- scene slots and batched rendering ------------------------------------------------------------
extern "C" {

rg_status rg_scene_create(rg_ctx* c, uint32_t* out) {
    if (!c || !out) return RG_ERR_INVALID_ARG;
    for (uint32_t k = 0; k < c->scenes.size(); ++k)
        if (!c->scenes[k]) {
            c->scenes[k] = new SceneState();
            *out = k;
            return RG_OK;
        }
    c->scenes.push_back(new SceneState());
    *out = (uint32_t)c->scenes.size() - 1;
    return RG_OK;
}

rg_status rg_scene_select(rg_ctx* c, uint32_t id) {
    if (!c) return RG_ERR_INVALID_ARG;
    if (id >= c->scenes.size() || !c->scenes[id]) return fail(c, RG_ERR_INVALID_ARG, "unknown scene " + std::to_string(id));
    c->sc = c->scenes[id];
    c->scId = id;
    return RG_OK;
}

rg_status rg_scene_destroy(rg_ctx* c, uint32_t id) {
    if (!c) return RG_ERR_INVALID_ARG;
    if (id >= c->scenes.size() || !c->scenes[id]) return fail(c, RG_ERR_INVALID_ARG, "unknown scene " + std::to_string(id));
    if (id == c->scId) return fail(c, RG_ERR_INVALID_ARG, "the selected scene cannot be destroyed");
    TRY(set_device(c));
    CK(cudaStreamSynchronize(c->stream));  // no queued work may still read the slot
    release_scene(c, *c->scenes[id]);
    delete c->scenes[id];
    c->scenes[id] = nullptr;
    return RG_OK;
}

rg_status rg_scene_bytes(rg_ctx* c, uint32_t id, uint64_t* out) {
    if (!c || !out) return RG_ERR_INVALID_ARG;
    if (id >= c->scenes.size() || !c->scenes[id]) return fail(c, RG_ERR_INVALID_ARG, "unknown scene " + std::to_string(id));
    *out = scene_bytes(*c->scenes[id]);
    return RG_OK;
}

rg_status rg_set_batch_tune(rg_ctx* c, const rg_batch_tune* t) {
    if (!c || !t) return RG_ERR_INVALID_ARG;
    TraceTune tt;
    tt.threads = t->threads;
    tt.depth = t->stack_depth;
    tt.sortKey = t->sort_key;
    if (!tune_supported(tt)) return fail(c, RG_ERR_INVALID_ARG, "unsupported batch tune (threads 64/128/256, depth 16/24/32/48, sort 0..2)");
    c->tune = tt;
    return RG_OK;
}

rg_status rg_get_batch_tune(rg_ctx* c, rg_batch_tune* t) {
    if (!c || !t) return RG_ERR_INVALID_ARG;
    t->threads = c->tune.threads;
    t->stack_depth = c->tune.depth;
    t->sort_key = c->tune.sortKey;
    return RG_OK;
}

rg_status rg_get_memory(rg_ctx* c, uint64_t* allocated, uint64_t* budget) {
    if (!c) return RG_ERR_INVALID_ARG;
    if (allocated) *allocated = c->allocated;
    if (budget) *budget = c->budget;
    return RG_OK;
}

rg_status rg_set_batch_slots(rg_ctx* c, uint32_t slots) {
    if (!c || slots < 1024) return fail(c, RG_ERR_INVALID_ARG, "batch path slots must be >= 1024");
    c->batchSlots = slots;
    return RG_OK;
}

rg_status rg_render_batch(rg_ctx* c, const rg_job* jobs, uint32_t n) {
    if (!c) return RG_ERR_INVALID_ARG;
    if (!jobs || n == 0) return fail(c, RG_ERR_INVALID_ARG, "empty batch");
    for (uint32_t j = 0; j < n; ++j)
        if ((jobs[j].options & RG_JOB_FILTER) && !c->filter)
            return fail(c, RG_ERR_INVALID_ARG, "job " + std::to_string(j) + ": learned filter asked for, none set (rg_set_filter)");
    std::vector<JobDesc> jd(n);
    uint64_t work = 0, samples = 0, pixels = 0, maxPixels = 0;
    for (uint32_t j = 0; j < n; ++j) {
        const rg_job& in = jobs[j];
        if (in.scene >= c->scenes.size() || !c->scenes[in.scene])
            return fail(c, RG_ERR_INVALID_ARG, "job " + std::to_string(j) + ": unknown scene");
        const SceneState& st = *c->scenes[in.scene];
        if (!st.tlasReady) return fail(c, RG_ERR_NOT_READY, "job " + std::to_string(j) + ": scene has no TLAS");
        if (in.width == 0 || in.height == 0 || in.width > 16384 || in.height > 16384)
            return fail(c, RG_ERR_INVALID_ARG, "job " + std::to_string(j) + ": resolution must be 1..16384");
        TRY(check_ubo(c, &in.ubo));
        const uint32_t S = (uint32_t)in.ubo.numSamples;
        const uint32_t tilesX = (in.width + 7) / 8, tilesY = (in.height + 3) / 4;
        const uint64_t jobWork = (uint64_t)tilesX * tilesY * 32 * S;
        const uint64_t jobPixels = (uint64_t)in.width * in.height;
        JobDesc& d = jd[j];
        std::memset(&d, 0, sizeof(d));
        d.scene = scene_of(st);
        d.ubo = in.ubo;
        d.W = in.width;
        d.H = in.height;
        d.S = S;
        d.tilesX = tilesX;
        d.workBase = (uint32_t)work;
        d.workCount = (uint32_t)jobWork;
        d.sampleBase = (uint32_t)samples;
        work += jobWork;
        samples += jobPixels * S;
        pixels += jobPixels;
        if (jobPixels > maxPixels) maxPixels = jobPixels;
        if (work >= (1ull << 31) || samples >= (1ull << 31))
            return fail(c, RG_ERR_TOO_LARGE, "batch too large: at most 2^31 samples per batch");
    }
    TRY(set_device(c));
    const uint32_t slots = (uint32_t)std::min<uint64_t>(work, c->batchSlots);
    TraceParams tp;
    std::memset(&tp, 0, sizeof(tp));
    TRY(ensure_wavefront(c, slots, tp.wf));
    TRY(ensure(c, c->samples, 48ull * samples));
    TRY(ensure(c, c->workCounter, 16));
    TRY(ensure(c, c->slotJob, 4ull * slots));
    TRY(ensure(c, c->slotSample, 4ull * slots));
    TRY(ensure(c, c->jobTable, sizeof(JobDesc) * n));
    SortScratch sort{};
    if (c->tune.sortKey != RG_SORT_NONE) {
        TRY(ensure(c, c->sortKeys, 4ull * slots));
        TRY(ensure(c, c->sortPerm, 4ull * slots));
        TRY(ensure(c, c->sortHist, 8192 * 4));
        sort.keysA = c->sortKeys.as<uint32_t>();
        sort.valsA = c->sortPerm.as<uint32_t>();
        sort.hist = c->sortHist.as<uint32_t>();
    }
    TRY(ensure(c, c->bBase, 8 * maxPixels));
    TRY(ensure(c, c->bNormal, 8 * maxPixels));
    TRY(ensure(c, c->bRough, 8 * maxPixels));
    TRY(ensure(c, c->bFinal, 8 * maxPixels));
    TRY(ensure(c, c->bFxaa, 8 * maxPixels));
    TRY(ensure(c, c->batchFb, 16 * pixels));
    CK(cudaMemcpyAsync(c->jobTable.p, jd.data(), sizeof(JobDesc) * n, cudaMemcpyHostToDevice, c->stream));
    tp.counters = c->counters.as<unsigned long long>();
    tp.countVisits = (c->flags & RG_FLAG_COUNT_VISITS) ? 1 : 0;
    tp.samples = c->samples.as<float4>();
    tp.workCounter = c->workCounter.as<uint32_t>();
    tp.jobs = c->jobTable.as<JobDesc>();
    tp.njobs = n;
    tp.totalWork = (uint32_t)work;
    tp.slots = slots;
    tp.slotJob = c->slotJob.as<uint32_t>();
    tp.slotSample = c->slotSample.as<uint32_t>();
    CK(cudaMemsetAsync(c->counters.p, 0, 64, c->stream));
    c->batchOffset.assign(n, 0);
    c->batchW.assign(n, 0);
    c->batchH.assign(n, 0);
    size_t off = 0;
    for (uint32_t j = 0; j < n; ++j) {
        c->batchOffset[j] = off;
        c->batchW[j] = jd[j].W;
        c->batchH[j] = jd[j].H;
        off += (size_t)jd[j].W * jd[j].H;
    }
    FrameEvents* fe;
    TRY(cur_events(c, &fe));
    CK(cudaEventRecord(fe->ev[EV_RT0], c->stream));
    bool filtered = false;
    for (uint32_t j = 0; j < n; ++j) filtered |= (jobs[j].options & RG_JOB_FILTER) != 0;
    const bool hostLoop = filtered || (c->flags & (RG_FLAG_HOST_LOOP | RG_FLAG_KERNEL_TIMING | RG_FLAG_COUNT_VISITS)) != 0;
    if (hostLoop) {
        if (c->flags & RG_FLAG_KERNEL_TIMING)
            CK(launch_trace_batch(tp, c->tune, sort, c->stream, c->hostCount, &c->lastIterations, next_kernel_events, fe));
        else
            CK(launch_trace_batch(tp, c->tune, sort, c->stream, c->hostCount, &c->lastIterations));
        CK(cudaEventRecord(fe->ev[EV_POST0], c->stream));
        CK(enqueue_batch_posts(c, jd.data(), jobs, n));
    } else {
        TRY(launch_batch_graph(c, tp, sort, jd.data(), jobs, n));
        CK(cudaEventRecord(fe->ev[EV_POST0], c->stream));
    }
    CK(cudaEventRecord(fe->ev[EV_ROUGH1], c->stream));
    CK(cudaEventRecord(fe->ev[EV_POST1], c->stream));
    fe->hasFrame = true;
    c->evPending.push_back(fe);
    c->evCur = nullptr;
    return RG_OK;
}

rg_status rg_autotune_batch(rg_ctx* c, const rg_job* jobs, uint32_t n, uint32_t reps, rg_batch_tune* best, float* msOut) {
    if (!c) return RG_ERR_INVALID_ARG;
    if (!jobs || n == 0 || reps == 0) return fail(c, RG_ERR_INVALID_ARG, "autotune needs jobs and reps >= 1");
    TRY(set_device(c));
    const int threads[3] = {64, 128, 256}, depths[4] = {16, 24, 32, 48}, keys[3] = {RG_SORT_NONE, RG_SORT_OCTANT, RG_SORT_MORTON};
    const TraceTune saved = c->tune;
    const uint32_t savedFlags = c->flags;
    c->flags &= ~(uint32_t)(RG_FLAG_KERNEL_TIMING | RG_FLAG_COUNT_VISITS);  // time the production (graph) loop
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float bestMs = -1.0f;
    TraceTune bestTune = saved;
    rg_status st = RG_OK;
    int idx = 0;
    for (int ti = 0; ti < 3 && st == RG_OK; ++ti)
        for (int di = 0; di < 4 && st == RG_OK; ++di)
            for (int ki = 0; ki < 3 && st == RG_OK; ++ki, ++idx) {
                c->tune.threads = threads[ti];
                c->tune.depth = depths[di];
                c->tune.sortKey = keys[ki];
                float ms = -1.0f;
                if (!tune_supported(c->tune)) {
                    if (msOut) msOut[idx] = ms;
                    continue;
                }
                st = rg_render_batch(c, jobs, n);
                rg_stats stats{};
                if (st == RG_OK) st = read_stats(c, &stats, 0);
                if (st == RG_OK && stats.stack_overflows == 0) {
                    cudaError_t e = cudaEventRecord(e0, c->stream);
                    for (uint32_t r = 0; r < reps && st == RG_OK && e == cudaSuccess; ++r) st = rg_render_batch(c, jobs, n);
                    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    if (st == RG_OK) st = settle_graph(c);
                    float el = 0.0f;
                    if (e == cudaSuccess) e = cudaEventElapsedTime(&el, e0, e1);
                    if (e != cudaSuccess && st == RG_OK) st = fail(c, RG_ERR_CUDA, cudaGetErrorString(e));
                    ms = el / (float)reps;
                    if (st == RG_OK && (bestMs < 0.0f || ms < bestMs)) {
                        bestMs = ms;
                        bestTune = c->tune;
                    }
                }
                if (msOut) msOut[idx] = ms;
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->flags = savedFlags;
    // the tuning renders are not frames of the caller's timeline
    for (FrameEvents* f : c->evPending) c->evPool.push_back(f);
    c->evPending.clear();
    c->tune = st == RG_OK && bestMs >= 0.0f ? bestTune : saved;
    if (st != RG_OK) return st;
    if (bestMs < 0.0f) return fail(c, RG_ERR_STACK_OVERFLOW, "every configuration overflowed the traversal stack");
    if (best) {
        best->threads = c->tune.threads;
        best->stack_depth = c->tune.depth;
        best->sort_key = c->tune.sortKey;
    }
    return RG_OK;
}

rg_status rg_batch_download_async(rg_ctx* c, float* host) {
    if (!c || !host) return RG_ERR_INVALID_ARG;
    if (c->batchOffset.empty()) return fail(c, RG_ERR_NOT_READY, "no batch rendered");
    TRY(set_device(c));
    const size_t last = c->batchOffset.size() - 1;
    const size_t bytes = 16ull * (c->batchOffset[last] + (size_t)c->batchW[last] * c->batchH[last]);
    const int k = c->readbackSlot;
    TRY(ensure(c, c->readback[k], bytes));
    if (c->copyIssued[k]) CK(cudaStreamWaitEvent(c->stream, c->copied[k], 0));  // the slot's previous copy left
    CK(cudaMemcpyAsync(c->readback[k].p, c->batchFb.p, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaEventRecord(c->staged[k], c->stream));
    CK(cudaStreamWaitEvent(c->copyStream, c->staged[k], 0));
    CK(cudaMemcpyAsync(host, c->readback[k].p, bytes, cudaMemcpyDeviceToHost, c->copyStream));
    CK(cudaEventRecord(c->copied[k], c->copyStream));
    c->copyIssued[k] = true;
    c->readbackSlot = k ^ 1;
    return RG_OK;
}

rg_status rg_batch_framebuffer(rg_ctx* c, uint32_t job, float** d) {
    if (!c || !d) return RG_ERR_INVALID_ARG;
    if (job >= c->batchOffset.size()) return fail(c, RG_ERR_INVALID_ARG, "no such job in the last batch");
    *d = reinterpret_cast<float*>(c->batchFb.as<float4>() + c->batchOffset[job]);
    return RG_OK;
}

rg_status rg_batch_download(rg_ctx* c, uint32_t job, float* host) {
    if (!c || !host) return RG_ERR_INVALID_ARG;
    if (job >= c->batchOffset.size()) return fail(c, RG_ERR_INVALID_ARG, "no such job in the last batch");
    TRY(set_device(c));
    CK(cudaMemcpyAsync(host, c->batchFb.as<float4>() + c->batchOffset[job], 16ull * c->batchW[job] * c->batchH[job],
                       cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    TRY(settle_graph(c));
    return RG_OK;
}

}  // extern "C"

// ---- learned roughness filter: frame inputs / targets, selection, glossy reference shading ---------
extern "C" {

rg_status rg_filter_input(rg_ctx* c, void* d_out) {
    if (!c || !d_out) return RG_ERR_INVALID_ARG;
    if (!c->haveFrame) return fail(c, RG_ERR_NOT_READY, "no frame rendered");
    TRY(set_device(c));
    CK(filter_gbuffer(c->base.as<uint2>(), c->normal.as<uint2>(), c->rough.as<uint2>(), (size_t)c->W * c->H, (float)c->lastSamples, d_out,
                      c->stream));
    return RG_OK;
}

rg_status rg_filter_target(rg_ctx* c, float* d_out) {
    if (!c || !d_out) return RG_ERR_INVALID_ARG;
    if (!c->haveFrame) return fail(c, RG_ERR_NOT_READY, "no frame rendered");
    TRY(set_device(c));
    CK(filter_target(c->rough.as<uint2>(), (size_t)c->W * c->H, reinterpret_cast<float4*>(d_out), c->stream));
    return RG_OK;
}

rg_status rg_set_filter(rg_ctx* c, rg_filter* f) {
    if (!c) return RG_ERR_INVALID_ARG;
    c->filter = f;
    return RG_OK;
}

rg_status rg_set_glossy(rg_ctx* c, uint32_t seed) {
    if (!c) return RG_ERR_INVALID_ARG;
    c->glossySeed = seed;
    return RG_OK;
}

}  // extern "C"
