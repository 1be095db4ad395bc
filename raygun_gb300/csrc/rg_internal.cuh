// rg_internal.cuh -- device-side layouts and helpers shared by the rgcuda kernels.
//
// All translation units are compiled with -fmad=false: every + - * / below is one IEEE operation,
// so the ray geometry (Morton codes, traversal, intersection, secondary ray set-up) reproduces the
// same bits as a plain C++ evaluation of the same expressions.  Fused multiply-adds are written
// out as fmaf() where they are wanted.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/rgcuda.h"

namespace rg {

constexpr uint32_t kLeaf = 0x80000000u;
#ifndef RG_STACK_DEPTH
#define RG_STACK_DEPTH 48
#endif
constexpr int kTraversalStack = RG_STACK_DEPTH;
constexpr int kMaxFrames = 10;  // maxRecursions (<= 8 supported) + primary + masked-miss leaf


// 4-wide record of BVH2 node i: the boxes and refs of i's grandchildren (a leaf child stands in
// for its own slot).  Traversal visits records only, so it skips every other BVH2 level; the
// BVH2 itself stays the built and checked structure.  Empty slots have ref kEmptySlot and an
// inverted box.  112 B = seven 16-byte loads.
constexpr uint32_t kEmptySlot = 0xFFFFFFFEu;
struct __align__(16) WideNode {
    float4 lox, hix, loy, hiy, loz, hiz;  // per slot
    uint4 ref;
};
static_assert(sizeof(WideNode) == 112, "wide node");

struct Box {
    float lo[3], hi[3];
};

// per-BLAS record read by the traversal kernel
struct DevBlas {
    const WideNode* wide;
    const float4* tris;  // 3 float4 per sorted leaf: v0 (w = primitive id bits), v1, v2
    uint32_t n;          // triangle count
    uint32_t maxMat;     // largest matIndex of the vertices its triangles reference
    float root[6];       // root box (lo xyz, hi xyz)
    uint32_t vOff, iOff; // vertex and index offsets it was built from (range-checked on the host)
    uint32_t pad0, pad1;
};
static_assert(sizeof(DevBlas) == 64, "BLAS table entry");

// per-instance record read by the traversal and shading code
struct __align__(16) DevInstance {
    float4 inv[3];  // world -> object rows
    float4 m[3];    // object -> world rows
    uint32_t blas, valid, vOff, iOff;
    uint32_t mOff, mask, pad0, pad1;
};
static_assert(sizeof(DevInstance) == 128, "instance");

// TLAS leaf record, in leaf (sorted) order: what the traversal needs to enter an instance, in one
// fetch of six independent 16-byte loads
struct __align__(16) InstRec {
    float4 inv[3];           // world -> object rows
    float4 lo;               // BLAS root box lo xyz; w = BLAS triangle count bits (0: invalid or empty)
    float4 hi;               // BLAS root box hi xyz; w = instance index bits
    const WideNode* wide;    // the BLAS's 4-wide records
    const float4* tris;      // its leaf-ordered triangles
};
static_assert(sizeof(InstRec) == 96, "instance record");

struct DevScene {
    const DevBlas* blas;
    const DevInstance* inst;
    const WideNode* tlasWide;
    const InstRec* tlasLeaves;  // sorted position -> instance record
    uint32_t tlasN;
    uint32_t pad;
    const float* tlasRoot;      // root box (lo xyz, hi xyz), device memory
    const rg_vertex* vertices;
    const uint32_t* indices;
    const rg_material* materials;
};

// ---- explicit-rounding helpers ------------------------------------------------------------------
__host__ __device__ inline uint32_t expand10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__device__ inline uint32_t quant10(float c, float lo, float inv) {
    float d = __fsub_rn(c, lo);
    float q = __fmul_rn(d, inv);
    float s = __fmul_rn(q, 1024.0f);
    s = fminf(fmaxf(s, 0.0f), 1023.0f);
    return (uint32_t)s;
}

// order-preserving float <-> uint mapping for atomic min/max
__device__ inline uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ inline float ord2f(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u); }

__host__ __device__ inline float3 f3(float x, float y, float z) { return make_float3(x, y, z); }

}  // namespace rg

// internal launchers implemented in the .cu files
namespace rg {

// kernels launched by this library in this process (rg_launch_count)
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

struct LbvhBuffers {  // scratch + outputs of one LBVH build, sized by the caller (n primitives)
    uint32_t n;
    // inputs
    float* primBoxes;      // n x 6, primitive order
    // outputs
    uint32_t* morton;      // n, primitive order
    uint32_t* order;       // n, sorted position -> primitive
    uint32_t* left;        // n-1
    uint32_t* right;       // n-1
    float* nodeBoxes;      // (n-1) x 6
    // scratch
    uint32_t* keysA; uint32_t* keysB; uint32_t* valsA; uint32_t* valsB;
    uint32_t* sortState;   // sort_state_words(n): digit histograms, tile counters, look-back words
    uint32_t* parents;     // 2n (internal n-1 then leaves n)
    uint32_t* flags;       // n-1
    uint32_t* bounds;      // 6 (ordered uints)
    // binned-SAH builds: the task queue of k_sah_tasks (sah_queue_bytes(n), 16-byte aligned) and a
    // status word set to 2 when one of its waits gave up (nullable)
    unsigned char* sahQueue = nullptr;
    int* status = nullptr;
};

// task queue of the SAH builder's task kernel: n task records (range, node id, level), n ready
// words, 8 counters (claims, pushes, first node id, tasks in total), 8 per-level task counts of its
// level kernels
struct SahQueue {
    uint4* tasks;
    uint32_t* ready;
    uint32_t* ctr;
};
constexpr size_t sah_queue_bytes(size_t n) { return 20 * n + 64; }

// onesweep radix sort of the Morton codes: keys per tile, and the layout of its state words (zeroed
// by each build): 4 passes x 256 digit counts, 4 tile counters, then per pass one status word per
// (tile, digit)
constexpr uint32_t kSortTileKeys = 2048;
constexpr uint32_t kSortTileCounters = 4 * 256;
constexpr uint32_t kSortStatusOffset = kSortTileCounters + 32;
constexpr size_t sort_tiles(size_t n) { return (n + kSortTileKeys - 1) / kSortTileKeys; }
constexpr size_t sort_state_words(size_t n) { return kSortStatusOffset + 4 * 256 * sort_tiles(n); }
cudaError_t lbvh_build(const LbvhBuffers& b, cudaStream_t s);
cudaError_t lbvh_refit(const LbvhBuffers& b, cudaStream_t s);  // topology kept, primBoxes changed
cudaError_t wide_records(const LbvhBuffers& b, WideNode* out, cudaStream_t s);  // after build / refit
// binned-SAH BVH2 over b.primBoxes in the LBVH's layout (order, left, right, nodeBoxes), one CTA;
// parents (for refits) on request.  *levels (device word, nullable) receives the number of levels.
// From level kSahMedianLevel on, ranges are halved without binning, so a tree has at most
// kSahMedianLevel + ceil(log2 n) levels.  The TLAS uses it up to kSahMaxPrims instances (it is
// rebuilt every frame), BLASes up to kSahBlasMaxPrims triangles (built once per scene load), the
// LBVH otherwise.
constexpr uint32_t kSahMaxPrims = 8192;
constexpr uint32_t kSahBlasMaxPrims = 1u << 18;
constexpr uint32_t kSahMedianLevel = 32;
cudaError_t sah_build(const LbvhBuffers& b, bool parents, uint32_t* levels, cudaStream_t s);
cudaError_t tri_boxes(const rg_vertex* v, const uint32_t* idx, uint32_t vOff, uint32_t iOff, uint32_t n, float* boxes,
                      cudaStream_t s);
cudaError_t tri_records(const rg_vertex* v, const uint32_t* idx, uint32_t vOff, uint32_t iOff, const uint32_t* order, uint32_t n,
                        float4* tris, cudaStream_t s);
// world boxes and shading records of n instances.  checkOffsets (instances from device memory, which
// the host never saw): an instance is also invalid -- never hit -- unless its vertex and index offsets
// are its BLAS's own and its material offset keeps the BLAS's materials below nm.
cudaError_t setup_instances(const rg_instance* in, uint32_t n, const DevBlas* blas, uint32_t nblas, DevInstance* out,
                            float* boxes, bool checkOffsets, uint32_t nm, cudaStream_t s);
// the TLAS leaf records (after the TLAS build; again after a BLAS refit, which moves root boxes)
cudaError_t inst_records(const uint32_t* order, uint32_t n, const DevInstance* inst, const DevBlas* blas, InstRec* out,
                         cudaStream_t s);

// device buffers of the wavefront path (one path per pixel sample; P = paths)
struct WavefrontBuffers {
    float4* payload;   // P x 4 float4: the reference payload (payload.h:29-39)
    int2* meta;        // P: frame-stack depth, miss index of the pending ray
    void* frames;      // P x kMaxFrames paused closest-hit frames (144 B each)
    float4* qO[2];     // ray queues: origin + tmin
    float4* qD[2];     //             direction + tmax
    uint32_t* qPath[2];
    float4* hitTUV;    // per queue slot: t, u, v, primitive bits
    uint32_t* hitInst; // per queue slot: instance or 0xFFFFFFFF (miss)
    uint32_t* counts;  // [0], [1] queue lengths, [2] trace work counter, [3] overflow list length,
                       // [4] trace blocks finished (both zero between launches)
    uint32_t* overflow; // per queue slot: slots of rays whose short traversal stack overflowed
};

// one render job of a batch: a scene, its UBO and its image size.  Work items of the batch are
// numbered job after job; job j owns [workBase, workBase + workCount) and writes its per-sample
// payload sums to samples[sampleBase + (y * W + x) * S + s].
struct JobDesc {
    DevScene scene;
    rg_ubo ubo;
    uint32_t W, H, S, tilesX;
    uint32_t workBase;    // first work item (work items: 8x4 pixel tiles x 32 pixels x S samples)
    uint32_t workCount;
    uint32_t sampleBase;  // first per-sample slot in TraceParams::samples
    uint32_t pad;
};

struct TraceParams {
    DevScene scene;
    rg_ubo ubo;
    uint32_t W, H;
    uint2* base;    // RGBA16F images (8 B per pixel)
    uint2* normal;
    uint2* rough;
    unsigned long long* counters;  // 8 per frame + 8 cumulative
    float4* samples;               // W*H*S*3 per-sample payload sums (k_trace -> k_resolve)
    uint32_t* workCounter;         // work-item counter of the persistent kernel
    int countVisits;
    WavefrontBuffers wf;
    // batch form of the wavefront loop (launch_trace_batch): the job table in device memory, the
    // batch's work-item count, and per path slot the job and the output sample index.  A slot whose
    // path finished takes the next work item (path regeneration), so `slots` bounds the path state.
    const JobDesc* jobs;
    uint32_t njobs;
    uint32_t totalWork;
    uint32_t slots;
    uint32_t pad2;
    uint32_t* slotJob;
    uint32_t* slotSample;
    const uint32_t* perm;  // nullable: order in which the trace kernel takes the queue's rays
    uint32_t glossySeed;   // 0: the reference's mirror shading; else glossy reference shading (seed)
    // frame loop: the first (trace, shade) round computes the camera rays and initial payloads of
    // work items 0 .. W*H*S-1 (8x4-tile order) itself instead of reading a raygen queue
    int firstRound;
    // ray query (rg_trace_rays_device): queryCount rays read from the caller's buffer (origin, tmin,
    // direction, tmax: two float4 per ray) and hits written in rg_trace_rays' layout, so the query
    // needs neither a queue copy before the traversal nor a read-out pass after it
    const float4* queryRays;
    float* queryTuv;
    uint32_t* queryIds;
    uint32_t queryCount;
};
cudaError_t launch_trace(const TraceParams& p, cudaStream_t s);
// Work items of the frame loop: W x H pixels padded to whole 8 x 4 tiles, times S samples.  The first
// round indexes its hit records by work item, so the hit buffers hold this many entries (more than
// W * H * S when W or H is not a multiple of the tile).
constexpr int kTileW = 8, kTileH = 4;
inline size_t frame_work_items(uint32_t W, uint32_t H, uint32_t S) {
    return (size_t)((W + kTileW - 1) / kTileW) * ((H + kTileH - 1) / kTileH) * (kTileW * kTileH) * S;
}
// hostCount: pinned host word used to poll the queue length; iterations: trace/shade rounds run
// kernelEvents (nullable): callback that returns a (start, end) event pair to record around each
// traversal launch
typedef bool (*EventPairFn)(void* user, cudaEvent_t* start, cudaEvent_t* end);
cudaError_t launch_trace_wavefront(const TraceParams& p, cudaStream_t s, uint32_t* hostCount, int* iterations,
                                   EventPairFn kernelEvents = nullptr, void* user = nullptr);
// traversal launch shape of the batch loop: block size {64,128,256}, stack entries {16,24,32,48},
// ray-sort key applied to each queue before it is traced
struct TraceTune {
    int threads = 128, depth = 48, sortKey = RG_SORT_NONE;
};
bool tune_supported(const TraceTune& t);
// scratch of the ray sort (each of the first three: `slots` words; hist: 8192 words)
struct SortScratch {
    uint32_t *keysA, *keysB, *valsA, *valsB, *hist;
};
// the wavefront loop over every job of p.jobs (raygen with regeneration, trace/shade rounds, tail);
// hostWords: two pinned words (queue length, work counter) polled every few rounds
cudaError_t launch_trace_batch(const TraceParams& p, const TraceTune& tune, const SortScratch& sort, cudaStream_t s,
                               uint32_t* hostWords, int* iterations, EventPairFn kernelEvents = nullptr, void* user = nullptr);
// graph form of launch_trace_batch, enqueued on stream s while it captures: prologue, a while node
// (body captured on the idle stream s2: two trace/shade rounds and the device-side loop condition)
// and the tail launch.  loopWords: 3 device words (body runs of the launch, sticky iteration-limit
// flag, body runs in total), the last two zeroed by the caller once.
cudaError_t capture_trace_batch(const TraceParams& p, const TraceTune& tune, const SortScratch& sort, cudaStream_t s,
                                cudaStream_t s2, uint32_t* loopWords);
// kernels of that graph outside the loop body; *perBody = kernels of one body run
int batch_graph_kernels(const TraceTune& tune, int* perBody);
// raygen.rgen:36-38 for one job of a batch: average its samples into RGBA16F G-buffers
cudaError_t launch_resolve_job(const float4* samples, const JobDesc& hostJob, uint2* base, uint2* normal, uint2* rough,
                               cudaStream_t s);
// closest hits of n rays (8 floats each, device memory, 16-byte aligned) by one launch of the frame
// loop's traversal kernel (k_wf_trace in its query form): the kernel takes the rays straight from
// `rays` and writes the hits in rg_trace_rays' layout; stack of `depth` (16, 24, 32 or 48) entries,
// 48 when p.countVisits
cudaError_t launch_trace_queue(const TraceParams& p, const float* rays, uint32_t n, float* tuv, uint32_t* ids, int depth,
                               cudaStream_t s);
// closest hits of n rays with a traversal stack of `depth` (16, 24, 32 or 48) entries
cudaError_t launch_trace_rays(const DevScene& sc, const float* rays, uint32_t n, float* tuv, uint32_t* ids,
                              unsigned long long* counters, int depth, cudaStream_t s);

// ---- learned roughness filter (filter.cu) ----
// one 3x3 convolution of NHWC BF16 activations (x 16-byte aligned): v = conv(x, w) + bias, then
// ReLU (relu), y = v, v += add, ya = v, ym = v where mask > 0 else 0, yf = v[0..3] in FP32
struct FilterConvArgs {
    const __nv_bfloat16* x;     // [B][H][W][CIN]
    const __nv_bfloat16* w;     // packed [9][CIN/8][COUT][8] (K = tap * CIN + ci, rows = output channels)
    const float* bias;          // nullable [COUT]
    const __nv_bfloat16* add;   // nullable [B][H][W][COUT]
    const __nv_bfloat16* mask;  // nullable [B][H][W][COUT] (required with ym)
    __nv_bfloat16* y;           // nullable [B][H][W][COUT]
    __nv_bfloat16* ya;          // nullable [B][H][W][COUT]
    __nv_bfloat16* ym;          // nullable [B][H][W][COUT]
    float* yf;                  // nullable [B][H][W][4]
    int B, H, W, relu;
    int* status;                // set when a tensor-core or copy completion wait gave up
};
cudaError_t filter_conv(int cin, int cout, const FilterConvArgs& a, cudaStream_t s);
int filter_dw_ctas();
cudaError_t filter_dw(int cin, int cout, const void* x, const void* x2, const void* g, int B, int H, int W, float* partial, int ctas,
                      int* status, cudaStream_t s);
cudaError_t filter_pack(const float* W, int coutReal, int cinReal, int cin, int cout, int transposed, void* out, cudaStream_t s);
cudaError_t filter_dw_reduce(const float* partial, int ctas, int cout, int cin, int coutReal, int cinReal, float* dW, cudaStream_t s);
cudaError_t filter_bias_grad(const void* g, size_t P, int C, int cReal, float* partial, int blocks, float* db, cudaStream_t s);
cudaError_t filter_loss(const float4* out, const float4* target, size_t P, float scale, void* g, float* partial, int blocks, cudaStream_t s);
cudaError_t filter_adam(float* w, const float* grad, float* m, float* v, int n, float lr, float b1, float b2, float eps, float c1,
                        float c2, cudaStream_t s);
cudaError_t filter_gbuffer(const uint2* base, const uint2* normal, const uint2* rough, size_t P, float samples, void* out, cudaStream_t s);
cudaError_t filter_composite(const uint2* base, const float4* pred, size_t P, const float fade[4], int showAlpha, uint2* finalImg,
                             cudaStream_t s);
cudaError_t filter_target(const uint2* rough, size_t P, float4* out, cudaStream_t s);
cudaError_t filter_bias_pad(const float* b, int cReal, int c, float* out, cudaStream_t s);
// the filter on one frame (G-buffers -> input -> network -> composite into finalImg); filter_api.cu.
// status: the rendering context's device-wait status word (3 when a wait of the filter gave up)
cudaError_t filter_frame(rg_filter* f, const uint2* base, const uint2* normal, const uint2* rough, uint32_t W, uint32_t H, float samples,
                         const float fade[4], int showAlpha, uint2* finalImg, int* status, cudaStream_t s);
const float4* filter_prediction(const rg_filter* f);  // [P] of the last frame: RGB, w unused

struct PostParams {
    uint32_t W, H;
    const uint2* base;     // half4 images (8 B per pixel)
    const uint2* normal;
    const uint2* rough;
    uint2* finalImg;       // half4, postprocess output (FXAA input)
    uint2* fxaaOut;        // half4, FXAA output (becomes the final image)
    float4* framebuffer;   // RGBA32F output
    // debug outputs (nullable)
    float* dbgTransition;  // W*H floats
    uint2* dbgA;           // half4
    uint2* dbgB;           // half4
    float fade[4];
    int showAlpha;
    int fxaa;
    int* status;           // nullable: set to 1 when a staged copy of the roughness pass never landed
    uint32_t waitLimit;    // polls of a staged copy before the pass gives up (see post_wait_limit)
};
cudaError_t launch_rough_post(const PostParams& p, cudaStream_t s);
cudaError_t launch_fxaa(const PostParams& p, cudaStream_t s);
cudaError_t f32_to_h16(const float4* in, uint2* out, size_t n, cudaStream_t s);
cudaError_t h16_to_f32(const uint2* in, float4* out, size_t n, cudaStream_t s);
cudaError_t r32_to_rgba(const float* in, float4* out, size_t n, cudaStream_t s);

}  // namespace rg
