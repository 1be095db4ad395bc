/* rgcuda.h -- C ABI of the GB300 ray-tracing core that replaces Raygun's Vulkan RT path.
 *
 * Every entry point returns rg_status (0 = RG_OK, negative = error; rg_last_error() gives text).
 * The library owns all device memory; inputs are copied; work is ordered on the context's stream
 * and rg_render() is asynchronous until rg_download()/rg_synchronize().  One context per host
 * thread, calls serialized per context (Raygun calls the renderer from its main loop only,
 * raygun/raygun.cpp:91-133); contexts on different threads run concurrently (the library's only
 * process-wide state, launch-shape caches and a launch counter, is locked or atomic).
 *
 * Data layouts are byte-identical to Raygun's shared GLSL/C++ structs.
 */
#ifndef RGCUDA_H
#define RGCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t rg_status;
enum {
    RG_OK = 0,
    RG_ERR_INVALID_ARG = -1,
    RG_ERR_CUDA = -2,
    RG_ERR_OUT_OF_MEMORY = -3,
    RG_ERR_NOT_READY = -4,     /* e.g. render before geometry/TLAS */
    RG_ERR_STACK_OVERFLOW = -5,
    RG_ERR_BUDGET = -6,        /* HBM budget of rg_device_opts exceeded */
    RG_ERR_NO_DEVICE = -7,
    RG_ERR_TOO_LARGE = -8      /* input beyond a fixed-size entry point's stated maximum */
};

typedef struct rg_ctx rg_ctx;

typedef struct {
    int32_t device;            /* CUDA ordinal */
    uint32_t flags;            /* RG_FLAG_* */
    uint64_t hbm_budget_bytes; /* 0 = unlimited */
} rg_device_opts;
#define RG_FLAG_DEBUG_IMAGES 1u /* keep roughTransitions / roughColorsA/B for rg_download_image */
#define RG_FLAG_COUNT_VISITS 2u /* count BVH node / triangle visits (roofline accounting) */
#define RG_FLAG_MEGAKERNEL 4u   /* trace + shade in one persistent kernel instead of the wavefront loop */
#define RG_FLAG_KERNEL_TIMING 8u /* CUDA events around every traversal launch (rg_timings.traceKernel) */
#define RG_FLAG_HOST_LOOP 16u    /* rg_render_batch: host-polled round loop instead of the CUDA graph */
#define RG_FLAG_TLAS_LBVH 32u    /* build the TLAS as an LBVH (Morton order) instead of by binned SAH; TLASes of more
                                    than 8192 instances are always LBVHs */
#define RG_FLAG_BLAS_LBVH 64u    /* build BLASes as LBVHs instead of by binned SAH; BLASes of more than 2^18 triangles
                                    are always LBVHs */

/* resources/shaders/vertex.def:3-7 (render/vertex.hpp:27-29): 32 B */
typedef struct {
    float position[3];
    uint32_t matIndex;
    float normal[3];
    float pad1;
} rg_vertex;

/* resources/shaders/gpu_material.def:11-26 (gpu/gpu_material.hpp:27-31): 64 B */
typedef struct {
    float diffuse[3];
    float transparency;
    float specular[3];
    float reflectivity;
    float roughness;
    float ior;
    uint32_t effectId;
    uint32_t rayConsumption;
    float emission;
    float pad0, pad1, pad2;
} rg_material;

/* resources/shaders/uniform_buffer_object.def:3-17 (gpu/uniform_buffer.hpp:29-31), std140: 192 B.
 * Matrices are column-major (glm).  showAlpha is a 32-bit bool as in std140. */
typedef struct {
    float viewInverse[16];
    float projInverse[16];
    float clearColor[3];
    int32_t numSamples;
    float lightDir[3];
    int32_t maxRecursions;
    float time;
    uint32_t showAlpha;
    float pad0, pad1;
    float fadeColor[4];
} rg_ubo;

/* One TLAS instance: the 3x4 row-major object-to-world transform of
 * VkAccelerationStructureInstanceKHR (render/acceleration_structure.cpp:34-51), the BLAS handle,
 * the cull mask (0xFF in Raygun) and the InstanceOffsetTableEntry
 * (resources/shaders/instance_offset_table.def:1-3).  customIndex = position in the array. 72 B. */
typedef struct {
    float transform[3][4];
    uint32_t blas;
    uint32_t mask;
    uint32_t vertexBufferOffset;
    uint32_t indexBufferOffset;
    uint32_t materialBufferOffset;
    uint32_t pad;
} rg_instance;

/* GPU time of the profiler ranges of raygun/profiler.def:6-10 in milliseconds: the last frame,
 * and sums over every frame since the previous rg_get_timings call (raygun/profiler.cpp keeps
 * 500-frame rolling statistics of the same ranges). */
typedef struct {
    float asBuild;   /* TLAS build (raytracer.cpp:78,84) */
    float rtTotal;   /* trace + post (raytracer.cpp:93,144) */
    float rtOnly;    /* trace (raytracer.cpp:95,104) */
    float postproc;  /* roughness + composite + FXAA (raytracer.cpp:106,142) */
    float rough;     /* roughness approximation (raytracer.cpp:111,123) */
    float refit;     /* BLAS refits issued before the frame (not in the reference) */
    uint32_t frames; /* frames in the sums below */
    float asBuildSum, rtTotalSum, rtOnlySum, postprocSum, roughSum, refitSum;
    float traceKernel, traceKernelSum; /* traversal launches only (RG_FLAG_KERNEL_TIMING), within rtOnly:
                                          the round loop's k_wf_trace and the tail kernel */
    uint32_t traceLaunches;            /* traversal launches in traceKernelSum */
} rg_timings;

/* Ray statistics of the last frame. */
typedef struct {
    uint64_t primary;    /* camera rays */
    uint64_t shadow;     /* SHADOW_TRACE / SHADOW_INTERNAL rays that traversed */
    uint64_t secondary;  /* reflection + refraction rays */
    uint64_t masked;     /* mask-0 traces (closesthit.rchit:144): miss shader only, no traversal */
    uint64_t nodes;      /* BVH node visits (RG_FLAG_COUNT_VISITS) */
    uint64_t tris;       /* triangle tests (RG_FLAG_COUNT_VISITS) */
    uint64_t stack_overflows; /* rays whose short traversal stack overflowed; each was traced again with a deep
                                 stack, so its hit is complete (a cost, not an error) */
    uint64_t iterations; /* trace/shade rounds of the wavefront loop (0 for the megakernel) */
    uint64_t deep_overflows; /* rays that overflowed even the deep stack: 0 for every tree this library builds
                                (at most 64 BVH2 levels); non-zero means hits may be missing */
} rg_stats;

/* Debug images of Raytracer::selectResultImage (raytracer.cpp:379-392). */
enum {
    RG_IMAGE_FINAL = 0,
    RG_IMAGE_BASE = 1,
    RG_IMAGE_NORMAL = 2,
    RG_IMAGE_ROUGH = 3,
    RG_IMAGE_ROUGH_TRANSITION = 4,
    RG_IMAGE_ROUGH_COLORS_A = 5,
    RG_IMAGE_ROUGH_COLORS_B = 6,
    RG_IMAGE_PRE_FXAA = 7,
    RG_IMAGE_FILTER_OUT = 8  /* the learned filter's prediction of the last frame (RGB; rg_set_filter) */
};

/* Replaces Raytracer::Raytracer (render/raytracer.cpp:38-52) and the device parts of
 * VulkanContext (raygun/vulkan_context.cpp). */
rg_status rg_create(rg_ctx** out, const rg_device_opts* opts);
rg_status rg_destroy(rg_ctx* ctx);
const char* rg_last_error(const rg_ctx* ctx);

/* Replaces RenderSystem::setupModelBuffers (render/render_system.cpp:192-223): copies the packed
 * vertex / index / material buffers to device memory. */
rg_status rg_upload_geometry(rg_ctx* ctx, const rg_vertex* vertices, uint32_t nv, const uint32_t* indices, uint32_t ni,
                             const rg_material* materials, uint32_t nm);
/* Replaces RenderSystem::updateModelBuffers (render/render_system.cpp:225-233) for a range:
 * changed vertices (the caller then refits) / materials (live material edit,
 * gpu/gpu_material.cpp:52-94).  A vertex update whose new matIndex would take an instance of the
 * current (host-built) TLAS past the material buffer is refused with RG_ERR_INVALID_ARG and changes
 * nothing. */
rg_status rg_update_vertices(rg_ctx* ctx, uint32_t first, const rg_vertex* vertices, uint32_t n);
rg_status rg_update_materials(rg_ctx* ctx, uint32_t first, const rg_material* materials, uint32_t n);
/* Same as rg_update_vertices from vertices already in device memory (device pointer).  The host
 * never sees these vertices: their matIndex values must stay as they were (or within the materials
 * every instance of them reaches); positions may change freely. */
rg_status rg_update_vertices_device(rg_ctx* ctx, uint32_t first, const rg_vertex* d_vertices, uint32_t n);

/* Replaces BottomLevelAS::BottomLevelAS (render/acceleration_structure.cpp:140-194) as driven by
 * Raytracer::setupBottomLevelAS (render/raytracer.cpp:54-74): triangles
 * indices[indexOffset + 3k + 0..2] + vertexOffset, k < triCount.  *out_blas receives the handle.
 * Checked on the host first (the reference relied on Vulkan's robustBufferAccess,
 * vulkan_context.cpp:256-257): a range past the index buffer, or vertexOffset + index past the
 * vertex buffer, returns RG_ERR_INVALID_ARG before any kernel runs.  The build is queued on the
 * context's stream; it can block the host while the scene's device buffers grow (cudaMalloc). */
rg_status rg_build_blas(rg_ctx* ctx, uint32_t vertexOffset, uint32_t indexOffset, uint32_t triCount, uint32_t* out_blas);
/* Refit of a BLAS after its vertices moved (same topology).  No reference counterpart: Raygun
 * never refits. */
rg_status rg_refit_blas(rg_ctx* ctx, uint32_t blas);

/* Replaces TopLevelAS::TopLevelAS + Raytracer::setupTopLevelAS (render/acceleration_structure.cpp:55-138,
 * render/raytracer.cpp:76-85): rebuilds the TLAS from scratch from host instances.  Every instance
 * that can be hit (known BLAS, non-zero mask) is checked on the host through its offset table entry
 * (closesthit.rchit:98-109): indexBufferOffset + 3 * triCount within the index buffer,
 * vertexBufferOffset + each index within the vertex buffer, materialBufferOffset + each referenced
 * vertex's matIndex within the material buffer; a violation returns RG_ERR_INVALID_ARG ("instance k:
 * ...") and builds nothing.  Instances with an unknown BLAS, a zero mask or a singular transform are
 * never hit. */
rg_status rg_build_tlas(rg_ctx* ctx, const rg_instance* instances, uint32_t n);
/* Same, from instances already in device memory (device pointer).  The host cannot check these;
 * the TLAS build does instead, and an instance is never hit unless its vertexBufferOffset and
 * indexBufferOffset are its BLAS's own (those of rg_build_blas, as in the reference, where every
 * instance's offsets are its model's, acceleration_structure.cpp:79-82) and materialBufferOffset
 * keeps the BLAS's materials inside the material buffer. */
rg_status rg_build_tlas_device(rg_ctx* ctx, const rg_instance* d_instances, uint32_t n);

/* Replaces the resize path RenderSystem::reload -> Raytracer::setupRaytracingImages
 * (render/render_system.cpp:66-81, render/raytracer.cpp:173-195). */
rg_status rg_set_resolution(rg_ctx* ctx, uint32_t width, uint32_t height);

/* Replaces RenderSystem::render's trace part: updateRenderTarget + doRaytracing
 * (render/render_system.cpp:88-100, render/raytracer.cpp:87-171): trace, roughness passes,
 * postprocess and FXAA into the RGBA32F framebuffer.  fxaa = 0 skips FXAA (ImGui checkbox,
 * raytracer.cpp:136). */
rg_status rg_render(rg_ctx* ctx, const rg_ubo* ubo, int32_t fxaa);

/* Framebuffer (width*height*4 floats) to host memory; waits for the frame. */
rg_status rg_download(rg_ctx* ctx, float* host_rgba);
/* The same read-back without waiting: the last rendered frame is staged on the device (one of two
 * slots) and copied to host_rgba (pinned memory for an overlapped copy) on the library's copy stream
 * while later frames render. host_rgba must stay valid and unread until rg_synchronize returns.
 * Stands where Raygun blits the frame to its swapchain image and presents it (render_system.cpp:130-161):
 * the render call returns before the image has left the GPU. */
rg_status rg_download_async(rg_ctx* ctx, float* host_rgba);
/* Device pointer of the RGBA32F framebuffer (valid until the next rg_set_resolution). */
rg_status rg_framebuffer_device(rg_ctx* ctx, float** d_rgba);
/* Any of the RG_IMAGE_* images as RGBA32F (roughTransition: value in .r). */
rg_status rg_download_image(rg_ctx* ctx, int32_t which, float* host_rgba);

rg_status rg_synchronize(rg_ctx* ctx);  /* waits for the render stream and for rg_download_async copies */
/* rg_download and rg_synchronize also read the context's device-wait status: every device-side wait
 * of this library is bounded, and one that gave up (a staged tile copy of the roughness pass that
 * never landed, a task of the SAH BVH builder that was never published, or a copy or tensor-core
 * wait of the learned filter in the frame) makes them return RG_ERR_CUDA, with rg_last_error
 * naming which.  No such wait ends this way in a correct run. */
/* Replaces Profiler (raygun/profiler.cpp:55-105): GPU ranges of the last frame. */
rg_status rg_get_timings(rg_ctx* ctx, rg_timings* out);
rg_status rg_get_stats(rg_ctx* ctx, rg_stats* out);
/* Ray statistics summed over every frame since the context was created or last reset. */
rg_status rg_get_total_stats(rg_ctx* ctx, rg_stats* out);
rg_status rg_reset_total_stats(rg_ctx* ctx);
/* Replace the RG_FLAG_* set of rg_device_opts (debug images, visit counting). */
rg_status rg_set_flags(rg_ctx* ctx, uint32_t flags);
/* Number of kernels this library has launched in this process. */
rg_status rg_launch_count(uint64_t* out);
/* The CUDA stream the context orders its work on (cudaStream_t). */
rg_status rg_get_stream(rg_ctx* ctx, void** stream);

/* ---- several scenes per context, batched rendering -------------------------------------------
 * The reference renders one Scene per RenderSystem, whose per-scene GPU state is the model buffers,
 * the BLASes and the TLAS (render/render_system.cpp:192-223, render/raytracer.cpp:54-85).  A scene
 * slot is that state; a context holds any number of slots side by side in device memory.  Slot 0
 * exists from rg_create.  rg_upload_geometry, rg_update_*, rg_build_blas, rg_refit_blas,
 * rg_build_tlas*, rg_render, rg_trace_rays, rg_bvh_info and rg_instance_inverse act on the
 * selected slot. */
rg_status rg_scene_create(rg_ctx* ctx, uint32_t* out_scene);
rg_status rg_scene_select(rg_ctx* ctx, uint32_t scene);
/* Frees the slot's device memory.  The selected slot cannot be destroyed. */
rg_status rg_scene_destroy(rg_ctx* ctx, uint32_t scene);
/* Device memory held by the slot (model buffers, BLASes, TLAS), in bytes. */
rg_status rg_scene_bytes(rg_ctx* ctx, uint32_t scene, uint64_t* out_bytes);

/* One render of a batch: RenderSystem::render (render/render_system.cpp:88-162) of the scene in
 * slot `scene` at width x height with this UBO.  options: RG_JOB_FXAA as rg_render's fxaa;
 * RG_JOB_FILTER: the learned roughness filter set with rg_set_filter stands in for the roughness
 * passes of this job (an error when the context has none); a batch with such a job runs its round
 * loop from the host (no graph capture). */
#define RG_JOB_FXAA 1
#define RG_JOB_FILTER 2
typedef struct rg_job {
    uint32_t scene;
    uint32_t width, height;
    int32_t options;
    rg_ubo ubo;
} rg_job;

/* Launch shape of the batch loop's traversal kernel and the order it takes rays in. */
enum { RG_SORT_NONE = 0, RG_SORT_OCTANT = 1, RG_SORT_MORTON = 2 };
typedef struct rg_batch_tune {
    int32_t threads;      /* block size: 64, 128 or 256 */
    int32_t stack_depth;  /* traversal stack words per thread: 16, 24, 32 or 48 (48: up to 128 threads); one word
                             flags an overflow, the rest hold entries.  A ray that overflows them is traced
                             again with a deep stack (rg_stats.stack_overflows counts them) */
    int32_t sort_key;     /* RG_SORT_*: rays sorted per round by direction octant or origin Morton code */
} rg_batch_tune;

/* Renders every job: one wavefront loop traces the paths of all jobs together (path slots that
 * finish take the next job's work), then each job's samples are resolved and run through the
 * roughness, postprocess and FXAA passes into its own RGBA32F image.  Each image equals what
 * rg_render of that job's scene, resolution and UBO produces.  rg_get_stats then counts the rays
 * of the whole batch.  The batch runs as one CUDA graph launch whose round loop is a device-side
 * while node (re-captured only when the batch's shape changes: job sizes, samples, post options,
 * tune); RG_FLAG_HOST_LOOP, RG_FLAG_KERNEL_TIMING and RG_FLAG_COUNT_VISITS use the host-polled
 * loop instead.  In graph mode rg_timings.rtOnly covers the whole batch (post included). */
rg_status rg_render_batch(rg_ctx* ctx, const rg_job* jobs, uint32_t n);
/* Device pointer of job `job`'s RGBA32F image of the last batch (width*height*4 floats). */
rg_status rg_batch_framebuffer(rg_ctx* ctx, uint32_t job, float** d_rgba);
/* Job `job`'s image of the last batch to host memory; waits for the batch. */
rg_status rg_batch_download(rg_ctx* ctx, uint32_t job, float* host_rgba);
/* Every image of the last batch to host memory without waiting: the images, in job order and
 * contiguous (sum of width*height*4 floats), are staged on the device (one of the two read-back
 * slots rg_download_async uses) and copied to host_rgba (pinned memory for an overlapped copy) on the
 * library's copy stream while later batches render.  host_rgba must stay valid and unread until
 * rg_synchronize returns. */
rg_status rg_batch_download_async(rg_ctx* ctx, float* host_rgba);
rg_status rg_set_batch_tune(rg_ctx* ctx, const rg_batch_tune* tune);
rg_status rg_get_batch_tune(rg_ctx* ctx, rg_batch_tune* out);
/* ---- learned roughness filter -------------------------------------------------------------------
 * A 5-layer 3x3 convolutional network (12-32-64-64-32-3 channels, ReLU, layer-1 output added to the
 * input of layer 5, BF16 weights and activations, FP32 accumulation on the tensor cores) that
 * predicts the rough-reflection radiance the composite mixes in (postprocess.comp:28-50), in place of
 * the screen-space roughness approximation (rough_prepare.comp + rough_blur_h/v,
 * raytracer.cpp:112-122).  No reference counterpart beyond the passes it replaces.
 * Parameters: per layer W[out][in][3][3] then b[out], FP32, real channel counts. */
typedef struct rg_filter rg_filter;
#define RG_FILTER_PARAMS 78243u
/* He-normal weights, on ctx's device with a stream of its own (frames of a context run it on the
 * context's stream); independent of ctx's lifetime */
rg_status rg_filter_create(rg_ctx* ctx, uint64_t seed, rg_filter** out);
rg_status rg_filter_destroy(rg_filter* f);
const char* rg_filter_last_error(const rg_filter* f);
rg_status rg_filter_get_params(rg_filter* f, float* host, uint32_t n);
rg_status rg_filter_set_params(rg_filter* f, const float* host, uint32_t n);  /* also resets the Adam state */
/* gradients of the last rg_filter_train_step, in the parameter layout */
rg_status rg_filter_get_grads(rg_filter* f, float* host, uint32_t n);
/* the network on `batch` images of height x width (device memory): d_input [batch][height][width][16]
 * BF16 (channels 12..15 zero), d_out [batch][height][width][4] FP32 (RGB used) */
rg_status rg_filter_forward(rg_filter* f, const void* d_input, uint32_t batch, uint32_t height, uint32_t width, float* d_out);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) on the mean squared error against d_target
 * [batch][height][width][4] FP32 (RGB used); lr 0 computes the gradients only.  *loss_out: the loss
 * before the step */
rg_status rg_filter_train_step(rg_filter* f, const void* d_input, const float* d_target, uint32_t batch, uint32_t height, uint32_t width,
                               float lr, float* loss_out);
/* the filter input of the context's last frame, d_out [H][W][16] BF16: rough RGB, normal, log-scaled
 * linear depth, roughness term (rough.a), base colour, reflect contribution */
rg_status rg_filter_input(rg_ctx* ctx, void* d_out);
/* the rough RGB of the context's last frame, d_out [H][W][4] FP32 (training target of a glossy frame) */
rg_status rg_filter_target(rg_ctx* ctx, float* d_out);
/* frames of this context (rg_render) use the filter in place of the roughness passes (NULL: the plain
 * passes); batch jobs use it when they ask for it (RG_JOB_FILTER) */
rg_status rg_set_filter(rg_ctx* ctx, rg_filter* f);
/* glossy reference shading (training targets; 0 = off, the default): at each sample's primary hit
 * the reflection and refraction directions are drawn around their mirror directions from a GGX lobe
 * of the material roughness (alpha = roughness^2), seeded per pixel sample from `seed` */
rg_status rg_set_glossy(rg_ctx* ctx, uint32_t seed);

/* Device memory the context holds (all scene slots, images, path state, scratch) and its budget
 * (rg_device_opts.hbm_budget_bytes, 0 = none), in bytes. */
rg_status rg_get_memory(rg_ctx* ctx, uint64_t* allocated_bytes, uint64_t* budget_bytes);
/* Path slots of the batch loop: at most this many samples are in flight, and a slot whose path ends
 * takes the next sample.  Default 2^25, about 1.6 KB of device memory each (54 GB when a batch has
 * that many samples; a batch of fewer samples takes one slot per sample).  Fewer slots narrow every
 * round: 2^23 slots rendered the 64-scene benchmark batch 4 % slower, 2^20 slots 34 % slower. */
rg_status rg_set_batch_slots(rg_ctx* ctx, uint32_t slots);
/* Autotuner of the batch loop: renders the batch once (warm-up, capture) and then `reps` times
 * with every launch shape of the grid threads {64,128,256} x stack depth {16,24,32,48} x sort key
 * {none, octant, morton} (36 configurations, in that nesting order), keeps the fastest one whose
 * render had no traversal-stack overflow (the results of every configuration are identical unless
 * the stack overflows) and selects it.  ms_out (nullable, 36 floats): mean milliseconds per batch
 * of each configuration, -1 where the stack overflowed or the shape is not built (256 threads with
 * 48 entries exceeds a block's static shared memory).  No reference counterpart. */
#define RG_AUTOTUNE_CONFIGS 36
rg_status rg_autotune_batch(rg_ctx* ctx, const rg_job* jobs, uint32_t n, uint32_t reps, rg_batch_tune* best, float* ms_out);

/* ---- parity / inspection entry points (no reference counterpart: the Vulkan driver's BVHs are
 * opaque) ---- */
/* BVH2 of a BLAS (blas) or of the TLAS (blas = 0xFFFFFFFF): Morton codes per primitive (LBVHs; zero
 * for a binned-SAH BLAS, unspecified for a binned-SAH TLAS), sorted order, children of the n-1
 * internal nodes (bit 31 = leaf, payload = sorted position) and the internal node boxes (6 floats: lo
 * xyz, hi xyz).  Pointers may be NULL.  *n_out = primitive count. */
rg_status rg_bvh_info(rg_ctx* ctx, uint32_t blas, uint32_t* n_out, uint32_t* morton, uint32_t* order, uint32_t* left,
                      uint32_t* right, float* nodeboxes);
/* The traversal's 4-wide records of a BLAS (blas) or of the TLAS (blas = 0xFFFFFFFF), one per
 * internal BVH2 node, 112 bytes each: float lo_x[4], hi_x[4], lo_y[4], hi_y[4], lo_z[4], hi_z[4] (the
 * boxes of the node's grandchildren, a leaf child standing in for its own slot); uint32 ref[4] (bit 31 =
 * leaf; 0xFFFFFFFE = empty slot, box lo = +inf, hi = -inf).  Copies min(capacity, n - 1) records to
 * out (may be NULL); *n_out = n - 1. */
rg_status rg_bvh_records(rg_ctx* ctx, uint32_t blas, void* out, uint32_t capacity, uint32_t* n_out);
/* World-to-object transforms the TLAS build computed (12 floats per instance). */
rg_status rg_instance_inverse(rg_ctx* ctx, float* out);
/* Closest hit of n rays (8 floats: origin.xyz, tmin, dir.xyz, tmax) through the current TLAS:
 * hit_tuv n x 3 (t, u, v), hit_ids n x 2 (instance, primitive; 0xFFFFFFFF = miss).  The traversal
 * stack has the batch launch shape's depth (rg_set_batch_tune; 48 by default).  Resets the per-frame
 * statistics: rg_get_stats afterwards reports this call's stack_overflows / deep_overflows. */
rg_status rg_trace_rays(rg_ctx* ctx, const float* rays, uint32_t n, float* hit_tuv, uint32_t* hit_ids);
/* The same closest hits from and into device memory, asynchronous on the context's stream, traced by
 * one launch of the frame loop's traversal kernel, which reads the rays where they are (d_rays
 * 16-byte aligned, else RG_ERR_INVALID_ARG) and writes the hits straight into d_hit_tuv / d_hit_ids;
 * no shading follows.  Stack depth as rg_trace_rays' (48 with RG_FLAG_COUNT_VISITS); rays that
 * overflow it are traced again with the deep stack.  The hits equal rg_trace_rays'.  Like the reference's traceRayEXT of a batch of rays with no
 * shading (closesthit.rchit:215,232,244 issue such rays), it is how incoherent secondary-ray
 * throughput is measured.  Resets the per-frame statistics (stack_overflows; nodes / tris with
 * RG_FLAG_COUNT_VISITS). */
rg_status rg_trace_rays_device(rg_ctx* ctx, const float* d_rays, uint32_t n, float* d_hit_tuv, uint32_t* d_hit_ids);
/* Post passes alone on host G-buffers (width*height*4 floats each, current resolution):
 * writes the framebuffer; used to check the post kernels on identical inputs. */
rg_status rg_post_only(rg_ctx* ctx, const rg_ubo* ubo, const float* base, const float* normal, const float* rough,
                       int32_t fxaa);

/* Raw LBVH build over host boxes (n x 6 floats), for the builder's parity tests. */
rg_status rg_lbvh_build_host(rg_ctx* ctx, const float* boxes, uint32_t n, uint32_t* morton, uint32_t* order,
                             uint32_t* left, uint32_t* right, float* nodeboxes);

/* L2 bandwidth of device `device` (no counterpart in the reference; the measure the traversal's
 * roofline is quoted against, since a frame's BVH records and triangles stay in L2): a working set
 * of working_set_bytes (1 MiB .. 1 GiB; well under the L2 size to measure L2) read with 16-byte
 * loads, and copied half into half, `reps` passes per launch, best of four launches timed with CUDA
 * events, in GB/s (copy counts read + write bytes).  Allocates and frees its own buffers. */
rg_status rg_measure_l2(int32_t device, uint64_t working_set_bytes, int32_t reps, double* read_gbs, double* copy_gbs);

/* LBVH build that allocates nothing (no counterpart in the reference).  For callers that must not
 * allocate device memory after start-up -- an engine that owns a fixed memory arena, or a frame
 * loop that cannot afford the device synchronisation a cudaMalloc may cause.  Same results as
 * rg_lbvh_build_host, but every pointer is a caller-owned DEVICE buffer (d_boxes: n x 6 floats;
 * d_morton, d_order: n; d_left, d_right: n-1; d_nodeboxes: (n-1) x 6 floats) and the work is queued
 * on `stream` (a cudaStream_t, NULL = legacy default stream) without waiting for it.  Scratch memory
 * is one fixed file-scope device array (about 1.9 MiB) that each GPU loading this library holds until
 * exit.  n > RG_LBVH_NOALLOC_MAX_PRIMS returns RG_ERR_TOO_LARGE.  All calls share that array: calls
 * whose GPU work overlaps (e.g. on two unsynchronised streams) race.  The first call on a device
 * looks up the array's device address with that device current; make it before any stream
 * capture. */
#define RG_LBVH_NOALLOC_MAX_PRIMS 65536u
rg_status rg_lbvh_build_device_noalloc(const float* d_boxes, uint32_t n, uint32_t* d_morton, uint32_t* d_order,
                                       uint32_t* d_left, uint32_t* d_right, float* d_nodeboxes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RGCUDA_H */
