// noalloc.cu -- LBVH build into caller-owned device buffers, with no device allocation at all.
//
// The context-based entry points grow their device buffers with cudaMalloc as scenes grow.  Some
// callers cannot allow that: a host engine that hands this library a fixed memory arena at start-up
// and forbids allocations afterwards (frame pacing, fragmentation, its own budget accounting), or a
// frame loop that must not stall, since cudaMalloc can synchronise the device.  For those callers
// this entry point builds the same LBVH as rg_lbvh_build_host, but all of its scratch memory lives
// in one file-scope __device__ array of fixed size, which the CUDA driver places when it loads this
// library onto a GPU and which every GPU that loads the library keeps until the process exits.
//
// Limits and rules (also stated in include/rgcuda.h):
//   * at most RG_LBVH_NOALLOC_MAX_PRIMS primitives per call; larger builds are rejected with
//     RG_ERR_TOO_LARGE before any work is queued;
//   * every call, on every stream, shares the one scratch array, so calls whose GPU work overlaps
//     race with each other; serialise them (one stream, or events between streams);
//   * the first call on a device resolves the array's device address (cudaGetSymbolAddress) with
//     that device current; make that first call before any stream capture.
#include <mutex>

#include "rg_internal.cuh"

namespace rg {
namespace {

constexpr uint32_t kMaxPrims = RG_LBVH_NOALLOC_MAX_PRIMS;
constexpr size_t kAlign = 256;

constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// scratch layout for kMaxPrims primitives
constexpr size_t kKeysBytes = align_up(4ull * kMaxPrims);
constexpr size_t kSortStateBytes = align_up(4ull * sort_state_words(kMaxPrims));
constexpr size_t kParentsBytes = align_up(8ull * kMaxPrims);
constexpr size_t kFlagsBytes = align_up(4ull * kMaxPrims);
constexpr size_t kBoundsBytes = align_up(64);
constexpr size_t kScratchBytes = 4 * kKeysBytes + kSortStateBytes + kParentsBytes + kFlagsBytes + kBoundsBytes;

static __device__ __align__(256) unsigned char g_lbvh_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// device address of g_lbvh_scratch on the current device (resolved once per device)
cudaError_t scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_lbvh_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace rg

extern "C" rg_status rg_lbvh_build_device_noalloc(const float* d_boxes, uint32_t n, uint32_t* d_morton, uint32_t* d_order,
                                                  uint32_t* d_left, uint32_t* d_right, float* d_nodeboxes, void* stream) {
    using namespace rg;
    if (n > kMaxPrims) return RG_ERR_TOO_LARGE;
    if (n == 0) return RG_OK;
    if (!d_boxes || !d_morton || !d_order) return RG_ERR_INVALID_ARG;
    if (n > 1 && (!d_left || !d_right || !d_nodeboxes)) return RG_ERR_INVALID_ARG;
    unsigned char* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return RG_ERR_CUDA;
    LbvhBuffers b;
    b.n = n;
    b.primBoxes = const_cast<float*>(d_boxes);  // read only by the build
    b.morton = d_morton;
    b.order = d_order;
    b.left = d_left;
    b.right = d_right;
    b.nodeBoxes = d_nodeboxes;
    unsigned char* p = base;
    b.keysA = reinterpret_cast<uint32_t*>(p); p += kKeysBytes;
    b.keysB = reinterpret_cast<uint32_t*>(p); p += kKeysBytes;
    b.valsA = reinterpret_cast<uint32_t*>(p); p += kKeysBytes;
    b.valsB = reinterpret_cast<uint32_t*>(p); p += kKeysBytes;
    b.sortState = reinterpret_cast<uint32_t*>(p); p += kSortStateBytes;  // zeroed by the build
    b.parents = reinterpret_cast<uint32_t*>(p); p += kParentsBytes;
    b.flags = reinterpret_cast<uint32_t*>(p); p += kFlagsBytes;  // zeroed inside lbvh_build (refit step)
    b.bounds = reinterpret_cast<uint32_t*>(p);                    // reset by the build's first kernel
    cudaError_t e = lbvh_build(b, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? RG_OK : RG_ERR_CUDA;
}
