// measure.cu -- the L2 bandwidth the traversal's roofline is measured against.
//
// A frame's BVH records, triangles and vertices (tens of MB) stay in the 126 MB L2 while the frame
// traces, so the traversal kernel's memory roof is the L2's bandwidth, not HBM's.  This measures it
// on the device at hand: a working set well inside L2 read (float4 loads, summed) and copied, many
// passes inside one launch, timed with CUDA events.  No counterpart in the reference.
#include <algorithm>

#include "rg_internal.cuh"

namespace rg {
namespace {

__global__ void k_bw_read(const float4* __restrict__ a, size_t n, int reps, float* __restrict__ sink) {
    float acc = 0.0f;
    for (int r = 0; r < reps; ++r)
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
            const float4 v = __ldcg(a + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    if (acc == 1234.5f) *sink = acc;  // keeps the loads
}

__global__ void k_bw_copy(const float4* __restrict__ a, float4* __restrict__ b, size_t n, int reps) {
    for (int r = 0; r < reps; ++r)
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
            __stcg(b + i, __ldcg(a + i));
}

}  // namespace
}  // namespace rg

extern "C" rg_status rg_measure_l2(int32_t device, uint64_t working_set_bytes, int32_t reps, double* read_gbs, double* copy_gbs) {
    using namespace rg;
    if (!read_gbs || !copy_gbs || reps < 1 || working_set_bytes < (1u << 20) || working_set_bytes > (1ull << 30))
        return RG_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return RG_ERR_NO_DEVICE;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return RG_ERR_CUDA;
    const size_t n = working_set_bytes / 32;  // float4 elements per buffer: read uses both halves, copy one into the other
    float4 *a = nullptr, *b = nullptr;
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    rg_status st = RG_OK;
    if (cudaMalloc(&a, 32 * n) != cudaSuccess || cudaMalloc(&sink, 4) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        st = RG_ERR_OUT_OF_MEMORY;
    } else {
        b = a + n;
        cudaMemset(a, 0, 32 * n);
        const int grid = sms * 8;
        float ms = 0.0f;
        double best = 0.0;
        for (int t = 0; t < 4; ++t) {  // best of four launches (the first warms L2)
            cudaEventRecord(e0);
            k_bw_read<<<grid, 256>>>(a, 2 * n, reps, sink);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
            best = std::max(best, 32.0 * n * reps / (ms * 1e-3) / 1e9);
        }
        *read_gbs = best;
        best = 0.0;
        for (int t = 0; t < 4; ++t) {
            cudaEventRecord(e0);
            k_bw_copy<<<grid, 256>>>(a, b, n, reps);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
            best = std::max(best, 32.0 * n * reps / (ms * 1e-3) / 1e9);
        }
        *copy_gbs = best;
        count_launch(8);
        if (cudaGetLastError() != cudaSuccess) st = RG_ERR_CUDA;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (a) cudaFree(a);
    if (sink) cudaFree(sink);
    return st;
}
