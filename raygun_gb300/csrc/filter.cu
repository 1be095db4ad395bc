// filter.cu -- the learned roughness filter on the 5th-generation tensor cores.
//
// A 5-layer 3x3 convolutional network stands in for the screen-space roughness approximation
// (rough_prepare.comp + 10 x rough_blur_h/v, raytracer.cpp:112-122): from the frame's G-buffers it
// predicts the rough-reflection radiance that the composite (postprocess.comp:28-50) mixes in.
//   layers: 16(12 used) -> 32 -> 64 -> 64 -> 32 -> 16(3 used), ReLU after layers 1-4, the output of
//   layer 1 added to the input of layer 5 (skip), every layer at full resolution.
// Activations are BF16 NHWC, accumulation FP32 in tensor memory.  Each convolution is an implicit
// GEMM: a CTA takes a tile of 2 image rows x 128 pixels (M = 128 output pixels per row), stages the
// 4 x 130 input patch in shared memory as channel-chunk planes [chunk][pixel][8 channels] (16 B per
// pixel and chunk) and issues, per row, 9 taps x Cin/16 tcgen05.mma (kind::f16, BF16 x BF16 -> F32)
// whose A descriptors point straight into the patch at the tap's offset: no im2col copy.  The data
// gradient is the same kernel on transposed, flipped weights; the weight gradient is a GEMM over
// pixels with both operands MN-major (channels contiguous), accumulated in tensor memory per CTA and
// reduced across CTAs in a fixed order (deterministic).
//
// Descriptor conventions (no swizzle): core matrix = 8 rows x 16 bytes; the leading-byte offset is
// the stride between core matrices along K, the stride-byte offset the stride along M / N.
#include <algorithm>
#include <atomic>

#include <cuda.h>
#include <cuda_bf16.h>

#include "rg_internal.cuh"
#include "rg_tma.cuh"

namespace rg {

namespace {

using bf16 = __nv_bfloat16;

// ---- tcgen05 / mbarrier helpers ----------------------------------------------------------------
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of tcgen05.mma kind::f16: D F32, A and B BF16, M x N, operand majors
__host__ __device__ constexpr uint32_t umma_idesc(int m, int n, bool aMN, bool bMN) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (aMN ? 1u << 15 : 0u) | (bMN ? 1u << 16 : 0u) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols));
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
          "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// 16 consecutive FP32 columns of this thread's TMEM lane, without waiting (tmem_wait_ld before use)
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
          "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint4 add_bf16x8(uint4 a, uint4 b) {
    const bf16* x = reinterpret_cast<const bf16*>(&a);
    const bf16* y = reinterpret_cast<const bf16*>(&b);
    uint4 o;
    bf16* z = reinterpret_cast<bf16*>(&o);
#pragma unroll
    for (int j = 0; j < 8; ++j) z[j] = __float2bfloat16(__bfloat162float(x[j]) + __bfloat162float(y[j]));
    return o;
}

constexpr int kTileRows = 2, kTilePx = 128, kPatchRows = kTileRows + 2, kPatchW = kTilePx + 2;
constexpr int kPatchPlane = kPatchRows * kPatchW * 16;  // bytes of one channel-chunk plane of the patch

// stages the (kTileRows + 2) x 130 input patch of tile (b, y0, x0) as [chunk][pixel][8]; x2 (nullable)
// is added element-wise; outside the image reads zero
template <int CIN>
__device__ __forceinline__ void load_patch(uint8_t* patch, const bf16* __restrict__ x, const bf16* __restrict__ x2, int b, int y0,
                                           int x0, int H, int W) {
    constexpr int CC = CIN / 8, NP = kPatchRows * kPatchW;
    for (int i = threadIdx.x; i < CC * NP; i += blockDim.x) {
        const int pix = i % NP, cc = i / NP;
        const int gy = y0 - 1 + pix / kPatchW, gx = x0 - 1 + pix % kPatchW;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
            const size_t off = (((size_t)b * H + gy) * W + gx) * CIN + cc * 8;
            v = *reinterpret_cast<const uint4*>(x + off);
            if (x2) v = add_bf16x8(v, *reinterpret_cast<const uint4*>(x2 + off));
        }
        *reinterpret_cast<uint4*>(patch + (size_t)cc * kPatchPlane + (size_t)pix * 16) = v;
    }
}

}  // namespace

namespace {

// Row-streaming convolution.  A work item is a strip of 128 output pixels x a segment of rows of
// one image; a CTA walks its items down the rows, three output rows (a group) at a time.  Input rows
// (130 pixels: the strip and a 1-pixel halo, zero outside the image) stream through a ring of
// shared-memory slots, each row loaded once per item as channel-chunk planes [chunk][pixel][8].  Input
// row i feeds output rows i+1, i, i-1 through the kernel rows dy = 0, 1, 2, so a group's accumulator is
// a window of three adjacent TMEM blocks and each of its five input rows r-1 .. r+3 feeds it with ONE
// tcgen05.mma per column tap dx and 16-channel step (M = 128 pixels, N = COUT, 2 COUT, 3 COUT, 2 COUT,
// COUT), the B operand stacking the kernel rows' weights.  62 MMAs instead of 108 per 3 rows of a
// 64-channel layer, each issued from fully unrolled code with constant offsets: one issuing thread
// must keep the tensor core fed, so the issue path carries no arithmetic beyond descriptor adds.
// Warp roles (320 threads):
//   warp 0     TMA producer: refills a slot once the MMAs of the last group reading its row completed;
//   warp 1     MMA issuer: group by group into alternating accumulator windows;
//   warps 2-9  epilogue, two warps per TMEM lane quarter (half the channels each): drain a completed
//              window (bias, ReLU, skip add, mask) and hand it back; BF16 rows leave through a small
//              swizzled shared-memory stage so that each store instruction writes whole sectors.
constexpr int kStripPx = 128, kRowW = kStripPx + 2;
constexpr int kRowPlane = 2176;  // 130 pixels x 16 B rounded up to 128 B (TMA destination alignment)
constexpr int kEpiWarps = 8;
constexpr int kConvThreads = 32 * (2 + kEpiWarps);
constexpr int kGroupRows = 3;

template <int CIN, int COUT>
struct ConvShape {
    static constexpr int CC = CIN / 8;
    static constexpr int kRing = 8;                               // input row slots
    static constexpr int kWin = 3 * COUT;                         // TMEM columns of one group's window
    static constexpr int kWindows = 3 * COUT * 4 <= 512 ? 4 : 2;  // accumulator windows (groups in flight)
    static constexpr int kRowBytes = CC * kRowPlane;              // one slot
    static constexpr uint32_t kRowTx = CC * kRowW * 16;           // bytes the TMA writes per row
    static constexpr int kWeightBytes = 9 * CIN * COUT * 2;       // [dx][ci/8][kernel row 2, 1, 0][co][8]
    static constexpr int kStageBytes = 32 * COUT;                 // per epilogue warp: 32 pixels x COUT/2 channels (BF16)
    static constexpr int kSmem = kWeightBytes + kRing * kRowBytes + kEpiWarps * kStageBytes + 1024;
    static constexpr uint32_t kCols = kWindows * kWin <= 32 ? 32 : (kWindows * kWin <= 64 ? 64 : (kWindows * kWin <= 128 ? 128 : (kWindows * kWin <= 256 ? 256 : 512)));
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && kWin <= 256 && kWindows * kWin <= 512, "shape");
    static_assert(kWeightBytes % 128 == 0, "ring slots 128-byte aligned");
};

// bounded wait that also gives up when another role has given up (abort flag in shared memory)
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* mbar, uint32_t phase, volatile int* abort, int* status) {
    for (int spin = 0; spin < (1 << 22); ++spin) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(phase)
            : "memory");
        if (done) return true;
        if ((spin & 255) == 255 && *abort) return false;
    }
    *abort = 1;
    if (status) atomicExch(status, 3);  // 3: a wait of the learned filter gave up
    return false;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// 8 consecutive FP32 columns of this thread's TMEM lane, without waiting (tmem_wait_ld before use)
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

// A warp's 32 pixels x NC 16-byte chunks in shared memory, chunk c of pixel p at slot c ^ f(p) so that
// both the per-pixel writes and the row-order reads below touch 8 distinct bank groups per phase.
template <int NC>
__device__ __forceinline__ uint32_t stage_off(int p, int c) {
    const int f = NC == 1 ? 0 : (p / (8 / NC)) % NC;
    return (uint32_t)(p * NC * 16 + ((c ^ f) * 16));
}
// copies the staged 32 x NC chunks to dst (pixel p at dst + p * pixStride bytes), pixels < valid only
template <int NC>
__device__ __forceinline__ void stage_out(const uint8_t* stage, uint8_t* dst, size_t pixStride, int valid, int lane) {
#pragma unroll
    for (int it = 0; it < NC; ++it) {
        const int k = it * 32 + lane, p = k / NC, c = k % NC;
        const uint4 v = *reinterpret_cast<const uint4*>(stage + stage_off<NC>(p, c));
        if (p < valid) *reinterpret_cast<uint4*>(dst + (size_t)p * pixStride + c * 16) = v;
    }
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(kConvThreads, 1) k_filter_conv(const __grid_constant__ CUtensorMap tmapX, const FilterConvArgs a,
                                                                 int segRows) {
    using S = ConvShape<CIN, COUT>;
    using bf16 = __nv_bfloat16;
    constexpr int CC = S::CC, NW = S::kWindows, KK = CIN / 16;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* wsm = smem;
    uint8_t* ring = smem + S::kWeightBytes;
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t full[S::kRing], empty[S::kRing], accFull[NW], accEmpty[NW], drain;
    __shared__ int abortFlag, issuedRows, consumedRows;
    __shared__ float biasSm[COUT];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // weights: packed [tap = dy * 3 + dx][ci/8][co][8] -> [dx][ci/8][kernel row 2, 1, 0][co][8]
    for (int i = tid; i < S::kWeightBytes / 16; i += blockDim.x) {
        const int co = i % COUT, dyr = (i / COUT) % 3, cc = (i / (3 * COUT)) % CC, dx = i / (3 * COUT * CC);
        const int tap = (2 - dyr) * 3 + dx;
        reinterpret_cast<uint4*>(wsm)[i] = reinterpret_cast<const uint4*>(a.w)[((size_t)tap * CC + cc) * COUT + co];
    }
    for (int i = tid; i < COUT; i += blockDim.x) biasSm[i] = a.bias ? a.bias[i] : 0.0f;
    if (tid == 0) {
        for (int k = 0; k < S::kRing; ++k) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], 1);
        }
        for (int k = 0; k < NW; ++k) {
            mbar_init(&accFull[k], 1);
            mbar_init(&accEmpty[k], kEpiWarps);
        }
        mbar_init(&drain, 1);
        abortFlag = 0;
        issuedRows = consumedRows = 0;
        mbar_init_fence();
    }
    async_proxy_fence();  // the weights are read by the tensor core
    if (warp == 1) tmem_alloc(&tmem_base, S::kCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    volatile int* abort = &abortFlag;
    // segRows is a multiple of 3; a segment's last group may run past the image (zero input rows,
    // results not stored)
    const int strips = (a.W + kStripPx - 1) / kStripPx, segs = (a.H + segRows - 1) / segRows;
    const int items = a.B * strips * segs;
    auto item_of = [&](int item, int& b, int& x0, int& ys, int& ng) {
        b = item / (strips * segs);
        const int rem = item % (strips * segs);
        x0 = (rem / segs) * kStripPx;
        ys = (rem % segs) * segRows;
        ng = (min(ys + segRows, a.H) - ys + kGroupRows - 1) / kGroupRows;
    };
    if (warp == 0) {
        if (lane == 0) {  // producer: input rows ys - 1 .. ys + 3 ng of each item
            int seq = 0;
            bool ok = true;
            for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
                int b, x0, ys, ng;
                item_of(item, b, x0, ys, ng);
                for (int k = 0; k < kGroupRows * ng + 2 && ok; ++k, ++seq) {
                    const int slot = seq % S::kRing, fill = seq / S::kRing;
                    if (fill > 0 && !mbar_wait_or_abort(&empty[slot], (uint32_t)((fill - 1) & 1), abort, a.status)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&full[slot], S::kRowTx);
#pragma unroll 1
                    for (int cc = 0; cc < CC; ++cc)
                        tma_load_4d(ring + slot * S::kRowBytes + cc * kRowPlane, &tmapX, cc * 8, x0 - 1, ys - 1 + k, b, &full[slot]);
                    issuedRows = seq + 1;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            // descriptors: the start address sits in the low 14 bits (address / 16) and every operand
            // lies below 256 KB, so offsets add to it without a carry
            const uint64_t adesc0 = umma_desc(smem_u32(ring), kRowPlane, 128), bdesc0 = umma_desc(smem_u32(wsm), 3 * COUT * 16, 128);
            constexpr uint32_t id1 = umma_idesc(128, COUT, false, false), id2 = umma_idesc(128, 2 * COUT, false, false),
                               id3 = umma_idesc(128, 3 * COUT, false, false);
            int base = 0, waited = 0, g = 0;  // first input row of the item, input rows waited for, groups issued
            bool ok = true;
            for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
                int b, x0, ys, ng;
                item_of(item, b, x0, ys, ng);
                for (int j = 0; j < ng && ok; ++j, ++g) {
                    const int w = g % NW;
                    if (g >= NW && !mbar_wait_or_abort(&accEmpty[w], (uint32_t)((g / NW - 1) & 1), abort, a.status)) {
                        ok = false;
                        break;
                    }
                    const int first = base + kGroupRows * j;  // input row r - 1 of this group
                    for (; waited < first + 5; ++waited)
                        if (!mbar_wait_or_abort(&full[waited % S::kRing], (uint32_t)((waited / S::kRing) & 1), abort, a.status)) {
                            ok = false;
                            break;
                        }
                    if (!ok) break;
                    consumedRows = waited;
                    tc_fence_after();
                    uint64_t arow[5];
#pragma unroll
                    for (int p = 0; p < 5; ++p) arow[p] = adesc0 + (uint64_t)((((first + p) % S::kRing) * S::kRowBytes) >> 4);
                    const uint32_t d0 = tmem + (uint32_t)(w * S::kWin);
#pragma unroll
                    for (int dx = 0; dx < 3; ++dx)
#pragma unroll
                        for (int kk = 0; kk < KK; ++kk) {
                            const uint64_t aoff = (uint64_t)((2 * kk * kRowPlane + dx * 16) >> 4);
                            const uint64_t bk = bdesc0 + (uint64_t)((dx * CC + 2 * kk) * 3 * COUT);
                            const bool f = dx == 0 && kk == 0;  // the step where rows r+1 and r+2 start
                            // input r - 1: row r (kernel row 0)
                            umma(d0, arow[0] + aoff, bk + 2 * COUT, id1, f ? 0u : 1u);
                            // input r: rows r, r + 1 (kernel rows 1, 0)
                            if (f) {
                                umma(d0, arow[1] + aoff, bk + COUT, id1, 1u);
                                umma(d0 + COUT, arow[1] + aoff, bk + 2 * COUT, id1, 0u);
                            } else {
                                umma(d0, arow[1] + aoff, bk + COUT, id2, 1u);
                            }
                            // input r + 1: rows r .. r + 2 (kernel rows 2, 1, 0)
                            if (f) {
                                umma(d0, arow[2] + aoff, bk, id2, 1u);
                                umma(d0 + 2 * COUT, arow[2] + aoff, bk + 2 * COUT, id1, 0u);
                            } else {
                                umma(d0, arow[2] + aoff, bk, id3, 1u);
                            }
                            // input r + 2: rows r + 1, r + 2 (kernel rows 2, 1); input r + 3: row r + 2
                            umma(d0 + COUT, arow[3] + aoff, bk, id2, 1u);
                            umma(d0 + 2 * COUT, arow[4] + aoff, bk, id1, 1u);
                        }
                    umma_commit(&accFull[w]);
                    // input rows no later group of the item reads
                    umma_commit(&empty[first % S::kRing]);
                    umma_commit(&empty[(first + 1) % S::kRing]);
                    umma_commit(&empty[(first + 2) % S::kRing]);
                    if (j == ng - 1) {
                        umma_commit(&empty[(first + 3) % S::kRing]);
                        umma_commit(&empty[(first + 4) % S::kRing]);
                    }
                }
                base += kGroupRows * ng + 2;
            }
            umma_commit(&drain);  // completes when every MMA issued above has
            mbar_wait(&drain, 0u, nullptr);
        }
    } else {  // epilogue: TMEM lane quarter warp % 4 = pixels 32 (warp % 4) .. + 31; channel half h
        constexpr int CH = COUT / 2, NC = CH / 8;
        const int q = warp & 3, h = (warp - 2) >> 2, cbase = h * CH;
        uint8_t* stage = ring + S::kRing * S::kRowBytes + (warp - 2) * S::kStageBytes;
        int g = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
            int b, x0, ys, ng;
            item_of(item, b, x0, ys, ng);
            const int ye = min(ys + segRows, a.H);
            const int xx = x0 + q * 32 + lane;
            for (int j = 0; j < ng; ++j, ++g) {
                const int w = g % NW;
                // narrow layers fetch the skip input of the group's rows before waiting for the
                // accumulators (registers allow it); 64-channel layers and masks load in place
                constexpr bool kPre = NC <= 2;
                constexpr int PR = kPre ? kGroupRows : 1;
                uint4 addPre[PR][NC];
                auto aux_load = [&](const bf16* src, int y, int c) {
                    return src && y < ye && xx < a.W ? reinterpret_cast<const uint4*>(src + (((size_t)b * a.H + y) * a.W + xx) * COUT + cbase)[c]
                                                     : make_uint4(0u, 0u, 0u, 0u);
                };
                if (kPre) {
#pragma unroll
                    for (int r = 0; r < PR; ++r)
#pragma unroll
                        for (int c = 0; c < NC; ++c) addPre[r][c] = aux_load(a.add, ys + kGroupRows * j + r, c);
                }
                if (!mbar_wait_or_abort(&accFull[w], (uint32_t)((g / NW) & 1), abort, a.status)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                uint32_t raw[kGroupRows][CH];
#pragma unroll
                for (int r = 0; r < kGroupRows; ++r)
#pragma unroll
                    for (int c = 0; c < CH; c += 8)
                        tmem_ld8_nowait(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(w * S::kWin + r * COUT + cbase + c), raw[r] + c);
                tmem_wait_ld();
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&accEmpty[w]);  // the window goes back before the math and stores
#pragma unroll
                for (int r = 0; r < kGroupRows; ++r) {
                    const int y = ys + kGroupRows * j + r;
                    if (y >= ye) continue;  // uniform across the warp
                    const size_t px0 = ((size_t)b * a.H + y) * a.W + x0 + q * 32;  // pixel of lane 0
                    const size_t px = px0 + lane;
                    const bool in = xx < a.W;
                    const int valid = min(32, a.W - (x0 + q * 32));
                    float v[CH];
#pragma unroll
                    for (int e = 0; e < CH; ++e) {
                        v[e] = __uint_as_float(raw[r][e]) + biasSm[cbase + e];
                        if (a.relu) v[e] = fmaxf(v[e], 0.0f);
                    }
                    auto put = [&](bf16* out, const float* vals, const uint4* mask) {  // BF16 row out through the stage
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            __align__(16) bf16 o[8];
                            if (mask) {
                                const bf16* mv = reinterpret_cast<const bf16*>(&mask[c]);
#pragma unroll
                                for (int e = 0; e < 8; ++e) o[e] = __float2bfloat16(__bfloat162float(mv[e]) > 0.0f ? vals[8 * c + e] : 0.0f);
                            } else {
#pragma unroll
                                for (int e = 0; e < 8; ++e) o[e] = __float2bfloat16(vals[8 * c + e]);
                            }
                            *reinterpret_cast<uint4*>(stage + stage_off<NC>(lane, c)) = *reinterpret_cast<uint4*>(o);
                        }
                        __syncwarp();
                        stage_out<NC>(stage, reinterpret_cast<uint8_t*>(out + px0 * COUT + cbase), (size_t)COUT * 2, valid, lane);
                        __syncwarp();
                    };
                    if (a.y) put(a.y, v, nullptr);
                    if (a.add) {
                        // forward skip (a.ya): the sum of the stored BF16 activations, x5 = bf16(bf16(y4) + y1);
                        // backward (the skip gradient into layer 1's): FP32 sum, rounded once on the way out
                        const bool storedSum = a.ya != nullptr;
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            const uint4 av = kPre ? addPre[kPre ? r : 0][c] : aux_load(a.add, y, c);
                            const bf16* hv = reinterpret_cast<const bf16*>(&av);
#pragma unroll
                            for (int e = 0; e < 8; ++e) {
                                const float own = storedSum ? __bfloat162float(__float2bfloat16(v[8 * c + e])) : v[8 * c + e];
                                v[8 * c + e] = own + __bfloat162float(hv[e]);
                            }
                        }
                    }
                    if (a.ya) put(a.ya, v, nullptr);
                    if (a.yf && cbase == 0 && in) reinterpret_cast<float4*>(a.yf)[px] = make_float4(v[0], v[1], v[2], v[3]);
                    if (a.ym) {
                        uint4 mk[NC];
#pragma unroll
                        for (int c = 0; c < NC; ++c) mk[c] = aux_load(a.mask, y, c);
                        put(a.ym, v, mk);
                    }
                }
            }
        }
    }
    __syncthreads();
    // an abandoned pipeline may still have row copies in flight: wait for them (bounded) before the
    // shared memory goes away; the MMA issuer already waited for its MMAs
    if (tid == 0 && abortFlag)
        for (int k = consumedRows; k < issuedRows; ++k) mbar_wait(&full[k % S::kRing], (uint32_t)((k / S::kRing) & 1), nullptr);
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, S::kCols);
}

// ---- weight gradient: dW[co][tap][ci] = sum_p g[p][co] * x[p + tap][ci] ----------------------------
// D (M = 128 rows: output channels, padded with zero planes) x (N = CIN per tap) over K = pixels.  Both
// operands MN-major: A = g tile [co chunk][pixel][8], B = the shifted input patch [ci chunk][pixel][8].
// Each CTA accumulates its tiles for a group of taps in TMEM, then writes its partial sums.
template <int CIN, int COUT>
struct DwShape {
    static constexpr int kTaps = CIN == 64 ? 5 : 9;          // taps per CTA (two tap groups for 64 channels)
    static constexpr int kGroups = CIN == 64 ? 2 : 1;
    static constexpr int kGPlane = kTileRows * kTilePx * 16;  // bytes of one chunk plane of the g tile
    static constexpr int kGBytes = 16 * kGPlane;              // 16 planes = 128 rows of A
    static constexpr int kPatchBytes = (CIN / 8) * kPatchPlane;
    // at least 120 KB so that one CTA holds an SM (and all 512 TMEM columns) at a time
    static constexpr int kSmem = kGBytes + kPatchBytes + 1024 > 120 * 1024 ? kGBytes + kPatchBytes + 1024 : 120 * 1024;
    static constexpr uint32_t kCols = 512;
    static_assert(kTaps * CIN <= 512, "TMEM columns");
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(128, 1) k_filter_dw(const bf16* __restrict__ x, const bf16* __restrict__ x2, const bf16* __restrict__ g,
                                                      int B, int H, int W, float* __restrict__ partial, int* status) {
    using S = DwShape<CIN, COUT>;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* gsm = smem;
    uint8_t* patch = smem + S::kGBytes;
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t mbar;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tap0 = blockIdx.y * S::kTaps, ntaps = min(S::kTaps, 9 - tap0);
    for (int i = tid; i < S::kGBytes / 16; i += blockDim.x) reinterpret_cast<uint4*>(gsm)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) mbar_init(&mbar, 1);
    if (warp == 0) tmem_alloc(&tmem_base, S::kCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    const int tilesX = (W + kTilePx - 1) / kTilePx, tilesY = (H + kTileRows - 1) / kTileRows;
    const int tiles = B * tilesY * tilesX;
    constexpr uint32_t idesc = umma_idesc(128, CIN, true, true);
    uint32_t phase = 0;
    bool ok = true, first = true;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        const int b = t / (tilesY * tilesX), rem = t % (tilesY * tilesX);
        const int y0 = (rem / tilesX) * kTileRows, x0 = (rem % tilesX) * kTilePx;
        load_patch<CIN>(patch, x, x2, b, y0, x0, H, W);
        for (int i = tid; i < (COUT / 8) * kTileRows * kTilePx; i += blockDim.x) {  // g tile, zero outside the image
            const int pix = i % (kTileRows * kTilePx), cc = i / (kTileRows * kTilePx);
            const int gy = y0 + pix / kTilePx, gx = x0 + pix % kTilePx;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (gy < H && gx < W) v = *reinterpret_cast<const uint4*>(g + (((size_t)b * H + gy) * W + gx) * COUT + cc * 8);
            *reinterpret_cast<uint4*>(gsm + (size_t)cc * S::kGPlane + (size_t)pix * 16) = v;
        }
        async_proxy_fence();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t pbase = smem_u32(patch), gbase = smem_u32(gsm);
#pragma unroll 1
            for (int j = 0; j < ntaps; ++j) {
                const int tap = tap0 + j, dy = tap / 3, dx = tap % 3;
#pragma unroll 1
                for (int r = 0; r < kTileRows; ++r)
#pragma unroll 1
                    for (int kk = 0; kk < kTilePx / 16; ++kk) {
                        const uint64_t ad = umma_desc(gbase + (uint32_t)((r * kTilePx + 16 * kk) * 16), 128, S::kGPlane);
                        const uint64_t bd = umma_desc(pbase + (uint32_t)(((r + dy) * kPatchW + 16 * kk + dx) * 16), 128, kPatchPlane);
                        umma(tmem + (uint32_t)(j * CIN), ad, bd, idesc, (first && r == 0 && kk == 0) ? 0u : 1u);
                    }
            }
            umma_commit(&mbar);
        }
        first = false;
        ok = __syncthreads_and(mbar_wait(&mbar, phase, status, 1u << 24, 3)) != 0;  // also: the next tile overwrites the operands
        phase ^= 1u;
        tc_fence_after();
    }
    // partial[blockIdx.x][co][tap][ci] for this CTA's taps (zero when it had no tile)
    const int co = warp * 32 + lane;
    float* out = partial + (size_t)blockIdx.x * COUT * 9 * CIN;
    if (warp * 32 < COUT) {
#pragma unroll 1
        for (int j = 0; j < ntaps; ++j)
#pragma unroll 1
            for (int c0 = 0; c0 < CIN; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * CIN + c0), v);
                if (co < COUT)
#pragma unroll
                    for (int q = 0; q < 16; ++q)
                        out[((size_t)co * 9 + tap0 + j) * CIN + c0 + q] = (ok && !first) ? v[q] : 0.0f;
            }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, S::kCols);
}

// ---- small kernels -------------------------------------------------------------------------------
// packs layer weights W[co][ci][3][3] (FP32, real sizes) into the B-operand layout [tap][ci/8][co][8]
// of the padded shape; transposed: the data-gradient weights W'[ci][co][8 - tap] with roles swapped
__global__ void k_filter_pack(const float* __restrict__ W, int coutReal, int cinReal, int cin, int cout, int transposed,
                              bf16* __restrict__ out) {
    const int n = 9 * cin * cout;  // in the packed (possibly transposed) shape: K = 9 * cin, N = cout
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int e = i % 8, row = (i / 8) % cout, kc = i / (8 * cout);
        const int tap = kc / (cin / 8), ci = (kc % (cin / 8)) * 8 + e;  // K index = tap * cin + ci
        float v = 0.0f;
        if (!transposed) {
            if (row < coutReal && ci < cinReal) v = W[((size_t)row * cinReal + ci) * 9 + tap];
        } else {  // packed cin = layer's cout, packed cout (row) = layer's cin
            const int lco = ci, lci = row;
            if (lco < coutReal && lci < cinReal) v = W[((size_t)lco * cinReal + lci) * 9 + (8 - tap)];
        }
        out[i] = __float2bfloat16(v);
    }
}

// dW (param layout [co][ci][3][3], real sizes) = sum over CTAs of the partials [cta][co][tap][ci]
__global__ void k_filter_dw_reduce(const float* __restrict__ partial, int ctas, int cout, int cin, int coutReal, int cinReal,
                                   float* __restrict__ dW) {
    const int n = coutReal * cinReal * 9;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int tap = i % 9, ci = (i / 9) % cinReal, co = i / (9 * cinReal);
        float s = 0.0f;
        for (int c = 0; c < ctas; ++c) s += partial[(((size_t)c * cout + co) * 9 + tap) * cin + ci];
        dW[i] = s;
    }
}

// per-block channel sums of g [P][C] -> partial[block][C] (C divides 256)
__global__ void __launch_bounds__(256) k_filter_bias_partial(const bf16* __restrict__ g, size_t P, int C, float* __restrict__ partial) {
    __shared__ float acc[256];
    const int c = threadIdx.x % C, rowsPer = 256 / C, r0 = threadIdx.x / C;
    float s = 0.0f;
    for (size_t p = (size_t)blockIdx.x * rowsPer + r0; p < P; p += (size_t)gridDim.x * rowsPer) s += __bfloat162float(g[p * C + c]);
    acc[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.0f;
        for (int k = 0; k < rowsPer; ++k) t += acc[k * C + threadIdx.x];
        partial[(size_t)blockIdx.x * C + threadIdx.x] = t;
    }
}

__global__ void k_filter_bias_reduce(const float* __restrict__ partial, int blocks, int C, int cReal, float* __restrict__ db) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cReal) return;
    float s = 0.0f;
    for (int b = 0; b < blocks; ++b) s += partial[(size_t)b * C + c];
    db[c] = s;
}

// mean-squared error over the 3 predicted channels; g = d(loss)/d(out) into channels 0..2 of [P][16]
__global__ void __launch_bounds__(256) k_filter_loss(const float4* __restrict__ out, const float4* __restrict__ target, size_t P,
                                                     float scale, bf16* __restrict__ g, float* __restrict__ partial) {
    __shared__ float red[256];
    float s = 0.0f;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const float4 o = out[p], t = target[p];
        const float d0 = o.x - t.x, d1 = o.y - t.y, d2 = o.z - t.z;
        s += d0 * d0 + d1 * d1 + d2 * d2;
        __align__(16) bf16 v[16];
        v[0] = __float2bfloat16(2.0f * scale * d0);
        v[1] = __float2bfloat16(2.0f * scale * d1);
        v[2] = __float2bfloat16(2.0f * scale * d2);
        for (int j = 3; j < 16; ++j) v[j] = __float2bfloat16(0.0f);
        uint4* dst = reinterpret_cast<uint4*>(g + p * 16);
        dst[0] = reinterpret_cast<uint4*>(v)[0];
        dst[1] = reinterpret_cast<uint4*>(v)[1];
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters
__global__ void k_filter_adam(float* __restrict__ w, const float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v, int n,
                              float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = grad[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__device__ __forceinline__ float4 unpack_half4(uint2 u) {
    const __half2 a = *reinterpret_cast<const __half2*>(&u.x), b = *reinterpret_cast<const __half2*>(&u.y);
    const float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}

// the 16-channel filter input of one frame from its RGBA16F G-buffers (channels 12..15 zero):
//   0-2 rough RGB (reflection / refraction radiance), 3-5 normal, 6 log-scaled linear depth,
//   7 roughness term (rough.a), 8-10 base colour, 11 reflect contribution
__global__ void k_filter_gbuffer(const uint2* __restrict__ base, const uint2* __restrict__ normal, const uint2* __restrict__ rough, size_t P,
                                 float samples, bf16* __restrict__ out) {
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const float4 b = unpack_half4(base[p]), n = unpack_half4(normal[p]), r = unpack_half4(rough[p]);
        // normal.w = log(sum of sample depths) * 0.25 / S  ->  mean depth
        const float depth = expf(n.w * 4.0f * samples) / samples;
        const float ld = log1pf(fmaxf(depth, 0.0f)) * 0.108574f;  // / log(10001)
        const float c[12] = {r.x, r.y, r.z, n.x, n.y, n.z, ld, r.w, b.x, b.y, b.z, b.w};
        __align__(16) bf16 v[16];
#pragma unroll
        for (int j = 0; j < 12; ++j) v[j] = __float2bfloat16(c[j]);
#pragma unroll
        for (int j = 12; j < 16; ++j) v[j] = __float2bfloat16(0.0f);
        uint4* dst = reinterpret_cast<uint4*>(out + p * 16);
        dst[0] = reinterpret_cast<uint4*>(v)[0];
        dst[1] = reinterpret_cast<uint4*>(v)[1];
    }
}

// postprocess.comp:28-50 with the filter's prediction in place of roughColorsA
__global__ void k_filter_composite(const uint2* __restrict__ base, const float4* __restrict__ pred, size_t P, float4 fade, int showAlpha,
                                   uint2* __restrict__ finalImg) {
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const float4 b = unpack_half4(base[p]), r = pred[p];
        float cr = fminf(fmaxf(b.x * (1.0f - b.w) + r.x * b.w, 0.0f), 1.0f);
        float cg = fminf(fmaxf(b.y * (1.0f - b.w) + r.y * b.w, 0.0f), 1.0f);
        float cb = fminf(fmaxf(b.z * (1.0f - b.w) + r.z * b.w, 0.0f), 1.0f);
        const float luma = (cr * 0.299f + cg * 0.587f) + cb * 0.114f;
        cr = cr * (1.0f - fade.w) + fade.x * fade.w;
        cg = cg * (1.0f - fade.w) + fade.y * fade.w;
        cb = cb * (1.0f - fade.w) + fade.z * fade.w;
        if (showAlpha) cr = cg = cb = luma;  // postprocess.comp:41-49 debug view
        const __half2 lo = __floats2half2_rn(cr, cg), hi = __floats2half2_rn(cb, luma);
        uint2 o;
        o.x = *reinterpret_cast<const uint32_t*>(&lo);
        o.y = *reinterpret_cast<const uint32_t*>(&hi);
        finalImg[p] = o;
    }
}

// RGBA16F rough image of a (glossy) reference render -> FP32 RGBx targets
__global__ void k_filter_target(const uint2* __restrict__ rough, size_t P, float4* __restrict__ out) {
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const float4 r = unpack_half4(rough[p]);
        out[p] = make_float4(r.x, r.y, r.z, 0.0f);
    }
}


// tensor map of an NHWC BF16 activation [B][H][W][C]: boxes of 8 channels x 130 pixels x 1 row
cudaError_t patch_map(CUtensorMap* map, const void* x, int B, int H, int W, int C) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return cudaErrorNotSupported;
    if ((reinterpret_cast<uintptr_t>(x) & 15u) != 0) return cudaErrorMisalignedAddress;
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    const cuuint32_t box[4] = {8, (cuuint32_t)kRowW, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// CTAs per SM of a persistent kernel: shared memory, registers and TMEM columns (512 per SM)
template <class K>
int ctas_per_sm(K kernel, int smem, uint32_t tmemCols, int threads) {
    int dev = 0, smemSm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smemSm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return 1;
    int per = smemSm / (smem + 1024);
    per = std::min(per, 65536 / std::max(1, fa.numRegs * threads));
    per = std::min(per, (int)(512 / tmemCols));
    per = std::min(per, 16);
    return std::max(per, 1);
}

template <int CIN, int COUT>
cudaError_t conv_launch(const FilterConvArgs& a, cudaStream_t s) {
    using S = ConvShape<CIN, COUT>;
    static std::atomic<int> gridCache{0};
    int grid = gridCache.load(std::memory_order_acquire);
    if (!grid) {
        cudaError_t e = cudaFuncSetAttribute(k_filter_conv<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kSmem);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = sms * ctas_per_sm(k_filter_conv<CIN, COUT>, S::kSmem, S::kCols, kConvThreads);
        gridCache.store(grid, std::memory_order_release);
    }
    if (a.B <= 0 || a.H <= 0 || a.W <= 0) return cudaSuccess;
    CUtensorMap map;
    cudaError_t e = patch_map(&map, a.x, a.B, a.H, a.W, CIN);
    if (e != cudaSuccess) return e;
    // segments of rows (a multiple of 3): about two items per CTA, at least 9 rows (each item re-reads
    // 2 halo rows)
    const long long strips = (a.W + kStripPx - 1) / kStripPx, rowsTotal = (long long)a.B * strips * a.H;
    int segRows = (int)std::min<long long>(a.H, std::max<long long>(9, (rowsTotal + 2LL * grid - 1) / (2LL * grid)));
    segRows = (segRows + kGroupRows - 1) / kGroupRows * kGroupRows;
    const long long items = (long long)a.B * strips * ((a.H + segRows - 1) / segRows);
    k_filter_conv<CIN, COUT><<<(int)std::min<long long>(items, grid), kConvThreads, S::kSmem, s>>>(map, a, segRows);
    count_launch();
    return cudaGetLastError();
}

template <int CIN, int COUT>
cudaError_t dw_launch(const bf16* x, const bf16* x2, const bf16* g, int B, int H, int W, float* partial, int ctas, int* status,
                      cudaStream_t s) {
    using S = DwShape<CIN, COUT>;
    static std::atomic<bool> attr{false};
    if (!attr.load(std::memory_order_acquire)) {
        cudaError_t e = cudaFuncSetAttribute(k_filter_dw<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kSmem);
        if (e != cudaSuccess) return e;
        attr.store(true, std::memory_order_release);
    }
    k_filter_dw<CIN, COUT><<<dim3(ctas, S::kGroups), 128, S::kSmem, s>>>(x, x2, g, B, H, W, partial, status);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

// ---- launchers (rg_internal.cuh) ---------------------------------------------------------------------
cudaError_t filter_conv(int cin, int cout, const FilterConvArgs& a, cudaStream_t s) {
    if (cin == 16 && cout == 32) return conv_launch<16, 32>(a, s);
    if (cin == 32 && cout == 64) return conv_launch<32, 64>(a, s);
    if (cin == 64 && cout == 64) return conv_launch<64, 64>(a, s);
    if (cin == 64 && cout == 32) return conv_launch<64, 32>(a, s);
    if (cin == 32 && cout == 16) return conv_launch<32, 16>(a, s);
    return cudaErrorInvalidValue;
}

int filter_dw_ctas() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

cudaError_t filter_dw(int cin, int cout, const void* x, const void* x2, const void* g, int B, int H, int W, float* partial, int ctas,
                      int* status, cudaStream_t s) {
    const bf16 *X = static_cast<const bf16*>(x), *X2 = static_cast<const bf16*>(x2), *G = static_cast<const bf16*>(g);
    if (cin == 16 && cout == 32) return dw_launch<16, 32>(X, X2, G, B, H, W, partial, ctas, status, s);
    if (cin == 32 && cout == 64) return dw_launch<32, 64>(X, X2, G, B, H, W, partial, ctas, status, s);
    if (cin == 64 && cout == 64) return dw_launch<64, 64>(X, X2, G, B, H, W, partial, ctas, status, s);
    if (cin == 64 && cout == 32) return dw_launch<64, 32>(X, X2, G, B, H, W, partial, ctas, status, s);
    if (cin == 32 && cout == 16) return dw_launch<32, 16>(X, X2, G, B, H, W, partial, ctas, status, s);
    return cudaErrorInvalidValue;
}

cudaError_t filter_pack(const float* W, int coutReal, int cinReal, int cin, int cout, int transposed, void* out, cudaStream_t s) {
    k_filter_pack<<<64, 256, 0, s>>>(W, coutReal, cinReal, cin, cout, transposed, static_cast<bf16*>(out));
    count_launch();
    return cudaGetLastError();
}

cudaError_t filter_dw_reduce(const float* partial, int ctas, int cout, int cin, int coutReal, int cinReal, float* dW, cudaStream_t s) {
    k_filter_dw_reduce<<<64, 256, 0, s>>>(partial, ctas, cout, cin, coutReal, cinReal, dW);
    count_launch();
    return cudaGetLastError();
}

cudaError_t filter_bias_grad(const void* g, size_t P, int C, int cReal, float* partial, int blocks, float* db, cudaStream_t s) {
    k_filter_bias_partial<<<blocks, 256, 0, s>>>(static_cast<const bf16*>(g), P, C, partial);
    k_filter_bias_reduce<<<1, 64, 0, s>>>(partial, blocks, C, cReal, db);
    count_launch(2);
    return cudaGetLastError();
}

cudaError_t filter_loss(const float4* out, const float4* target, size_t P, float scale, void* g, float* partial, int blocks, cudaStream_t s) {
    k_filter_loss<<<blocks, 256, 0, s>>>(out, target, P, scale, static_cast<bf16*>(g), partial);
    count_launch();
    return cudaGetLastError();
}

cudaError_t filter_adam(float* w, const float* grad, float* m, float* v, int n, float lr, float b1, float b2, float eps, float c1,
                        float c2, cudaStream_t s) {
    k_filter_adam<<<128, 256, 0, s>>>(w, grad, m, v, n, lr, b1, b2, eps, c1, c2);
    count_launch();
    return cudaGetLastError();
}

cudaError_t filter_gbuffer(const uint2* base, const uint2* normal, const uint2* rough, size_t P, float samples, void* out, cudaStream_t s) {
    k_filter_gbuffer<<<(unsigned)((P + 255) / 256 < 4096 ? (P + 255) / 256 : 4096), 256, 0, s>>>(base, normal, rough, P, samples,
                                                                                                 static_cast<bf16*>(out));
    count_launch();
    return cudaGetLastError();
}

cudaError_t filter_composite(const uint2* base, const float4* pred, size_t P, const float fade[4], int showAlpha, uint2* finalImg,
                             cudaStream_t s) {
    k_filter_composite<<<(unsigned)((P + 255) / 256 < 4096 ? (P + 255) / 256 : 4096), 256, 0, s>>>(
        base, pred, P, make_float4(fade[0], fade[1], fade[2], fade[3]), showAlpha, finalImg);
    count_launch();
    return cudaGetLastError();
}

namespace {
__global__ void k_filter_bias_pad(const float* __restrict__ b, int cReal, int c, float* __restrict__ out) {
    const int i = threadIdx.x;
    if (i < c) out[i] = i < cReal ? b[i] : 0.0f;
}
}  // namespace

cudaError_t filter_bias_pad(const float* b, int cReal, int c, float* out, cudaStream_t s) {
    k_filter_bias_pad<<<1, 64, 0, s>>>(b, cReal, c, out);
    count_launch();
    return cudaGetLastError();
}

cudaError_t filter_target(const uint2* rough, size_t P, float4* out, cudaStream_t s) {
    k_filter_target<<<(unsigned)((P + 255) / 256 < 4096 ? (P + 255) / 256 : 4096), 256, 0, s>>>(rough, P, out);
    count_launch();
    return cudaGetLastError();
}

}  // namespace rg
