// lbvh.cu -- linear BVH builder (BLAS over triangles, TLAS over instance boxes).
//
// Replaces the driver-side builds of BottomLevelAS / TopLevelAS
// (render/acceleration_structure.cpp:55-194), which the reference leaves opaque:
//   1. primitive boxes (triangles: min/max of the three vertices)
//   2. centroid bounds (order-preserving uint atomics: exact, order independent)
//   3. 30-bit Morton codes of the centroids, normalised to the cube of the largest centroid extent
//   4. stable LSD radix sort of (code, primitive) in four 8-bit passes, one onesweep kernel each
//   5. Karras 2012 hierarchy (n-1 internal nodes; equal codes split on the index)
//   6. bottom-up boxes: one thread per leaf climbs; the second arrival at a node writes its box
// Refit (topology kept, boxes recomputed) reruns step 6 only.
#include <cstdlib>

#include "rg_internal.cuh"

namespace rg {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortRounds = 8;
static_assert(kSortWarps * kSortRounds * 32 == kSortTileKeys, "one onesweep tile per block");
constexpr uint32_t kMortonMaxBlocks = 608;  // grid-stride: bounds the global histogram atomics

__global__ void k_tri_boxes(const rg_vertex* __restrict__ v, const uint32_t* __restrict__ idx, uint32_t vOff, uint32_t iOff,
                            uint32_t n, float* __restrict__ boxes) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        const float* pos = v[vOff + idx[iOff + 3 * p + k]].position;
        for (int a = 0; a < 3; ++a) {
            float x = pos[a];
            lo[a] = k == 0 ? x : fminf(lo[a], x);
            hi[a] = k == 0 ? x : fmaxf(hi[a], x);
        }
    }
    float* o = boxes + 6 * (size_t)p;
    o[0] = lo[0]; o[1] = lo[1]; o[2] = lo[2]; o[3] = hi[0]; o[4] = hi[1]; o[5] = hi[2];
}

// triangle records in leaf order: v0 (w = primitive id), v1, v2
__global__ void k_tri_records(const rg_vertex* __restrict__ v, const uint32_t* __restrict__ idx, uint32_t vOff, uint32_t iOff,
                              const uint32_t* __restrict__ order, uint32_t n, float4* __restrict__ tris) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t p = order[k];
    const float* a = v[vOff + idx[iOff + 3 * p + 0]].position;
    const float* b = v[vOff + idx[iOff + 3 * p + 1]].position;
    const float* c = v[vOff + idx[iOff + 3 * p + 2]].position;
    tris[3 * (size_t)k + 0] = make_float4(a[0], a[1], a[2], __uint_as_float(p));
    tris[3 * (size_t)k + 1] = make_float4(b[0], b[1], b[2], 0.0f);
    tris[3 * (size_t)k + 2] = make_float4(c[0], c[1], c[2], 0.0f);
}

__device__ inline void centroid(const float* b, float* c) {
    if (!(b[0] <= b[3])) {  // empty box (invalid instance): keyed at the origin
        c[0] = c[1] = c[2] = 0.0f;
        return;
    }
    for (int a = 0; a < 3; ++a) c[a] = __fmul_rn(__fadd_rn(b[a], b[3 + a]), 0.5f);
}

__global__ void k_bounds_init(uint32_t* bounds) {
    if (threadIdx.x < 3) bounds[threadIdx.x] = 0xFFFFFFFFu;
    else if (threadIdx.x < 6) bounds[threadIdx.x] = 0u;
}

__global__ void __launch_bounds__(256) k_centroid_bounds(const float* __restrict__ boxes, uint32_t n, uint32_t* bounds) {
    __shared__ float red[6][8];
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        float c[3];
        centroid(boxes + 6 * (size_t)p, c);
        for (int a = 0; a < 3; ++a) {
            mn[a] = fminf(mn[a], c[a]);
            mx[a] = fmaxf(mx[a], c[a]);
        }
    }
    for (int off = 16; off > 0; off >>= 1)
        for (int a = 0; a < 3; ++a) {
            mn[a] = fminf(mn[a], __shfl_xor_sync(0xFFFFFFFFu, mn[a], off));
            mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xFFFFFFFFu, mx[a], off));
        }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) {
            red[a][w] = mn[a];
            red[3 + a][w] = mx[a];
        }
    __syncthreads();
    // one atomic per block and bound (same-address atomics from every warp serialise in L2)
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        float lo = red[a][0], hi = red[3 + a][0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            lo = fminf(lo, red[a][k]);
            hi = fmaxf(hi, red[3 + a][k]);
        }
        if (lo <= hi) {  // the block saw a centroid
            atomicMin(&bounds[a], f2ord(lo));
            atomicMax(&bounds[3 + a], f2ord(hi));
        }
    }
}

// codes, the sort's input (keys, and values = primitive ids in BOTH value buffers, so that every
// word of either is a valid primitive id whatever a pass writes), and the four digit histograms of
// the sort (grid-stride; one shared-memory histogram per block, flushed with global atomics)
__global__ void __launch_bounds__(256) k_morton(const float* __restrict__ boxes, uint32_t n, const uint32_t* __restrict__ bounds,
                                                uint32_t* __restrict__ morton, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                uint32_t* __restrict__ valsAlt, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[4 * 256];
    for (int i = threadIdx.x; i < 4 * 256; i += 256) h[i] = 0;
    // every axis is scaled by the LARGEST centroid extent (a cube), so a thin axis spends few of its
    // 10 bits and the hierarchy splits mostly along the long axes
    float lo[3], inv[3];
    float emax = 0.0f;
    for (int a = 0; a < 3; ++a) {
        lo[a] = ord2f(bounds[a]);
        emax = fmaxf(emax, __fsub_rn(ord2f(bounds[3 + a]), lo[a]));
    }
    for (int a = 0; a < 3; ++a) inv[a] = emax > 0.0f ? __fdiv_rn(1.0f, emax) : 0.0f;
    __syncthreads();
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        float c[3];
        centroid(boxes + 6 * (size_t)p, c);
        uint32_t x = quant10(c[0], lo[0], inv[0]), y = quant10(c[1], lo[1], inv[1]), z = quant10(c[2], lo[2], inv[2]);
        uint32_t m = (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
        morton[p] = m;
        keys[p] = m;
        vals[p] = p;
        valsAlt[p] = p;
#pragma unroll
        for (int d = 0; d < 4; ++d) atomicAdd(&h[256 * d + ((m >> (8 * d)) & 0xFFu)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += 256)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// ---- onesweep LSD radix sort (Adinets & Merrill 2022) --------------------------------------------
// k_morton counts the four 8-bit digit histograms of the codes as it writes them.  Each of the four
// passes is then ONE kernel: a block takes the next tile in launch order (an atomic counter, so every
// earlier tile belongs to a block that is already running), ranks its kSortTileKeys keys by digit
// (stable: warp chunks in key order, lanes in key order), publishes its per-digit counts, and finds
// how many keys of each digit precede it by decoupled look-back over the earlier tiles' published
// words, then scatters.  A status word is flag (bits 31:30) | count (bits 29:0): 0 = not yet
// published, kStatAgg = this tile's own count, kStatIncl = count over this and all earlier tiles.
// A look-back that finds a predecessor unpublished polls it a bounded number of times and then
// counts that tile's keys of the digit directly from the input, so no wait is unbounded and the
// result does not depend on the bound.
constexpr uint32_t kStatAgg = 1u << 30;
constexpr uint32_t kStatIncl = 2u << 30;
constexpr uint32_t kStatCount = (1u << 30) - 1u;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// exclusive prefix sum over the block's 256 threads (one value each); `warpSums` holds 8 words
__device__ __forceinline__ uint32_t block_exclusive_256(uint32_t v, uint32_t* warpSums) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warpSums[w] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int k = 0; k < w; ++k) before += warpSums[k];
    return before + x - v;
}

__global__ void __launch_bounds__(kSortThreads) k_sort_onesweep(const uint32_t* __restrict__ keysIn, const uint32_t* __restrict__ valsIn,
                                                                 uint32_t* __restrict__ keysOut, uint32_t* __restrict__ valsOut,
                                                                 uint32_t n, int pass, uint32_t* __restrict__ state, uint32_t nTiles,
                                                                 uint32_t spinLimit) {
    __shared__ uint32_t wc[kSortWarps][256];
    __shared__ uint32_t digitBase[256];
    __shared__ uint32_t warpSums[kSortWarps];
    __shared__ uint32_t tileShared;
    const int shift = 8 * pass;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) tileShared = atomicAdd(state + kSortTileCounters + pass, 1u);
    for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads) (&wc[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = tileShared;
    const uint32_t ltmask = (1u << lane) - 1u;
    const uint32_t base = tile * kSortTileKeys + w * (kSortRounds * 32);
    uint32_t key[kSortRounds], val[kSortRounds], pos[kSortRounds];
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        uint32_t i = base + r * 32 + lane;
        bool ok = i < n;
        key[r] = ok ? keysIn[i] : 0u;
        val[r] = ok ? valsIn[i] : 0u;
        uint32_t digit = ok ? ((key[r] >> shift) & 0xFFu) : (256u + lane);
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
        uint32_t before = ok ? wc[w][digit] : 0u;
        __syncwarp();
        pos[r] = before + __popc(peers & ltmask);
        if (ok && (peers & ltmask) == 0) wc[w][digit] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // thread d: this tile's count of digit d, and each warp's exclusive offset within the tile
    const uint32_t d = threadIdx.x;
    uint32_t cnt = 0;
    for (int ww = 0; ww < kSortWarps; ++ww) {
        uint32_t t = wc[ww][d];
        wc[ww][d] = cnt;
        cnt += t;
    }
    uint32_t* status = state + kSortStatusOffset + (size_t)pass * nTiles * 256;
    st_relaxed(status + (size_t)tile * 256 + d, (tile == 0 ? kStatIncl : kStatAgg) | cnt);
    // keys of smaller digits in the whole input (this pass's histogram)
    const uint32_t globalBefore = block_exclusive_256(state[256 * pass + d], warpSums);
    // keys of digit d in earlier tiles
    uint32_t earlier = 0;
    for (int64_t t = (int64_t)tile - 1; t >= 0; --t) {
        const uint32_t* sp = status + (size_t)t * 256 + d;
        uint32_t v = ld_relaxed(sp);
        for (uint32_t spins = 0; (v >> 30) == 0 && spins < spinLimit; ++spins) {
            __nanosleep(100);
            v = ld_relaxed(sp);
        }
        if ((v >> 30) == 0) {  // still unpublished: count tile t's keys of digit d from the input
            uint32_t c = 0;
            const uint32_t b0 = (uint32_t)t * kSortTileKeys, b1 = min(n, b0 + kSortTileKeys);
            for (uint32_t i = b0; i < b1; ++i) c += ((keysIn[i] >> shift) & 0xFFu) == d;
            v = kStatAgg | c;
        }
        earlier += v & kStatCount;
        if ((v >> 30) == 2) break;
    }
    if (tile > 0) st_relaxed(status + (size_t)tile * 256 + d, kStatIncl | (earlier + cnt));
    digitBase[d] = globalBefore + earlier;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r) {
        uint32_t i = base + r * 32 + lane;
        if (i < n) {
            uint32_t dg = (key[r] >> shift) & 0xFFu;
            uint32_t dst = digitBase[dg] + wc[w][dg] + pos[r];
            if (dst < n) {  // always true: the counts are exact
                keysOut[dst] = key[r];
                valsOut[dst] = val[r];
            }
        }
    }
}

// TLAS leaf k: the instance at sorted position k with its inverse rows and its BLAS's root box
// and record pointers copied in
__global__ void k_inst_records(const uint32_t* __restrict__ order, uint32_t n, const DevInstance* __restrict__ inst,
                               const DevBlas* __restrict__ blas, InstRec* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t ii = order[k];
    const DevInstance& d = inst[ii];
    InstRec r;
    r.inv[0] = d.inv[0];
    r.inv[1] = d.inv[1];
    r.inv[2] = d.inv[2];
    r.lo = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0u));
    r.hi = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(ii));
    r.wide = nullptr;
    r.tris = nullptr;
    if (d.valid) {
        const DevBlas& b = blas[d.blas];
        r.lo = make_float4(b.root[0], b.root[1], b.root[2], __uint_as_float(b.n));
        r.hi = make_float4(b.root[3], b.root[4], b.root[5], __uint_as_float(ii));
        r.wide = b.wide;
        r.tris = b.tris;
    }
    out[k] = r;
}

// ---- Karras 2012 hierarchy ----------------------------------------------------------------------
__device__ inline int delta(const uint32_t* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = k[i], b = k[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ left, uint32_t* __restrict__ right,
                         uint32_t* __restrict__ parents) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = (int)n;
    if (i >= N - 1) return;
    int d = (delta(keys, N, i, i + 1) - delta(keys, N, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, N, i, i - d);
    int lmax = 2;
    while (delta(keys, N, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(keys, N, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, N, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, N, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    uint32_t L = (lo == gamma) ? (kLeaf | (uint32_t)gamma) : (uint32_t)gamma;
    uint32_t R = (hi == gamma + 1) ? (kLeaf | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    left[i] = L;
    right[i] = R;
    parents[(L & kLeaf) ? (n - 1) + (L & ~kLeaf) : L] = (uint32_t)i;
    parents[(R & kLeaf) ? (n - 1) + (R & ~kLeaf) : R] = (uint32_t)i;
    if (i == 0) parents[0] = 0xFFFFFFFFu;
}

// ---- bottom-up boxes ----------------------------------------------------------------------------
__device__ inline void load_box_cg(const float* p, float* b) {
    for (int a = 0; a < 6; ++a) b[a] = __ldcg(p + a);
}

__device__ __forceinline__ uint32_t arrive(uint32_t* flag) {  // release my box, acquire my sibling's
    uint32_t old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(flag) : "memory");
    return old;
}

// one thread per leaf climbs towards the root and writes each node's box as the union of its
// children's.  The climbing thread keeps the box of the child it comes from in registers and loads
// only its sibling's.  A leaf sibling's box is input data, so a node with a leaf child needs no
// arrival: the thread from its inner child (or, for two leaves, from its left leaf) goes on and the
// other stops at once.  A node with two inner children takes the arrival counter: the first
// arrival stops, the second (which then sees the first's box: release / acquire) goes on.
__global__ void k_bottom_up(const float* __restrict__ primBoxes, const uint32_t* __restrict__ order, uint32_t n,
                            const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                            const uint32_t* __restrict__ parents, uint32_t* flags, float* nodeBoxes) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t node = parents[(n - 1) + k];
    uint32_t from = kLeaf | k;
    float cur[6];  // loaded once this thread knows that it goes on from its leaf
    // a finished tree has at most 64 levels and in-range parents; the bounds keep a tree that a
    // failed build left unfinished from sending the climb out of range or round in circles
    for (int level = 0; node < n - 1u && level < 128; ++level) {  // the root's parent is 0xFFFFFFFF
        const uint32_t L = left[node], R = right[node];
        const uint32_t other = L == from ? R : L;
        if ((other & kLeaf) ? (other & ~kLeaf) >= n : other >= n - 1u) break;  // in range in a finished tree
        if (other & kLeaf) {
            if ((from & kLeaf) && L != from) return;  // two leaves: the left one goes on
        } else if (from & kLeaf) {
            return;  // the thread from the inner child goes on
        } else if (arrive(&flags[node]) == 0) {
            return;  // two inner children: the second arrival goes on
        }
        if (level == 0) load_box_cg(primBoxes + 6 * (size_t)order[k], cur);
        float ob[6];
        if (other & kLeaf) load_box_cg(primBoxes + 6 * (size_t)order[other & ~kLeaf], ob);
        else load_box_cg(nodeBoxes + 6 * (size_t)other, ob);
        const float* bl = L == from ? cur : ob;
        const float* br = L == from ? ob : cur;
        float nb[6];
        for (int a = 0; a < 3; ++a) {
            nb[a] = fminf(bl[a], br[a]);
            nb[3 + a] = fmaxf(bl[3 + a], br[3 + a]);
        }
        float* o = nodeBoxes + 6 * (size_t)node;
        for (int a = 0; a < 6; ++a) {
            __stcg(o + a, nb[a]);
            cur[a] = nb[a];
        }
        from = node;
        node = parents[node];
    }
}

// ---- 4-wide records ----------------------------------------------------------------------------
__device__ inline void child_box(const float* __restrict__ primBoxes, const uint32_t* __restrict__ order, const float* nodeBoxes,
                                 uint32_t ref, float* b) {
    const float* p = (ref & kLeaf) ? primBoxes + 6 * (size_t)order[ref & ~kLeaf] : nodeBoxes + 6 * (size_t)ref;
    for (int a = 0; a < 6; ++a) b[a] = p[a];
}

__global__ void k_wide_records(const float* __restrict__ primBoxes, const uint32_t* __restrict__ order, uint32_t n,
                               const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                               const float* __restrict__ nodeBoxes, WideNode* __restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 >= n) return;
    uint32_t refs[4];
    int k = 0;
    for (uint32_t c : {left[i], right[i]}) {
        if (c & kLeaf) {
            refs[k++] = c;
        } else {
            refs[k++] = left[c];
            refs[k++] = right[c];
        }
    }
    float lo[3][4], hi[3][4];
    uint32_t r[4];
    for (int j = 0; j < 4; ++j) {
        if (j < k) {
            float b[6];
            child_box(primBoxes, order, nodeBoxes, refs[j], b);
            for (int a = 0; a < 3; ++a) {
                lo[a][j] = b[a];
                hi[a][j] = b[3 + a];
            }
            r[j] = refs[j];
        } else {
            for (int a = 0; a < 3; ++a) {
                lo[a][j] = INFINITY;
                hi[a][j] = -INFINITY;
            }
            r[j] = kEmptySlot;
        }
    }
    WideNode w;
    w.lox = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
    w.hix = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
    w.loy = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
    w.hiy = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
    w.loz = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
    w.hiz = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
    w.ref = make_uint4(r[0], r[1], r[2], r[3]);
    out[i] = w;
}

// ---- binned-SAH BVH2 (TLAS, and BLASes up to kSahBlasMaxPrims triangles) ------------------------
// One CTA builds a BVH2 over the primitive boxes, top-down, level by level: each warp takes a node
// task (a range of the order array), reduces the range's box and centroid box, bins the centroids into
// 16 bins per axis (shared-memory atomics on order-preserving integer images of the bounds), evaluates
// the 45 surface-area-heuristic splits, partitions the range stably with ballots, and emits its
// children (single primitives become leaf refs, the rest next-level tasks).  Every split leaves both
// sides non-empty, so each level shortens every range.  From level medianLevel on, ranges are halved
// without binning, so no tree is deeper than medianLevel + ceil(log2 n) levels, whatever the centroid
// distribution (a surface-area split can peel one primitive off a range per level).
// Internal nodes are numbered in level order (a level's tasks follow the previous levels' nodes), so
// a task is just its range.  The result has the LBVH's layout (order, left, right, nodeBoxes), so
// records, refits and traversal are shared.
constexpr int kSahBins = 16;
constexpr int kSahWarps = 32;
constexpr int kSahTaskWarps = 8;               // warps per block of k_sah_tasks
constexpr uint32_t kSahHandoff = 64;           // tasks of a level from which k_sah_tasks takes over
constexpr int kSahParallelLevels = 6;          // levels built by k_sah_level, one launch each
constexpr uint32_t kSahWaitLimit = 1u << 22;   // polls of an unpublished task before k_sah_tasks gives up

__device__ __forceinline__ int ord_float(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float unord_float(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }
__device__ __forceinline__ float half_area3(const float* lo, const float* hi) {
    const float dx = fmaxf(hi[0] - lo[0], 0.0f), dy = fmaxf(hi[1] - lo[1], 0.0f), dz = fmaxf(hi[2] - lo[2], 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

// The cheapest of the 3 x 15 surface-area splits of a task's bins (ties to the lowest candidate),
// reduced over the calling warp (all 32 lanes call it); -1 when no split leaves both sides
// non-empty.  cnt(a, k), lo(a, k, c), hi(a, k, c) read bin k of axis a (bounds as ordered ints).
template <class Cnt, class Lo, class Hi>
__device__ __forceinline__ int sah_best_split(const float* scale, int lane, Cnt cnt, Lo lo, Hi hi) {
    float bestCost = INFINITY;
    int bestCand = -1;
    for (int cand = lane; cand < 3 * (kSahBins - 1); cand += 32) {
        const int a = cand / (kSahBins - 1), sp = cand % (kSahBins - 1) + 1;
        if (scale[a] <= 0.0f) continue;
        float L0[3] = {INFINITY, INFINITY, INFINITY}, L1[3] = {-INFINITY, -INFINITY, -INFINITY};
        float R0[3] = {INFINITY, INFINITY, INFINITY}, R1[3] = {-INFINITY, -INFINITY, -INFINITY};
        int nl = 0, nr = 0;
        for (int k = 0; k < kSahBins; ++k) {
            const int n = cnt(a, k);
            if (!n) continue;
            float* X0 = k < sp ? L0 : R0;
            float* X1 = k < sp ? L1 : R1;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                X0[c] = fminf(X0[c], unord_float(lo(a, k, c)));
                X1[c] = fmaxf(X1[c], unord_float(hi(a, k, c)));
            }
            if (k < sp) nl += n;
            else nr += n;
        }
        if (!nl || !nr) continue;
        const float cost = half_area3(L0, L1) * (float)nl + half_area3(R0, R1) * (float)nr;
        if (cost < bestCost) {
            bestCost = cost;
            bestCand = cand;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float oc = __shfl_xor_sync(0xFFFFFFFFu, bestCost, off);
        const int oi = __shfl_xor_sync(0xFFFFFFFFu, bestCand, off);
        if (oi >= 0 && (bestCand < 0 || oc < bestCost || (oc == bestCost && oi < bestCand))) {
            bestCost = oc;
            bestCand = oi;
        }
    }
    return bestCand;
}

// One level with fewer tasks than warps: G warps share a task (G * count <= 32), each taking a
// contiguous chunk of the task's range.  The same computation as one warp per task -- bounds and bin
// contents are order-independent minima, maxima and counts, the split is chosen by the same rule, and
// the partition stays stable (each warp writes its chunk at the offsets of the chunks before it) --
// so the tree is the same; the top levels just run on the whole CTA instead of a few warps.
__device__ __forceinline__ void sah_level_grouped(const float* __restrict__ boxes, uint32_t* __restrict__ order, uint32_t* __restrict__ tmp,
                                                  uint32_t* __restrict__ left, uint32_t* __restrict__ right, float* __restrict__ nodeBoxes,
                                                  const uint2* cur, uint2* nxt, uint32_t count, bool median, uint32_t baseCur,
                                                  uint32_t baseNext, uint32_t& nNext, int (*bLo)[3][kSahBins][3],
                                                  int (*bHi)[3][kSahBins][3], int (*bCnt)[3][kSahBins], float (*gPart)[12],
                                                  float (*tClo)[3], float (*tScale)[3], int* tBest, uint32_t* wLeft) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t G = kSahWarps;
    while (G * count > (uint32_t)kSahWarps) G >>= 1;
    const uint32_t t = (uint32_t)warp / G, m = (uint32_t)warp % G;
    const bool has = t < count;  // warp-uniform
    const int lw = (int)(t * G);  // the task's leader warp (owner of its bins)
    uint32_t b = 0, e = 0, cb = 0, ce = 0, node = 0;
    if (has) {
        const uint2 tk = cur[t];
        b = tk.x;
        e = tk.y;
        node = baseCur + t;
        const uint32_t chunk = (e - b + G - 1) / G;
        cb = min(e, b + m * chunk);
        ce = min(e, cb + chunk);
    }
    // bounds and centroid bounds of the chunk, then of the task
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = cb + lane; i < ce; i += 32) {
        const float* bx = boxes + 6 * (size_t)order[i];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], bx[a]);
            hi[a] = fmaxf(hi[a], bx[3 + a]);
            const float c = 0.5f * (bx[a] + bx[3 + a]);
            clo[a] = fminf(clo[a], c);
            chi[a] = fmaxf(chi[a], c);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xFFFFFFFFu, lo[a], off));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xFFFFFFFFu, hi[a], off));
            clo[a] = fminf(clo[a], __shfl_xor_sync(0xFFFFFFFFu, clo[a], off));
            chi[a] = fmaxf(chi[a], __shfl_xor_sync(0xFFFFFFFFu, chi[a], off));
        }
    if (lane == 0)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            gPart[warp][a] = lo[a];
            gPart[warp][3 + a] = hi[a];
            gPart[warp][6 + a] = clo[a];
            gPart[warp][9 + a] = chi[a];
        }
    __syncthreads();
    if (has && m == 0) {
        if (lane == 0) {
            for (uint32_t g = 1; g < G; ++g)
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    lo[a] = fminf(lo[a], gPart[lw + g][a]);
                    hi[a] = fmaxf(hi[a], gPart[lw + g][3 + a]);
                    clo[a] = fminf(clo[a], gPart[lw + g][6 + a]);
                    chi[a] = fmaxf(chi[a], gPart[lw + g][9 + a]);
                }
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                nodeBoxes[6 * (size_t)node + a] = lo[a];
                nodeBoxes[6 * (size_t)node + 3 + a] = hi[a];
                const float ext = chi[a] - clo[a];
                tClo[t][a] = clo[a];
                tScale[t][a] = ext > 0.0f ? (float)kSahBins / ext : 0.0f;
            }
        }
    }
    __syncthreads();
    float tc[3] = {0.0f, 0.0f, 0.0f}, ts[3] = {0.0f, 0.0f, 0.0f};
    if (has)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            tc[a] = tClo[t][a];
            ts[a] = tScale[t][a];
        }
    auto bin_of = [&](const float* bx, int a) {
        const float c = 0.5f * (bx[a] + bx[3 + a]);
        return max(0, min((int)((c - tc[a]) * ts[a]), kSahBins - 1));
    };
    if (has && !median) {  // every warp bins its chunk into its own bins (no atomics across warps)
        for (int k = lane; k < 3 * kSahBins; k += 32) {
            const int a = k / kSahBins, bn = k % kSahBins;
            bCnt[warp][a][bn] = 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                bLo[warp][a][bn][c] = ord_float(INFINITY);
                bHi[warp][a][bn][c] = ord_float(-INFINITY);
            }
        }
        __syncwarp();
        for (uint32_t i = cb + lane; i < ce; i += 32) {
            const float* bx = boxes + 6 * (size_t)order[i];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (ts[a] <= 0.0f) continue;
                const int k = bin_of(bx, a);
                atomicAdd(&bCnt[warp][a][k], 1);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    atomicMin(&bLo[warp][a][k][c], ord_float(bx[c]));
                    atomicMax(&bHi[warp][a][k][c], ord_float(bx[3 + c]));
                }
            }
        }
    }
    __syncthreads();
    if (has && m == 0) {  // the leader picks the split: cheapest surface-area cost, ties to the lowest candidate
        int bestCand = -1;
        if (!median) {
            // the group's bins into the leader's (counts add, bounds are minima and maxima: exact)
            for (int k = lane; k < 3 * kSahBins; k += 32) {
                const int a = k / kSahBins, bn = k % kSahBins;
                int cnt = bCnt[lw][a][bn];
                int l[3], h[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    l[c] = bLo[lw][a][bn][c];
                    h[c] = bHi[lw][a][bn][c];
                }
                for (uint32_t g = 1; g < G; ++g) {
                    cnt += bCnt[lw + g][a][bn];
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        l[c] = min(l[c], bLo[lw + g][a][bn][c]);
                        h[c] = max(h[c], bHi[lw + g][a][bn][c]);
                    }
                }
                bCnt[lw][a][bn] = cnt;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    bLo[lw][a][bn][c] = l[c];
                    bHi[lw][a][bn][c] = h[c];
                }
            }
            __syncwarp();
            bestCand = sah_best_split(ts, lane, [&](int a, int k) { return bCnt[lw][a][k]; },
                                      [&](int a, int k, int c) { return bLo[lw][a][k][c]; },
                                      [&](int a, int k, int c) { return bHi[lw][a][k][c]; });
        }
        if (lane == 0) tBest[t] = bestCand;
    }
    __syncthreads();
    const int best = has ? tBest[t] : -1;
    const int sa = best >= 0 ? best / (kSahBins - 1) : 0, sp = best >= 0 ? best % (kSahBins - 1) + 1 : 0;
    if (best >= 0) {  // left count of the chunk
        uint32_t nl = 0;
        for (uint32_t i0 = cb; i0 < ce; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool isL = i < ce && bin_of(boxes + 6 * (size_t)order[i], sa) < sp;
            nl += __popc(__ballot_sync(0xFFFFFFFFu, isL));
        }
        if (lane == 0) wLeft[warp] = nl;
    }
    __syncthreads();
    uint32_t nlTotal = 0;
    if (best >= 0) {  // stable partition: this chunk's lefts after the lefts of the chunks before it, rights likewise
        uint32_t before = 0;
        for (uint32_t g = 0; g < G; ++g) {
            const uint32_t c = wLeft[lw + g];
            if (g < m) before += c;
            nlTotal += c;
        }
        uint32_t lb = b + before, rb = b + nlTotal + ((cb - b) - before);
        for (uint32_t i0 = cb; i0 < ce; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool valid = i < ce;
            const uint32_t prim = valid ? order[i] : 0u;
            const bool isL = valid && bin_of(boxes + 6 * (size_t)prim, sa) < sp;
            const unsigned lm = __ballot_sync(0xFFFFFFFFu, isL), rm = __ballot_sync(0xFFFFFFFFu, valid && !isL);
            const unsigned below = (1u << lane) - 1u;
            if (isL) tmp[lb + __popc(lm & below)] = prim;
            else if (valid) tmp[rb + __popc(rm & below)] = prim;
            lb += __popc(lm);
            rb += __popc(rm);
        }
    }
    __syncthreads();
    if (best >= 0)
        for (uint32_t i = cb + lane; i < ce; i += 32) order[i] = tmp[i];
    if (has && m == 0 && lane == 0) {  // children: single primitives become leaf refs, the rest next-level tasks
        const uint32_t mid = best >= 0 ? b + nlTotal : b + (e - b) / 2;
        const uint32_t rb0[2] = {b, mid}, re0[2] = {mid, e};
        uint32_t ref[2];
        for (int c = 0; c < 2; ++c) {
            if (re0[c] - rb0[c] == 1) {
                ref[c] = kLeaf | rb0[c];
            } else {
                const uint32_t idx = atomicAdd(&nNext, 1u);
                nxt[idx] = make_uint2(rb0[c], re0[c]);
                ref[c] = baseNext + idx;
            }
        }
        left[node] = ref[0];
        right[node] = ref[1];
    }
}

// One node task on one warp: the range's box (written as the node's box) and centroid box, 16 bins
// per axis in this warp's shared-memory bins, the cheapest of the 45 surface-area splits (ties to
// the lowest candidate; no usable split or `median`: halve the range), a stable ballot partition of
// order[b, e) through tmp, then emit(mid) creates the children and writes the node's refs.
// COHERENT: order[] and tmp[] may have been written by other SMs (the task kernel), so they are read
// through L2.
// The same for a task of at most 32 * R primitives, with each lane's primitives (ids and boxes)
// loaded once into registers: every pass reads them there, and the partition writes order[]
// directly.  Same bounds, bins, costs and stable partition, so the same split.
template <int R, bool COHERENT, class Emit>
__device__ __forceinline__ void sah_task_warp_small(const float* __restrict__ boxes, uint32_t* __restrict__ order,
                                                    float* __restrict__ nodeBoxes, uint32_t b, uint32_t e, uint32_t node, bool median,
                                                    int (&wLo)[3][kSahBins][3], int (&wHi)[3][kSahBins][3], int (&wCnt)[3][kSahBins],
                                                    int lane, Emit&& emit) {
    uint32_t prim[R];
    float bx[R][6];
    bool valid[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const uint32_t i = b + (uint32_t)(32 * j + lane);
        valid[j] = i < e;
        prim[j] = valid[j] ? (COHERENT ? __ldcg(order + i) : order[i]) : 0u;
    }
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
        for (int c = 0; c < 6; ++c) bx[j][c] = valid[j] ? boxes[6 * (size_t)prim[j] + c] : 0.0f;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
#pragma unroll
    for (int j = 0; j < R; ++j)
        if (valid[j])
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], bx[j][a]);
                hi[a] = fmaxf(hi[a], bx[j][3 + a]);
                const float c = 0.5f * (bx[j][a] + bx[j][3 + a]);
                clo[a] = fminf(clo[a], c);
                chi[a] = fmaxf(chi[a], c);
            }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xFFFFFFFFu, lo[a], off));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xFFFFFFFFu, hi[a], off));
            clo[a] = fminf(clo[a], __shfl_xor_sync(0xFFFFFFFFu, clo[a], off));
            chi[a] = fmaxf(chi[a], __shfl_xor_sync(0xFFFFFFFFu, chi[a], off));
        }
    if (lane == 0)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            nodeBoxes[6 * (size_t)node + a] = lo[a];
            nodeBoxes[6 * (size_t)node + 3 + a] = hi[a];
        }
    float scale[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float ext = chi[a] - clo[a];
        scale[a] = ext > 0.0f ? (float)kSahBins / ext : 0.0f;
    }
    // bin of primitive j on axis a (a may be a runtime value: selects, not indexing, keep the boxes
    // in registers)
    auto bin_of = [&](int j, int a) {
        const float l = a == 0 ? bx[j][0] : (a == 1 ? bx[j][1] : bx[j][2]);
        const float h = a == 0 ? bx[j][3] : (a == 1 ? bx[j][4] : bx[j][5]);
        const float o = a == 0 ? clo[0] : (a == 1 ? clo[1] : clo[2]);
        const float s = a == 0 ? scale[0] : (a == 1 ? scale[1] : scale[2]);
        const float c = 0.5f * (l + h);
        return max(0, min((int)((c - o) * s), kSahBins - 1));
    };
    int bestCand = -1;
    if (!median) {
        for (int k = lane; k < 3 * kSahBins; k += 32) {
            const int a = k / kSahBins, bn = k % kSahBins;
            wCnt[a][bn] = 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                wLo[a][bn][c] = ord_float(INFINITY);
                wHi[a][bn][c] = ord_float(-INFINITY);
            }
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < R; ++j)
            if (valid[j])
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    if (scale[a] <= 0.0f) continue;
                    const int k = bin_of(j, a);
                    atomicAdd(&wCnt[a][k], 1);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        atomicMin(&wLo[a][k][c], ord_float(bx[j][c]));
                        atomicMax(&wHi[a][k][c], ord_float(bx[j][3 + c]));
                    }
                }
        __syncwarp();
        bestCand = sah_best_split(scale, lane, [&](int a, int k) { return wCnt[a][k]; },
                                  [&](int a, int k, int c) { return wLo[a][k][c]; },
                                  [&](int a, int k, int c) { return wHi[a][k][c]; });
    }
    uint32_t mid = b + (e - b) / 2;  // no usable split (coincident centroids): halve the range
    if (bestCand >= 0) {
        const int a = bestCand / (kSahBins - 1), sp = bestCand % (kSahBins - 1) + 1;
        bool isL[R];
        uint32_t nl = 0;
#pragma unroll
        for (int j = 0; j < R; ++j) {
            isL[j] = valid[j] && bin_of(j, a) < sp;
            nl += __popc(__ballot_sync(0xFFFFFFFFu, isL[j]));
        }
        uint32_t lb = 0, rb = 0;
        const unsigned below = (1u << lane) - 1u;
#pragma unroll
        for (int j = 0; j < R; ++j) {  // every lane holds its primitives already: write order[] in place
            const unsigned lm = __ballot_sync(0xFFFFFFFFu, isL[j]), rm = __ballot_sync(0xFFFFFFFFu, valid[j] && !isL[j]);
            if (isL[j]) order[b + lb + __popc(lm & below)] = prim[j];
            else if (valid[j]) order[b + nl + rb + __popc(rm & below)] = prim[j];
            lb += __popc(lm);
            rb += __popc(rm);
        }
        __syncwarp();
        mid = b + nl;
    }
    emit(mid);
    __syncwarp();
}

template <bool COHERENT, class Emit>
__device__ __forceinline__ void sah_task_warp(const float* __restrict__ boxes, uint32_t* __restrict__ order, uint32_t* __restrict__ tmp,
                                              float* __restrict__ nodeBoxes, uint32_t b, uint32_t e, uint32_t node, bool median,
                                              int (&wLo)[3][kSahBins][3], int (&wHi)[3][kSahBins][3], int (&wCnt)[3][kSahBins],
                                              int lane, Emit&& emit) {
    if (e - b <= 64) {
        sah_task_warp_small<2, COHERENT>(boxes, order, nodeBoxes, b, e, node, median, wLo, wHi, wCnt, lane, emit);
        return;
    }
    auto ord = [&](uint32_t i) { return COHERENT ? __ldcg(order + i) : order[i]; };
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = b + lane; i < e; i += 32) {
        const float* bx = boxes + 6 * (size_t)ord(i);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], bx[a]);
            hi[a] = fmaxf(hi[a], bx[3 + a]);
            const float c = 0.5f * (bx[a] + bx[3 + a]);
            clo[a] = fminf(clo[a], c);
            chi[a] = fmaxf(chi[a], c);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xFFFFFFFFu, lo[a], off));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xFFFFFFFFu, hi[a], off));
            clo[a] = fminf(clo[a], __shfl_xor_sync(0xFFFFFFFFu, clo[a], off));
            chi[a] = fmaxf(chi[a], __shfl_xor_sync(0xFFFFFFFFu, chi[a], off));
        }
    if (lane == 0)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            nodeBoxes[6 * (size_t)node + a] = lo[a];
            nodeBoxes[6 * (size_t)node + 3 + a] = hi[a];
        }
    float scale[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float ext = chi[a] - clo[a];
        scale[a] = ext > 0.0f ? (float)kSahBins / ext : 0.0f;
    }
    auto bin_of = [&](const float* bx, int a) {
        const float c = 0.5f * (bx[a] + bx[3 + a]);
        return max(0, min((int)((c - clo[a]) * scale[a]), kSahBins - 1));
    };
    int bestCand = -1;
    if (!median) {
        for (int k = lane; k < 3 * kSahBins; k += 32) {
            const int a = k / kSahBins, bn = k % kSahBins;
            wCnt[a][bn] = 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                wLo[a][bn][c] = ord_float(INFINITY);
                wHi[a][bn][c] = ord_float(-INFINITY);
            }
        }
        __syncwarp();
        for (uint32_t i = b + lane; i < e; i += 32) {
            const float* bx = boxes + 6 * (size_t)ord(i);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (scale[a] <= 0.0f) continue;
                const int k = bin_of(bx, a);
                atomicAdd(&wCnt[a][k], 1);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    atomicMin(&wLo[a][k][c], ord_float(bx[c]));
                    atomicMax(&wHi[a][k][c], ord_float(bx[3 + c]));
                }
            }
        }
        __syncwarp();
        bestCand = sah_best_split(scale, lane, [&](int a, int k) { return wCnt[a][k]; },
                                  [&](int a, int k, int c) { return wLo[a][k][c]; },
                                  [&](int a, int k, int c) { return wHi[a][k][c]; });
    }
    uint32_t mid = b + (e - b) / 2;  // no usable split (coincident centroids): halve the range
    if (bestCand >= 0) {
        const int a = bestCand / (kSahBins - 1), sp = bestCand % (kSahBins - 1) + 1;
        uint32_t nl = 0;
        for (uint32_t i0 = b; i0 < e; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool isL = i < e && bin_of(boxes + 6 * (size_t)ord(i), a) < sp;
            nl += __popc(__ballot_sync(0xFFFFFFFFu, isL));
        }
        uint32_t lb = 0, rb = 0;
        for (uint32_t i0 = b; i0 < e; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool valid = i < e;
            const uint32_t prim = valid ? ord(i) : 0u;
            const bool isL = valid && bin_of(boxes + 6 * (size_t)prim, a) < sp;
            const unsigned lm = __ballot_sync(0xFFFFFFFFu, isL), rm = __ballot_sync(0xFFFFFFFFu, valid && !isL);
            const unsigned below = (1u << lane) - 1u;
            if (isL) tmp[b + lb + __popc(lm & below)] = prim;
            else if (valid) tmp[b + nl + rb + __popc(rm & below)] = prim;
            lb += __popc(lm);
            rb += __popc(rm);
        }
        __syncwarp();
        for (uint32_t i = b + lane; i < e; i += 32) order[i] = COHERENT ? __ldcg(tmp + i) : tmp[i];
        __syncwarp();
        mid = b + nl;
    }
    emit(mid);
    __syncwarp();
}

// The first kSahParallelLevels levels, one launch per level: CTA t of level L splits task t of the
// level with all 32 of its warps (the grouped routine with one task), so the levels' tasks run on
// separate SMs.  Level L's tasks are the node ids from base_L = 1 + count_1 + ... + count_(L-1) on
// (count_0 = 1: the root), listed in tasksA for even L and tasksB for odd L; a child task takes the
// next slot of level L + 1 from the global counter lvCount[L + 1].  Level 0 also prepares order[]
// (identity) and the node refs (every node starts as (leaf 0, leaf 0), so a tree left unfinished by
// a task wait that gave up only refers to nodes and leaves in range).
__global__ void __launch_bounds__(kSahWarps * 32, 1) k_sah_level(const float* __restrict__ boxes, uint32_t n, uint32_t* __restrict__ order,
                                                                 uint32_t* __restrict__ tmp, uint32_t* __restrict__ left,
                                                                 uint32_t* __restrict__ right, float* __restrict__ nodeBoxes,
                                                                 uint2* __restrict__ tasksA, uint2* __restrict__ tasksB,
                                                                 uint32_t* __restrict__ lvCount, int level, uint32_t medianLevel) {
    __shared__ int bLo[kSahWarps][3][kSahBins][3], bHi[kSahWarps][3][kSahBins][3];
    __shared__ int bCnt[kSahWarps][3][kSahBins];
    __shared__ float gPart[kSahWarps][12];
    __shared__ float tClo[kSahWarps][3], tScale[kSahWarps][3];
    __shared__ int tBest[kSahWarps];
    __shared__ uint32_t wLeft[kSahWarps];
    uint2* cur = (level & 1) ? tasksB : tasksA;
    uint2* nxt = (level & 1) ? tasksA : tasksB;
    if (level == 0) {
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) order[i] = i;
        for (uint32_t i = threadIdx.x; i + 1 < n; i += blockDim.x) left[i] = right[i] = kLeaf;
        if (threadIdx.x == 0) cur[0] = make_uint2(0u, n);
        __syncthreads();
    }
    const uint32_t count = level == 0 ? 1u : lvCount[level];
    if (blockIdx.x >= count) return;
    uint32_t base = level == 0 ? 0u : 1u;
    for (int k = 1; k < level; ++k) base += lvCount[k];
    sah_level_grouped(boxes, order, tmp, left, right, nodeBoxes, cur + blockIdx.x, nxt, 1u, (uint32_t)level >= medianLevel,
                      base + blockIdx.x, base + count, lvCount[level + 1], bLo, bHi, bCnt, gPart, tClo, tScale, tBest, wLeft);
}

// ---- one task over many CTAs (the top levels of large builds) -------------------------------------
// For builds of at least kSahSplitMin primitives, the first kSahSplitLevels levels split each task
// over kSplitCtas CTAs, in five launches per level, because one SM would otherwise bin a whole
// level's primitives.  CTA (t, m) takes chunk m of task t.
//   0 bounds: the chunk's box and centroid box          -> part[t][m]
//   1 bins:   the task's frame from all parts (minima and maxima: every CTA gets the same), the
//             chunk binned per warp, the warps merged    -> bins[t][m]
//   2 choose: all CTAs' bins merged (counts add, bounds are minima and maxima: exact), the split
//             chosen as the one-CTA builder chooses it (every CTA gets the same), the chunk's lefts
//             counted                                    -> left[t][m]; CTA m = 0: node box, best[t]
//   3 scatter: the chunk partitioned stably into tmp, its lefts after the lefts of the chunks (and
//             warps) before it
//   4 finish: tmp back into order; CTA m = 0 emits the children as k_sah_level does
// The tree is the one-CTA builder's: same bounds, bins, costs and candidate order, same stable
// partition.
constexpr int kSplitCtas = 32;
constexpr int kSahSplitLevels = 3;
constexpr uint32_t kSahSplitMin = 32768;
constexpr int kBinInts = 3 * kSahBins * 7;  // counts, then lo xyz, then hi xyz per (axis, bin)

struct SplitScratch {
    float* part;  // [4][kSplitCtas][12]
    int* bins;    // [4][kSplitCtas][kBinInts]
    uint32_t* left;  // [4][kSplitCtas]
    int* best;       // [4]
};

__device__ __forceinline__ int bin_slot_cnt(int a, int bn) { return a * kSahBins + bn; }
__device__ __forceinline__ int bin_slot_lo(int a, int bn, int c) { return 3 * kSahBins + (a * kSahBins + bn) * 3 + c; }
__device__ __forceinline__ int bin_slot_hi(int a, int bn, int c) { return 3 * kSahBins + 9 * kSahBins + (a * kSahBins + bn) * 3 + c; }

// the task's frame (box, centroid origin and bin scale) from the parts of all its CTAs
__device__ __forceinline__ void split_frame(const float* part, float* lo, float* hi, float* clo, float* scale) {
    float chi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = clo[a] = INFINITY;
        hi[a] = chi[a] = -INFINITY;
    }
    for (int m = 0; m < kSplitCtas; ++m) {
        const float* p = part + 12 * m;
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], p[a]);
            hi[a] = fmaxf(hi[a], p[3 + a]);
            clo[a] = fminf(clo[a], p[6 + a]);
            chi[a] = fmaxf(chi[a], p[9 + a]);
        }
    }
    for (int a = 0; a < 3; ++a) {
        const float ext = chi[a] - clo[a];
        scale[a] = ext > 0.0f ? (float)kSahBins / ext : 0.0f;
    }
}

__global__ void __launch_bounds__(kSahWarps * 32, 1) k_sah_init(uint32_t n, uint32_t* __restrict__ order, uint32_t* __restrict__ left,
                                                                uint32_t* __restrict__ right, uint2* __restrict__ tasksA) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        order[i] = i;
        if (i + 1 < n) left[i] = right[i] = kLeaf;  // every node starts as (leaf 0, leaf 0)
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) tasksA[0] = make_uint2(0u, n);
}

__global__ void __launch_bounds__(kSahWarps * 32, 1) k_sah_split(const float* __restrict__ boxes, uint32_t* __restrict__ order,
                                                                 uint32_t* __restrict__ tmp, uint32_t* __restrict__ left,
                                                                 uint32_t* __restrict__ right, float* __restrict__ nodeBoxes,
                                                                 uint2* __restrict__ tasksA, uint2* __restrict__ tasksB,
                                                                 uint32_t* __restrict__ lvCount, SplitScratch X, int level, int phase,
                                                                 uint32_t medianLevel) {
    __shared__ int sb[kSahWarps][kBinInts];  // per-warp bins; merged bins in sb[0]
    __shared__ float red[kSahWarps][12];
    __shared__ uint32_t wl[kSahWarps];
    __shared__ int sBest;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t t = blockIdx.x / kSplitCtas, m = blockIdx.x % kSplitCtas;
    const uint32_t count = level == 0 ? 1u : lvCount[level];
    if (t >= count) return;
    uint2* cur = (level & 1) ? tasksB : tasksA;
    uint2* nxt = (level & 1) ? tasksA : tasksB;
    uint32_t base = level == 0 ? 0u : 1u;
    for (int k = 1; k < level; ++k) base += lvCount[k];
    const uint2 tk = cur[t];
    const uint32_t b = tk.x, e = tk.y, node = base + t;
    const uint32_t chunk = (e - b + kSplitCtas - 1) / kSplitCtas;
    const uint32_t cb = min(e, b + m * chunk), ce = min(e, cb + chunk);
    float* part = X.part + (size_t)t * kSplitCtas * 12;
    int* binsT = X.bins + (size_t)t * kSplitCtas * kBinInts;
    uint32_t* leftT = X.left + (size_t)t * kSplitCtas;
    const bool median = (uint32_t)level >= medianLevel;
    if (phase == 0) {  // the chunk's box and centroid box
        float v[12];
        for (int a = 0; a < 3; ++a) {
            v[a] = v[6 + a] = INFINITY;
            v[3 + a] = v[9 + a] = -INFINITY;
        }
        for (uint32_t i = cb + threadIdx.x; i < ce; i += blockDim.x) {
            const float* bx = boxes + 6 * (size_t)order[i];
            for (int a = 0; a < 3; ++a) {
                v[a] = fminf(v[a], bx[a]);
                v[3 + a] = fmaxf(v[3 + a], bx[3 + a]);
                const float c = 0.5f * (bx[a] + bx[3 + a]);
                v[6 + a] = fminf(v[6 + a], c);
                v[9 + a] = fmaxf(v[9 + a], c);
            }
        }
        for (int off = 16; off > 0; off >>= 1)
            for (int k = 0; k < 12; ++k) {
                const float o = __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
                v[k] = (k % 6) < 3 ? fminf(v[k], o) : fmaxf(v[k], o);
            }
        if (lane == 0)
            for (int k = 0; k < 12; ++k) red[warp][k] = v[k];
        __syncthreads();
        if (threadIdx.x < 12) {
            const int k = threadIdx.x;
            float r = red[0][k];
            for (int w = 1; w < kSahWarps; ++w) r = (k % 6) < 3 ? fminf(r, red[w][k]) : fmaxf(r, red[w][k]);
            part[12 * m + k] = r;
        }
        return;
    }
    float lo[3], hi[3], clo[3], scale[3];
    split_frame(part, lo, hi, clo, scale);
    auto bin_of = [&](const float* bx, int a) {
        const float c = 0.5f * (bx[a] + bx[3 + a]);
        return max(0, min((int)((c - clo[a]) * scale[a]), kSahBins - 1));
    };
    if (phase == 1) {  // the chunk binned per warp, the warps merged into this CTA's bins
        if (median) return;
        for (int k = lane; k < 3 * kSahBins; k += 32) {
            const int a = k / kSahBins, bn = k % kSahBins;
            sb[warp][bin_slot_cnt(a, bn)] = 0;
            for (int c = 0; c < 3; ++c) {
                sb[warp][bin_slot_lo(a, bn, c)] = ord_float(INFINITY);
                sb[warp][bin_slot_hi(a, bn, c)] = ord_float(-INFINITY);
            }
        }
        __syncwarp();
        for (uint32_t i = cb + threadIdx.x; i < ce; i += blockDim.x) {
            const float* bx = boxes + 6 * (size_t)order[i];
            for (int a = 0; a < 3; ++a) {
                if (scale[a] <= 0.0f) continue;
                const int k = bin_of(bx, a);
                atomicAdd(&sb[warp][bin_slot_cnt(a, k)], 1);
                for (int c = 0; c < 3; ++c) {
                    atomicMin(&sb[warp][bin_slot_lo(a, k, c)], ord_float(bx[c]));
                    atomicMax(&sb[warp][bin_slot_hi(a, k, c)], ord_float(bx[3 + c]));
                }
            }
        }
        __syncthreads();
        for (int k = threadIdx.x; k < kBinInts; k += blockDim.x) {
            int r = sb[0][k];
            for (int w = 1; w < kSahWarps; ++w)
                r = k < 3 * kSahBins ? r + sb[w][k] : (k < 3 * kSahBins + 9 * kSahBins ? min(r, sb[w][k]) : max(r, sb[w][k]));
            binsT[(size_t)m * kBinInts + k] = r;
        }
        return;
    }
    if (phase == 2) {  // every CTA's bins merged, the split chosen, the chunk's lefts counted
        if (!median)
            for (int k = threadIdx.x; k < kBinInts; k += blockDim.x) {
                int r = binsT[k];
                for (int c = 1; c < kSplitCtas; ++c) {
                    const int o = binsT[(size_t)c * kBinInts + k];
                    r = k < 3 * kSahBins ? r + o : (k < 3 * kSahBins + 9 * kSahBins ? min(r, o) : max(r, o));
                }
                sb[0][k] = r;
            }
        __syncthreads();
        if (warp == 0) {  // cheapest surface-area cost, ties to the lowest candidate
            int bestCand = -1;
            if (!median) {
                bestCand = sah_best_split(scale, lane, [&](int a, int k) { return sb[0][bin_slot_cnt(a, k)]; },
                                          [&](int a, int k, int c) { return sb[0][bin_slot_lo(a, k, c)]; },
                                          [&](int a, int k, int c) { return sb[0][bin_slot_hi(a, k, c)]; });
            }
            if (lane == 0) sBest = bestCand;
        }
        __syncthreads();
        const int best = sBest;
        if (m == 0 && threadIdx.x == 0) {
            X.best[t] = best;
            for (int a = 0; a < 3; ++a) {
                nodeBoxes[6 * (size_t)node + a] = lo[a];
                nodeBoxes[6 * (size_t)node + 3 + a] = hi[a];
            }
        }
        if (best < 0) return;
        const int sa = best / (kSahBins - 1), sp = best % (kSahBins - 1) + 1;
        uint32_t nl = 0;
        for (uint32_t i = cb + threadIdx.x; i < ce; i += blockDim.x) nl += bin_of(boxes + 6 * (size_t)order[i], sa) < sp;
        for (int off = 16; off > 0; off >>= 1) nl += __shfl_xor_sync(0xFFFFFFFFu, nl, off);
        if (lane == 0) wl[warp] = nl;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t s = 0;
            for (int w = 0; w < kSahWarps; ++w) s += wl[w];
            leftT[m] = s;
        }
        return;
    }
    const int best = X.best[t];
    if (phase == 3) {  // stable partition of the chunk: warp sub-chunks in order, lanes in order
        if (best < 0) return;
        const int sa = best / (kSahBins - 1), sp = best % (kSahBins - 1) + 1;
        uint32_t nlTotal = 0, before = 0;
        for (uint32_t c = 0; c < (uint32_t)kSplitCtas; ++c) {
            const uint32_t x = leftT[c];
            if (c < m) before += x;
            nlTotal += x;
        }
        const uint32_t sub = (ce - cb + kSahWarps - 1) / kSahWarps;
        const uint32_t wb = min(ce, cb + warp * sub), we = min(ce, wb + sub);
        uint32_t nl = 0;
        for (uint32_t i0 = wb; i0 < we; i0 += 32) {
            const uint32_t i = i0 + lane;
            nl += __popc(__ballot_sync(0xFFFFFFFFu, i < we && bin_of(boxes + 6 * (size_t)order[i], sa) < sp));
        }
        if (lane == 0) wl[warp] = nl;
        __syncthreads();
        uint32_t wBefore = 0;
        for (int w = 0; w < warp; ++w) wBefore += wl[w];
        const uint32_t lefts = before + wBefore;  // lefts ahead of this warp's sub-chunk in the task
        uint32_t lb = b + lefts, rb = b + nlTotal + ((wb - b) - lefts);
        for (uint32_t i0 = wb; i0 < we; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool valid = i < we;
            const uint32_t prim = valid ? order[i] : 0u;
            const bool isL = valid && bin_of(boxes + 6 * (size_t)prim, sa) < sp;
            const unsigned lm = __ballot_sync(0xFFFFFFFFu, isL), rm = __ballot_sync(0xFFFFFFFFu, valid && !isL);
            const unsigned below = (1u << lane) - 1u;
            if (isL) tmp[lb + __popc(lm & below)] = prim;
            else if (valid) tmp[rb + __popc(rm & below)] = prim;
            lb += __popc(lm);
            rb += __popc(rm);
        }
        return;
    }
    // phase 4: tmp back into order, the children
    if (best >= 0)
        for (uint32_t i = cb + threadIdx.x; i < ce; i += blockDim.x) order[i] = tmp[i];
    if (m == 0 && threadIdx.x == 0) {
        uint32_t nlTotal = 0;
        for (uint32_t c = 0; c < (uint32_t)kSplitCtas; ++c) nlTotal += leftT[c];
        const uint32_t mid = best >= 0 ? b + nlTotal : b + (e - b) / 2;
        const uint32_t rb0[2] = {b, mid}, re0[2] = {mid, e};
        uint32_t ref[2];
        for (int c = 0; c < 2; ++c) {
            if (re0[c] - rb0[c] == 1) {
                ref[c] = kLeaf | rb0[c];
            } else {
                const uint32_t idx = atomicAdd(&lvCount[level + 1], 1u);
                nxt[idx] = make_uint2(rb0[c], re0[c]);
                ref[c] = base + count + idx;
            }
        }
        left[node] = ref[0];
        right[node] = ref[1];
    }
}

// The rest of the top of the tree: one CTA, level by level from level kSahParallelLevels on (levels
// with fewer tasks than warps spread each task over a group of warps), until a level has `handoff`
// tasks or more.  That level's tasks go to the queue Q, whose slots are the node ids from baseCur
// on, and k_sah_tasks finishes the tree.
__global__ void __launch_bounds__(kSahWarps * 32, 1) k_sah_build(const float* __restrict__ boxes, uint32_t n, uint32_t* __restrict__ order,
                                                                 uint32_t* __restrict__ tmp, uint32_t* __restrict__ left,
                                                                 uint32_t* __restrict__ right, float* __restrict__ nodeBoxes,
                                                                 uint2* __restrict__ tasksA, uint2* __restrict__ tasksB,
                                                                 uint32_t medianLevel, uint32_t handoff, SahQueue Q,
                                                                 const uint32_t* __restrict__ lvCount, uint32_t* __restrict__ levelsOut) {
    __shared__ int bLo[kSahWarps][3][kSahBins][3], bHi[kSahWarps][3][kSahBins][3];
    __shared__ int bCnt[kSahWarps][3][kSahBins];
    __shared__ uint32_t nCur, nNext, baseCur, baseNext, levels;
    // levels with fewer tasks than warps: per-warp partial bounds, per-task centroid frame and split,
    // per-warp left counts
    __shared__ float gPart[kSahWarps][12];
    __shared__ float tClo[kSahWarps][3], tScale[kSahWarps][3];
    __shared__ int tBest[kSahWarps];
    __shared__ uint32_t wLeft[kSahWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {  // the state after the level kernels (their counts; level 0: the root)
        uint32_t base = 1, lv = 1;
        while (lv < (uint32_t)kSahParallelLevels && lvCount[lv]) base += lvCount[lv++];
        nCur = lv < (uint32_t)kSahParallelLevels ? 0u : lvCount[lv];
        nNext = 0;
        baseCur = base;          // node id of the current level's first task
        baseNext = base + nCur;  // node id of the next level's first task
        levels = lv;
    }
    __syncthreads();
    uint2* cur = (kSahParallelLevels & 1) ? tasksB : tasksA;
    uint2* nxt = (kSahParallelLevels & 1) ? tasksA : tasksB;
    for (;;) {
        const uint32_t count = nCur;
        if (count == 0) break;
        if (count >= handoff) {  // the rest of the tree on every SM
            for (uint32_t t = threadIdx.x; t < count; t += blockDim.x) {
                const uint2 tk = cur[t];
                Q.tasks[t] = make_uint4(tk.x, tk.y, baseCur + t, levels);
                Q.ready[t] = 1u;  // the task kernel starts after this one
            }
            if (threadIdx.x == 0) {
                Q.ctr[1] = count;
                Q.ctr[2] = baseCur;
                Q.ctr[3] = n - 1 - baseCur;
            }
            break;
        }
        const bool median = levels >= medianLevel;  // from here on ranges are halved: the depth stays bounded
        if (count < (uint32_t)kSahWarps) {
            sah_level_grouped(boxes, order, tmp, left, right, nodeBoxes, cur, nxt, count, median, baseCur, baseNext, nNext, bLo, bHi,
                              bCnt, gPart, tClo, tScale, tBest, wLeft);
        } else
        for (uint32_t t = warp; t < count; t += kSahWarps) {
            const uint2 tk = cur[t];
            const uint32_t b = tk.x, e = tk.y, node = baseCur + t;
            sah_task_warp<false>(boxes, order, tmp, nodeBoxes, b, e, node, median, bLo[warp], bHi[warp], bCnt[warp], lane,
                                 [&](uint32_t mid) {  // single primitives become leaf refs, the rest next-level tasks
                                     if (lane != 0) return;
                                     const uint32_t rb0[2] = {b, mid}, re0[2] = {mid, e};
                                     uint32_t ref[2];
                                     for (int c = 0; c < 2; ++c) {
                                         if (re0[c] - rb0[c] == 1) {
                                             ref[c] = kLeaf | rb0[c];
                                         } else {
                                             const uint32_t idx = atomicAdd(&nNext, 1u);
                                             nxt[idx] = make_uint2(rb0[c], re0[c]);
                                             ref[c] = baseNext + idx;
                                         }
                                     }
                                     left[node] = ref[0];
                                     right[node] = ref[1];
                                 });
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            baseCur = baseNext;
            baseNext += nNext;
            nCur = nNext;
            nNext = 0;
            ++levels;
        }
        uint2* sw = cur;
        cur = nxt;
        nxt = sw;
        __syncthreads();
    }
    if (threadIdx.x == 0 && levelsOut) *levelsOut = levels;
}

// The rest of the tree on every SM: a warp claims the next queue slot, waits (bounded) until the
// slot's task is published, splits it as k_sah_build does, and publishes its children's tasks in
// the next free slots (node id = first node id of the queue + slot).  Every internal node is one
// task, so the queue holds exactly n - 1 - (first node id) tasks and a warp whose claim lies beyond
// that is done.  A slot's task is published by the warp that split its parent, which claimed an
// earlier slot and runs, so every wait ends; a wait that still runs out sets *status to 2 and
// leaves that subtree as prepared (valid refs, unset boxes).
__global__ void __launch_bounds__(kSahTaskWarps * 32, 3) k_sah_tasks(const float* __restrict__ boxes, uint32_t* __restrict__ order,
                                                                  uint32_t* __restrict__ tmp, uint32_t* __restrict__ left,
                                                                  uint32_t* __restrict__ right, float* __restrict__ nodeBoxes,
                                                                  SahQueue Q, uint32_t medianLevel, uint32_t* __restrict__ levelsOut,
                                                                  int* __restrict__ status, uint32_t waitLimit) {
    __shared__ int bLo[kSahTaskWarps][3][kSahBins][3], bHi[kSahTaskWarps][3][kSahBins][3];
    __shared__ int bCnt[kSahTaskWarps][3][kSahBins];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t total = Q.ctr[3], base = Q.ctr[2];  // written by k_sah_build
    uint32_t deepest = 0;
    for (;;) {
        uint32_t slot = 0, ok = 1;
        if (lane == 0) {
            slot = atomicAdd(Q.ctr, 1u);
            if (slot < total) {
                for (uint32_t spins = 0; ld_relaxed(Q.ready + slot) == 0; ++spins) {
                    if (spins >= waitLimit) {
                        ok = 0;
                        if (status) atomicExch(status, 2);
                        break;
                    }
                    __nanosleep(128);
                }
            }
        }
        slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
        ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
        if (slot >= total || !ok) break;
        __threadfence();  // after the publication: the task and its order[] range
        const uint4 tk = __ldcg(Q.tasks + slot);
        const uint32_t b = tk.x, e = tk.y, node = tk.z, level = tk.w;
        deepest = max(deepest, level + 1);
        sah_task_warp<true>(boxes, order, tmp, nodeBoxes, b, e, node, level >= medianLevel, bLo[warp], bHi[warp], bCnt[warp], lane,
                            [&](uint32_t mid) {
                                const uint32_t rb0[2] = {b, mid}, re0[2] = {mid, e};
                                uint32_t ref[2] = {0u, 0u};
                                if (lane == 0) {
                                    for (int c = 0; c < 2; ++c) {
                                        if (re0[c] - rb0[c] == 1) {
                                            ref[c] = kLeaf | rb0[c];
                                        } else {
                                            const uint32_t q = atomicAdd(Q.ctr + 1, 1u);
                                            ref[c] = base + q;
                                            Q.tasks[q] = make_uint4(rb0[c], re0[c], base + q, level + 1);
                                        }
                                    }
                                    left[node] = ref[0];
                                    right[node] = ref[1];
                                }
                                __threadfence();  // every lane's order[] writes and the new tasks, then the publication
                                __syncwarp();
                                if (lane == 0)
                                    for (int c = 0; c < 2; ++c)
                                        if (!(ref[c] & kLeaf)) st_relaxed(Q.ready + (ref[c] - base), 1u);
                            });
    }
    if (lane == 0 && levelsOut && deepest) atomicMax(levelsOut, deepest);
}

// parents of a BVH2 in the LBVH layout (internal node i at parents[i], the leaf at sorted position k
// at parents[n - 1 + k], the root's 0xFFFFFFFF), which the bottom-up refit walks
__global__ void k_parents(const uint32_t* __restrict__ left, const uint32_t* __restrict__ right, uint32_t n,
                          uint32_t* __restrict__ parents) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 >= n) return;
    const uint32_t L = left[i], R = right[i];
    for (const uint32_t c : {L, R}) {  // child refs of a finished tree are in range; anything else is skipped
        const uint32_t slot = (c & kLeaf) ? (n - 1) + (c & ~kLeaf) : c;
        if (((c & kLeaf) && (c & ~kLeaf) < n) || (!(c & kLeaf) && c > 0 && c + 1 < n)) parents[slot] = i;
    }
    if (i == 0) parents[0] = 0xFFFFFFFFu;
}

// ---- instances ----------------------------------------------------------------------------------
__global__ void k_instances(const rg_instance* __restrict__ in, uint32_t n, const DevBlas* __restrict__ blas, uint32_t nblas,
                            DevInstance* __restrict__ out, float* __restrict__ boxes, bool checkOffsets, uint32_t nm) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rg_instance I = in[i];
    const float* m = &I.transform[0][0];
    float a00 = m[0], a01 = m[1], a02 = m[2], t0 = m[3];
    float a10 = m[4], a11 = m[5], a12 = m[6], t1 = m[7];
    float a20 = m[8], a21 = m[9], a22 = m[10], t2 = m[11];
    float c00 = a11 * a22 - a12 * a21, c01 = a02 * a21 - a01 * a22, c02 = a01 * a12 - a02 * a11;
    float c10 = a12 * a20 - a10 * a22, c11 = a00 * a22 - a02 * a20, c12 = a02 * a10 - a00 * a12;
    float c20 = a10 * a21 - a11 * a20, c21 = a01 * a20 - a00 * a21, c22 = a00 * a11 - a01 * a10;
    float det = (a00 * c00 + a01 * c10) + a02 * c20;
    bool ok = (det != 0.0f) && isfinite(det) && I.blas < nblas && (I.mask & 0xFFu) != 0u;
    if (ok && checkOffsets && blas[I.blas].n > 0) {
        const DevBlas& B = blas[I.blas];
        ok = I.vertexBufferOffset == B.vOff && I.indexBufferOffset == B.iOff && (uint64_t)I.materialBufferOffset + B.maxMat < nm;
    }
    float id = ok ? 1.0f / det : 0.0f;
    float r[9] = {c00 * id, c01 * id, c02 * id, c10 * id, c11 * id, c12 * id, c20 * id, c21 * id, c22 * id};
    DevInstance d;
    for (int row = 0; row < 3; ++row) {
        float tr = -((r[3 * row + 0] * t0 + r[3 * row + 1] * t1) + r[3 * row + 2] * t2);
        d.inv[row] = make_float4(r[3 * row + 0], r[3 * row + 1], r[3 * row + 2], tr);
        d.m[row] = make_float4(m[4 * row + 0], m[4 * row + 1], m[4 * row + 2], m[4 * row + 3]);
    }
    d.blas = ok ? I.blas : 0u;
    d.valid = ok ? 1u : 0u;
    d.vOff = I.vertexBufferOffset;
    d.iOff = I.indexBufferOffset;
    d.mOff = I.materialBufferOffset;
    d.mask = I.mask;
    d.pad0 = d.pad1 = 0;
    out[i] = d;
    float* o = boxes + 6 * (size_t)i;
    if (ok && blas[I.blas].n > 0) {
        const float* rb = blas[I.blas].root;
        for (int row = 0; row < 3; ++row) {
            float lo = m[4 * row + 3], hi = m[4 * row + 3];
            for (int j = 0; j < 3; ++j) {
                float e = m[4 * row + j] * rb[j], f = m[4 * row + j] * rb[3 + j];
                lo = lo + fminf(e, f);
                hi = hi + fmaxf(e, f);
            }
            o[row] = lo;
            o[3 + row] = hi;
        }
    } else {
        o[0] = o[1] = o[2] = INFINITY;
        o[3] = o[4] = o[5] = -INFINITY;
    }
}

inline uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

}  // namespace

cudaError_t tri_boxes(const rg_vertex* v, const uint32_t* idx, uint32_t vOff, uint32_t iOff, uint32_t n, float* boxes, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_tri_boxes<<<blocks(n, 256), 256, 0, s>>>(v, idx, vOff, iOff, n, boxes);
    count_launch();
    return cudaGetLastError();
}

cudaError_t tri_records(const rg_vertex* v, const uint32_t* idx, uint32_t vOff, uint32_t iOff, const uint32_t* order, uint32_t n,
                        float4* tris, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_tri_records<<<blocks(n, 256), 256, 0, s>>>(v, idx, vOff, iOff, order, n, tris);
    count_launch();
    return cudaGetLastError();
}

cudaError_t inst_records(const uint32_t* order, uint32_t n, const DevInstance* inst, const DevBlas* blas, InstRec* out,
                         cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_inst_records<<<blocks(n, 128), 128, 0, s>>>(order, n, inst, blas, out);
    count_launch();
    return cudaGetLastError();
}

cudaError_t setup_instances(const rg_instance* in, uint32_t n, const DevBlas* blas, uint32_t nblas, DevInstance* out, float* boxes,
                            bool checkOffsets, uint32_t nm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_instances<<<blocks(n, 128), 128, 0, s>>>(in, n, blas, nblas, out, boxes, checkOffsets, nm);
    count_launch();
    return cudaGetLastError();
}

cudaError_t lbvh_refit(const LbvhBuffers& b, cudaStream_t s) {
    if (b.n <= 1) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(b.flags, 0, sizeof(uint32_t) * (b.n - 1), s);
    if (e != cudaSuccess) return e;
    k_bottom_up<<<blocks(b.n, 256), 256, 0, s>>>(b.primBoxes, b.order, b.n, b.left, b.right, b.parents, b.flags, b.nodeBoxes);
    count_launch();
    return cudaGetLastError();
}

static int sah_task_grid() {  // persistent grid of k_sah_tasks (every resident block)
    static std::atomic<int> grid{0};
    int g = grid.load(std::memory_order_acquire);
    if (g) return g;
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sah_tasks, kSahTaskWarps * 32, 0) != cudaSuccess)
        return 0;
    g = sms * max(per, 1);
    grid.store(g, std::memory_order_release);
    return g;
}

cudaError_t sah_build(const LbvhBuffers& b, bool parents, uint32_t* levels, cudaStream_t s) {
    if (b.n <= 1) return cudaSuccess;
    if (!b.sahQueue) return cudaErrorInvalidValue;
    const int grid = sah_task_grid();
    if (!grid) return cudaErrorUnknown;
    SahQueue Q;
    Q.tasks = reinterpret_cast<uint4*>(b.sahQueue);
    Q.ready = reinterpret_cast<uint32_t*>(b.sahQueue + 16 * (size_t)b.n);
    Q.ctr = Q.ready + b.n;
    uint32_t* lvCount = Q.ctr + 8;  // tasks per level of the level kernels
    cudaError_t e = cudaMemsetAsync(Q.ready, 0, 4 * (size_t)b.n + 64, s);  // ready words and counters
    if (e != cudaSuccess) return e;
    // scratch: the sort buffers (n words each); at most n / 2 tasks per level, 2 words each
    uint2* tasksA = reinterpret_cast<uint2*>(b.valsA);
    uint2* tasksB = reinterpret_cast<uint2*>(b.valsB);
    int lv0 = 0;
    if (b.n >= kSahSplitMin) {  // the first levels with each task over kSplitCtas CTAs
        SplitScratch X;  // in the queue's task records, which k_sah_build fills only later
        X.part = reinterpret_cast<float*>(Q.tasks);
        X.bins = reinterpret_cast<int*>(X.part + 4 * kSplitCtas * 12);
        X.left = reinterpret_cast<uint32_t*>(X.bins + 4 * kSplitCtas * kBinInts);
        X.best = reinterpret_cast<int*>(X.left + 4 * kSplitCtas);
        k_sah_init<<<2 * kSplitCtas, kSahWarps * 32, 0, s>>>(b.n, b.order, b.left, b.right, tasksA);
        count_launch();
        for (; lv0 < kSahSplitLevels; ++lv0)
            for (int ph = 0; ph < 5; ++ph) {
                k_sah_split<<<(1u << lv0) * kSplitCtas, kSahWarps * 32, 0, s>>>(b.primBoxes, b.order, b.keysA, b.left, b.right,
                                                                                 b.nodeBoxes, tasksA, tasksB, lvCount, X, lv0, ph,
                                                                                 kSahMedianLevel);
                count_launch();
            }
    }
    for (int lv = lv0; lv < kSahParallelLevels; ++lv)
        k_sah_level<<<1u << lv, kSahWarps * 32, 0, s>>>(b.primBoxes, b.n, b.order, b.keysA, b.left, b.right, b.nodeBoxes, tasksA,
                                                         tasksB, lvCount, lv, kSahMedianLevel);
    k_sah_build<<<1, kSahWarps * 32, 0, s>>>(b.primBoxes, b.n, b.order, b.keysA, b.left, b.right, b.nodeBoxes, tasksA, tasksB,
                                              kSahMedianLevel, kSahHandoff, Q, lvCount, levels);
    // polls of an unpublished task before a warp gives up (RG_SAH_WAIT_LIMIT overrides; 0 makes
    // the first unpublished slot end the wait, which tests use to check the reported status)
    uint32_t waitLimit = kSahWaitLimit;
    if (const char* env = getenv("RG_SAH_WAIT_LIMIT")) waitLimit = (uint32_t)strtoul(env, nullptr, 10);
    k_sah_tasks<<<grid, kSahTaskWarps * 32, 0, s>>>(b.primBoxes, b.order, b.keysA, b.left, b.right, b.nodeBoxes, Q, kSahMedianLevel,
                                                     levels, b.status, waitLimit);
    count_launch(kSahParallelLevels - lv0 + 2);
    if (parents) {
        k_parents<<<blocks(b.n - 1, 256), 256, 0, s>>>(b.left, b.right, b.n, b.parents);
        count_launch();
    }
    return cudaGetLastError();
}

cudaError_t wide_records(const LbvhBuffers& b, WideNode* out, cudaStream_t s) {
    if (b.n <= 1) return cudaSuccess;
    k_wide_records<<<blocks(b.n - 1, 256), 256, 0, s>>>(b.primBoxes, b.order, b.n, b.left, b.right, b.nodeBoxes, out);
    count_launch();
    return cudaGetLastError();
}

cudaError_t lbvh_build(const LbvhBuffers& b, cudaStream_t s) {
    const uint32_t n = b.n;
    if (n == 0) return cudaSuccess;
    if (n > kStatCount) return cudaErrorInvalidValue;  // the sort's status words count in 30 bits
    const uint32_t nTiles = (uint32_t)sort_tiles(n);
    cudaError_t e = cudaMemsetAsync(b.sortState, 0, 4 * sort_state_words(n), s);
    if (e != cudaSuccess) return e;
    k_bounds_init<<<1, 32, 0, s>>>(b.bounds);
    uint32_t gb = min(blocks(n, 256), 1024u);
    k_centroid_bounds<<<gb, 256, 0, s>>>(b.primBoxes, n, b.bounds);
    k_morton<<<min(blocks(n, 256), kMortonMaxBlocks), 256, 0, s>>>(b.primBoxes, n, b.bounds, b.morton, b.keysA, b.valsA, b.valsB,
                                                                   b.sortState);
    count_launch(3);
    // polls of an unpublished predecessor tile before a look-back counts that tile itself
    // (RG_SORT_SPIN_LIMIT overrides; 0 makes every such look-back count, which tests use)
    uint32_t spinLimit = 1u << 16;
    if (const char* env = getenv("RG_SORT_SPIN_LIMIT")) spinLimit = (uint32_t)strtoul(env, nullptr, 10);
    uint32_t *kin = b.keysA, *vin = b.valsA, *kout = b.keysB, *vout = b.valsB;
    for (int pass = 0; pass < 4; ++pass) {
        k_sort_onesweep<<<nTiles, kSortThreads, 0, s>>>(kin, vin, kout, vout, n, pass, b.sortState, nTiles, spinLimit);
        count_launch();
        uint32_t* t = kin; kin = kout; kout = t;
        t = vin; vin = vout; vout = t;
    }
    // after 4 passes the sorted data is back in keysA / valsA
    e = cudaMemcpyAsync(b.order, vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    if (n == 1) return cudaGetLastError();
    k_karras<<<blocks(n - 1, 256), 256, 0, s>>>(kin, n, b.left, b.right, b.parents);
    count_launch();
    return lbvh_refit(b, s);
}

}  // namespace rg
