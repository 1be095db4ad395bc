// trace.cu -- per-pixel ray generation, two-level BVH traversal and closest-hit / miss shading.
//
// Replaces traceRaysKHR with the raygen / closest-hit / miss / shadow-miss programs
// (render/raytracer.cpp:99-100; resources/shaders/raygen.h:69-115, raygen.rgen:30-39,
// closesthit.rchit:74-268, miss.rmiss:38-83, shadowMiss.rmiss:30-34).
//
// GB300 has no RT cores, so traversal is software: 4-wide records derived from the BVH2 (one
// 112-byte record = six 16-byte plane loads plus the refs tests four children), nearest-child-first
// stack traversal, TLAS leaves switch to the instance's BLAS with the ray moved into object space, and
// a watertight ray/triangle test (Woop, Benthin, Wald 2013).  Closest-hit ties (equal t) resolve to
// the smaller (instance, primitive).  Box tests only ever accept more than the exact test would (see
// the ray set-up below), so the hit found does not depend on the tree: it is the brute-force answer.
//
// The reference's recursion (nested traceRayEXT calls sharing ONE payload, payload.h:29-43) runs
// here as an explicit state machine per thread: a paused closest-hit invocation is a Frame on a
// small per-thread stack with a resume code, and every trace (of any depth) happens in the same
// outer loop so the threads of a warp traverse together.  Payload fields that the reference leaves
// stale (depth, rayType, curIOR, refDepth) leak exactly as in the reference.
//
// GLSL-undefined cases follow fixed policies: r/(tr+r) with tr+r == 0 -> 0; pow(x, n) with
// integer n -> repeated multiply; a zero direction (refract at total internal reflection) -> no
// traversal, miss shader; clamp/min/max treat a NaN operand as absent (fminf/fmaxf).
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "rg_internal.cuh"

namespace rg {
namespace {

// ---------------------------------------------------------------------------------------------
// ray set-up and primitive tests
//
// Box tests use one fused multiply-add per plane: t = l * j + C with j = 1/d and C = -o/d.  C is a
// rounded product, so it is kept as a bracket [cl, ch] around -o*j, and the products-sums are rounded
// down for entry planes and up for exit planes: every computed entry is at or below the exact one and
// every exit at or above, and the remaining rounding of 1/d itself is covered by the kInflate margin
// (Ize 2013).  |j| is clamped to [2^-60, 2^64] so that nothing overflows.  Past 2^64 (a zero or tiny
// direction component) the entry plane's t stays a lower bound where it is positive.  The exit
// plane's t is raised by the ray's current far bound tfar (ch = -o*j + tfar, rounded up): an exit
// plane ahead of the origin then lies at or beyond tfar and never rejects the box, while one behind
// the origin still does (its exact t is at or below the clamped one, so raising it stays an upper
// bound).  tfar only shrinks during a traversal, so terms set with an earlier tfar stay valid.
// Below 2^-60 the exit plane's t stays an upper bound where it is positive and the entry plane is
// dropped (cl = -inf).  Boxes are therefore never rejected when the exact test accepts them,
// including rays that start on a plane with a zero direction component.  Which of a box's two
// planes is the entry one follows from the sign of j (the ray's octant).
struct Ray {
    float ox, oy, oz;              // origin of the current level (world, or the instance's object space)
    float dx, dy, dz;              // WORLD direction (kept while inside a BLAS: only instance entry reads it)
    float jx, jy, jz;              // 1/d of the current level, magnitude clamped to [2^-60, 2^64]
    float clx, cly, clz;           // -o*j rounded down (-inf: entry planes dropped)
    float chx, chy, chz;           // -o*j rounded up (plus the far bound where |j| = 2^64)
    float Sx, Sy, Sz;              // shear of the watertight triangle test (BLAS level)
    uint32_t bits;                 // kx | ky << 2 | kz << 4 (triangle test axes) | octant << 6
};

__device__ __forceinline__ float comp(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

// j, cl, ch from the origin, 1/d and the ray's current far bound tfar
__device__ __forceinline__ void box_terms(float o, float inv, float tfar, float& j, float& cl, float& ch) {
    const float ai = fabsf(inv);
    j = copysignf(fminf(fmaxf(ai, 0x1p-60f), 0x1p64f), inv);
    const float c = -(o * j);
    const float err = fabsf(c) * 0x1p-22f;  // |c - (-o j)| <= 2^-24 |c| (one rounding)
    // the clamp rules read j alone (so that a saved j restores valid terms); at exactly 2^64 or
    // 2^-60 they only accept more
    cl = fabsf(j) > 0x1p-60f ? __fsub_rd(c, err) : -INFINITY;
    ch = fabsf(j) < 0x1p64f ? __fadd_ru(c, err) : __fadd_ru(__fadd_ru(c, err), tfar);
}

__device__ __forceinline__ uint32_t octant(float jx, float jy, float jz) {
    return (jx < 0.0f ? 1u : 0u) | (jy < 0.0f ? 2u : 0u) | (jz < 0.0f ? 4u : 0u);
}

__device__ __forceinline__ void set_box_terms(Ray& r, float ix, float iy, float iz, float tfar) {
    box_terms(r.ox, ix, tfar, r.jx, r.clx, r.chx);
    box_terms(r.oy, iy, tfar, r.jy, r.cly, r.chy);
    box_terms(r.oz, iz, tfar, r.jz, r.clz, r.chz);
    r.bits = (r.bits & 63u) | octant(r.jx, r.jy, r.jz) << 6;
}

// object-space ray at instance entry: origin, box terms and the triangle test's shear; the world
// direction in r stays untouched
__device__ __forceinline__ void ray_pre(Ray& r, float ox, float oy, float oz, float dx, float dy, float dz, float tfar) {
    r.ox = ox; r.oy = oy; r.oz = oz;
    float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    float dkz = comp(dx, dy, dz, kz);
    if (dkz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.bits = (uint32_t)kx | (uint32_t)ky << 2 | (uint32_t)kz << 4;
    r.Sx = comp(dx, dy, dz, kx) / dkz;
    r.Sy = comp(dx, dy, dz, ky) / dkz;
    r.Sz = 1.0f / dkz;
    set_box_terms(r, 1.0f / dx, 1.0f / dy, 1.0f / dz, tfar);
}

// the world-space ray at the TLAS level (no triangle is tested there)
__device__ __forceinline__ void ray_pre_world(Ray& r, float ox, float oy, float oz, float dx, float dy, float dz, float tfar) {
    r.ox = ox; r.oy = oy; r.oz = oz;
    r.dx = dx; r.dy = dy; r.dz = dz;
    r.bits = 0u;
    set_box_terms(r, 1.0f / dx, 1.0f / dy, 1.0f / dz, tfar);
}

constexpr float kInflate = 1.0000004f;  // 1 + 2*gamma_3 (Ize 2013) rounded up



// entry and exit t of one box given its entry planes (n) and exit planes (f)
__device__ __forceinline__ float box_test(const Ray& r, float nx, float ny, float nz, float fx, float fy, float fz, float tmin,
                                          float tbest) {
    const float tn = fmaxf(fmaxf(__fmaf_rd(nx, r.jx, r.clx), __fmaf_rd(ny, r.jy, r.cly)), fmaxf(__fmaf_rd(nz, r.jz, r.clz), tmin));
    const float tf = fminf(fminf(__fmaf_ru(fx, r.jx, r.chx), __fmaf_ru(fy, r.jy, r.chy)), fminf(__fmaf_ru(fz, r.jz, r.chz), tbest));
    return tn <= tf * kInflate ? tn : INFINITY;
}

// a box given as lo xyz, hi xyz
__device__ __forceinline__ float box_test6(const Ray& r, const float* lo, const float* hi, float tmin, float tbest) {
    const uint32_t o = r.bits >> 6;
    return box_test(r, (o & 1) ? hi[0] : lo[0], (o & 2) ? hi[1] : lo[1], (o & 4) ? hi[2] : lo[2],
                    (o & 1) ? lo[0] : hi[0], (o & 2) ? lo[1] : hi[1], (o & 4) ? lo[2] : hi[2], tmin, tbest);
}

struct Hit {
    float t, u, v;
    uint32_t inst, prim;
    bool hit;
};

__device__ __forceinline__ bool accept(float t, float tmin, uint32_t inst, uint32_t prim, const Hit& h) {
    if (!(t >= tmin)) return false;
    if (!h.hit) return t <= h.t;
    if (t < h.t) return true;
    if (t == h.t) return inst < h.inst || (inst == h.inst && prim < h.prim);
    return false;
}

__device__ __forceinline__ void tri_test(const Ray& r, float4 a, float4 b, float4 c, float tmin, uint32_t inst, Hit& h) {
    const int kx = (int)(r.bits & 3u), ky = (int)((r.bits >> 2) & 3u), kz = (int)((r.bits >> 4) & 3u);
    float A0 = a.x - r.ox, A1 = a.y - r.oy, A2 = a.z - r.oz;
    float B0 = b.x - r.ox, B1 = b.y - r.oy, B2 = b.z - r.oz;
    float C0 = c.x - r.ox, C1 = c.y - r.oy, C2 = c.z - r.oz;
    float Akz = comp(A0, A1, A2, kz), Bkz = comp(B0, B1, B2, kz), Ckz = comp(C0, C1, C2, kz);
    float Ax = comp(A0, A1, A2, kx) - r.Sx * Akz, Ay = comp(A0, A1, A2, ky) - r.Sy * Akz;
    float Bx = comp(B0, B1, B2, kx) - r.Sx * Bkz, By = comp(B0, B1, B2, ky) - r.Sy * Bkz;
    float Cx = comp(C0, C1, C2, kx) - r.Sx * Ckz, Cy = comp(C0, C1, C2, ky) - r.Sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return;
    float det = (U + V) + W;
    if (det == 0.0f) return;
    float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
    float T = (U * Az + V * Bz) + W * Cz;
    float rc = 1.0f / det;
    float t = T * rc;
    uint32_t prim = __float_as_uint(a.w);
    if (!accept(t, tmin, inst, prim, h)) return;
    h.t = t;
    h.u = V * rc;
    h.v = W * rc;
    h.inst = inst;
    h.prim = prim;
    h.hit = true;
}

constexpr uint32_t kMarker = 0xFFFFFFFFu;  // stack entry: leave the BLAS, back to the TLAS

struct VisitCounts {
    unsigned long long nodes, tris, overflow;
};

constexpr int kTraceThreads = 128;
#ifndef RG_TRACE_MIN_BLOCKS
#define RG_TRACE_MIN_BLOCKS 4
#endif

// per-thread traversal stack in shared memory, laid out [depth][thread] so that the 32 lanes of a
// warp touching the same depth hit 32 different banks.  THREADS = block size, DEPTH = entries.
// Beside it, six floats per thread keep the world-space ray's origin and clamped inverse direction
// while the ray is inside a BLAS (the world direction itself stays in registers), so leaving the BLAS
// restores them instead of dividing again.
// The last of the DEPTH words flags an overflow (a push that found the other DEPTH - 1 entries
// full), so the flag costs the traversal loop neither a register nor shared memory beyond the stack.
template <int THREADS, int DEPTH>
struct SmemStackT {
    static constexpr int kDepth = DEPTH - 1;
    uint32_t* base;  // &stack[0][threadIdx.x]
    float* saved;    // &world[0][threadIdx.x]
    __device__ __forceinline__ uint32_t& operator[](int i) const { return base[i * THREADS]; }
    __device__ __forceinline__ float& w(int i) const { return saved[i * THREADS]; }
    __device__ __forceinline__ uint32_t& over() const { return base[(DEPTH - 1) * THREADS]; }
};
// the same stack in (L1-cached) local memory
#ifndef RG_STACK_SMEM
#define RG_STACK_SMEM 1
#endif
template <int DEPTH>
struct LocalStackT {
    static constexpr int kDepth = DEPTH - 1;
    uint32_t* base;
    float* saved;
    __device__ __forceinline__ uint32_t& operator[](int i) const { return base[i]; }
    __device__ __forceinline__ float& w(int i) const { return saved[i]; }
    __device__ __forceinline__ uint32_t& over() const { return base[DEPTH - 1]; }
};
#define RG_DECLARE_SMEM_STACK(name, THREADS, DEPTH)      \
    __shared__ uint32_t name##_mem[DEPTH][THREADS];      \
    __shared__ float name##_world[6][THREADS];           \
    const SmemStackT<THREADS, DEPTH> name{&name##_mem[0][threadIdx.x], &name##_world[0][threadIdx.x]}
#if RG_STACK_SMEM
#define RG_DECLARE_STACK(name) RG_DECLARE_SMEM_STACK(name, kTraceThreads, kTraversalStack)
using TravStack = SmemStackT<kTraceThreads, kTraversalStack>;
#else
#define RG_DECLARE_STACK(name)                 \
    uint32_t name##_mem[kTraversalStack];      \
    float name##_world[6];                     \
    const LocalStackT<kTraversalStack> name{name##_mem, name##_world}
using TravStack = LocalStackT<kTraversalStack>;
#endif
#ifndef RG_WF_MIN_BLOCKS
#define RG_WF_MIN_BLOCKS 7
#endif
#ifndef RG_TAIL_RAYS
#define RG_TAIL_RAYS 32768
#endif
#ifndef RG_POLL_ROUNDS
#define RG_POLL_ROUNDS 4
#endif

// Resumable traversal of one ray: trav_begin sets it up, each trav_step processes one record or one
// leaf (a record tests up to eight children and descends into the nearest hit; a TLAS leaf moves
// the ray into the instance's object space and descends into its BLAS behind a marker entry; a BLAS
// leaf runs the triangle test).  The kernel interleaves trav_step with shading so that a lane whose
// ray finished does not idle.
struct Trav {
    float tmin;
    Ray r;  // the ray of the current level (world or object space); its shear terms are used in BLASes only
    Hit h;
    const WideNode* nodes;
    const float4* tris;
    uint32_t ref, inst;
    int sp;
    bool inBlas, active;
};

template <class STACK>
__device__ __forceinline__ void trav_begin(Trav& T, const DevScene& sc, float ox, float oy, float oz, float dx, float dy, float dz,
                                           float tmin, float tmax, const STACK& stack) {
    stack.over() = 0u;
    T.h.hit = false;
    T.h.t = tmax;
    T.h.u = T.h.v = 0.0f;
    T.h.inst = T.h.prim = 0xFFFFFFFFu;
    T.active = false;
    if ((dx == 0.0f && dy == 0.0f && dz == 0.0f) || sc.tlasN == 0) return;
    T.tmin = tmin;
    ray_pre_world(T.r, ox, oy, oz, dx, dy, dz, tmax);
    if (sc.tlasN > 1 && box_test6(T.r, sc.tlasRoot, sc.tlasRoot + 3, tmin, T.h.t) == INFINITY) return;
    T.sp = 0;
    T.nodes = sc.tlasWide;
    T.tris = nullptr;
    T.inBlas = false;
    T.inst = 0;
    T.ref = sc.tlasN == 1 ? kLeaf : 0u;
    T.active = true;
}

template <bool COUNT, class STACK>
__device__ __forceinline__ void trav_step(Trav& T, const DevScene& sc, const STACK& stack, VisitCounts& vc) {
    const uint32_t ref = T.ref;
    const float tmin = T.tmin;
    if (!(ref & kLeaf)) {
        if (COUNT) vc.nodes++;
        const WideNode* nd = T.nodes + ref;
        // entry and exit plane vectors of the ray's octant (lox, hix, loy, hiy, loz, hiz in order)
        const float4* pl = &nd->lox;
        const uint32_t o = T.r.bits >> 6;
        const uint32_t ox = o & 1u, oy = (o >> 1) & 1u, oz = (o >> 2) & 1u;
        const float4 nx = __ldg(pl + ox), fx = __ldg(pl + (ox ^ 1u));
        const float4 ny = __ldg(pl + 2 + oy), fy = __ldg(pl + 2 + (oy ^ 1u));
        const float4 nz = __ldg(pl + 4 + oz), fz = __ldg(pl + 4 + (oz ^ 1u));
        const uint4 rf = __ldg(&nd->ref);
        float t[4];
        uint32_t r[4] = {rf.x, rf.y, rf.z, rf.w};
        t[0] = box_test(T.r, nx.x, ny.x, nz.x, fx.x, fy.x, fz.x, tmin, T.h.t);
        t[1] = box_test(T.r, nx.y, ny.y, nz.y, fx.y, fy.y, fz.y, tmin, T.h.t);
        t[2] = r[2] != kEmptySlot ? box_test(T.r, nx.z, ny.z, nz.z, fx.z, fy.z, fz.z, tmin, T.h.t) : INFINITY;
        t[3] = r[3] != kEmptySlot ? box_test(T.r, nx.w, ny.w, nz.w, fx.w, fy.w, fz.w, tmin, T.h.t) : INFINITY;
        // nearest first: 5 compare-exchanges sort the four (t, ref) pairs
#define RG_CSWAP(a, b)                                           \
        if (t[b] < t[a]) {                                       \
            float tt = t[a]; t[a] = t[b]; t[b] = tt;             \
            uint32_t rr = r[a]; r[a] = r[b]; r[b] = rr;          \
        }
        RG_CSWAP(0, 1) RG_CSWAP(2, 3) RG_CSWAP(0, 2) RG_CSWAP(1, 3) RG_CSWAP(1, 2)
#undef RG_CSWAP
        if (t[0] != INFINITY) {
#pragma unroll
            for (int j = 3; j >= 1; --j)
                if (t[j] != INFINITY) {
                    if (T.sp < STACK::kDepth) stack[T.sp++] = r[j];
                    else stack.over() = 1u;
                }
            T.ref = r[0];
            return;
        }
    } else if (T.inBlas) {
        if (COUNT) vc.tris++;
        const float4* tp = T.tris + 3 * (size_t)(ref & ~kLeaf);
        tri_test(T.r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), tmin, T.inst, T.h);
    } else {
        const InstRec* ir = sc.tlasLeaves + (ref & ~kLeaf);
        const float4 i0 = __ldg(&ir->inv[0]), i1 = __ldg(&ir->inv[1]), i2 = __ldg(&ir->inv[2]);
        const float4 lo = __ldg(&ir->lo), hi = __ldg(&ir->hi);
        const uint32_t bn = __float_as_uint(lo.w);
        if (bn > 0) {
            const float ox = T.r.ox, oy = T.r.oy, oz = T.r.oz, dx = T.r.dx, dy = T.r.dy, dz = T.r.dz;  // world ray (TLAS level)
            float qx = ((i0.x * ox + i0.y * oy) + i0.z * oz) + i0.w;
            float qy = ((i1.x * ox + i1.y * oy) + i1.z * oz) + i1.w;
            float qz = ((i2.x * ox + i2.y * oy) + i2.z * oz) + i2.w;
            float ex = (i0.x * dx + i0.y * dy) + i0.z * dz;
            float ey = (i1.x * dx + i1.y * dy) + i1.z * dz;
            float ez = (i2.x * dx + i2.y * dy) + i2.z * dz;
            if (!(ex == 0.0f && ey == 0.0f && ez == 0.0f)) {
                Ray orr;
                orr.dx = dx; orr.dy = dy; orr.dz = dz;  // the world direction stays in the ray
                ray_pre(orr, qx, qy, qz, ex, ey, ez, T.h.t);
                const float blo[3] = {lo.x, lo.y, lo.z}, bhi[3] = {hi.x, hi.y, hi.z};
                if (box_test6(orr, blo, bhi, tmin, T.h.t) != INFINITY) {
                    if (T.sp < STACK::kDepth) {
                        const ulonglong2 pp = __ldg(reinterpret_cast<const ulonglong2*>(&ir->wide));
                        stack.w(0) = ox; stack.w(1) = oy; stack.w(2) = oz;
                        stack.w(3) = T.r.jx; stack.w(4) = T.r.jy; stack.w(5) = T.r.jz;
                        stack[T.sp++] = kMarker;
                        T.r = orr;
                        T.nodes = reinterpret_cast<const WideNode*>(pp.x);
                        T.tris = reinterpret_cast<const float4*>(pp.y);
                        T.inst = __float_as_uint(hi.w);
                        T.inBlas = true;
                        T.ref = bn == 1 ? kLeaf : 0u;
                        return;
                    }
                    stack.over() = 1u;
                }
            }
        }
    }
    // pop (a marker leaves the BLAS: back to the world-space ray and the TLAS)
    for (;;) {
        if (T.sp == 0) {
            T.active = false;
            return;
        }
        uint32_t nr = stack[--T.sp];
        if (nr != kMarker) {
            T.ref = nr;
            return;
        }
        T.inBlas = false;
        T.nodes = sc.tlasWide;
        T.r.ox = stack.w(0); T.r.oy = stack.w(1); T.r.oz = stack.w(2);
        box_terms(T.r.ox, stack.w(3), T.h.t, T.r.jx, T.r.clx, T.r.chx);
        box_terms(T.r.oy, stack.w(4), T.h.t, T.r.jy, T.r.cly, T.r.chy);
        box_terms(T.r.oz, stack.w(5), T.h.t, T.r.jz, T.r.clz, T.r.chz);
        T.r.bits = octant(T.r.jx, T.r.jy, T.r.jz) << 6;
        }
}

// Deep re-trace.  The short stack of the kernels (kTraversalStack entries in shared memory, or the
// batch tuner's depth) holds the far children of the records on the ray's current path: up to 3 per
// 4-wide record level, plus one marker while the ray is inside a BLAS.  Deep trees whose boxes the
// ray hits many at a time can need more.  A push that finds the short stack full sets Trav::over
// instead, and when that ray's traversal ends it is traced again from the start with this stack of
// kDeepStack entries in local memory, so its result is complete.  Every tree this library builds has
// at most 64 BVH2 levels (LBVH: 30 code bits plus at most 32 index bits of tie-break, one level per
// bit; binned SAH: kSahMedianLevel + 18), i.e. at most 32 record levels, so a TLAS path, a marker and
// a BLAS path take at most 3 * 32 + 1 + 3 * 32 = 193 entries.  Should a push still find it full, the
// ray is counted in counters[7] (rg_stats.deep_overflows), never silently.
constexpr int kDeepStack = 196;  // 195 entries and the overflow flag
__device__ __noinline__ void retrace_deep(const DevScene* sc, float4 o, float4 d, Hit* out, unsigned long long* counters) {
    uint32_t mem[kDeepStack];
    float world[6];
    const LocalStackT<kDeepStack> st{mem, world};
    VisitCounts vc = {0, 0, 0};
    Trav T;
    trav_begin(T, *sc, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, st);
    while (T.active) trav_step<false>(T, *sc, st, vc);
    if (st.over() && counters) {
        atomicAdd(counters + 7, 1ull);
        atomicAdd(counters + 15, 1ull);
    }
    *out = T.h;
}

template <bool COUNT, class STACK>
__device__ Hit closest_hit(const DevScene& sc, float ox, float oy, float oz, float dx, float dy, float dz, float tmin, float tmax,
                           const STACK& stack, VisitCounts& vc, unsigned long long* counters) {
    Trav T;
    trav_begin(T, sc, ox, oy, oz, dx, dy, dz, tmin, tmax, stack);
    while (T.active) trav_step<COUNT>(T, sc, stack, vc);
    if (stack.over()) {
        vc.overflow++;
        retrace_deep(&sc, make_float4(ox, oy, oz, tmin), make_float4(dx, dy, dz, tmax), &T.h, counters);
    }
    return T.h;
}

// ---------------------------------------------------------------------------------------------
// GLSL helpers with the oracle's operation order
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ V3 v3s(float s) { return {s, s, s}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ V3 normalize(V3 v) {
    float l = sqrtf(dot(v, v));
    return {v.x / l, v.y / l, v.z / l};
}
__device__ __forceinline__ float mixs(float x, float y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ V3 mix(V3 x, V3 y, float a) { return {mixs(x.x, y.x, a), mixs(x.y, y.y, a), mixs(x.z, y.z, a)}; }
__device__ __forceinline__ V3 reflect(V3 I, V3 N) {
    float k = 2.0f * dot(N, I);
    return I - N * k;
}
__device__ __forceinline__ V3 refract(V3 I, V3 N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return v3s(0.0f);
    float s = eta * d + sqrtf(k);
    return I * eta - N * s;
}
__device__ __forceinline__ float glsl_mod(float x, float y) { return x - y * floorf(x / y); }
__device__ __forceinline__ float len(V3 v) { return sqrtf(dot(v, v)); }

enum : int { RT_GENERIC = 0, RT_SHADOW_TRACE = 1, RT_SHADOW_INTERNAL = 2 };

struct Payload {  // payload.h:29-39
    V3 hitValue;
    float reflectContribution;
    V3 normal;
    V3 roughRGB;
    float roughA;
    float depth, curIOR, refDepth;
    int rayType, recDepth;
    uint32_t seed;  // glossy reference shading: per-sample random seed (0: mirror shading); not in payload.h
};

// resume codes of a paused closest-hit invocation
enum : int {
    R_G_SHADOW = 0,    // GENERIC, after the shadow ray (closesthit.rchit:193)
    R_G_REFLECT = 1,   // GENERIC, after the reflection ray (:215)
    R_G_REFR_F = 2,    // GENERIC, after the front-face refraction ray (:232)
    R_G_REFR_B = 3,    // GENERIC, after the back-face refraction ray (:244)
    R_SI_A = 4,        // SHADOW_INTERNAL, after the shadow-trace ray (:133)
    R_SI_B = 5,        // SHADOW_INTERNAL, after the mask-0 trace (:144)
    R_ST_C = 6         // SHADOW_TRACE, after the shadow-internal ray (:158)
};

struct __align__(16) Frame {
    int kind, front, rayConsumption, pad;
    V3 origin, D, n;
    float t;
    V3 diffuse, specular;
    float transparency, reflectivity, roughness, ior, emission;
    V3 base;          // GENERIC: baseColor; SHADOW_INTERNAL: shadowCol
    V3 shadow;        // GENERIC: shadowColor
    V3 reflectColor;  // GENERIC
    float reflectDepth;
    float pad1;
};
static_assert(sizeof(Frame) == 144, "frame");

// miss.rmiss:38-83
__device__ void sky(Payload& p, V3 D, V3 L) {
    const V3 sunTone = v3(1.0f, 0.6f, 0.05f), skyTone = v3(0.2f, 0.4f, 0.8f), scatterTone = v3(1.0f, 0.3f, 0.0f);
    const float scatterFactor = 1.3f, powFactor = 80.0f;
    V3 rayDir = normalize(D);
    float y = fabsf(D.y + 1.5f) / 3.0f;
    float sun = 1.0f - len(rayDir - normalize(-L));
    sun = clampf(sun, 0.0f, 2.0f);
    float glow = sun;
    glow = clampf(glow, 0.0f, 1.0f);
    sun = powf(sun, powFactor);
    sun = sun * 1000.0f;
    sun = clampf(sun, 0.0f, 16.0f);
    glow = glow * glow * glow * glow * glow * glow * 1.0f;
    glow = powf(glow, y);
    glow = clampf(glow, 0.0f, 1.0f);
    sun = sun * powf(y * y, 1.0f / 1.65f);
    glow = glow * powf(y * y, 1.0f / 2.0f);
    sun = sun + glow;
    V3 sunColor = sunTone * sun;
    float atmosphere = sqrtf(1.0f - y);
    float scatter = powf(4.0f - L.y, 1.0f / 15.0f);
    scatter = 1.0f - clampf(scatter, 0.8f, 1.0f);
    V3 scatterColor = mix(v3s(1.0f), scatterTone * 1.5f, scatter);
    V3 skyScatter = mix(skyTone, scatterColor, atmosphere / scatterFactor);
    V3 res = sunColor + skyScatter;
    p.hitValue = res;
    p.roughRGB = res;
    p.roughA = 0.0f;
    p.depth = 10000.0f;
}

__device__ __forceinline__ uint2 pack_half4(float a, float b, float c, float d) {
    __half2 lo = __floats2half2_rn(a, b), hi = __floats2half2_rn(c, d);
    return make_uint2(*reinterpret_cast<uint32_t*>(&lo), *reinterpret_cast<uint32_t*>(&hi));
}

__constant__ float kAA[9][8][2] = {
    {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}},
    {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}},
    {{0.25f, 0.25f}, {-0.25f, -0.25f}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}},
    {{-0.125f, -0.375f}, {0.375f, -0.125f}, {-0.375f, 0.125f}, {0.125f, 0.375f}, {0, 0}, {0, 0}, {0, 0}, {0, 0}},
    {{-0.125f, -0.375f}, {0.375f, -0.125f}, {-0.375f, 0.125f}, {0.125f, 0.375f}, {0, 0}, {0, 0}, {0, 0}, {0, 0}},
    {{0.0625f, -0.1875f}, {-0.0625f, 0.1875f}, {0.3125f, 0.0625f}, {-0.1875f, -0.3125f}, {-0.3125f, 0.3125f}, {-0.4375f, -0.0625f}, {0.1875f, 0.4375f}, {0.4375f, -0.4375f}},
    {{0.0625f, -0.1875f}, {-0.0625f, 0.1875f}, {0.3125f, 0.0625f}, {-0.1875f, -0.3125f}, {-0.3125f, 0.3125f}, {-0.4375f, -0.0625f}, {0.1875f, 0.4375f}, {0.4375f, -0.4375f}},
    {{0.0625f, -0.1875f}, {-0.0625f, 0.1875f}, {0.3125f, 0.0625f}, {-0.1875f, -0.3125f}, {-0.3125f, 0.3125f}, {-0.4375f, -0.0625f}, {0.1875f, 0.4375f}, {0.4375f, -0.4375f}},
    {{0.0625f, -0.1875f}, {-0.0625f, 0.1875f}, {0.3125f, 0.0625f}, {-0.1875f, -0.3125f}, {-0.3125f, 0.3125f}, {-0.4375f, -0.0625f}, {0.1875f, 0.4375f}, {0.4375f, -0.4375f}},
};

// column-major mat4 * vec4 with the oracle's summation order
__device__ __forceinline__ void mul4(const float* m, float v0, float v1, float v2, float v3, float* o) {
#pragma unroll
    for (int r = 0; r < 4; ++r) o[r] = ((m[r] * v0 + m[4 + r] * v1) + m[8 + r] * v2) + m[12 + r] * v3;
}

enum : int { PH_HIT, PH_G_REFLECT, PH_G_REFRACT, PH_G_COMPOSE, PH_RETURN };

struct RayReq {
    V3 o, d;
    float tmin, tmax;
    int missIndex;
    bool masked;
};

struct RayCounts {  // per thread (flushed as 64-bit sums)
    uint32_t primary, shadow, secondary, masked;
};

__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {  // PCG-RXS-M-XS (O'Neill 2014) output permutation
    const uint32_t st = v * 747796405u + 2891336453u;
    const uint32_t w = ((st >> ((st >> 28u) + 4u)) ^ st) * 277803737u;
    return (w >> 22u) ^ w;
}

// Glossy reference shading: a GGX microfacet normal (Walter et al. 2007, alpha = roughness^2) drawn
// around n from two uniforms of the sample's seed and stream k
__device__ __forceinline__ V3 ggx_normal(V3 n, float roughness, uint32_t seed, uint32_t k) {
    const uint32_t h1 = pcg_hash(seed * 2654435761u + k), h2 = pcg_hash(h1 ^ 0x9E3779B9u);
    const float u1 = (float)(h1 >> 8) * (1.0f / 16777216.0f), u2 = (float)(h2 >> 8) * (1.0f / 16777216.0f);
    const float a = roughness * roughness;
    const float tan2 = a * a * u1 / fmaxf(1.0f - u1, 1e-7f);
    const float cosT = rsqrtf(1.0f + tan2), sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
    const float phi = 6.28318530718f * u2;
    // orthonormal basis around n (Duff et al. 2017)
    const float sg = copysignf(1.0f, n.z), aa = -1.0f / (sg + n.z), bb = n.x * n.y * aa;
    const V3 t = v3(1.0f + sg * n.x * n.x * aa, sg * bb, -sg * n.x), b = v3(bb, sg + n.y * n.y * aa, -n.y);
    return normalize(t * (sinT * cosf(phi)) + b * (sinT * sinf(phi)) + n * cosT);
}

// One step of the closest-hit / miss state machine: consume the result `h` of the pending trace and
// run the paused invocations on the frame stack until the next trace is needed (returns true, `ray`
// set) or the sample's primary trace has returned (returns false).
template <bool GLOSSY = true>
__device__ __forceinline__ bool shade_step(const DevScene& sc, const V3 L, const int maxRec, const Hit& h, Payload& p, RayReq& ray,
                                           Frame* frames, int& fsp, Frame& cur, RayCounts& cnt) {
    int ph;
    if (!h.hit) {
        if (ray.missIndex == 0) sky(p, ray.d, L);
        else p.hitValue = v3s(1.0f);  // shadowMiss.rmiss:30-34
        ph = PH_RETURN;
    } else {
        ph = PH_HIT;
    }
    bool newRay = false;
    V3 refractColor = v3s(1.0f);
    while (!newRay) {
        if (ph == PH_HIT) {
            // closesthit.rchit:95-122 -- fetch, world position, world normal, grid effect
            const DevInstance* in = sc.inst + h.inst;
            const uint32_t vOff = __ldg(&in->vOff), iOff = __ldg(&in->iOff), mOff = __ldg(&in->mOff);
            const float4 m0 = __ldg(&in->m[0]), m1 = __ldg(&in->m[1]), m2 = __ldg(&in->m[2]);
            const float hitT = h.t;
            const float bx = (1.0f - h.u) - h.v, by = h.u, bz = h.v;
            const uint32_t ib = iOff + 3 * h.prim;
            const rg_vertex* v0 = sc.vertices + vOff + __ldg(sc.indices + ib);
            const rg_vertex* v1 = sc.vertices + vOff + __ldg(sc.indices + ib + 1);
            const rg_vertex* v2 = sc.vertices + vOff + __ldg(sc.indices + ib + 2);
            const uint32_t matIndex = __ldg(&v0->matIndex);
            V3 n0 = v3(__ldg(&v0->normal[0]), __ldg(&v0->normal[1]), __ldg(&v0->normal[2]));
            V3 n1 = v3(__ldg(&v1->normal[0]), __ldg(&v1->normal[1]), __ldg(&v1->normal[2]));
            V3 n2 = v3(__ldg(&v2->normal[0]), __ldg(&v2->normal[1]), __ldg(&v2->normal[2]));
            const rg_material* M = sc.materials + mOff + matIndex;
            cur.diffuse = v3(__ldg(&M->diffuse[0]), __ldg(&M->diffuse[1]), __ldg(&M->diffuse[2]));
            cur.specular = v3(__ldg(&M->specular[0]), __ldg(&M->specular[1]), __ldg(&M->specular[2]));
            cur.transparency = __ldg(&M->transparency);
            cur.reflectivity = __ldg(&M->reflectivity);
            cur.roughness = __ldg(&M->roughness);
            cur.ior = __ldg(&M->ior);
            cur.emission = __ldg(&M->emission);
            cur.rayConsumption = (int)__ldg(&M->rayConsumption);
            const uint32_t effectId = __ldg(&M->effectId);
            cur.origin = ray.o + ray.d * hitT;
            cur.D = ray.d;
            cur.t = hitT;
            V3 vn = (n0 * bx + n1 * by) + n2 * bz;
            V3 wn = v3((m0.x * vn.x + m0.y * vn.y) + m0.z * vn.z, (m1.x * vn.x + m1.y * vn.y) + m1.z * vn.z,
                       (m2.x * vn.x + m2.y * vn.y) + m2.z * vn.z);
            cur.n = normalize(wn);
            if (effectId == 1) {  // gridEffect, closesthit.rchit:74-91
                V3 pos = cur.origin;
                float aa = ((p.refDepth + hitT) + 8.0f) / 30.0f;
                float aa2 = aa / 2.0f;
                float minmod = fminf(fabsf(glsl_mod((pos.x + 1000.0f) * 10.0f + aa2, 20.0f) - aa2),
                                     fabsf(glsl_mod((pos.z + 1000.0f) * 10.0f + aa2, 20.0f) - aa2));
                if (minmod < aa2) {
                    float aa_sq = aa * aa;
                    minmod = minmod - (aa2 - aa_sq / 3.0f);
                    minmod = minmod * (3.0f / aa_sq);
                    float f = mixs(aa / 10.0f, 1.0f, minmod);
                    cur.diffuse = cur.diffuse * f;
                    cur.specular = cur.specular * f;
                    cur.reflectivity = cur.reflectivity * f;
                }
                if (glsl_mod((pos.x + 1000.0f) * 5.0f, 20.0f) < 10.0f && glsl_mod((pos.z + 1000.0f) * 5.0f, 20.0f) < 10.0f)
                    cur.reflectivity = cur.reflectivity * 1.5f;
            }
            if (p.rayType == RT_SHADOW_INTERNAL) {  // :125-152
                float thick = clampf(hitT * (1.0f - cur.transparency) * 10.0f, 0.0f, 1.0f);
                V3 shadowCol = p.hitValue - mix(v3s(0.0f), normalize(v3s(1.1f) - cur.diffuse) + v3s(0.1f), thick);
                if (p.recDepth < maxRec) {
                    p.rayType = RT_SHADOW_TRACE;
                    p.recDepth++;
                    cnt.shadow++;
                    cur.base = shadowCol;
                    cur.kind = R_SI_A;
                    frames[fsp++] = cur;
                    ray.o = cur.origin; ray.d = cur.D; ray.tmin = 0.01f; ray.tmax = 1000.0f; ray.missIndex = 0; ray.masked = false;
                    newRay = true;
                } else {
                    p.hitValue = shadowCol * 0.4f;
                    ph = PH_RETURN;
                }
            } else if (p.rayType == RT_SHADOW_TRACE) {  // :153-166
                if (cur.transparency > 0.0f) {
                    if (p.recDepth < maxRec) {
                        p.rayType = RT_SHADOW_INTERNAL;
                        p.recDepth++;
                        cnt.shadow++;
                        cur.kind = R_ST_C;
                        frames[fsp++] = cur;
                        ray.o = cur.origin; ray.d = cur.D; ray.tmin = 0.01f; ray.tmax = 1000.0f; ray.missIndex = 1; ray.masked = false;
                        newRay = true;
                    } else {
                        ph = PH_RETURN;
                    }
                } else {
                    float f = mixs(0.4f, 0.8f, clampf(logf(hitT) / 8.0f, 0.0f, 1.0f));
                    p.hitValue = p.hitValue * f;
                    ph = PH_RETURN;
                }
            } else {  // GENERIC, :168-204
                cur.front = dot(-cur.D, cur.n) > 0.0f;
                if (!cur.front) cur.n = normalize(-cur.n);
                float ndl = dot(-L, cur.n);
                float dp = fmaxf(ndl, 0.2f);
                cur.base = cur.diffuse * dp;
                cur.reflectColor = v3s(1.0f);
                cur.reflectDepth = 0.0f;
                if (ndl > 0.07f) {
                    if (p.recDepth < maxRec) {
                        p.hitValue = v3s(1.0f);
                        p.rayType = RT_SHADOW_TRACE;
                        p.recDepth++;
                        cnt.shadow++;
                        cur.kind = R_G_SHADOW;
                        frames[fsp++] = cur;
                        ray.o = cur.origin; ray.d = -L; ray.tmin = 0.01f * 10.0f; ray.tmax = 1000.0f; ray.missIndex = 1; ray.masked = false;
                        newRay = true;
                    } else {
                        cur.shadow = v3s(1.0f);
                        ph = PH_G_REFLECT;
                    }
                } else {
                    float tr = cur.transparency;
                    float sm = tr * tr;
                    cur.shadow = tr < 1.0f ? mix(v3s(1.0f), cur.diffuse * sm, tr) : v3s(0.4f);
                    ph = PH_G_REFLECT;
                }
            }
        } else if (ph == PH_G_REFLECT) {  // :206-221
            if (p.recDepth < maxRec && cur.reflectivity > 0.0f) {
                V3 dir = reflect(cur.D, cur.n);
                if (GLOSSY && p.seed && p.recDepth == 0 && cur.roughness > 0.0f) {  // glossy reference shading
                    const V3 g = reflect(cur.D, ggx_normal(cur.n, cur.roughness, p.seed, 1u));
                    if (dot(g, cur.n) > 0.0f) dir = g;
                }
                p.recDepth += cur.rayConsumption;
                p.refDepth = p.refDepth + cur.t;
                cnt.secondary++;
                cur.kind = R_G_REFLECT;
                frames[fsp++] = cur;
                ray.o = cur.origin; ray.d = dir; ray.tmin = 0.01f; ray.tmax = 1000.0f; ray.missIndex = 0; ray.masked = false;
                newRay = true;
            } else {
                ph = PH_G_REFRACT;
            }
        } else if (ph == PH_G_REFRACT) {  // :223-251
            if (p.recDepth < maxRec && cur.transparency > 0.0f) {
                V3 dir;
                const bool glossy = GLOSSY && p.seed && p.recDepth == 0 && cur.roughness > 0.0f;
                const V3 mn = glossy ? ggx_normal(cur.n, cur.roughness, p.seed, 2u) : cur.n;
                if (cur.front) {
                    float eta = p.curIOR / cur.ior;
                    dir = refract(cur.D, cur.n, eta);
                    if (glossy) {  // glossy reference shading: refraction through the sampled microfacet
                        const V3 g = refract(cur.D, mn, eta);
                        if (!(g.x == 0.0f && g.y == 0.0f && g.z == 0.0f)) dir = g;
                    }
                    p.curIOR = cur.ior;
                    cur.kind = R_G_REFR_F;
                } else {
                    float eta = cur.ior / 1.0f;
                    dir = refract(cur.D, cur.n, eta);
                    if (glossy) {
                        const V3 g = refract(cur.D, mn, eta);
                        if (!(g.x == 0.0f && g.y == 0.0f && g.z == 0.0f)) dir = g;
                    }
                    p.curIOR = 1.0f;
                    cur.kind = R_G_REFR_B;
                }
                p.recDepth++;
                if (!(dir.x == 0.0f && dir.y == 0.0f && dir.z == 0.0f)) cnt.secondary++;  // only rays that traverse
                frames[fsp++] = cur;
                ray.o = cur.origin; ray.d = dir; ray.tmin = 0.01f; ray.tmax = 1000.0f; ray.missIndex = 0; ray.masked = false;
                newRay = true;
            } else {
                refractColor = v3s(1.0f);
                ph = PH_G_COMPOSE;
            }
        } else if (ph == PH_G_COMPOSE) {  // :253-267
            V3 baseColor = cur.base * cur.shadow;
            baseColor = baseColor + cur.diffuse * cur.emission;
            float total = fmaxf(cur.transparency, cur.reflectivity);
            float den = cur.transparency + cur.reflectivity;
            float w = den == 0.0f ? 0.0f : cur.reflectivity / den;
            V3 roughCol = mix(refractColor, cur.reflectColor, w);
            p.hitValue = mix(baseColor, roughCol, total);
            if (p.recDepth == 0) {
                p.hitValue = baseColor;
                p.normal = cur.n;
                p.roughRGB = roughCol;
                p.roughA = fminf((cur.reflectDepth / 50.0f) * cur.roughness, cur.roughness / 2.1f);
                p.reflectContribution = total;
            }
            p.depth = cur.t;
            ph = PH_RETURN;
        } else {  // PH_RETURN: resume the paused invocation
            if (fsp == 0) break;
            cur = frames[--fsp];
            switch (cur.kind) {
                case R_G_SHADOW:
                    p.recDepth--;
                    cur.shadow = p.hitValue;
                    p.rayType = RT_GENERIC;
                    ph = PH_G_REFLECT;
                    break;
                case R_G_REFLECT:
                    p.recDepth -= cur.rayConsumption;
                    cur.reflectColor = p.hitValue * cur.specular;
                    cur.reflectDepth = p.depth;
                    ph = PH_G_REFRACT;
                    break;
                case R_G_REFR_F:
                    p.recDepth--;
                    refractColor = p.hitValue;
                    ph = PH_G_COMPOSE;
                    break;
                case R_G_REFR_B:
                    p.recDepth--;
                    refractColor = mix(v3s(1.0f), cur.diffuse, logf(1.0f + cur.t)) * p.hitValue;
                    ph = PH_G_COMPOSE;
                    break;
                case R_SI_A:
                    p.recDepth--;
                    if (p.depth < 1000.0f) {
                        p.hitValue = p.hitValue * cur.base;
                        ph = PH_RETURN;
                    } else {
                        float eta = cur.ior / 1.0f;
                        V3 dir = refract(cur.D, cur.n, eta);
                        float x = dot(L, dir);
                        float dp = x * x * x * x * x + 0.75f;
                        cur.base = cur.base * dp;
                        cur.kind = R_SI_B;
                        frames[fsp++] = cur;
                        cnt.masked++;
                        ray.o = cur.origin; ray.d = -dir; ray.tmin = 0.01f; ray.tmax = 1000.0f; ray.missIndex = 0; ray.masked = true;
                        newRay = true;
                    }
                    break;
                case R_SI_B:
                    p.hitValue = cur.base + p.hitValue * 0.1f;
                    ph = PH_RETURN;
                    break;
                default:  // R_ST_C
                    p.recDepth--;
                    ph = PH_RETURN;
                    break;
            }
        }
    }
    return newRay;
}

// raygen.h:84-102: camera ray of one sample and the payload initialisation
__device__ __forceinline__ void start_sample(const rg_ubo& U, const V3 camO, uint32_t px, uint32_t py, uint32_t W, uint32_t H,
                                             int sample, int aaRow, Payload& p, RayReq& ray, uint32_t glossySeed = 0u) {
    float pcx = ((float)px + 0.5f) + kAA[aaRow][sample & 7][0];
    float pcy = ((float)py + 0.5f) + kAA[aaRow][sample & 7][1];
    float ux = pcx / (float)W, uy = pcy / (float)H;
    float dx = ux * 2.0f - 1.0f, dy = uy * 2.0f - 1.0f;
    float tg[4], dw[4];
    mul4(U.projInverse, dx, dy, 1.0f, 1.0f, tg);
    V3 tn = normalize(v3(tg[0], tg[1], tg[2]));
    mul4(U.viewInverse, tn.x, tn.y, tn.z, 0.0f, dw);
    ray.o = camO;
    ray.d = v3(dw[0], dw[1], dw[2]);
    ray.tmin = 0.001f;
    ray.tmax = 10000.0f;
    ray.missIndex = 0;
    ray.masked = false;
    p.hitValue = v3s(0.0f);
    p.normal = v3s(0.0f);
    p.roughRGB = v3s(0.0f);
    p.roughA = 0.0f;
    p.depth = 0.0f;
    p.refDepth = 0.0f;
    p.curIOR = 1.0f;
    p.rayType = RT_GENERIC;
    p.recDepth = 0;
    p.reflectContribution = 0.0f;
    p.seed = glossySeed ? ((pcg_hash(glossySeed ^ pcg_hash(px + pcg_hash(py + pcg_hash((uint32_t)sample)))) & 0xFFFFFFu) | 1u) : 0u;
}

#ifndef RG_TRACE_STEPS
#define RG_TRACE_STEPS 4
#endif
#ifndef RG_SHADE_THRESHOLD
#define RG_SHADE_THRESHOLD 16
#endif
enum : int { kIdle = 0, kTraverse = 1, kResult = 2 };

// starts the traversal of the pending trace; mask-0 traces and zero directions need none
template <class STACK>
__device__ __forceinline__ int begin_ray(Trav& T, const DevScene& sc, const RayReq& ray, const STACK& stack) {
    if (ray.masked) {
        T.h.hit = false;
        T.active = false;
        stack.over() = 0u;
        return kResult;
    }
    trav_begin(T, sc, ray.o.x, ray.o.y, ray.o.z, ray.d.x, ray.d.y, ray.d.z, ray.tmin, ray.tmax, stack);
    return T.active ? kTraverse : kResult;
}

// (kTileW x kTileH, the 32 pixels of one work tile, are declared in rg_internal.cuh)

// Persistent kernel: each lane takes (pixel, sample) work items from a global counter -- in
// warp-aggregated batches -- and runs the sample's whole depth-first trace sequence.  Traversal is
// resumable: every loop iteration advances each lane's ray by up to RG_TRACE_STEPS nodes, and a
// lane whose ray finished shades it and starts its next ray (or takes the next work item) while
// the other lanes keep traversing, so no lane idles behind the longest ray of its warp.  Work items
// enumerate 8x4 pixel tiles, then pixels, then samples, so consecutive items are coherent.
// Each sample's payload sums go to `samples` (12 floats); k_resolve averages them in sample order.
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, RG_TRACE_MIN_BLOCKS) k_trace(const __grid_constant__ TraceParams P) {
    RG_DECLARE_STACK(stk);
    const DevScene& sc = P.scene;
    const rg_ubo& U = P.ubo;
    const V3 L = v3(U.lightDir[0], U.lightDir[1], U.lightDir[2]);
    const int maxRec = U.maxRecursions;
    const uint32_t S = (uint32_t)U.numSamples;
    const int aaRow = S < 8 ? (int)S : 8;
    const uint32_t tilesX = (P.W + kTileW - 1) / kTileW, tilesY = (P.H + kTileH - 1) / kTileH;
    const uint32_t total = tilesX * tilesY * (kTileW * kTileH) * S;
    const unsigned lane = threadIdx.x & 31;
    const unsigned ltmask = (1u << lane) - 1u;

    float org[4];
    mul4(U.viewInverse, 0.0f, 0.0f, 0.0f, 1.0f, org);
    const V3 camO = v3(org[0], org[1], org[2]);

    RayCounts cnt = {0, 0, 0, 0};
    VisitCounts vc = {0, 0, 0};
    Frame frames[kMaxFrames];
    int fsp = 0;
    Payload p;
    RayReq ray;
    Frame cur;
    Trav T;
    T.active = false;
    bool alive = true;
    int state = kIdle;
    uint32_t px = 0, py = 0, sample = 0;

    for (;;) {
        // A shading round runs when at least RG_SHADE_THRESHOLD lanes of the warp wait (finished ray
        // or no work) or no lane is traversing: the waiting lanes shade together, idle lanes take new
        // work items (one atomic per warp), then every lane with a ray continues traversing.
        const unsigned travMask = __ballot_sync(0xFFFFFFFFu, state == kTraverse);
        const unsigned waitMask = __ballot_sync(0xFFFFFFFFu, state == kResult || (alive && state == kIdle));
        if (travMask == 0 || __popc(waitMask) >= RG_SHADE_THRESHOLD) {
            if (state == kResult) {
                // closest-hit / miss shading of the finished trace, up to the next trace
                if (shade_step(sc, L, maxRec, T.h, p, ray, frames, fsp, cur, cnt)) {
                    state = begin_ray(T, sc, ray, stk);
                } else {
                    float4* o = P.samples + 3 * ((size_t)(py * P.W + px) * S + sample);
                    o[0] = make_float4(p.hitValue.x, p.hitValue.y, p.hitValue.z, p.reflectContribution);
                    o[1] = make_float4(p.normal.x, p.normal.y, p.normal.z, p.depth);
                    o[2] = make_float4(p.roughRGB.x, p.roughRGB.y, p.roughRGB.z, p.roughA);
                    state = kIdle;
                }
            }
            const bool need = alive && state == kIdle;
            const unsigned needMask = __ballot_sync(0xFFFFFFFFu, need);
            if (needMask) {
                const int leader = __ffs(needMask) - 1;
                uint32_t base = 0;
                if ((int)lane == leader) base = atomicAdd(P.workCounter, (uint32_t)__popc(needMask));
                base = __shfl_sync(0xFFFFFFFFu, base, leader);
                if (need) {
                    const uint32_t id = base + (uint32_t)__popc(needMask & ltmask);
                    if (id >= total) {
                        alive = false;
                    } else {
                        sample = id % S;
                        const uint32_t pid = id / S, tile = pid / (kTileW * kTileH), within = pid % (kTileW * kTileH);
                        px = (tile % tilesX) * kTileW + within % kTileW;
                        py = (tile / tilesX) * kTileH + within / kTileW;
                        if (px < P.W && py < P.H) {
                            start_sample(U, camO, px, py, P.W, P.H, (int)sample, aaRow, p, ray, P.glossySeed);
                            cnt.primary++;
                            fsp = 0;
                            state = begin_ray(T, sc, ray, stk);
                        }
                    }
                }
            }
            if (!__any_sync(0xFFFFFFFFu, alive)) break;
        }
        if (state == kTraverse) {
#pragma unroll 1
            for (int k = 0; k < RG_TRACE_STEPS; ++k) {
                trav_step<COUNT>(T, sc, stk, vc);
                if (!T.active) {
                    if (stk.over()) {
                        vc.overflow++;
                        retrace_deep(&sc, make_float4(ray.o.x, ray.o.y, ray.o.z, ray.tmin), make_float4(ray.d.x, ray.d.y, ray.d.z, ray.tmax),
                                     &T.h, P.counters);
                    }
                    state = kResult;
                    break;
                }
            }
        }
    }

    // ray statistics: warp reduction then one atomic per warp (all lanes are here)
    unsigned long long c[7] = {cnt.primary, cnt.shadow, cnt.secondary, cnt.masked, vc.nodes, vc.tris, vc.overflow};
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        unsigned long long v = c[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
        if (lane == 0 && v) {
            atomicAdd(P.counters + k, v);
            atomicAdd(P.counters + 8 + k, v);
        }
    }
}

// raygen.h:116 + raygen.rgen:36-38: average one pixel's S samples (in sample order) into the three
// RGBA16F G-buffer images; normal.w = log(sum of depths) * 0.25 / S
__device__ __forceinline__ void resolve_pixel(const float4* s, uint32_t S, size_t pix, uint2* base, uint2* normal, uint2* rough) {
    float4 a = s[0], b = s[1], c = s[2];
    for (uint32_t k = 1; k < S; ++k) {
        const float4 a2 = s[3 * k], b2 = s[3 * k + 1], c2 = s[3 * k + 2];
        a.x = a.x + a2.x; a.y = a.y + a2.y; a.z = a.z + a2.z; a.w = a.w + a2.w;
        b.x = b.x + b2.x; b.y = b.y + b2.y; b.z = b.z + b2.z; b.w = b.w + b2.w;
        c.x = c.x + c2.x; c.y = c.y + c2.y; c.z = c.z + c2.z; c.w = c.w + c2.w;
    }
    const float fs = (float)S;
    base[pix] = pack_half4(a.x / fs, a.y / fs, a.z / fs, a.w / fs);
    normal[pix] = pack_half4(b.x / fs, b.y / fs, b.z / fs, (logf(b.w) * 0.25f) / fs);
    rough[pix] = pack_half4(c.x / fs, c.y / fs, c.z / fs, c.w / fs);
}

__global__ void k_resolve(const TraceParams P) {
    const uint32_t x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= P.W || y >= P.H) return;
    const uint32_t S = (uint32_t)P.ubo.numSamples;
    const size_t pix = (size_t)y * P.W + x;
    resolve_pixel(P.samples + 3 * pix * S, S, pix, P.base, P.normal, P.rough);
}

// samples: the job's first sample (samples + 3 * sampleBase)
__global__ void k_resolve_job(const float4* __restrict__ samples, uint32_t W, uint32_t H, uint32_t S, uint2* base, uint2* normal,
                              uint2* rough) {
    const uint32_t x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const size_t pix = (size_t)y * W + x;
    resolve_pixel(samples + 3 * pix * S, S, pix, base, normal, rough);
}

// ---------------------------------------------------------------------------------------------
// Wavefront form of the same path: every (pixel, sample) is a path with exactly one outstanding
// ray at a time (the reference's recursion is depth-first on one payload), so a frame is a loop of
// (trace all pending rays, shade all their results).  The trace kernel only traverses: few
// registers, high occupancy, dynamic ray fetch.  The shade kernel runs the same state machine as
// the megakernel on the path's payload and frame stack, which live in device memory between the
// two kernels, and appends each path's next ray to the other queue.

struct PathMeta {
    int fsp, missIndex;
};

__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want) {
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, want);
    if (!mask) return 0;
    const unsigned lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void store_payload(float4* dst, const Payload& p) {
    dst[0] = make_float4(p.hitValue.x, p.hitValue.y, p.hitValue.z, p.reflectContribution);
    dst[1] = make_float4(p.normal.x, p.normal.y, p.normal.z, p.depth);
    dst[2] = make_float4(p.roughRGB.x, p.roughRGB.y, p.roughRGB.z, p.roughA);
    dst[3] = make_float4(p.curIOR, p.refDepth, __uint_as_float((uint32_t)p.rayType | (p.seed << 8)), __int_as_float(p.recDepth));
}

__device__ __forceinline__ void load_payload(const float4* src, Payload& p) {
    const float4 a = src[0], b = src[1], c = src[2], d = src[3];
    p.hitValue = v3(a.x, a.y, a.z);
    p.reflectContribution = a.w;
    p.normal = v3(b.x, b.y, b.z);
    p.depth = b.w;
    p.roughRGB = v3(c.x, c.y, c.z);
    p.roughA = c.w;
    p.curIOR = d.x;
    p.refDepth = d.y;
    p.rayType = (int)(__float_as_uint(d.z) & 0xFFu);
    p.seed = __float_as_uint(d.z) >> 8;
    p.recDepth = __float_as_int(d.w);
}

__device__ __forceinline__ void emit_ray(const WavefrontBuffers& wf, int q, uint32_t pos, uint32_t path, const RayReq& ray) {
    wf.qO[q][pos] = make_float4(ray.o.x, ray.o.y, ray.o.z, ray.tmin);
    wf.qD[q][pos] = make_float4(ray.d.x, ray.d.y, ray.d.z, ray.tmax);
    wf.qPath[q][pos] = path;
}

__device__ __forceinline__ void flush_counts(const TraceParams& P, unsigned long long* c, int n) {
    const unsigned lane = threadIdx.x & 31;
    for (int k = 0; k < n; ++k) {
        unsigned long long v = c[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
        c[k] = v;
    }
    if (lane == 0)
        for (int k = 0; k < n; ++k)
            if (c[k]) {
                atomicAdd(P.counters + k, c[k]);
                atomicAdd(P.counters + 8 + k, c[k]);
            }
}

// work item -> pixel and sample: work items enumerate 8x4 pixel tiles (row-major over the tile
// grid), then the 32 pixels of a tile (row-major), then the samples of a pixel
__device__ __forceinline__ bool decode_work(uint32_t id, uint32_t W, uint32_t H, uint32_t S, uint32_t tilesX, uint32_t& px,
                                            uint32_t& py, uint32_t& sample) {
    sample = id % S;
    const uint32_t pid = id / S, tile = pid / (kTileW * kTileH), within = pid % (kTileW * kTileH);
    px = (tile % tilesX) * kTileW + within % kTileW;
    py = (tile / tilesX) * kTileH + within / kTileW;
    return px < W && py < H;
}

// the job owning work item `id`: the last job whose workBase <= id (jobs are in work order)
__device__ __forceinline__ uint32_t find_job(const JobDesc* __restrict__ jobs, uint32_t n, uint32_t id) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].workBase <= id) lo = mid;
        else hi = mid;
    }
    return lo;
}

// camera ray and fresh payload of work item `id` of a batch (raygen.h:84-102 with the job's UBO);
// false when the item's pixel lies outside its image
__device__ __forceinline__ bool batch_primary(const TraceParams& P, uint32_t id, uint32_t& job, uint32_t& sampleIdx, Payload& p,
                                              RayReq& ray) {
    job = find_job(P.jobs, P.njobs, id);
    const JobDesc& J = P.jobs[job];
    uint32_t px, py, s;
    if (!decode_work(id - J.workBase, J.W, J.H, J.S, J.tilesX, px, py, s)) return false;
    float org[4];
    mul4(J.ubo.viewInverse, 0.0f, 0.0f, 0.0f, 1.0f, org);
    const int aaRow = J.S < 8 ? (int)J.S : 8;
    start_sample(J.ubo, v3(org[0], org[1], org[2]), px, py, J.W, J.H, (int)s, aaRow, p, ray, P.glossySeed);
    sampleIdx = J.sampleBase + (py * J.W + px) * J.S + s;
    return true;
}

__device__ __forceinline__ void store_sample(float4* so, const Payload& p) {
    so[0] = make_float4(p.hitValue.x, p.hitValue.y, p.hitValue.z, p.reflectContribution);
    so[1] = make_float4(p.normal.x, p.normal.y, p.normal.z, p.depth);
    so[2] = make_float4(p.roughRGB.x, p.roughRGB.y, p.roughRGB.z, p.roughA);
}

// work items of the frame loop: one path per (pixel, sample) in 8x4-tile order, all of them in the
// first round; path = (py * W + px) * S + sample
__device__ __forceinline__ uint32_t frame_work_total(const TraceParams& P) {
    const uint32_t S = (uint32_t)P.ubo.numSamples;
    return ((P.W + kTileW - 1) / kTileW) * ((P.H + kTileH - 1) / kTileH) * (kTileW * kTileH) * S;
}
// camera ray and initial payload of work item id (raygen.h:84-102); false outside the image
__device__ __forceinline__ bool frame_work_item(const TraceParams& P, uint32_t id, uint32_t& path, Payload& p, RayReq& ray) {
    const rg_ubo& U = P.ubo;
    const uint32_t S = (uint32_t)U.numSamples;
    const uint32_t tilesX = (P.W + kTileW - 1) / kTileW;
    uint32_t px = 0, py = 0, sample = 0;
    if (!decode_work(id, P.W, P.H, S, tilesX, px, py, sample)) return false;
    float org[4];
    mul4(U.viewInverse, 0.0f, 0.0f, 0.0f, 1.0f, org);
    start_sample(U, v3(org[0], org[1], org[2]), px, py, P.W, P.H, (int)sample, S < 8 ? (int)S : 8, p, ray, P.glossySeed);
    path = (py * P.W + px) * S + sample;
    return true;
}

// raygen of a batch: path slot k starts work item k (k < min(totalWork, slots)); the shade kernel
// hands later work items to slots whose paths finished
__global__ void __launch_bounds__(256) k_wfb_raygen(const TraceParams P) {
    const WavefrontBuffers& wf = P.wf;
    const uint32_t total = min(P.totalWork, P.slots);
    if (blockIdx.x == 0 && threadIdx.x == 0) *P.workCounter = total;
    unsigned long long c[1] = {0};
    for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
        const uint32_t id = base + threadIdx.x;
        Payload p;
        RayReq ray;
        uint32_t job = 0, si = 0;
        const bool valid = id < total && batch_primary(P, id, job, si, p, ray);
        const uint32_t pos = warp_append(wf.counts + 0, valid);
        if (valid) {
            store_payload(wf.payload + 4 * (size_t)id, p);
            wf.meta[id] = make_int2(0, 0);
            P.slotJob[id] = job;
            P.slotSample[id] = si;
            emit_ray(wf, 0, pos, id, ray);
            c[0]++;
        }
    }
    flush_counts(P, c, 1);
}

// closest hit of every ray of queue q.  Lanes whose ray finished take new rays from the queue (one
// atomic per warp) as soon as RG_FETCH_THRESHOLD lanes of the warp are idle, so a warp does not wait
// for its longest ray; between fetches every lane advances its ray by RG_WF_STEPS steps.  BATCH: the
// ray's scene is its path's job's scene.  P.perm (nullable) gives the order the rays are taken in.
#ifndef RG_FETCH_THRESHOLD
#define RG_FETCH_THRESHOLD 8
#endif
#ifndef RG_WF_STEPS
#define RG_WF_STEPS 6
#endif
#ifndef RG_WHILE_WHILE
#define RG_WHILE_WHILE 1
#endif
#ifndef RG_INNER_ROUNDS
#define RG_INNER_ROUNDS 3
#endif
// Shared memory: the stack (DEPTH words) and the parked world ray (6 words) per thread, nothing else:
// at 128 threads x 48 words that is 27,648 B, and 7 blocks (plus the 1 KB the driver reserves per
// block) fill the 196 KB shared-memory carve-out exactly.  One more byte per block moves the SM to
// the 228 KB carve-out and halves the L1 left for BVH records (measured: trace stage +5 %).
// a finished ray's hit: the frame loop's hit record (t, u, v, primitive; instance or 0xFFFFFFFF), or
// for a ray query rg_trace_rays' layout in the caller's buffers (t, u, v and (instance, primitive);
// zeros and 0xFFFFFFFF for a miss)
template <bool QUERY>
__device__ __forceinline__ void put_hit(const TraceParams& P, uint32_t slot, const Hit& h, bool hit) {
    if (QUERY) {
        float* t = P.queryTuv + 3 * (size_t)slot;
        uint32_t* id = P.queryIds + 2 * (size_t)slot;
        t[0] = hit ? h.t : 0.0f;
        t[1] = hit ? h.u : 0.0f;
        t[2] = hit ? h.v : 0.0f;
        id[0] = hit ? h.inst : 0xFFFFFFFFu;
        id[1] = hit ? h.prim : 0xFFFFFFFFu;
    } else {
        P.wf.hitTUV[slot] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
        P.wf.hitInst[slot] = hit ? h.inst : 0xFFFFFFFFu;
    }
}

// QUERY: the ray-query form (rg_trace_rays_device), rays and hits in the caller's buffers
template <bool COUNT, bool BATCH, int THREADS, int DEPTH, bool QUERY = false>
__global__ void __launch_bounds__(THREADS, (RG_WF_MIN_BLOCKS * 128) / THREADS) k_wf_trace(const __grid_constant__ TraceParams P, int q) {
    RG_DECLARE_SMEM_STACK(stk, THREADS, DEPTH);
    const WavefrontBuffers& wf = P.wf;
    const bool first = !BATCH && !QUERY && P.firstRound;
    const uint32_t count = QUERY ? P.queryCount : first ? frame_work_total(P) : *(volatile uint32_t*)(wf.counts + q);
    if (blockIdx.x == 0 && threadIdx.x == 0) wf.counts[q ^ 1] = 0;  // the shade kernel appends there next
    const unsigned lane = threadIdx.x & 31;
    const unsigned ltmask = (1u << lane) - 1u;
    VisitCounts vc = {0, 0, 0};
    Trav T;
    T.active = false;
    uint32_t slot = 0;
    const DevScene* scp = nullptr;  // BATCH: scene of the lane's ray
#define RG_SC (BATCH ? *scp : P.scene)
    // a finished ray's hit record; a ray whose short stack overflowed also joins the overflow list,
    // whose rays the kernel's last block traces again with the deep stack (below)
#define RG_WF_HIT_OUT()                                                                      \
    do {                                                                                     \
        if (stk.over()) {                                                                    \
            vc.overflow++;                                                                   \
            wf.overflow[atomicAdd(wf.counts + 3, 1u)] = slot;                                \
        }                                                                                    \
        put_hit<QUERY>(P, slot, T.h, T.h.hit);                                               \
    } while (0)
    bool exhausted = false;
    for (;;) {
        const unsigned idle = __ballot_sync(0xFFFFFFFFu, !T.active);
        if (__popc(idle) >= RG_FETCH_THRESHOLD || idle == 0xFFFFFFFFu) {
            const bool need = !T.active && !exhausted;
            const unsigned needMask = __ballot_sync(0xFFFFFFFFu, need);
            if (needMask) {
                const int leader = __ffs(needMask) - 1;
                uint32_t base = 0;
                if ((int)lane == leader) base = atomicAdd(wf.counts + 2, (uint32_t)__popc(needMask));
                base = __shfl_sync(0xFFFFFFFFu, base, leader);
                if (need) {
                    const uint32_t k = base + (uint32_t)__popc(needMask & ltmask);
                    if (k >= count) {
                        exhausted = true;
                    } else if (first) {  // camera ray of work item k, computed here
                        slot = k;
                        uint32_t path;
                        Payload p0;
                        RayReq r0;
                        if (frame_work_item(P, k, path, p0, r0)) {
                            trav_begin(T, P.scene, r0.o.x, r0.o.y, r0.o.z, r0.d.x, r0.d.y, r0.d.z, r0.tmin, r0.tmax, stk);
                            if (!T.active) {
                                wf.hitTUV[slot] = make_float4(T.h.t, T.h.u, T.h.v, __uint_as_float(T.h.prim));
                                wf.hitInst[slot] = 0xFFFFFFFFu;
                            }
                        }
                    } else {
                        slot = P.perm ? P.perm[k] : k;
                        if (BATCH) scp = &P.jobs[P.slotJob[wf.qPath[q][slot]]].scene;
                        const float4 o = QUERY ? P.queryRays[2 * (size_t)slot] : wf.qO[q][slot];
                        const float4 d = QUERY ? P.queryRays[2 * (size_t)slot + 1] : wf.qD[q][slot];
                        trav_begin(T, RG_SC, o.x, o.y, o.z, d.x, d.y, d.z, o.w, d.w, stk);
                        if (!T.active) put_hit<QUERY>(P, slot, T.h, false);  // zero direction or the scene box missed
                    }
                }
            }
            if (!__any_sync(0xFFFFFFFFu, T.active || !exhausted)) break;
        }
#if RG_WHILE_WHILE
        // while-while: lanes on inner nodes descend together (the others wait), then every lane at a
        // leaf processes it, so each pass runs one kind of step across most of the warp
#pragma unroll 1
        for (int k = 0; k < RG_WF_STEPS; ++k) {
#pragma unroll 1
            for (int j = 0; j < RG_INNER_ROUNDS; ++j) {
                const bool inner = T.active && !(T.ref & kLeaf);
                if (!__any_sync(0xFFFFFFFFu, inner)) break;
                if (inner) {
                    trav_step<COUNT>(T, RG_SC, stk, vc);
                    if (!T.active) RG_WF_HIT_OUT();
                }
            }
            if (T.active && (T.ref & kLeaf)) {
                trav_step<COUNT>(T, RG_SC, stk, vc);
                if (!T.active) RG_WF_HIT_OUT();
            }
        }
#else
        if (T.active) {
#pragma unroll 1
            for (int k = 0; k < RG_WF_STEPS; ++k) {
                trav_step<COUNT>(T, RG_SC, stk, vc);
                if (!T.active) {
                    RG_WF_HIT_OUT();
                    break;
                }
            }
        }
#endif
    }
#undef RG_WF_HIT_OUT
#undef RG_SC
    unsigned long long c[3] = {vc.nodes, vc.tris, vc.overflow};
    for (int k = 0; k < 3; ++k) {
        unsigned long long v = c[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
        if (lane == 0 && v) {
            atomicAdd(P.counters + 4 + k, v);
            atomicAdd(P.counters + 12 + k, v);
        }
    }
    // Rays whose short stack overflowed: the last block to finish (every other block has appended its
    // rays to the list and fenced) traces them again from the start with the deep stack and rewrites
    // their hit records, then clears the list for the next launch.  No block waits for another.
    // (thread 0's stack word carries the verdict: every stack is idle once the block is here; no
    // shared memory is added, which would cost the kernel L1 at 7 blocks per SM)
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        stk.over() = atomicAdd(wf.counts + 4, 1u) == gridDim.x - 1 ? 1u : 0u;
    }
    __syncthreads();
    const uint32_t lastBlock = *reinterpret_cast<volatile uint32_t*>(&stk_mem[DEPTH - 1][0]);
    if (!lastBlock) return;
    __threadfence();
    const uint32_t nOver = __ldcg(wf.counts + 3);
    for (uint32_t i = threadIdx.x; i < nOver; i += blockDim.x) {
        const uint32_t s = __ldcg(wf.overflow + i);
        float4 o, d;
        const DevScene* sc = &P.scene;
        if (first) {  // work item s's camera ray, as the first round computed it
            uint32_t path;
            Payload p0;
            RayReq r0;
            frame_work_item(P, s, path, p0, r0);
            o = make_float4(r0.o.x, r0.o.y, r0.o.z, r0.tmin);
            d = make_float4(r0.d.x, r0.d.y, r0.d.z, r0.tmax);
        } else if (QUERY) {
            o = P.queryRays[2 * (size_t)s];
            d = P.queryRays[2 * (size_t)s + 1];
        } else {
            o = __ldcg(&wf.qO[q][s]);
            d = __ldcg(&wf.qD[q][s]);
            if (BATCH) sc = &P.jobs[P.slotJob[__ldcg(&wf.qPath[q][s])]].scene;
        }
        Hit h;
        retrace_deep(sc, o, d, &h, P.counters);
        put_hit<QUERY>(P, s, h, h.hit);
    }
    if (threadIdx.x == 0) {
        wf.counts[3] = 0;
        wf.counts[4] = 0;
    }
}

// shading of one path from a trace result up to its next traversed ray (false) or to the end of
// its sample (true); mask-0 traces and zero directions run their miss shader right away
template <bool GLOSSY>
__device__ __forceinline__ bool shade_until_trace(const DevScene& sc, const V3 L, const int maxRec, Hit h, Payload& p, RayReq& ray,
                                                  Frame* frames, int& fsp, Frame& cur, RayCounts& cnt) {
    for (;;) {
        if (!shade_step<GLOSSY>(sc, L, maxRec, h, p, ray, frames, fsp, cur, cnt)) return true;
        if (ray.masked || (ray.d.x == 0.0f && ray.d.y == 0.0f && ray.d.z == 0.0f)) {
            h.hit = false;
            continue;
        }
        return false;
    }
}

// shading of every result of queue q; next rays go to queue q^1, finished samples to P.samples.
// BATCH: a slot whose path finished starts the batch's next work item in place.
#ifndef RG_SHADE_MIN_BLOCKS
#define RG_SHADE_MIN_BLOCKS 6  // 85 registers, a few spilled: 6 blocks of 128 per SM beat 4 unspilled
#endif
template <bool BATCH, bool GLOSSY = false>
__global__ void __launch_bounds__(128, BATCH ? 1 : RG_SHADE_MIN_BLOCKS) k_wf_shade(const TraceParams P, int q) {
    const WavefrontBuffers& wf = P.wf;
    const V3 L = v3(P.ubo.lightDir[0], P.ubo.lightDir[1], P.ubo.lightDir[2]);
    const int maxRec = P.ubo.maxRecursions;
    const bool first = !BATCH && P.firstRound;
    const uint32_t count = first ? frame_work_total(P) : *(volatile uint32_t*)(wf.counts + q);
    if (blockIdx.x == 0 && threadIdx.x == 0) wf.counts[2] = 0;  // the next trace kernel's work counter
    const unsigned lane = threadIdx.x & 31;
    RayCounts cnt = {0, 0, 0, 0};
    Frame* framesBase = static_cast<Frame*>(wf.frames);
    bool exhausted = false;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool emit = false, regen = false;
        uint32_t path = 0;
        Payload p;
        Frame cur;
        RayReq ray;
        int fsp = 0;
        bool live = i < count;
        if (live && first) {  // the work item's camera ray and initial payload, as the trace kernel made them
            live = frame_work_item(P, i, path, p, ray);
            fsp = 0;
            if (live) cnt.primary++;
        } else if (live) {
            path = wf.qPath[q][i];
            const float4 o = wf.qO[q][i], d = wf.qD[q][i];
            const int2 meta = wf.meta[path];
            fsp = meta.x;
            ray.o = v3(o.x, o.y, o.z);
            ray.tmin = o.w;
            ray.d = v3(d.x, d.y, d.z);
            ray.tmax = d.w;
            ray.missIndex = meta.y;
            ray.masked = false;
            load_payload(wf.payload + 4 * (size_t)path, p);
        }
        if (live) {
            const float4 ht = wf.hitTUV[i];
            Hit h;
            h.inst = wf.hitInst[i];
            h.hit = h.inst != 0xFFFFFFFFu;
            h.t = ht.x;
            h.u = ht.y;
            h.v = ht.z;
            h.prim = __float_as_uint(ht.w);
            Frame* frames = framesBase + (size_t)path * kMaxFrames;
            bool done;
            if constexpr (BATCH) {
                const JobDesc& J = P.jobs[P.slotJob[path]];
                done = shade_until_trace<GLOSSY>(J.scene, v3(J.ubo.lightDir[0], J.ubo.lightDir[1], J.ubo.lightDir[2]), J.ubo.maxRecursions, h,
                                                 p, ray, frames, fsp, cur, cnt);
            } else {
                done = shade_until_trace<GLOSSY>(P.scene, L, maxRec, h, p, ray, frames, fsp, cur, cnt);
            }
            if (done) {
                store_sample(P.samples + 3 * (size_t)(BATCH ? P.slotSample[path] : path), p);
                regen = BATCH;
            } else {
                emit = true;
            }
        }
        if constexpr (BATCH) {
            // path regeneration: finished slots take the next work items (one atomic per warp and try)
            for (;;) {
                const bool need = regen && !exhausted;
                const unsigned needMask = __ballot_sync(0xFFFFFFFFu, need);
                if (!needMask) break;
                const int leader = __ffs(needMask) - 1;
                uint32_t b0 = 0;
                if ((int)lane == leader) b0 = atomicAdd(P.workCounter, (uint32_t)__popc(needMask));
                b0 = __shfl_sync(0xFFFFFFFFu, b0, leader);
                if (need) {
                    const uint32_t id = b0 + (uint32_t)__popc(needMask & ((1u << lane) - 1u));
                    uint32_t job = 0, si = 0;
                    if (id >= P.totalWork) {
                        exhausted = true;
                    } else if (batch_primary(P, id, job, si, p, ray)) {
                        P.slotJob[path] = job;
                        P.slotSample[path] = si;
                        fsp = 0;
                        regen = false;
                        emit = true;
                        cnt.primary++;
                    }
                }
            }
        }
        const uint32_t pos = warp_append(wf.counts + (q ^ 1), emit);
        if (emit) {
            emit_ray(wf, q ^ 1, pos, path, ray);
            store_payload(wf.payload + 4 * (size_t)path, p);
            wf.meta[path] = make_int2(fsp, ray.missIndex);
        }
    }
    unsigned long long c[4] = {cnt.primary, cnt.shadow, cnt.secondary, cnt.masked};
    flush_counts(P, c, 4);
}

// the rest of one path, traced and shaded back to back
template <bool GLOSSY, class STACK>
__device__ __forceinline__ void finish_path(const DevScene& sc, const V3 L, const int maxRec, RayReq& ray, Payload& p, Frame* frames,
                                            int& fsp, const STACK& stk, VisitCounts& vc, RayCounts& cnt, unsigned long long* counters) {
    Frame cur;
    for (;;) {
        Hit h;
        h.hit = false;
        if (!ray.masked)
            h = closest_hit<false>(sc, ray.o.x, ray.o.y, ray.o.z, ray.d.x, ray.d.y, ray.d.z, ray.tmin, ray.tmax, stk, vc, counters);
        if (!shade_step<GLOSSY>(sc, L, maxRec, h, p, ray, frames, fsp, cur, cnt)) break;
    }
}

// Tail of the wavefront loop: once few paths remain, one launch finishes every remaining path --
// each thread traces and shades its path's remaining sequence back to back -- instead of one
// (trace, shade) launch pair per remaining round.  BATCH: only after the last work item was taken.
template <bool BATCH, bool GLOSSY = false>
__global__ void __launch_bounds__(kTraceThreads) k_wf_tail(const __grid_constant__ TraceParams P, int q) {
    RG_DECLARE_STACK(stk);
    const WavefrontBuffers& wf = P.wf;
    const V3 L0 = v3(P.ubo.lightDir[0], P.ubo.lightDir[1], P.ubo.lightDir[2]);
    const int maxRec0 = P.ubo.maxRecursions;
    const uint32_t count = *(volatile uint32_t*)(wf.counts + q);
    RayCounts cnt = {0, 0, 0, 0};
    VisitCounts vc = {0, 0, 0};
    Frame* framesBase = static_cast<Frame*>(wf.frames);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t path = wf.qPath[q][i];
        const float4 o = wf.qO[q][i], d = wf.qD[q][i];
        const int2 meta = wf.meta[path];
        int fsp = meta.x;
        RayReq ray;
        ray.o = v3(o.x, o.y, o.z);
        ray.tmin = o.w;
        ray.d = v3(d.x, d.y, d.z);
        ray.tmax = d.w;
        ray.missIndex = meta.y;
        ray.masked = false;
        Payload p;
        load_payload(wf.payload + 4 * (size_t)path, p);
        Frame* frames = framesBase + (size_t)path * kMaxFrames;
        if constexpr (BATCH) {
            const JobDesc& J = P.jobs[P.slotJob[path]];
            finish_path<GLOSSY>(J.scene, v3(J.ubo.lightDir[0], J.ubo.lightDir[1], J.ubo.lightDir[2]), J.ubo.maxRecursions, ray, p, frames, fsp,
                        stk, vc, cnt, P.counters);
        } else {
            finish_path<GLOSSY>(P.scene, L0, maxRec0, ray, p, frames, fsp, stk, vc, cnt, P.counters);
        }
        store_sample(P.samples + 3 * (size_t)(BATCH ? P.slotSample[path] : path), p);
    }
    unsigned long long c[6] = {cnt.shadow, cnt.secondary, cnt.masked, vc.nodes, vc.tris, vc.overflow};
    const int slot[6] = {1, 2, 3, 4, 5, 6};
    const unsigned lane = threadIdx.x & 31;
    for (int k = 0; k < 6; ++k) {
        unsigned long long v = c[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
        if (lane == 0 && v) {
            atomicAdd(P.counters + slot[k], v);
            atomicAdd(P.counters + 8 + slot[k], v);
        }
    }
}

// ---- ray sort of a queue (batch loop, optional) ------------------------------------------------
// Bucket keys: direction octant (8 buckets) or the Morton code of the origin quantised to 16 cells
// per axis of the scene's root box (4096 buckets).  The order within a bucket is arbitrary: every
// ray's result is a function of the ray alone, so the sort changes which lane traces a ray, not
// what it returns.
template <int KEY>
struct SortBuckets {
    static constexpr int n = KEY == RG_SORT_OCTANT ? 8 : 4096;
};

template <bool BATCH, int KEY>
__device__ __forceinline__ uint32_t ray_sort_key(const TraceParams& P, const float4 o, const float4 d, uint32_t path) {
    if (KEY == RG_SORT_OCTANT) return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    const DevScene& sc = BATCH ? P.jobs[P.slotJob[path]].scene : P.scene;
    if (sc.tlasN == 0) return 0u;
    const float* b = sc.tlasRoot;
    const float x = fminf(fmaxf((o.x - b[0]) / (b[3] - b[0]) * 16.0f, 0.0f), 15.0f);
    const float y = fminf(fmaxf((o.y - b[1]) / (b[4] - b[1]) * 16.0f, 0.0f), 15.0f);
    const float z = fminf(fmaxf((o.z - b[2]) / (b[5] - b[2]) * 16.0f, 0.0f), 15.0f);
    return (expand10((uint32_t)x) << 2) | (expand10((uint32_t)y) << 1) | expand10((uint32_t)z);
}

// per block: histogram of the queue's keys in shared memory, added to the global bucket counts
template <bool BATCH, int KEY>
__global__ void __launch_bounds__(256) k_sort_count(const TraceParams P, int q, uint32_t* __restrict__ keys,
                                                     uint32_t* __restrict__ buckets) {
    constexpr int NB = SortBuckets<KEY>::n;
    __shared__ uint32_t h[NB];
    for (int i = threadIdx.x; i < NB; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const WavefrontBuffers& wf = P.wf;
    const uint32_t count = *(volatile uint32_t*)(wf.counts + q);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t k = ray_sort_key<BATCH, KEY>(P, wf.qO[q][i], wf.qD[q][i], BATCH ? wf.qPath[q][i] : 0u);
        keys[i] = k;
        atomicAdd(&h[k], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NB; i += blockDim.x)
        if (h[i]) atomicAdd(&buckets[i], h[i]);
}

// exclusive scan of the bucket counts into offsets (one block of 1024 threads); clears the counts
template <int NB>
__global__ void __launch_bounds__(1024) k_sort_offsets(uint32_t* __restrict__ buckets, uint32_t* __restrict__ offsets) {
    constexpr int PER = (NB + 1023) / 1024;
    __shared__ uint32_t part[1024];
    uint32_t v[PER], sum = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int b = threadIdx.x * PER + k;
        v[k] = b < NB ? buckets[b] : 0u;
        sum += v[k];
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const uint32_t t = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int b = threadIdx.x * PER + k;
        if (b < NB) {
            offsets[b] = run;
            buckets[b] = 0u;
        }
        run += v[k];
    }
}

// perm[offsets[key]++] = ray: each block reserves one range per bucket, then fills it
template <int KEY>
__global__ void __launch_bounds__(256) k_sort_scatter(const TraceParams P, int q, const uint32_t* __restrict__ keys,
                                                       uint32_t* __restrict__ offsets, uint32_t* __restrict__ perm) {
    constexpr int NB = SortBuckets<KEY>::n;
    __shared__ uint32_t h[NB], start[NB];
    for (int i = threadIdx.x; i < NB; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const uint32_t count = *(volatile uint32_t*)(P.wf.counts + q);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) atomicAdd(&h[keys[i]], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < NB; i += blockDim.x) {
        start[i] = h[i] ? atomicAdd(&offsets[i], h[i]) : 0u;
        h[i] = 0;
    }
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        perm[start[k] + atomicAdd(&h[k], 1u)] = i;
    }
}

template <int DEPTH>
__global__ void __launch_bounds__(kTraceThreads) k_trace_rays(const __grid_constant__ DevScene sc, const float* __restrict__ rays,
                                                               uint32_t n, float* __restrict__ tuv, uint32_t* __restrict__ ids,
                                                               unsigned long long* counters) {
    RG_DECLARE_SMEM_STACK(stk, kTraceThreads, DEPTH);
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float* r = rays + 8 * (size_t)k;
    VisitCounts vc = {0, 0, 0};
    Hit h = closest_hit<false>(sc, r[0], r[1], r[2], r[4], r[5], r[6], r[3], r[7], stk, vc, counters);
    if (vc.overflow) {  // rays re-traced deep, counted like the frame's
        atomicAdd(counters + 6, vc.overflow);
        atomicAdd(counters + 14, vc.overflow);
    }
    if (h.hit) {
        tuv[3 * k] = h.t; tuv[3 * k + 1] = h.u; tuv[3 * k + 2] = h.v;
        ids[2 * k] = h.inst; ids[2 * k + 1] = h.prim;
    } else {
        tuv[3 * k] = tuv[3 * k + 1] = tuv[3 * k + 2] = 0.0f;
        ids[2 * k] = ids[2 * k + 1] = 0xFFFFFFFFu;
    }
}

}  // namespace

cudaError_t launch_trace(const TraceParams& p, cudaStream_t s) {
    static std::atomic<int> gridBlocks[2];  // zero-initialised (static storage); first use computes them
    const int c = p.countVisits ? 1 : 0;
    if (!gridBlocks[c].load(std::memory_order_acquire)) {
        int dev = 0, sms = 0, perSm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = c ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_trace<true>, kTraceThreads, 0)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_trace<false>, kTraceThreads, 0);
        if (e != cudaSuccess) return e;
        gridBlocks[c].store(sms * (perSm > 0 ? perSm : 1), std::memory_order_release);
    }
    const int gBlocks = gridBlocks[c].load(std::memory_order_acquire);
    cudaError_t e = cudaMemsetAsync(p.workCounter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    if (p.countVisits) k_trace<true><<<gBlocks, kTraceThreads, 0, s>>>(p);
    else k_trace<false><<<gBlocks, kTraceThreads, 0, s>>>(p);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dim3 grid((p.W + 31) / 32, (p.H + 7) / 8);
    k_resolve<<<grid, 256, 0, s>>>(p);
    count_launch();
    return cudaGetLastError();
}

static int persistent_grid(const void* fn, int threads, int smem) {
    int dev = 0, sms = 0, perSm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, fn, threads, smem) != cudaSuccess) return 0;
    return sms * (perSm > 0 ? perSm : 1);
}

// persistent grid sizes, one per kernel (computed on first use; contexts on several host threads
// share the table)
static int grid_of(const void* fn, int threads) {
    static std::mutex mu;
    static const void* fns[64];
    static int grids[64];
    static int n = 0;
    std::lock_guard<std::mutex> lock(mu);
    for (int k = 0; k < n; ++k)
        if (fns[k] == fn) return grids[k];
    const int g = persistent_grid(fn, threads, 0);
    if (g && n < 64) {
        fns[n] = fn;
        grids[n] = g;
        ++n;
    }
    return g;
}

typedef void (*TraceKernel)(const TraceParams, int);

// the traversal kernel of one launch shape
static TraceKernel trace_kernel(bool batch, bool count, int threads, int depth) {
    if (count) return batch ? k_wf_trace<true, true, kTraceThreads, kTraversalStack> : k_wf_trace<true, false, kTraceThreads, kTraversalStack>;
    if (!batch) return k_wf_trace<false, false, kTraceThreads, kTraversalStack>;
#define RG_TK(T, D) \
    if (threads == T && depth == D) return k_wf_trace<false, true, T, D>;
    RG_TK(64, 16) RG_TK(64, 24) RG_TK(64, 32) RG_TK(64, 48)
    RG_TK(128, 16) RG_TK(128, 24) RG_TK(128, 32) RG_TK(128, 48)
    RG_TK(256, 16) RG_TK(256, 24) RG_TK(256, 32)  // 256 x 48 exceeds the 48 KB of static shared memory
#undef RG_TK
    return nullptr;
}

bool tune_supported(const TraceTune& t) {
    return trace_kernel(true, false, t.threads, t.depth) != nullptr && t.sortKey >= RG_SORT_NONE && t.sortKey <= RG_SORT_MORTON;
}

// the query form of the traversal kernel for a stack depth (visit counting: the default depth only)
static TraceKernel query_kernel(bool count, int depth) {
    if (count) return k_wf_trace<true, false, kTraceThreads, kTraversalStack, true>;
    switch (depth) {
        case 16: return k_wf_trace<false, false, kTraceThreads, 16, true>;
        case 24: return k_wf_trace<false, false, kTraceThreads, 24, true>;
        case 32: return k_wf_trace<false, false, kTraceThreads, 32, true>;
        case 48: return k_wf_trace<false, false, kTraceThreads, 48, true>;
        default: return nullptr;
    }
}

cudaError_t launch_trace_queue(const TraceParams& p, const float* rays, uint32_t n, float* tuv, uint32_t* ids, int depth,
                               cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (reinterpret_cast<uintptr_t>(rays) & 15u) return cudaErrorInvalidValue;  // read as float4
    const TraceKernel trace = query_kernel(p.countVisits != 0, depth);
    if (!trace) return cudaErrorInvalidValue;
    const int g = grid_of((const void*)trace, kTraceThreads);
    if (!g) return cudaErrorUnknown;
    TraceParams q = p;
    q.firstRound = 0;
    q.perm = nullptr;
    q.queryRays = reinterpret_cast<const float4*>(rays);
    q.queryTuv = tuv;
    q.queryIds = ids;
    q.queryCount = n;
    // the fetch counter, the overflow-list length and the finished-block count (the kernel's last
    // block clears the latter two again)
    cudaError_t e = cudaMemsetAsync(q.wf.counts + 2, 0, 3 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    trace<<<g, kTraceThreads, 0, s>>>(q, 0);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_trace_wavefront(const TraceParams& p, cudaStream_t s, uint32_t* hostCount, int* iterations,
                                   EventPairFn kernelEvents, void* user) {
    const int c = p.countVisits ? 1 : 0;
    const TraceKernel trace = trace_kernel(false, c, kTraceThreads, kTraversalStack);
    const int gTrace = grid_of((const void*)trace, kTraceThreads);
    // glossy reference shading has kernels of its own; the reference's shading keeps the lean ones
    typedef void (*WfKernel)(const TraceParams, int);
    const WfKernel shade = p.glossySeed ? k_wf_shade<false, true> : k_wf_shade<false, false>;
    const WfKernel tail = p.glossySeed ? k_wf_tail<false, true> : k_wf_tail<false, false>;
    const int gShade = grid_of((const void*)shade, 128);
    const int gTail = grid_of((const void*)tail, kTraceThreads);
    if (!gTrace || !gShade || !gTail) return cudaErrorUnknown;
    cudaError_t e = cudaMemsetAsync(p.wf.counts, 0, 4 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    // the first round generates the camera rays itself (no raygen queue)
    TraceParams p1 = p;
    p1.firstRound = 1;
    // the pending-ray count below which the remaining paths finish in one k_wf_tail launch; the
    // visit-counting build stays in the round loop (the tail kernel does not count visits)
    const uint32_t tailBelow = c ? 0u : (uint32_t)RG_TAIL_RAYS;
    int q = 0, it = 0;
    const int kChunk = RG_POLL_ROUNDS, kMaxIterations = 100000;
    for (;;) {
        for (int k = 0; k < kChunk; ++k, ++it) {
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (kernelEvents && !kernelEvents(user, &e0, &e1)) e0 = e1 = nullptr;
            if (e0) cudaEventRecord(e0, s);
            trace<<<gTrace, kTraceThreads, 0, s>>>(it == 0 ? p1 : p, q);
            if (e1) cudaEventRecord(e1, s);
            shade<<<gShade, 128, 0, s>>>(it == 0 ? p1 : p, q);
            count_launch(2);
            q ^= 1;
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(hostCount, p.wf.counts + q, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        if (*hostCount == 0) break;
        if (*hostCount < tailBelow) {
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (kernelEvents && !kernelEvents(user, &e0, &e1)) e0 = e1 = nullptr;
            if (e0) cudaEventRecord(e0, s);
            tail<<<gTail, kTraceThreads, 0, s>>>(p, q);
            if (e1) cudaEventRecord(e1, s);
            count_launch();
            break;
        }
        if (it >= kMaxIterations) return cudaErrorLaunchTimeout;
    }
    if (iterations) *iterations = it;
    dim3 grid((p.W + 31) / 32, (p.H + 7) / 8);
    k_resolve<<<grid, 256, 0, s>>>(p);
    count_launch();
    return cudaGetLastError();
}

// sort of queue q by the tune's key into p.perm (the scratch's valsA)
static cudaError_t enqueue_sort(const TraceParams& p, int key, const SortScratch& sc, int grid, int q, cudaStream_t s) {
    if (key == RG_SORT_OCTANT) {
        k_sort_count<true, RG_SORT_OCTANT><<<grid, 256, 0, s>>>(p, q, sc.keysA, sc.hist);
        k_sort_offsets<SortBuckets<RG_SORT_OCTANT>::n><<<1, 1024, 0, s>>>(sc.hist, sc.hist + 4096);
        k_sort_scatter<RG_SORT_OCTANT><<<grid, 256, 0, s>>>(p, q, sc.keysA, sc.hist + 4096, sc.valsA);
    } else {
        k_sort_count<true, RG_SORT_MORTON><<<grid, 256, 0, s>>>(p, q, sc.keysA, sc.hist);
        k_sort_offsets<SortBuckets<RG_SORT_MORTON>::n><<<1, 1024, 0, s>>>(sc.hist, sc.hist + 4096);
        k_sort_scatter<RG_SORT_MORTON><<<grid, 256, 0, s>>>(p, q, sc.keysA, sc.hist + 4096, sc.valsA);
    }
    count_launch(3);
    return cudaGetLastError();
}

cudaError_t launch_trace_batch(const TraceParams& p0, const TraceTune& tune, const SortScratch& sort, cudaStream_t s,
                               uint32_t* hostWords, int* iterations, EventPairFn kernelEvents, void* user) {
    TraceParams p = p0;
    const int c = p.countVisits ? 1 : 0;
    const int threads = c ? kTraceThreads : tune.threads;
    const TraceKernel trace = trace_kernel(true, c, threads, c ? kTraversalStack : tune.depth);
    if (!trace || !tune_supported(tune)) return cudaErrorInvalidValue;
    const int gTrace = grid_of((const void*)trace, threads);
    const int gShade = grid_of((const void*)k_wf_shade<true>, 128);
    const int gRaygen = grid_of((const void*)k_wfb_raygen, 256);
    const int gTail = grid_of((const void*)k_wf_tail<true>, kTraceThreads);
    const int gSort = grid_of((const void*)k_sort_scatter<RG_SORT_MORTON>, 256);
    if (!gTrace || !gShade || !gRaygen || !gTail || !gSort) return cudaErrorUnknown;
    const bool sorted = tune.sortKey != RG_SORT_NONE;
    p.perm = sorted ? sort.valsA : nullptr;
    cudaError_t e = cudaMemsetAsync(p.wf.counts, 0, 4 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    if (sorted && (e = cudaMemsetAsync(sort.hist, 0, 4096 * sizeof(uint32_t), s)) != cudaSuccess) return e;
    k_wfb_raygen<<<gRaygen, 256, 0, s>>>(p);
    count_launch();
    const uint32_t tailBelow = c ? 0u : (uint32_t)RG_TAIL_RAYS;
    int q = 0, it = 0;
    const int kChunk = RG_POLL_ROUNDS, kMaxIterations = 100000;
    for (;;) {
        for (int k = 0; k < kChunk; ++k, ++it) {
            if (sorted && (e = enqueue_sort(p, tune.sortKey, sort, gSort, q, s)) != cudaSuccess) return e;
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (kernelEvents && !kernelEvents(user, &e0, &e1)) e0 = e1 = nullptr;
            if (e0) cudaEventRecord(e0, s);
            trace<<<gTrace, threads, 0, s>>>(p, q);
            if (e1) cudaEventRecord(e1, s);
            k_wf_shade<true><<<gShade, 128, 0, s>>>(p, q);
            count_launch(2);
            q ^= 1;
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(hostWords, p.wf.counts + q, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(hostWords + 1, p.workCounter, sizeof(uint32_t), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        if (hostWords[0] == 0) break;  // nothing queued: every path finished and no work item is left
        if (hostWords[1] >= p.totalWork && hostWords[0] < tailBelow) {
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (kernelEvents && !kernelEvents(user, &e0, &e1)) e0 = e1 = nullptr;
            if (e0) cudaEventRecord(e0, s);
            k_wf_tail<true><<<gTail, kTraceThreads, 0, s>>>(p, q);
            if (e1) cudaEventRecord(e1, s);
            count_launch();
            break;
        }
        if (it >= kMaxIterations) return cudaErrorLaunchTimeout;
    }
    if (iterations) *iterations = it;
    return cudaGetLastError();
}

// loop condition of the graph form: continue while rays are queued and either many are queued or
// work items remain; stop (and flag) after maxIter body runs.  loop[0] = body runs, loop[1] = flag.
__global__ void k_batch_continue(cudaGraphConditionalHandle h, const uint32_t* __restrict__ counts, const uint32_t* __restrict__ work,
                                 uint32_t totalWork, uint32_t tailBelow, uint32_t maxIter, uint32_t* __restrict__ loop) {
    const uint32_t c = *(volatile const uint32_t*)counts, it = loop[0] + 1u;
    loop[0] = it;
    loop[2] += 1u;  // body runs since the words were allocated (launch accounting)
    bool more = c != 0u && (c >= tailBelow || *(volatile const uint32_t*)work < totalWork);
    if (more && it >= maxIter) {
        loop[1] = 1u;
        more = false;
    }
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

int batch_graph_kernels(const TraceTune& tune, int* perBody) {
    const int round = 2 + (tune.sortKey != RG_SORT_NONE ? 3 : 0);
    if (perBody) *perBody = 2 * round + 1;
    return 2;  // raygen + tail
}

cudaError_t capture_trace_batch(const TraceParams& p0, const TraceTune& tune, const SortScratch& sort, cudaStream_t s,
                                cudaStream_t s2, uint32_t* loopWords) {
    TraceParams p = p0;
    if (p.countVisits) return cudaErrorInvalidValue;  // the visit-counting build runs the host loop
    const TraceKernel trace = trace_kernel(true, false, tune.threads, tune.depth);
    if (!trace || !tune_supported(tune)) return cudaErrorInvalidValue;
    const int gTrace = grid_of((const void*)trace, tune.threads);
    const int gShade = grid_of((const void*)k_wf_shade<true>, 128);
    const int gRaygen = grid_of((const void*)k_wfb_raygen, 256);
    const int gTail = grid_of((const void*)k_wf_tail<true>, kTraceThreads);
    const int gSort = grid_of((const void*)k_sort_scatter<RG_SORT_MORTON>, 256);
    if (!gTrace || !gShade || !gRaygen || !gTail || !gSort) return cudaErrorUnknown;
    const bool sorted = tune.sortKey != RG_SORT_NONE;
    p.perm = sorted ? sort.valsA : nullptr;
    cudaError_t e;
    if ((e = cudaMemsetAsync(p.wf.counts, 0, 4 * sizeof(uint32_t), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(loopWords, 0, sizeof(uint32_t), s)) != cudaSuccess) return e;
    if (sorted && (e = cudaMemsetAsync(sort.hist, 0, 4096 * sizeof(uint32_t), s)) != cudaSuccess) return e;
    k_wfb_raygen<<<gRaygen, 256, 0, s>>>(p);
    // while node after the prologue; its body is captured on s2
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if ((e = cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd)) != cudaSuccess) return e;
    if (st != cudaStreamCaptureStatusActive) return cudaErrorStreamCaptureInvalidated;
    cudaGraphConditionalHandle h;
    if ((e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if ((e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp)) != cudaSuccess) return e;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(s2, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) != cudaSuccess) return e;
    for (int q = 0; q < 2; ++q) {
        if (sorted) enqueue_sort(p, tune.sortKey, sort, gSort, q, s2);
        trace<<<gTrace, tune.threads, 0, s2>>>(p, q);
        k_wf_shade<true><<<gShade, 128, 0, s2>>>(p, q);
    }
    // body runs before the loop stops with its limit flag set (RG_BATCH_LOOP_LIMIT overrides, read
    // when the graph is captured; tests use a small limit to check the reported error)
    uint32_t maxIter = 50000u;
    if (const char* env = getenv("RG_BATCH_LOOP_LIMIT")) maxIter = (uint32_t)strtoul(env, nullptr, 10);
    k_batch_continue<<<1, 1, 0, s2>>>(h, p.wf.counts, p.workCounter, p.totalWork, (uint32_t)RG_TAIL_RAYS, maxIter, loopWords);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(s2, &captured);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) != cudaSuccess) return e;
    // after an even number of rounds the pending rays are in queue 0
    k_wf_tail<true><<<gTail, kTraceThreads, 0, s>>>(p, 0);
    return cudaGetLastError();
}

cudaError_t launch_resolve_job(const float4* samples, const JobDesc& j, uint2* base, uint2* normal, uint2* rough, cudaStream_t s) {
    dim3 grid((j.W + 31) / 32, (j.H + 7) / 8);
    k_resolve_job<<<grid, 256, 0, s>>>(samples + 3 * (size_t)j.sampleBase, j.W, j.H, j.S, base, normal, rough);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const DevScene& sc, const float* rays, uint32_t n, float* tuv, uint32_t* ids,
                              unsigned long long* counters, int depth, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t g = (n + kTraceThreads - 1) / kTraceThreads;
    switch (depth) {
        case 16: k_trace_rays<16><<<g, kTraceThreads, 0, s>>>(sc, rays, n, tuv, ids, counters); break;
        case 24: k_trace_rays<24><<<g, kTraceThreads, 0, s>>>(sc, rays, n, tuv, ids, counters); break;
        case 32: k_trace_rays<32><<<g, kTraceThreads, 0, s>>>(sc, rays, n, tuv, ids, counters); break;
        case 48: k_trace_rays<48><<<g, kTraceThreads, 0, s>>>(sc, rays, n, tuv, ids, counters); break;
        default: return cudaErrorInvalidValue;
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace rg
