// trace.cu -- per-pixel ray generation, two-level BVH traversal and closest-hit / miss shading.
//
// Replaces traceRaysKHR with the raygen / closest-hit / miss / shadow-miss programs
// (render/raytracer.cpp:99-100; resources/shaders/raygen.h:69-115, raygen.rgen:30-39,
// closesthit.rchit:74-268, miss.rmiss:38-83, shadowMiss.rmiss:30-34).
//
// GB300 has no RT cores, so traversal is software: a BVH2 whose nodes carry both children's
// boxes (one 64-byte node = four 16-byte loads tests two children), near-child-first stack
// traversal, TLAS leaves switch to the instance's BLAS with the ray moved into object space, and a
// watertight ray/triangle test (Woop, Benthin, Wald 2013).  Closest-hit ties (equal t) resolve to
// the smaller (instance, primitive).
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
#include "rg_internal.cuh"

namespace rg {
namespace {

// ---------------------------------------------------------------------------------------------
// ray set-up and primitive tests
struct Ray {
    float ox, oy, oz, dx, dy, dz, ix, iy, iz;  // origin, direction, 1/direction
    float Sx, Sy, Sz;
    int kx, ky, kz;
};

__device__ __forceinline__ float comp(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ void ray_pre(Ray& r, float ox, float oy, float oz, float dx, float dy, float dz) {
    r.ox = ox; r.oy = oy; r.oz = oz;
    r.dx = dx; r.dy = dy; r.dz = dz;
    r.ix = 1.0f / dx; r.iy = 1.0f / dy; r.iz = 1.0f / dz;
    float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    float dkz = comp(dx, dy, dz, kz);
    if (dkz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = comp(dx, dy, dz, kx) / dkz;
    r.Sy = comp(dx, dy, dz, ky) / dkz;
    r.Sz = 1.0f / dkz;
}

constexpr float kInflate = 1.0000004f;  // 1 + 2*gamma_3 (Ize 2013) rounded up

// slab test of one box against [tmin, tbest]; returns entry distance or +inf
__device__ __forceinline__ float slab(const Ray& r, float lx, float hx, float ly, float hy, float lz, float hz, float tmin, float tbest) {
    float t0x = (lx - r.ox) * r.ix, t1x = (hx - r.ox) * r.ix;
    float t0y = (ly - r.oy) * r.iy, t1y = (hy - r.oy) * r.iy;
    float t0z = (lz - r.oz) * r.iz, t1z = (hz - r.oz) * r.iz;
    float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tbest));
    return tn <= tf * kInflate ? tn : INFINITY;
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
    float A0 = a.x - r.ox, A1 = a.y - r.oy, A2 = a.z - r.oz;
    float B0 = b.x - r.ox, B1 = b.y - r.oy, B2 = b.z - r.oz;
    float C0 = c.x - r.ox, C1 = c.y - r.oy, C2 = c.z - r.oz;
    float Akz = comp(A0, A1, A2, r.kz), Bkz = comp(B0, B1, B2, r.kz), Ckz = comp(C0, C1, C2, r.kz);
    float Ax = comp(A0, A1, A2, r.kx) - r.Sx * Akz, Ay = comp(A0, A1, A2, r.ky) - r.Sy * Akz;
    float Bx = comp(B0, B1, B2, r.kx) - r.Sx * Bkz, By = comp(B0, B1, B2, r.ky) - r.Sy * Bkz;
    float Cx = comp(C0, C1, C2, r.kx) - r.Sx * Ckz, Cy = comp(C0, C1, C2, r.ky) - r.Sy * Ckz;
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

template <bool COUNT>
__device__ Hit closest_hit(const DevScene& sc, float ox, float oy, float oz, float dx, float dy, float dz, float tmin, float tmax,
                           VisitCounts& vc) {
    Hit h;
    h.hit = false;
    h.t = tmax;
    h.u = h.v = 0.0f;
    h.inst = h.prim = 0xFFFFFFFFu;
    if ((dx == 0.0f && dy == 0.0f && dz == 0.0f) || sc.tlasN == 0) return h;
    Ray wr;
    ray_pre(wr, ox, oy, oz, dx, dy, dz);
    if (sc.tlasN > 1 && slab(wr, sc.tlasRoot[0], sc.tlasRoot[3], sc.tlasRoot[1], sc.tlasRoot[4], sc.tlasRoot[2], sc.tlasRoot[5], tmin, h.t) == INFINITY)
        return h;
    uint32_t stack[kTraversalStack];
    int sp = 0;
    Ray r = wr;
    const BvhNode* nodes = sc.tlasNodes;
    const float4* tris = nullptr;
    bool inBlas = false;
    uint32_t inst = 0;
    uint32_t ref = sc.tlasN == 1 ? kLeaf : 0u;
    for (;;) {
        if (!(ref & kLeaf)) {
            if (COUNT) vc.nodes++;
            const BvhNode* nd = nodes + ref;
            float4 a = __ldg(&nd->a), b = __ldg(&nd->b), c = __ldg(&nd->c);
            uint4 d = __ldg(&nd->d);
            float tl = slab(r, a.x, a.y, a.z, a.w, b.x, b.y, tmin, h.t);
            float tr = slab(r, b.z, b.w, c.x, c.y, c.z, c.w, tmin, h.t);
            bool hl = tl != INFINITY, hr = tr != INFINITY;
            if (hl && hr) {
                bool rFirst = tr < tl;
                uint32_t nearR = rFirst ? d.y : d.x, farR = rFirst ? d.x : d.y;
                if (sp < kTraversalStack) stack[sp++] = farR;
                else if (COUNT || true) vc.overflow++;
                ref = nearR;
                continue;
            }
            if (hl) { ref = d.x; continue; }
            if (hr) { ref = d.y; continue; }
        } else if (inBlas) {
            if (COUNT) vc.tris++;
            const float4* tp = tris + 3 * (size_t)(ref & ~kLeaf);
            tri_test(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), tmin, inst, h);
        } else {
            uint32_t ii = __ldg(sc.tlasOrder + (ref & ~kLeaf));
            const DevInstance* in = sc.inst + ii;
            if (__ldg(&in->valid)) {
                float4 i0 = __ldg(&in->inv[0]), i1 = __ldg(&in->inv[1]), i2 = __ldg(&in->inv[2]);
                float qx = ((i0.x * ox + i0.y * oy) + i0.z * oz) + i0.w;
                float qy = ((i1.x * ox + i1.y * oy) + i1.z * oz) + i1.w;
                float qz = ((i2.x * ox + i2.y * oy) + i2.z * oz) + i2.w;
                float ex = (i0.x * dx + i0.y * dy) + i0.z * dz;
                float ey = (i1.x * dx + i1.y * dy) + i1.z * dz;
                float ez = (i2.x * dx + i2.y * dy) + i2.z * dz;
                if (!(ex == 0.0f && ey == 0.0f && ez == 0.0f)) {
                    const DevBlas* bl = sc.blas + __ldg(&in->blas);
                    uint32_t bn = __ldg(&bl->n);
                    Ray orr;
                    ray_pre(orr, qx, qy, qz, ex, ey, ez);
                    const float* rb = bl->root;
                    if (bn > 0 && slab(orr, __ldg(rb + 0), __ldg(rb + 3), __ldg(rb + 1), __ldg(rb + 4), __ldg(rb + 2), __ldg(rb + 5), tmin, h.t) != INFINITY) {
                        if (sp < kTraversalStack) {
                            stack[sp++] = kMarker;
                            r = orr;
                            nodes = bl->nodes;
                            tris = bl->tris;
                            inst = ii;
                            inBlas = true;
                            ref = bn == 1 ? kLeaf : 0u;
                            continue;
                        }
                        vc.overflow++;
                    }
                }
            }
        }
        // pop
        for (;;) {
            if (sp == 0) return h;
            ref = stack[--sp];
            if (ref != kMarker) break;
            inBlas = false;
            r = wr;
            nodes = sc.tlasNodes;
        }
    }
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

struct Frame {
    int kind, front, rayConsumption, pad;
    V3 origin, D, n;
    float t;
    V3 diffuse, specular;
    float transparency, reflectivity, roughness, ior, emission;
    V3 base;          // GENERIC: baseColor; SHADOW_INTERNAL: shadowCol
    V3 shadow;        // GENERIC: shadowColor
    V3 reflectColor;  // GENERIC
    float reflectDepth;
};

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

template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace(const TraceParams P) {
    const uint32_t px = blockIdx.x * 16 + (threadIdx.x & 15);
    const uint32_t py = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (px >= P.W || py >= P.H) return;
    const DevScene& sc = P.scene;
    const rg_ubo& U = P.ubo;
    const V3 L = v3(U.lightDir[0], U.lightDir[1], U.lightDir[2]);
    const int maxRec = U.maxRecursions;
    const int S = U.numSamples;
    const int aaRow = S < 8 ? S : 8;

    unsigned long long nPrimary = 0, nShadow = 0, nSecondary = 0, nMasked = 0;
    VisitCounts vc = {0, 0, 0};

    float org[4];
    mul4(U.viewInverse, 0.0f, 0.0f, 0.0f, 1.0f, org);
    const V3 camO = v3(org[0], org[1], org[2]);

    V3 accColor = v3s(0.0f), accNormal = v3s(0.0f), accRough = v3s(0.0f);
    float accRoughA = 0.0f, accReflect = 0.0f, accDepth = 0.0f;

    Frame stack[kMaxFrames];
    int fsp = 0;
    Payload p;
    RayReq ray;
    Frame cur;

    for (int sample = 0; sample < S; ++sample) {
        // raygen.h:84-102 -- camera ray of this sample, payload initialisation
        {
            float pcx = ((float)px + 0.5f) + kAA[aaRow][sample & 7][0];
            float pcy = ((float)py + 0.5f) + kAA[aaRow][sample & 7][1];
            float ux = pcx / (float)P.W, uy = pcy / (float)P.H;
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
            nPrimary++;
        }
        for (;;) {
            // ---- traceRayEXT ----
            Hit h;
            h.hit = false;
            if (!ray.masked) h = closest_hit<COUNT>(sc, ray.o.x, ray.o.y, ray.o.z, ray.d.x, ray.d.y, ray.d.z, ray.tmin, ray.tmax, vc);
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
                            nShadow++;
                            cur.base = shadowCol;
                            cur.kind = R_SI_A;
                            stack[fsp++] = cur;
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
                                nShadow++;
                                cur.kind = R_ST_C;
                                stack[fsp++] = cur;
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
                                nShadow++;
                                cur.kind = R_G_SHADOW;
                                stack[fsp++] = cur;
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
                        p.recDepth += cur.rayConsumption;
                        p.refDepth = p.refDepth + cur.t;
                        nSecondary++;
                        cur.kind = R_G_REFLECT;
                        stack[fsp++] = cur;
                        ray.o = cur.origin; ray.d = dir; ray.tmin = 0.01f; ray.tmax = 1000.0f; ray.missIndex = 0; ray.masked = false;
                        newRay = true;
                    } else {
                        ph = PH_G_REFRACT;
                    }
                } else if (ph == PH_G_REFRACT) {  // :223-251
                    if (p.recDepth < maxRec && cur.transparency > 0.0f) {
                        V3 dir;
                        if (cur.front) {
                            float eta = p.curIOR / cur.ior;
                            dir = refract(cur.D, cur.n, eta);
                            p.curIOR = cur.ior;
                            cur.kind = R_G_REFR_F;
                        } else {
                            float eta = cur.ior / 1.0f;
                            dir = refract(cur.D, cur.n, eta);
                            p.curIOR = 1.0f;
                            cur.kind = R_G_REFR_B;
                        }
                        p.recDepth++;
                        nSecondary++;
                        stack[fsp++] = cur;
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
                    cur = stack[--fsp];
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
                                stack[fsp++] = cur;
                                nMasked++;
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
            if (!newRay) break;  // sample finished
        }
        accColor = accColor + p.hitValue;
        accNormal = accNormal + p.normal;
        accRough = accRough + p.roughRGB;
        accRoughA = accRoughA + p.roughA;
        accReflect = accReflect + p.reflectContribution;
        accDepth = accDepth + p.depth;
    }
    const float fs = (float)S;
    const size_t pix = (size_t)py * P.W + px;
    P.base[pix] = pack_half4(accColor.x / fs, accColor.y / fs, accColor.z / fs, accReflect / fs);
    P.normal[pix] = pack_half4(accNormal.x / fs, accNormal.y / fs, accNormal.z / fs, (logf(accDepth) * 0.25f) / fs);
    P.rough[pix] = pack_half4(accRough.x / fs, accRough.y / fs, accRough.z / fs, accRoughA / fs);

    // ray statistics: warp reduction then one atomic per warp
    unsigned long long c[7] = {nPrimary, nShadow, nSecondary, nMasked, vc.nodes, vc.tris, vc.overflow};
    const unsigned mask = __activemask();
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        unsigned long long v = c[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off);
        c[k] = v;
    }
    // with a partial warp the xor-reduction is incomplete; fall back to per-thread atomics then
    if (mask == 0xFFFFFFFFu) {
        if ((threadIdx.x & 31) == 0)
            for (int k = 0; k < 7; ++k)
                if (c[k]) {
                    atomicAdd(P.counters + k, c[k]);
                    atomicAdd(P.counters + 8 + k, c[k]);
                }
    } else {
        unsigned long long own[7] = {nPrimary, nShadow, nSecondary, nMasked, vc.nodes, vc.tris, vc.overflow};
        for (int k = 0; k < 7; ++k)
            if (own[k]) {
                atomicAdd(P.counters + k, own[k]);
                atomicAdd(P.counters + 8 + k, own[k]);
            }
    }
}

__global__ void k_trace_rays(const DevScene sc, const float* __restrict__ rays, uint32_t n, float* __restrict__ tuv, uint32_t* __restrict__ ids) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float* r = rays + 8 * (size_t)k;
    VisitCounts vc = {0, 0, 0};
    Hit h = closest_hit<false>(sc, r[0], r[1], r[2], r[4], r[5], r[6], r[3], r[7], vc);
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
    dim3 grid((p.W + 15) / 16, (p.H + 7) / 8);
    if (p.countVisits) k_trace<true><<<grid, 128, 0, s>>>(p);
    else k_trace<false><<<grid, 128, 0, s>>>(p);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const DevScene& sc, const float* rays, uint32_t n, float* tuv, uint32_t* ids, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_trace_rays<<<(n + 127) / 128, 128, 0, s>>>(sc, rays, n, tuv, ids);
    count_launch();
    return cudaGetLastError();
}

}  // namespace rg
