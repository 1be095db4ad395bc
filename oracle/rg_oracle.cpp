// rg_oracle.cpp -- CPU oracle for the Raygun ray-tracing path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the smoke check and the
// CPU-baseline leg of the benchmark call it; nothing in the product links or calls it.
//
// Pinned to the reference: the reference's own shader sources, compiled as C++ through a GLSL shim
// (oracle/ref, built from the reference tree), produce the golden fixtures of tests/golden, and this
// restatement reproduces them bit for bit (G-buffers, debug images, final frame, ray counts).  The
// BVH, traversal and triangle test are the Vulkan driver's in the reference and have no reference
// counterpart; both checkers share them from this file.
//
// It is a scalar C++ restatement of the reference's per-frame path:
//   * LBVH over triangle / instance boxes (30-bit Morton, stable sort, Karras 2012 hierarchy,
//     bottom-up boxes), and the binned-SAH BVH2 the CUDA library builds by default.  The reference
//     leaves BVHs to the Vulkan driver (render/acceleration_structure.cpp:55-194), so this part has
//     no reference counterpart.
//   * watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013) with closest-hit ties broken
//     by the smaller (instance, primitive) pair.
//   * raygen / closest-hit / miss / shadow-miss (resources/shaders/raygen.h:69-115,
//     raygen.rgen:30-39, closesthit.rchit:74-268, miss.rmiss:38-83, shadowMiss.rmiss:30-34)
//     evaluated depth-first on ONE payload that every nested trace mutates (payload.h:29-43),
//     so stale fields leak exactly as they do on the GPU.
//   * rough_prepare.comp:28-54, rough_blur.h:23-40 (x10 H/V, raytracer.cpp:116-121),
//     postprocess.comp:28-50 and FXAA 3.11 PC quality preset 39 (fxaa.comp:29-36,
//     fxaa.h:615-1136) with every imageStore rounded to the image's storage format.
//
// Policies for GLSL-undefined cases (the product implements the same ones):
//   P1 r/(tr+r) with tr+r == 0 -> weight 0            (closesthit.rchit:257)
//   P2 pow(x, n) for integer n -> repeated multiply   (closesthit.rchit:81-82,142,202)
//   P3 a zero ray direction (refract TIR) -> no traversal, miss shader of that trace
//   P4 imageLoad out of bounds -> vec4(0); FXAA samples clamp to edge
//   P5 roughTransitions (R8_SNORM) stores rint(clamp(t,-1,1)*127)/127
//   P6 RGBA16F stores round to nearest even
//   P7 equal t -> smaller (instance, primitive)
//   P8 clamp/min/max follow fminf/fmaxf (a NaN operand yields the other operand)
//   P9 FXAA taps: a coordinate equal to a texel centre ((i+0.5)/W in FP32) samples that texel,
//      others are FP32 bilinear x = u*W - 0.5, weights (1-f, f); clamp to edge
//
// Built with -ffp-contract=off: every + - * / is a separately rounded IEEE operation, sqrt and /
// are correctly rounded, so ray geometry is reproducible bit for bit.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ------------------------------------------------------------------------------------------------
// layouts (resources/shaders/*.def)
struct Vertex {  // vertex.def:3-7
    float position[3];
    uint32_t matIndex;
    float normal[3];
    float pad1;
};
struct Material {  // gpu_material.def:11-26
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
};
struct Ubo {  // uniform_buffer_object.def:3-17 (std140)
    float viewInverse[16];  // column-major
    float projInverse[16];
    float clearColor[3];
    int32_t numSamples;
    float lightDir[3];
    int32_t maxRecursions;
    float time;
    uint32_t showAlpha;
    float pad0, pad1;
    float fadeColor[4];
};
struct Instance {
    float transform[12];  // 3x4 row-major (acceleration_structure.cpp:43-45)
    uint32_t blas;
    uint32_t mask;
    uint32_t vertexBufferOffset, indexBufferOffset, materialBufferOffset;  // instance_offset_table.def
    uint32_t pad;
};
static_assert(sizeof(Vertex) == 32 && sizeof(Material) == 64 && sizeof(Ubo) == 192 && sizeof(Instance) == 72, "layout");

// ------------------------------------------------------------------------------------------------
// small vector type, templated on the scalar (float for parity and timing, double for error
// accounting)
template <class T>
struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit V3(T s) : x(s), y(s), z(s) {}
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> T dot(V3<T> a, V3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> T fmin_(T a, T b) { return std::fmin(a, b); }
template <class T> T fmax_(T a, T b) { return std::fmax(a, b); }
template <class T> T clampT(T x, T lo, T hi) { return fmin_(fmax_(x, lo), hi); }  // P8
template <class T> V3<T> normalize(V3<T> v) {
    T l = std::sqrt(dot(v, v));
    return {v.x / l, v.y / l, v.z / l};
}
template <class T> T mixs(T x, T y, T a) { return x * (T(1) - a) + y * a; }  // GLSL mix definition
template <class T> V3<T> mix(V3<T> x, V3<T> y, T a) { return {mixs(x.x, y.x, a), mixs(x.y, y.y, a), mixs(x.z, y.z, a)}; }
template <class T> V3<T> mix(V3<T> x, V3<T> y, V3<T> a) { return {mixs(x.x, y.x, a.x), mixs(x.y, y.y, a.y), mixs(x.z, y.z, a.z)}; }
template <class T> V3<T> reflect(V3<T> I, V3<T> N) {  // GLSL: I - 2*dot(N,I)*N
    T d = dot(N, I);
    T k = T(2) * d;
    return I - N * k;
}
template <class T> V3<T> refract(V3<T> I, V3<T> N, T eta) {  // GLSL refract definition
    T d = dot(N, I);
    T k = T(1) - eta * eta * (T(1) - d * d);
    if (k < T(0)) return V3<T>(T(0));
    T s = eta * d + std::sqrt(k);
    return I * eta - N * s;
}
template <class T> T glsl_mod(T x, T y) { return x - y * std::floor(x / y); }
template <class T> T len(V3<T> v) { return std::sqrt(dot(v, v)); }

template <class T> V3<T> cvt(const float* p) { return {T(p[0]), T(p[1]), T(p[2])}; }

// ------------------------------------------------------------------------------------------------
// half precision round trip (P6)
static inline uint16_t f2h(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7FFFFFFFu;
    if (ax >= 0x7F800000u) return (uint16_t)(sign | 0x7C00u | (ax > 0x7F800000u ? 0x200u : 0u));
    if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // rounds to inf
    if (ax < 0x38800000u) {                                   // subnormal half or zero
        if (ax < 0x33000000u) return (uint16_t)sign;
        uint32_t e = ax >> 23;
        uint32_t m = (ax & 0x7FFFFFu) | 0x800000u;
        uint32_t shift = 126 - e;  // 14 + (113 - e) ... result = m >> (shift) with rounding
        uint32_t r = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1u);
        uint32_t half = 1u << (shift - 1);
        if (rem > half || (rem == half && (r & 1u))) r++;
        return (uint16_t)(sign | r);
    }
    uint32_t r = (ax >> 13) - (112u << 10);
    uint32_t rem = ax & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;
    return (uint16_t)(sign | r);
}
static inline float h2f(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
    uint32_t x;
    if (e == 0) {
        if (m == 0) x = sign;
        else {
            float f = std::ldexp((float)m, -24);
            std::memcpy(&x, &f, 4);
            x |= sign;
        }
    } else if (e == 31) x = sign | 0x7F800000u | (m << 13);
    else x = sign | ((e + 112u) << 23) | (m << 13);
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}
static inline float rh(float f) { return h2f(f2h(f)); }

// ------------------------------------------------------------------------------------------------
// LBVH (Morton30 -> stable sort -> Karras hierarchy -> bottom-up boxes)
static inline uint32_t expand10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
static inline uint32_t quant10(float c, float lo, float inv) {
    float d = c - lo;
    float q = d * inv;
    float s = q * 1024.0f;
    s = std::fmin(std::fmax(s, 0.0f), 1023.0f);
    return (uint32_t)s;
}

struct Box {
    float lo[3], hi[3];
};

struct Lbvh {
    uint32_t n = 0;
    std::vector<uint32_t> morton;     // per primitive (input order)
    std::vector<uint32_t> order;      // sorted position -> primitive
    std::vector<uint32_t> left, right;  // n-1 internal nodes; bit31 = leaf (sorted position)
    std::vector<uint32_t> parent;     // internal parents (n-1), leaf parents (n) appended
    std::vector<Box> nodeBox;         // n-1 internal boxes
    std::vector<Box> leafBox;         // sorted position -> box
    uint32_t rootRef() const { return n == 1 ? 0x80000000u : 0u; }
};

static inline int delta(const std::vector<uint32_t>& keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = keys[i], b = keys[j];
    if (a == b) return 32 + __builtin_clz((uint32_t)i ^ (uint32_t)j);
    return __builtin_clz(a ^ b);
}

static void lbvh_refit(Lbvh& b) {
    const uint32_t n = b.n;
    if (n <= 1) return;
    // internal node indices are not topologically ordered; evaluate recursively with a stack
    std::vector<uint32_t> post;
    post.reserve(n);
    std::vector<uint32_t> st{0};
    while (!st.empty()) {
        uint32_t i = st.back();
        st.pop_back();
        post.push_back(i);
        if (!(b.left[i] & 0x80000000u)) st.push_back(b.left[i]);
        if (!(b.right[i] & 0x80000000u)) st.push_back(b.right[i]);
    }
    for (size_t k = post.size(); k-- > 0;) {
        uint32_t i = post[k];
        const Box& L = (b.left[i] & 0x80000000u) ? b.leafBox[b.left[i] & 0x7FFFFFFFu] : b.nodeBox[b.left[i]];
        const Box& R = (b.right[i] & 0x80000000u) ? b.leafBox[b.right[i] & 0x7FFFFFFFu] : b.nodeBox[b.right[i]];
        Box& o = b.nodeBox[i];
        for (int a = 0; a < 3; ++a) {
            o.lo[a] = std::fmin(L.lo[a], R.lo[a]);
            o.hi[a] = std::fmax(L.hi[a], R.hi[a]);
        }
    }
}

static void lbvh_build(Lbvh& b, const std::vector<Box>& prim) {
    const uint32_t n = (uint32_t)prim.size();
    b.n = n;
    b.morton.assign(n, 0);
    b.order.resize(n);
    if (n == 0) return;
    // centroid bounds
    float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    std::vector<float> cen(3 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            float c = (prim[i].lo[a] + prim[i].hi[a]) * 0.5f;
            cen[3 * (size_t)i + a] = c;
            cmin[a] = std::fmin(cmin[a], c);
            cmax[a] = std::fmax(cmax[a], c);
        }
    // every axis is scaled by the LARGEST centroid extent (a cube), so a thin axis spends few of its
    // 10 bits and the hierarchy splits mostly along the long axes
    float inv[3];
    float emax = 0.0f;
    for (int a = 0; a < 3; ++a) emax = std::fmax(emax, cmax[a] - cmin[a]);
    for (int a = 0; a < 3; ++a) inv[a] = emax > 0.0f ? 1.0f / emax : 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t x = quant10(cen[3 * (size_t)i + 0], cmin[0], inv[0]);
        uint32_t y = quant10(cen[3 * (size_t)i + 1], cmin[1], inv[1]);
        uint32_t z = quant10(cen[3 * (size_t)i + 2], cmin[2], inv[2]);
        b.morton[i] = (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
    }
    for (uint32_t i = 0; i < n; ++i) b.order[i] = i;
    std::stable_sort(b.order.begin(), b.order.end(), [&](uint32_t p, uint32_t q) { return b.morton[p] < b.morton[q]; });
    std::vector<uint32_t> keys(n);
    for (uint32_t i = 0; i < n; ++i) keys[i] = b.morton[b.order[i]];
    b.leafBox.resize(n);
    for (uint32_t i = 0; i < n; ++i) b.leafBox[i] = prim[b.order[i]];
    b.left.assign(n > 1 ? n - 1 : 0, 0);
    b.right.assign(n > 1 ? n - 1 : 0, 0);
    b.nodeBox.assign(n > 1 ? n - 1 : 0, Box{});
    b.parent.assign(2 * (size_t)n, 0xFFFFFFFFu);
    const int N = (int)n;
    for (int i = 0; i + 1 < N; ++i) {
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
        int gamma = i + s * d + std::min(d, 0);
        int lo = std::min(i, j), hi = std::max(i, j);
        b.left[i] = (lo == gamma) ? (0x80000000u | (uint32_t)gamma) : (uint32_t)gamma;
        b.right[i] = (hi == gamma + 1) ? (0x80000000u | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    }
    for (uint32_t i = 0; i + 1 < n; ++i) {
        for (uint32_t c : {b.left[i], b.right[i]}) {
            if (c & 0x80000000u) b.parent[(n - 1) + (c & 0x7FFFFFFFu)] = i;
            else b.parent[c] = i;
        }
    }
    lbvh_refit(b);
}

// Binned-SAH BVH2 (the default BLAS and TLAS builder of the CUDA library), in the LBVH's layout.  Top
// down, level by level: a node's range of the order array gets its box and centroid box; centroids
// fall into 16 bins per axis (bin = trunc((c - clo) * 16 / ext), clamped); the 45 splits between
// bins are scored by half-area(left) * count(left) + half-area(right) * count(right) and the
// cheapest wins, ties to the lowest (axis, split); the range is partitioned stably; a range with no
// usable split (coincident centroids, or every cost infinite) is halved.  Children of one primitive
// are leaf refs.  Internal nodes are numbered in level order, tasks of a level in order (the GPU
// numbers a level's nodes in the order its warps emit them, so trees compare up to that numbering).
// From level medianLevel on (root = level 0) every range is halved without binning, so no tree is
// deeper than medianLevel + ceil(log2 n) levels however the centroids are spread.  Returns the
// number of levels.
static float half_area3(const float* lo, const float* hi) {
    const float dx = std::fmax(hi[0] - lo[0], 0.0f), dy = std::fmax(hi[1] - lo[1], 0.0f), dz = std::fmax(hi[2] - lo[2], 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

static uint32_t sah_build(Lbvh& l, const std::vector<Box>& prim, uint32_t medianLevel) {
    const int kBins = 16;
    const uint32_t n = (uint32_t)prim.size();
    l.n = n;
    l.order.resize(n);
    for (uint32_t i = 0; i < n; ++i) l.order[i] = i;
    l.left.assign(n > 1 ? n - 1 : 0, 0u);
    l.right.assign(n > 1 ? n - 1 : 0, 0u);
    l.nodeBox.assign(n > 1 ? n - 1 : 0, Box{});
    l.leafBox.resize(n);
    if (n <= 1) {
        for (uint32_t i = 0; i < n; ++i) l.leafBox[i] = prim[i];
        return 0;
    }
    std::vector<std::pair<uint32_t, uint32_t>> cur{{0u, n}}, nxt;
    std::vector<uint32_t> tmp(n);
    uint32_t baseCur = 0, baseNext = 1, levels = 0;
    while (!cur.empty()) {
        const bool median = levels >= medianLevel;
        nxt.clear();
        for (uint32_t t = 0; t < cur.size(); ++t) {
            const uint32_t b = cur[t].first, e = cur[t].second, node = baseCur + t;
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (uint32_t i = b; i < e; ++i) {
                const Box& x = prim[l.order[i]];
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::fmin(lo[a], x.lo[a]);
                    hi[a] = std::fmax(hi[a], x.hi[a]);
                    const float c = 0.5f * (x.lo[a] + x.hi[a]);
                    clo[a] = std::fmin(clo[a], c);
                    chi[a] = std::fmax(chi[a], c);
                }
            }
            for (int a = 0; a < 3; ++a) {
                l.nodeBox[node].lo[a] = lo[a];
                l.nodeBox[node].hi[a] = hi[a];
            }
            float scale[3];
            for (int a = 0; a < 3; ++a) {
                const float ext = chi[a] - clo[a];
                scale[a] = ext > 0.0f ? (float)kBins / ext : 0.0f;
            }
            auto bin_of = [&](const Box& x, int a) {
                const float c = 0.5f * (x.lo[a] + x.hi[a]);
                return std::max(0, std::min((int)((c - clo[a]) * scale[a]), kBins - 1));
            };
            int cnt[3][kBins] = {};
            float blo[3][kBins][3], bhi[3][kBins][3];
            for (int a = 0; a < 3; ++a)
                for (int k = 0; k < kBins; ++k)
                    for (int c = 0; c < 3; ++c) {
                        blo[a][k][c] = INFINITY;
                        bhi[a][k][c] = -INFINITY;
                    }
            for (uint32_t i = b; i < e; ++i) {
                const Box& x = prim[l.order[i]];
                for (int a = 0; a < 3; ++a) {
                    if (scale[a] <= 0.0f) continue;
                    const int k = bin_of(x, a);
                    cnt[a][k]++;
                    for (int c = 0; c < 3; ++c) {
                        blo[a][k][c] = std::fmin(blo[a][k][c], x.lo[c]);
                        bhi[a][k][c] = std::fmax(bhi[a][k][c], x.hi[c]);
                    }
                }
            }
            float bestCost = INFINITY;
            int bestCand = -1;
            for (int cand = 0; !median && cand < 3 * (kBins - 1); ++cand) {
                const int a = cand / (kBins - 1), sp = cand % (kBins - 1) + 1;
                if (scale[a] <= 0.0f) continue;
                float L0[3] = {INFINITY, INFINITY, INFINITY}, L1[3] = {-INFINITY, -INFINITY, -INFINITY};
                float R0[3] = {INFINITY, INFINITY, INFINITY}, R1[3] = {-INFINITY, -INFINITY, -INFINITY};
                int nl = 0, nr = 0;
                for (int k = 0; k < kBins; ++k) {
                    if (!cnt[a][k]) continue;
                    float* X0 = k < sp ? L0 : R0;
                    float* X1 = k < sp ? L1 : R1;
                    for (int c = 0; c < 3; ++c) {
                        X0[c] = std::fmin(X0[c], blo[a][k][c]);
                        X1[c] = std::fmax(X1[c], bhi[a][k][c]);
                    }
                    if (k < sp) nl += cnt[a][k];
                    else nr += cnt[a][k];
                }
                if (!nl || !nr) continue;
                const float cost = half_area3(L0, L1) * (float)nl + half_area3(R0, R1) * (float)nr;
                if (cost < bestCost) {
                    bestCost = cost;
                    bestCand = cand;
                }
            }
            uint32_t mid = b + (e - b) / 2;
            if (bestCand >= 0) {
                const int a = bestCand / (kBins - 1), sp = bestCand % (kBins - 1) + 1;
                uint32_t nl = 0;
                for (uint32_t i = b; i < e; ++i) nl += bin_of(prim[l.order[i]], a) < sp ? 1u : 0u;
                uint32_t lb = 0, rb = 0;
                for (uint32_t i = b; i < e; ++i) {
                    const uint32_t p = l.order[i];
                    if (bin_of(prim[p], a) < sp) tmp[b + lb++] = p;
                    else tmp[b + nl + rb++] = p;
                }
                for (uint32_t i = b; i < e; ++i) l.order[i] = tmp[i];
                mid = b + nl;
            }
            const uint32_t rb0[2] = {b, mid}, re0[2] = {mid, e};
            uint32_t ref[2];
            for (int c = 0; c < 2; ++c) {
                if (re0[c] - rb0[c] == 1) {
                    ref[c] = 0x80000000u | rb0[c];
                } else {
                    ref[c] = baseNext + (uint32_t)nxt.size();
                    nxt.push_back({rb0[c], re0[c]});
                }
            }
            l.left[node] = ref[0];
            l.right[node] = ref[1];
        }
        baseCur = baseNext;
        baseNext += (uint32_t)nxt.size();
        cur.swap(nxt);
        ++levels;
    }
    for (uint32_t k = 0; k < n; ++k) l.leafBox[k] = prim[l.order[k]];
    return levels;
}

// ------------------------------------------------------------------------------------------------
// scene
struct Blas {
    uint32_t vertexOffset, indexOffset, triCount;
    Lbvh bvh;
    std::vector<float> tri;  // sorted position -> 9 floats (v0, v1, v2 positions)
    Box root;
};

struct Inst {
    float m[12];     // object -> world
    float inv[12];   // world -> object
    uint32_t blas;
    uint32_t vOff, iOff, mOff;
    bool valid;
};

struct Scene {
    std::vector<Vertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<Material> materials;
    std::vector<Blas> blas;
    std::vector<Inst> inst;
    Lbvh tlas;
};

static void tri_box(const Scene& s, const Blas& b, uint32_t p, Box& out, float* v9) {
    for (int k = 0; k < 3; ++k) {
        uint32_t vi = b.vertexOffset + s.indices[b.indexOffset + 3 * p + k];
        const float* pos = s.vertices[vi].position;
        for (int a = 0; a < 3; ++a) {
            v9[3 * k + a] = pos[a];
            if (k == 0) out.lo[a] = out.hi[a] = pos[a];
            else {
                out.lo[a] = std::fmin(out.lo[a], pos[a]);
                out.hi[a] = std::fmax(out.hi[a], pos[a]);
            }
        }
    }
}

static void build_blas(const Scene& s, Blas& b, bool refit_only) {
    std::vector<Box> boxes(b.triCount);
    std::vector<float> v9(9 * (size_t)b.triCount);
    for (uint32_t p = 0; p < b.triCount; ++p) tri_box(s, b, p, boxes[p], &v9[9 * (size_t)p]);
    if (!refit_only) lbvh_build(b.bvh, boxes);
    else {
        for (uint32_t k = 0; k < b.bvh.n; ++k) b.bvh.leafBox[k] = boxes[b.bvh.order[k]];
        lbvh_refit(b.bvh);
    }
    b.tri.resize(9 * (size_t)b.triCount);
    for (uint32_t k = 0; k < b.triCount; ++k)
        std::memcpy(&b.tri[9 * (size_t)k], &v9[9 * (size_t)b.bvh.order[k]], 9 * sizeof(float));
    if (b.triCount == 0) {
        b.root = Box{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
    } else if (b.triCount == 1) b.root = b.bvh.leafBox[0];
    else b.root = b.bvh.nodeBox[0];
}

// 3x4 affine inverse via the adjugate; identical operation order in the product.
static bool affine_inverse(const float* m, float* o) {
    float a00 = m[0], a01 = m[1], a02 = m[2], t0 = m[3];
    float a10 = m[4], a11 = m[5], a12 = m[6], t1 = m[7];
    float a20 = m[8], a21 = m[9], a22 = m[10], t2 = m[11];
    float c00 = a11 * a22 - a12 * a21, c01 = a02 * a21 - a01 * a22, c02 = a01 * a12 - a02 * a11;
    float c10 = a12 * a20 - a10 * a22, c11 = a00 * a22 - a02 * a20, c12 = a02 * a10 - a00 * a12;
    float c20 = a10 * a21 - a11 * a20, c21 = a01 * a20 - a00 * a21, c22 = a00 * a11 - a01 * a10;
    float det = (a00 * c00 + a01 * c10) + a02 * c20;
    if (!(det != 0.0f) || !std::isfinite(det)) return false;
    float id = 1.0f / det;
    float r[9] = {c00 * id, c01 * id, c02 * id, c10 * id, c11 * id, c12 * id, c20 * id, c21 * id, c22 * id};
    for (int i = 0; i < 3; ++i) {
        o[4 * i + 0] = r[3 * i + 0];
        o[4 * i + 1] = r[3 * i + 1];
        o[4 * i + 2] = r[3 * i + 2];
        o[4 * i + 3] = -((r[3 * i + 0] * t0 + r[3 * i + 1] * t1) + r[3 * i + 2] * t2);
    }
    return true;
}

// world box of a transformed object box (per output row: t + sum_j min/max(m_ij*lo_j, m_ij*hi_j))
static Box xform_box(const float* m, const Box& b) {
    Box o;
    for (int i = 0; i < 3; ++i) {
        float lo = m[4 * i + 3], hi = m[4 * i + 3];
        for (int j = 0; j < 3; ++j) {
            float e = m[4 * i + j] * b.lo[j], f = m[4 * i + j] * b.hi[j];
            lo = lo + std::fmin(e, f);
            hi = hi + std::fmax(e, f);
        }
        o.lo[i] = lo;
        o.hi[i] = hi;
    }
    return o;
}

static void build_tlas(Scene& s) {
    std::vector<Box> boxes(s.inst.size());
    for (size_t i = 0; i < s.inst.size(); ++i) {
        const Inst& in = s.inst[i];
        if (in.valid && s.blas[in.blas].triCount > 0) boxes[i] = xform_box(in.m, s.blas[in.blas].root);
        else boxes[i] = Box{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
    }
    // empty boxes get centroid NaN-free placement: put them at the origin of the Morton grid
    for (auto& b : boxes)
        if (!(b.lo[0] <= b.hi[0])) {
            for (int a = 0; a < 3; ++a) { b.lo[a] = INFINITY; b.hi[a] = -INFINITY; }
        }
    // centroids of empty boxes would be NaN; substitute 0 boxes for keying but keep them empty
    std::vector<Box> keyed = boxes;
    for (auto& b : keyed)
        if (!(b.lo[0] <= b.hi[0]))
            for (int a = 0; a < 3; ++a) { b.lo[a] = 0.0f; b.hi[a] = 0.0f; }
    lbvh_build(s.tlas, keyed);
    for (uint32_t k = 0; k < s.tlas.n; ++k) s.tlas.leafBox[k] = boxes[s.tlas.order[k]];
    lbvh_refit(s.tlas);
}

// ------------------------------------------------------------------------------------------------
// traversal
struct RayPre {
    float o[3], d[3], idir[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

static void ray_pre(RayPre& r, const float* o, const float* d) {
    for (int a = 0; a < 3; ++a) {
        r.o[a] = o[a];
        r.d[a] = d[a];
        r.idir[a] = 1.0f / d[a];
    }
    float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
}

static const float kInflate = 1.0000004f;  // 1 + 2*gamma_3 (Ize 2013) rounded up

// One axis of the slab test: the interval [min(t0, t1), max(t0, t1)].  A zero direction component
// whose plane passes through the origin gives 0 * inf = NaN: the ray then runs inside that closed
// slab, so the axis does not constrain t (-inf, +inf).  Without that rule min/max would drop the NaN
// and reject boxes the ray lies on.
static inline void slab_axis(float lo, float hi, float o, float id, float& n, float& f) {
    const float t0 = (lo - o) * id, t1 = (hi - o) * id;
    if (t0 != t0 || t1 != t1) {
        n = -INFINITY;
        f = INFINITY;
        return;
    }
    n = std::fmin(t0, t1);
    f = std::fmax(t0, t1);
}

// slab test against [tmin, tbest]; returns entry distance or +inf when missed
static inline float slab(const RayPre& r, const Box& b, float tmin, float tbest) {
    float nx, fx, ny, fy, nz, fz;
    slab_axis(b.lo[0], b.hi[0], r.o[0], r.idir[0], nx, fx);
    slab_axis(b.lo[1], b.hi[1], r.o[1], r.idir[1], ny, fy);
    slab_axis(b.lo[2], b.hi[2], r.o[2], r.idir[2], nz, fz);
    float tn = std::fmax(std::fmax(nx, ny), std::fmax(nz, tmin));
    float tf = std::fmin(std::fmin(fx, fy), std::fmin(fz, tbest));
    return tn <= tf * kInflate ? tn : INFINITY;
}

struct Hit {
    float t, u, v;
    uint32_t inst, prim;
    bool hit;
};

// candidate acceptance: inside [tmin, bound] and, once something was hit, closer than it or an
// equal-t tie with a smaller (instance, primitive) pair (P7)
static inline bool accept(float t, float tmin, uint32_t inst, uint32_t prim, const Hit& h) {
    if (!(t >= tmin)) return false;
    if (!h.hit) return t <= h.t;
    if (t < h.t) return true;
    if (t == h.t) return inst < h.inst || (inst == h.inst && prim < h.prim);
    return false;
}

// watertight test; identical operation order in the product
static inline void tri_test(const RayPre& r, const float* v, float tmin, uint32_t inst, uint32_t prim, Hit& h) {
    float A[3] = {v[0] - r.o[0], v[1] - r.o[1], v[2] - r.o[2]};
    float B[3] = {v[3] - r.o[0], v[4] - r.o[1], v[5] - r.o[2]};
    float C[3] = {v[6] - r.o[0], v[7] - r.o[1], v[8] - r.o[2]};
    const int kx = r.kx, ky = r.ky, kz = r.kz;
    float Ax = A[kx] - r.Sx * A[kz], Ay = A[ky] - r.Sy * A[kz];
    float Bx = B[kx] - r.Sx * B[kz], By = B[ky] - r.Sy * B[kz];
    float Cx = C[kx] - r.Sx * C[kz], Cy = C[ky] - r.Sy * C[kz];
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
    float Az = r.Sz * A[kz], Bz = r.Sz * B[kz], Cz = r.Sz * C[kz];
    float T = (U * Az + V * Bz) + W * Cz;
    float rc = 1.0f / det;
    float t = T * rc;
    if (!accept(t, tmin, inst, prim, h)) return;
    h.t = t;
    h.u = V * rc;
    h.v = W * rc;
    h.inst = inst;
    h.prim = prim;
    h.hit = true;
}

struct TraceStats {
    uint64_t nodes = 0, tris = 0;
};

static inline const Box& child_box(const Lbvh& b, uint32_t ref) {
    return (ref & 0x80000000u) ? b.leafBox[ref & 0x7FFFFFFFu] : b.nodeBox[ref];
}

// near-child-first stack traversal of one BLAS; h.t is the current upper bound
static void trace_blas(const Blas& b, const RayPre& r, float tmin, uint32_t inst, Hit& h, TraceStats& st) {
    if (b.triCount == 0) return;
    uint32_t stack[128];
    int sp = 0;
    uint32_t ref = b.bvh.rootRef();
    for (;;) {
        if (ref & 0x80000000u) {
            uint32_t k = ref & 0x7FFFFFFFu;
            ++st.tris;
            tri_test(r, &b.tri[9 * (size_t)k], tmin, inst, b.bvh.order[k], h);
        } else {
            ++st.nodes;
            uint32_t L = b.bvh.left[ref], R = b.bvh.right[ref];
            float tl = slab(r, child_box(b.bvh, L), tmin, h.t), tr = slab(r, child_box(b.bvh, R), tmin, h.t);
            bool hl = tl != INFINITY, hr = tr != INFINITY;
            if (hl && hr) {
                uint32_t nearR = (tr < tl) ? R : L, farR = (tr < tl) ? L : R;
                if (sp < 128) stack[sp++] = farR;
                ref = nearR;
                continue;
            }
            if (hl) { ref = L; continue; }
            if (hr) { ref = R; continue; }
        }
        if (sp == 0) break;
        ref = stack[--sp];
    }
}

static inline void object_ray(const Inst& in, const float* o, const float* d, float* oo, float* dd) {
    const float* m = in.inv;
    for (int a = 0; a < 3; ++a) {
        oo[a] = ((m[4 * a + 0] * o[0] + m[4 * a + 1] * o[1]) + m[4 * a + 2] * o[2]) + m[4 * a + 3];
        dd[a] = (m[4 * a + 0] * d[0] + m[4 * a + 1] * d[1]) + m[4 * a + 2] * d[2];
    }
}

static Hit closest_hit(const Scene& s, const float* o, const float* d, float tmin, float tmax, TraceStats& st) {
    Hit h{};
    h.hit = false;
    h.t = tmax;
    if (d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f) return h;  // P3
    if (s.tlas.n == 0) return h;
    RayPre wr;
    ray_pre(wr, o, d);
    uint32_t stack[64];
    int sp = 0;
    uint32_t ref = s.tlas.rootRef();
    if (slab(wr, child_box(s.tlas, ref == 0x80000000u ? ref : 0u), tmin, h.t) == INFINITY && s.tlas.n > 1) return h;
    for (;;) {
        if (ref & 0x80000000u) {
            uint32_t ii = s.tlas.order[ref & 0x7FFFFFFFu];
            const Inst& in = s.inst[ii];
            if (in.valid) {
                float oo[3], dd[3];
                object_ray(in, o, d, oo, dd);
                if (!(dd[0] == 0.0f && dd[1] == 0.0f && dd[2] == 0.0f)) {
                    RayPre orr;
                    ray_pre(orr, oo, dd);
                    const Blas& b = s.blas[in.blas];
                    if (b.triCount > 0 && slab(orr, b.root, tmin, h.t) != INFINITY) trace_blas(b, orr, tmin, ii, h, st);
                }
            }
        } else {
            ++st.nodes;
            uint32_t L = s.tlas.left[ref], R = s.tlas.right[ref];
            float tl = slab(wr, child_box(s.tlas, L), tmin, h.t), tr = slab(wr, child_box(s.tlas, R), tmin, h.t);
            bool hl = tl != INFINITY, hr = tr != INFINITY;
            if (hl && hr) {
                uint32_t nearR = (tr < tl) ? R : L, farR = (tr < tl) ? L : R;
                if (sp < 64) stack[sp++] = farR;
                ref = nearR;
                continue;
            }
            if (hl) { ref = L; continue; }
            if (hr) { ref = R; continue; }
        }
        if (sp == 0) break;
        ref = stack[--sp];
    }
    return h;
}

// brute force over every instance and triangle (validation of the traversal)
static Hit closest_hit_brute(const Scene& s, const float* o, const float* d, float tmin, float tmax) {
    Hit h{};
    h.hit = false;
    h.t = tmax;
    if (d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f) return h;
    for (uint32_t ii = 0; ii < s.inst.size(); ++ii) {
        const Inst& in = s.inst[ii];
        if (!in.valid) continue;
        float oo[3], dd[3];
        object_ray(in, o, d, oo, dd);
        if (dd[0] == 0.0f && dd[1] == 0.0f && dd[2] == 0.0f) continue;
        RayPre r;
        ray_pre(r, oo, dd);
        const Blas& b = s.blas[in.blas];
        for (uint32_t k = 0; k < b.triCount; ++k) tri_test(r, &b.tri[9 * (size_t)k], tmin, ii, b.bvh.order[k], h);
    }
    return h;
}

// ------------------------------------------------------------------------------------------------
// shading (closesthit.rchit / miss.rmiss / shadowMiss.rmiss / raygen.h), depth-first on one payload
enum { RT_GENERIC = 0, RT_SHADOW_TRACE = 1, RT_SHADOW_INTERNAL = 2 };

template <class T>
struct Payload {  // payload.h:29-39
    V3<T> hitValue;
    T reflectContribution;
    V3<T> normal;
    V3<T> roughRGB;
    T roughA;
    T depth, curIOR, refDepth;
    int rayType, recDepth;
};

struct Counters {
    uint64_t primary = 0, shadow = 0, secondary = 0, masked = 0, nodes = 0, tris = 0;
};

template <class T>
struct Shader {
    const Scene& s;
    const Ubo& u;
    Payload<T> p;
    Counters& c;
    TraceStats ts;
    V3<T> lightDir;
    Shader(const Scene& sc, const Ubo& ub, Counters& cc) : s(sc), u(ub), c(cc) { lightDir = cvt<T>(u.lightDir); }

    // miss.rmiss:38-83 (skyMix with the constants of main())
    void miss(V3<T> D) {
        const V3<T> sunTone(T(1.0), T(0.6), T(0.05)), skyTone(T(0.2), T(0.4), T(0.8)), scatterTone(T(1.0), T(0.3), T(0.0));
        const T scatterFactor = T(1.3), powFactor = T(80);
        V3<T> rayDir = normalize(D);
        T y = std::fabs(D.y + T(1.5)) / T(3.0);
        T sun = T(1.0) - len(rayDir - normalize(-lightDir));
        sun = clampT(sun, T(0), T(2));
        T glow = sun;
        glow = clampT(glow, T(0), T(1));
        sun = std::pow(sun, powFactor);
        sun = sun * T(1000.0);
        sun = clampT(sun, T(0), T(16));
        glow = glow * glow * glow * glow * glow * glow * T(1.0);  // pow(glow, 6.0) (P2)
        glow = std::pow(glow, y);
        glow = clampT(glow, T(0), T(1));
        sun = sun * std::pow(y * y, T(1.0) / T(1.65));
        glow = glow * std::pow(y * y, T(1.0) / T(2.0));
        sun = sun + glow;
        V3<T> sunColor = sunTone * sun;
        T atmosphere = std::sqrt(T(1.0) - y);
        T scatter = std::pow(T(4) - lightDir.y, T(1.0) / T(15.0));
        scatter = T(1.0) - clampT(scatter, T(0.8), T(1.0));
        V3<T> scatterColor = mix(V3<T>(T(1.0)), scatterTone * T(1.5), scatter);
        V3<T> skyScatter = mix(skyTone, scatterColor, atmosphere / scatterFactor);
        V3<T> res = sunColor + skyScatter;
        p.hitValue = res;
        p.roughRGB = res;
        p.roughA = T(0);
        p.depth = T(10000);
    }

    // traceRayEXT: traverse (unless mask == 0), then closest-hit or the miss shader `missIndex`
    void trace(V3<T> O, T tmin, V3<T> D, T tmax, bool masked, int missIndex) {
        float of[3] = {(float)O.x, (float)O.y, (float)O.z}, df[3] = {(float)D.x, (float)D.y, (float)D.z};
        Hit h{};
        h.hit = false;
        bool zero = (df[0] == 0.0f && df[1] == 0.0f && df[2] == 0.0f);
        if (masked) c.masked++;
        else if (!zero) {
            TraceStats t2;
            h = closest_hit(s, of, df, (float)tmin, (float)tmax, t2);
            c.nodes += t2.nodes;
            c.tris += t2.tris;
        }
        if (h.hit) closesthit(O, D, h);
        else if (missIndex == 0) miss(D);
        else p.hitValue = V3<T>(T(1));  // shadowMiss.rmiss:30-34
    }

    void gridEffect(V3<T>& diffuse, V3<T>& specular, T& reflectivity, V3<T> pos, T hitT) {  // closesthit.rchit:74-91
        T aa = (p.refDepth + hitT + T(8)) / T(30);
        T aa2 = aa / T(2.0);
        T minmod = std::fmin(std::fabs(glsl_mod((pos.x + T(1000)) * T(10) + aa2, T(20)) - aa2),
                             std::fabs(glsl_mod((pos.z + T(1000)) * T(10) + aa2, T(20)) - aa2));
        if (minmod < aa2) {
            T aa_sq = aa * aa;  // pow(aa, 2) (P2)
            minmod = minmod - (aa2 - aa_sq / T(3.0));
            minmod = minmod * (T(3.0) / aa_sq);
            T f = mixs(aa / T(10), T(1.0), minmod);
            diffuse = diffuse * f;
            specular = specular * f;
            reflectivity = reflectivity * f;
        }
        if (glsl_mod((pos.x + T(1000)) * T(5), T(20)) < T(10) && glsl_mod((pos.z + T(1000)) * T(5), T(20)) < T(10))
            reflectivity = reflectivity * T(1.5);
    }

    void closesthit(V3<T> WO, V3<T> WD, const Hit& h) {  // closesthit.rchit:93-268
        const int maxRec = u.maxRecursions;
        const T hitT = T(h.t);
        const Inst& in = s.inst[h.inst];
        V3<T> bary(T(1.0) - T(h.u) - T(h.v), T(h.u), T(h.v));
        uint32_t ib = in.iOff + 3 * h.prim;
        const Vertex& v0 = s.vertices[in.vOff + s.indices[ib + 0]];
        const Vertex& v1 = s.vertices[in.vOff + s.indices[ib + 1]];
        const Vertex& v2 = s.vertices[in.vOff + s.indices[ib + 2]];
        const Material& M = s.materials[in.mOff + v0.matIndex];
        V3<T> diffuse = cvt<T>(M.diffuse), specular = cvt<T>(M.specular);
        T transparency = T(M.transparency), reflectivity = T(M.reflectivity), roughness = T(M.roughness), ior = T(M.ior);
        T emission = T(M.emission);
        const T tmin = T(0.01f), tmax = T(1000.0f);
        V3<T> origin = WO + WD * hitT;
        V3<T> vn = (cvt<T>(v0.normal) * bary.x + cvt<T>(v1.normal) * bary.y) + cvt<T>(v2.normal) * bary.z;
        const float* m = in.m;
        V3<T> wn((T(m[0]) * vn.x + T(m[1]) * vn.y) + T(m[2]) * vn.z,
                 (T(m[4]) * vn.x + T(m[5]) * vn.y) + T(m[6]) * vn.z,
                 (T(m[8]) * vn.x + T(m[9]) * vn.y) + T(m[10]) * vn.z);
        V3<T> n = normalize(wn);
        if (M.effectId == 1) gridEffect(diffuse, specular, reflectivity, origin, hitT);

        if (p.rayType == RT_SHADOW_INTERNAL) {
            T thick = clampT(hitT * (T(1) - transparency) * T(10), T(0), T(1));
            V3<T> shadowCol = p.hitValue - mix(V3<T>(T(0)), normalize(V3<T>(T(1.1f)) - diffuse) + V3<T>(T(0.1f)), thick);
            if (p.recDepth < maxRec) {
                p.rayType = RT_SHADOW_TRACE;
                p.recDepth++;
                c.shadow++;
                trace(origin, tmin, WD, tmax, false, 0);
                p.recDepth--;
                if (p.depth < T(1000)) {
                    p.hitValue = p.hitValue * shadowCol;
                } else {
                    T eta = ior / T(1.0);
                    V3<T> dir = refract(WD, n, eta);
                    T x = dot(lightDir, dir);
                    T dp = x * x * x * x * x + T(0.75);  // pow(x, 5) (P2)
                    shadowCol = shadowCol * dp;
                    trace(origin, tmin, -dir, tmax, true, 0);
                    p.hitValue = shadowCol + p.hitValue * T(0.1f);
                }
            } else {
                p.hitValue = shadowCol * T(0.4f);
            }
            return;
        }
        if (p.rayType == RT_SHADOW_TRACE) {
            if (transparency > T(0)) {
                if (p.recDepth < maxRec) {
                    p.rayType = RT_SHADOW_INTERNAL;
                    p.recDepth++;
                    c.shadow++;
                    trace(origin, tmin, WD, tmax, false, 1);
                    p.recDepth--;
                }
            } else {
                T f = mixs(T(0.4f), T(0.8f), clampT(std::log(hitT) / T(8), T(0), T(1)));
                p.hitValue = p.hitValue * f;
            }
            return;
        }
        bool front = dot(-WD, n) > T(0);
        if (!front) n = normalize(-n);
        T ndl = dot(-lightDir, n);
        T dp = std::fmax(ndl, T(0.2f));
        V3<T> baseColor = diffuse * dp;
        V3<T> shadowColor(T(1));
        if (ndl > T(0.07f)) {
            if (p.recDepth < maxRec) {
                p.hitValue = V3<T>(T(1.0));
                p.rayType = RT_SHADOW_TRACE;
                p.recDepth++;
                c.shadow++;
                trace(origin, tmin * T(10), -lightDir, tmax, false, 1);
                p.recDepth--;
                shadowColor = p.hitValue;
                p.rayType = RT_GENERIC;
            }
        } else {
            T sm = transparency * transparency;  // pow(transparency, 2) (P2)
            shadowColor = transparency < T(1) ? mix(V3<T>(T(1)), diffuse * sm, transparency) : V3<T>(T(0.4f));
        }
        V3<T> reflectColor(T(1));
        T reflectDepth = T(0);
        if (p.recDepth < maxRec && reflectivity > T(0)) {
            V3<T> dir = reflect(WD, n);
            p.recDepth += (int)M.rayConsumption;
            p.refDepth = p.refDepth + hitT;
            c.secondary++;
            trace(origin, tmin, dir, tmax, false, 0);
            p.recDepth -= (int)M.rayConsumption;
            reflectColor = p.hitValue * specular;
            reflectDepth = p.depth;
        }
        V3<T> refractColor(T(1));
        if (p.recDepth < maxRec && transparency > T(0)) {
            if (front) {
                T eta = p.curIOR / ior;
                V3<T> dir = refract(WD, n, eta);
                p.recDepth++;
                p.curIOR = ior;
                if (!(dir.x == T(0) && dir.y == T(0) && dir.z == T(0))) c.secondary++;  // only rays that traverse
                trace(origin, tmin, dir, tmax, false, 0);
                p.recDepth--;
                refractColor = p.hitValue;
            } else {
                T eta = ior / T(1.0);
                V3<T> dir = refract(WD, n, eta);
                p.recDepth++;
                p.curIOR = T(1.0);
                if (!(dir.x == T(0) && dir.y == T(0) && dir.z == T(0))) c.secondary++;
                trace(origin, tmin, dir, tmax, false, 0);
                p.recDepth--;
                V3<T> tm = mix(V3<T>(T(1)), diffuse, std::log(T(1) + hitT));
                refractColor = tm * p.hitValue;
            }
        }
        baseColor = baseColor * shadowColor;
        baseColor = baseColor + diffuse * emission;
        T total = std::fmax(transparency, reflectivity);
        T den = transparency + reflectivity;
        T w = den == T(0) ? T(0) : reflectivity / den;  // P1
        V3<T> roughCol = mix(refractColor, reflectColor, w);
        p.hitValue = mix(baseColor, roughCol, total);
        if (p.recDepth == 0) {
            p.hitValue = baseColor;
            p.normal = n;
            p.roughRGB = roughCol;
            p.roughA = std::fmin((reflectDepth / T(50.f)) * roughness, roughness / T(2.1f));
            p.reflectContribution = total;
        }
        p.depth = hitT;
    }
};

// raygen.h:37-53 (vAAOffsets)
static const float kAA[9][8][2] = {
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

// mat4 (column-major) * vec4
template <class T>
static void mul4(const float* m, const T* v, T* o) {
    for (int r = 0; r < 4; ++r) o[r] = ((T(m[0 * 4 + r]) * v[0] + T(m[1 * 4 + r]) * v[1]) + T(m[2 * 4 + r]) * v[2]) + T(m[3 * 4 + r]) * v[3];
}

// raygen.h:69-115 + raygen.rgen:30-39 for one pixel; writes 12 floats (image, normalImage, roughImage)
template <class T>
static void raygen_pixel(const Scene& s, const Ubo& u, uint32_t px, uint32_t py, uint32_t W, uint32_t H, float* out12, Counters& c) {
    Shader<T> sh(s, u, c);
    V3<T> color(T(0)), normal(T(0));
    T rough[4] = {0, 0, 0, 0};
    T reflectContrib = T(0), depth = T(0);
    T o4[4], z4[4] = {T(0), T(0), T(0), T(1)};
    mul4<T>(u.viewInverse, z4, o4);
    V3<T> origin(o4[0], o4[1], o4[2]);
    const int S = u.numSamples;
    const int row = std::min(S, 8);
    for (int i = 0; i < S; ++i) {
        T pcx = (T(px) + T(0.5)) + T(kAA[row][i % 8][0]);
        T pcy = (T(py) + T(0.5)) + T(kAA[row][i % 8][1]);
        T ux = pcx / T(W), uy = pcy / T(H);
        T dx = ux * T(2.0) - T(1.0), dy = uy * T(2.0) - T(1.0);
        T tv[4] = {dx, dy, T(1), T(1)}, tg[4];
        mul4<T>(u.projInverse, tv, tg);
        V3<T> tn = normalize(V3<T>(tg[0], tg[1], tg[2]));
        T dv[4] = {tn.x, tn.y, tn.z, T(0)}, dw[4];
        mul4<T>(u.viewInverse, dv, dw);
        V3<T> dir(dw[0], dw[1], dw[2]);
        auto& p = sh.p;
        p.hitValue = V3<T>(T(0));
        p.normal = V3<T>(T(0));
        p.roughRGB = V3<T>(T(0));
        p.roughA = T(0);
        p.depth = T(0);
        p.refDepth = T(0);
        p.curIOR = T(1);
        p.rayType = RT_GENERIC;
        p.recDepth = 0;
        p.reflectContribution = T(0);
        c.primary++;
        sh.trace(origin, T(0.001f), dir, T(10000.0f), false, 0);
        color = color + p.hitValue;
        normal = normal + p.normal;
        rough[0] = rough[0] + p.roughRGB.x;
        rough[1] = rough[1] + p.roughRGB.y;
        rough[2] = rough[2] + p.roughRGB.z;
        rough[3] = rough[3] + p.roughA;
        reflectContrib = reflectContrib + p.reflectContribution;
        depth = depth + p.depth;
    }
    T fs = T(S);
    T v[12] = {color.x, color.y, color.z, reflectContrib, normal.x, normal.y, normal.z, std::log(depth) * T(0.25),
               rough[0], rough[1], rough[2], rough[3]};
    for (int k = 0; k < 12; ++k) out12[k] = rh((float)(v[k] / fs));
}

// ------------------------------------------------------------------------------------------------
// post passes
struct Img {
    uint32_t W, H;
    std::vector<float> px;  // RGBA
    Img(uint32_t w, uint32_t h) : W(w), H(h), px(4 * (size_t)w * h, 0.0f) {}
    const float* at(int x, int y) const { return &px[4 * ((size_t)y * W + x)]; }
    float* at(int x, int y) { return &px[4 * ((size_t)y * W + x)]; }
    void load(int x, int y, float* o) const {  // P4
        if (x < 0 || y < 0 || x >= (int)W || y >= (int)H) { o[0] = o[1] = o[2] = o[3] = 0.0f; return; }
        std::memcpy(o, at(x, y), 16);
    }
};

static float dist4(const float* a, const float* b) {
    float d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2], d3 = a[3] - b[3];
    return std::sqrt(((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3);
}

template <class F>
static void parallel_rows(uint32_t r0, uint32_t r1, int nthreads, F&& f);

static void rough_passes(const Img& rough, const Img& normal, Img& trans, Img& A, Img& B, int nt = 1) {
    const int W = rough.W, H = rough.H;
    // rough_prepare.comp:28-54
    parallel_rows(0, (uint32_t)H, nt, [&](uint32_t yy, int) {
        const int y = (int)yy;
        for (int x = 0; x < W; ++x) {
            float r[4], ru[4], rd[4], rl[4], rr[4], n[4], nu[4], nd[4], nl[4], nr[4];
            rough.load(x, y, r); rough.load(x, y + 1, ru); rough.load(x, y - 1, rd); rough.load(x + 1, y, rl); rough.load(x - 1, y, rr);
            normal.load(x, y, n); normal.load(x, y + 1, nu); normal.load(x, y - 1, nd); normal.load(x + 1, y, nl); normal.load(x - 1, y, nr);
            float uf = std::fmin(ru[3], r[3]) * clampT(1.0f - dist4(nu, n) * 10.0f, 0.0f, 1.0f);
            float df = std::fmin(rd[3], r[3]) * clampT(1.0f - dist4(nd, n) * 10.0f, 0.0f, 1.0f);
            float lf = std::fmin(rl[3], r[3]) * clampT(1.0f - dist4(nl, n) * 10.0f, 0.0f, 1.0f);
            float rf = std::fmin(rr[3], r[3]) * clampT(1.0f - dist4(nr, n) * 10.0f, 0.0f, 1.0f);
            float t = std::fmin(std::fmin(std::fmin(uf, df), lf), rf);
            float q = std::rint(clampT(t, -1.0f, 1.0f) * 127.0f) / 127.0f;  // P5
            float* tp = trans.at(x, y);
            tp[0] = q; tp[1] = 0.0f; tp[2] = 0.0f; tp[3] = 1.0f;
            std::memcpy(A.at(x, y), r, 16);
            std::memcpy(B.at(x, y), r, 16);
        }
    });
    // rough_blur.h:23-40, 10 x (H: A->B, V: B->A); a pass reads only the previous pass's image
    for (int it = 0; it < 10; ++it) {
        for (int pass = 0; pass < 2; ++pass) {
            const Img& in = pass == 0 ? A : B;
            Img& out = pass == 0 ? B : A;
            int ox = pass == 0 ? 1 : 0, oy = pass == 0 ? 0 : 1;
            parallel_rows(0, (uint32_t)H, nt, [&](uint32_t yy, int) {
                const int y = (int)yy;
                for (int x = 0; x < W; ++x) {
                    float t = trans.at(x, y)[0];
                    if (t < 0.001f) continue;
                    float c[4], a[4], b[4];
                    in.load(x, y, c);
                    in.load(x + ox, y + oy, a);
                    in.load(x - ox, y - oy, b);
                    float w = (1.0f - t) - t;
                    float* o = out.at(x, y);
                    for (int k = 0; k < 3; ++k) o[k] = rh((c[k] * w + a[k] * t) + b[k] * t);
                    o[3] = rh(c[3]);
                }
            });
        }
    }
}

// postprocess.comp:28-50 (without the showAlpha branch, applied separately)
static void postprocess(const Img& base, const Img& A, const Ubo& u, Img& fin) {
    for (uint32_t y = 0; y < base.H; ++y)
        for (uint32_t x = 0; x < base.W; ++x) {
            const float* b = base.at(x, y);
            const float* r = A.at(x, y);
            float col[3];
            for (int k = 0; k < 3; ++k) col[k] = clampT(mixs(b[k], r[k], b[3]), 0.0f, 1.0f);
            float luma = (col[0] * 0.299f + col[1] * 0.587f) + col[2] * 0.114f;
            for (int k = 0; k < 3; ++k) col[k] = mixs(col[k], u.fadeColor[k], u.fadeColor[3]);
            float* o = fin.at(x, y);
            o[0] = rh(col[0]); o[1] = rh(col[1]); o[2] = rh(col[2]); o[3] = rh(luma);
        }
}

// FXAA 3.11, PC quality, preset 39, FXAA_GREEN_AS_LUMA = 1 (fxaa.h:180,201,487-500,615-1136)
struct Fxaa {
    const Img& im;
    float rcpW, rcpH;
    Fxaa(const Img& i) : im(i) {
        rcpW = 1.0f / (float)i.W;
        rcpH = 1.0f / (float)i.H;
    }
    const float* texel(int x, int y) const {
        x = std::min(std::max(x, 0), (int)im.W - 1);
        y = std::min(std::max(y, 0), (int)im.H - 1);
        return im.at(x, y);
    }
    // P9: a coordinate equal to a texel centre as the shader computes it ((i + 0.5) / size in FP32)
    // samples that texel; any other coordinate is FP32 bilinear x = u*size - 0.5, weights (1-f, f)
    static void axis(float u, int size, int& i0, float& f) {
        int c = (int)std::floor(u * (float)size);
        if (u == ((float)c + 0.5f) / (float)size) {
            i0 = c;
            f = 0.0f;
            return;
        }
        float fx = u * (float)size - 0.5f;
        float x0 = std::floor(fx);
        f = fx - x0;
        i0 = (int)x0;
    }
    void bilinear(float u, float v, float* o) const {
        int ix, iy;
        float ax, ay;
        axis(u, (int)im.W, ix, ax);
        axis(v, (int)im.H, iy, ay);
        const float *t00 = texel(ix, iy), *t10 = texel(ix + 1, iy), *t01 = texel(ix, iy + 1), *t11 = texel(ix + 1, iy + 1);
        for (int k = 0; k < 4; ++k) {
            float top = t00[k] * (1.0f - ax) + t10[k] * ax;
            float bot = t01[k] * (1.0f - ax) + t11[k] * ax;
            o[k] = top * (1.0f - ay) + bot * ay;
        }
    }
    float lumaAt(float u, float v) const {
        float o[4];
        bilinear(u, v, o);
        return o[1];
    }
    void pixel(int x, int y, float* out) const {
        static const float P[12] = {1.0f, 1.0f, 1.0f, 1.0f, 1.0f, 1.5f, 2.0f, 2.0f, 2.0f, 2.0f, 4.0f, 8.0f};
        const float subpix = 1.0f, edgeThreshold = 0.063f, edgeThresholdMin = 0.0312f;
        float posMx = ((float)x + 0.5f) / (float)im.W;  // fxaa.comp:31
        float posMy = ((float)y + 0.5f) / (float)im.H;
        const float* rgbyM = texel(x, y);
        float lumaM = rgbyM[1];
        float lumaS = texel(x, y + 1)[1], lumaE = texel(x + 1, y)[1], lumaN = texel(x, y - 1)[1], lumaW = texel(x - 1, y)[1];
        float maxSM = std::fmax(lumaS, lumaM), minSM = std::fmin(lumaS, lumaM);
        float maxESM = std::fmax(lumaE, maxSM), minESM = std::fmin(lumaE, minSM);
        float maxWN = std::fmax(lumaN, lumaW), minWN = std::fmin(lumaN, lumaW);
        float rangeMax = std::fmax(maxWN, maxESM), rangeMin = std::fmin(minWN, minESM);
        float rangeMaxScaled = rangeMax * edgeThreshold;
        float range = rangeMax - rangeMin;
        float rangeMaxClamped = std::fmax(edgeThresholdMin, rangeMaxScaled);
        if (range < rangeMaxClamped) {
            std::memcpy(out, rgbyM, 16);
            return;
        }
        float lumaNW = texel(x - 1, y - 1)[1], lumaSE = texel(x + 1, y + 1)[1];
        float lumaNE = texel(x + 1, y - 1)[1], lumaSW = texel(x - 1, y + 1)[1];
        float lumaNS = lumaN + lumaS, lumaWE = lumaW + lumaE;
        float subpixRcpRange = 1.0f / range;
        float subpixNSWE = lumaNS + lumaWE;
        float edgeHorz1 = (-2.0f * lumaM) + lumaNS, edgeVert1 = (-2.0f * lumaM) + lumaWE;
        float lumaNESE = lumaNE + lumaSE, lumaNWNE = lumaNW + lumaNE;
        float edgeHorz2 = (-2.0f * lumaE) + lumaNESE, edgeVert2 = (-2.0f * lumaN) + lumaNWNE;
        float lumaNWSW = lumaNW + lumaSW, lumaSWSE = lumaSW + lumaSE;
        float edgeHorz4 = (std::fabs(edgeHorz1) * 2.0f) + std::fabs(edgeHorz2);
        float edgeVert4 = (std::fabs(edgeVert1) * 2.0f) + std::fabs(edgeVert2);
        float edgeHorz3 = (-2.0f * lumaW) + lumaNWSW, edgeVert3 = (-2.0f * lumaS) + lumaSWSE;
        float edgeHorz = std::fabs(edgeHorz3) + edgeHorz4, edgeVert = std::fabs(edgeVert3) + edgeVert4;
        float subpixNWSWNESE = lumaNWSW + lumaNESE;
        float lengthSign = rcpW;
        bool horzSpan = edgeHorz >= edgeVert;
        float subpixA = subpixNSWE * 2.0f + subpixNWSWNESE;
        if (!horzSpan) lumaN = lumaW;
        if (!horzSpan) lumaS = lumaE;
        if (horzSpan) lengthSign = rcpH;
        float subpixB = (subpixA * (1.0f / 12.0f)) - lumaM;
        float gradientN = lumaN - lumaM, gradientS = lumaS - lumaM;
        float lumaNN = lumaN + lumaM, lumaSS = lumaS + lumaM;
        bool pairN = std::fabs(gradientN) >= std::fabs(gradientS);
        float gradient = std::fmax(std::fabs(gradientN), std::fabs(gradientS));
        if (pairN) lengthSign = -lengthSign;
        float subpixC = clampT(std::fabs(subpixB) * subpixRcpRange, 0.0f, 1.0f);
        float posBx = posMx, posBy = posMy;
        float offNPx = (!horzSpan) ? 0.0f : rcpW;
        float offNPy = (horzSpan) ? 0.0f : rcpH;
        if (!horzSpan) posBx = posBx + lengthSign * 0.5f;
        if (horzSpan) posBy = posBy + lengthSign * 0.5f;
        float posNx = posBx - offNPx * P[0], posNy = posBy - offNPy * P[0];
        float posPx = posBx + offNPx * P[0], posPy = posBy + offNPy * P[0];
        float subpixD = ((-2.0f) * subpixC) + 3.0f;
        float lumaEndN = lumaAt(posNx, posNy);
        float subpixE = subpixC * subpixC;
        float lumaEndP = lumaAt(posPx, posPy);
        if (!pairN) lumaNN = lumaSS;
        float gradientScaled = gradient * 1.0f / 4.0f;
        float lumaMM = lumaM - lumaNN * 0.5f;
        float subpixF = subpixD * subpixE;
        bool lumaMLTZero = lumaMM < 0.0f;
        lumaEndN = lumaEndN - lumaNN * 0.5f;
        lumaEndP = lumaEndP - lumaNN * 0.5f;
        bool doneN = std::fabs(lumaEndN) >= gradientScaled;
        bool doneP = std::fabs(lumaEndP) >= gradientScaled;
        if (!doneN) { posNx = posNx - offNPx * P[1]; posNy = posNy - offNPy * P[1]; }
        bool doneNP = (!doneN) || (!doneP);
        if (!doneP) { posPx = posPx + offNPx * P[1]; posPy = posPy + offNPy * P[1]; }
        for (int k = 2; k < 12 && doneNP; ++k) {
            if (!doneN) lumaEndN = lumaAt(posNx, posNy);
            if (!doneP) lumaEndP = lumaAt(posPx, posPy);
            if (!doneN) lumaEndN = lumaEndN - lumaNN * 0.5f;
            if (!doneP) lumaEndP = lumaEndP - lumaNN * 0.5f;
            doneN = std::fabs(lumaEndN) >= gradientScaled;
            doneP = std::fabs(lumaEndP) >= gradientScaled;
            if (!doneN) { posNx = posNx - offNPx * P[k]; posNy = posNy - offNPy * P[k]; }
            doneNP = (!doneN) || (!doneP);
            if (!doneP) { posPx = posPx + offNPx * P[k]; posPy = posPy + offNPy * P[k]; }
        }
        float dstN = posMx - posNx, dstP = posPx - posMx;
        if (!horzSpan) dstN = posMy - posNy;
        if (!horzSpan) dstP = posPy - posMy;
        bool goodSpanN = (lumaEndN < 0.0f) != lumaMLTZero;
        float spanLength = (dstP + dstN);
        bool goodSpanP = (lumaEndP < 0.0f) != lumaMLTZero;
        float spanLengthRcp = 1.0f / spanLength;
        bool directionN = dstN < dstP;
        float dst = std::fmin(dstN, dstP);
        bool goodSpan = directionN ? goodSpanN : goodSpanP;
        float subpixG = subpixF * subpixF;
        float pixelOffset = (dst * (-spanLengthRcp)) + 0.5f;
        float subpixH = subpixG * subpix;
        float pixelOffsetGood = goodSpan ? pixelOffset : 0.0f;
        float pixelOffsetSubpix = std::fmax(pixelOffsetGood, subpixH);
        if (!horzSpan) posMx = posMx + pixelOffsetSubpix * lengthSign;
        if (horzSpan) posMy = posMy + pixelOffsetSubpix * lengthSign;
        float o[4];
        bilinear(posMx, posMy, o);
        out[0] = o[0]; out[1] = o[1]; out[2] = o[2]; out[3] = lumaM;
    }
};

template <class F>
static void parallel_rows(uint32_t r0, uint32_t r1, int nthreads, F&& f) {
    if (nthreads <= 1) {
        for (uint32_t y = r0; y < r1; ++y) f(y, 0);
        return;
    }
    std::atomic<uint32_t> next{r0};
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t] {
            for (;;) {
                uint32_t y = next.fetch_add(1);
                if (y >= r1) break;
                f(y, t);
            }
        });
    for (auto& x : th) x.join();
}

}  // namespace

// ================================================================================================
// C API
extern "C" {

struct orc_scene;

uint32_t orc_lbvh(const float* boxes, uint32_t n, uint32_t* morton, uint32_t* order, uint32_t* left, uint32_t* right, float* nodeboxes) {
    std::vector<Box> b(n);
    for (uint32_t i = 0; i < n; ++i) std::memcpy(&b[i], boxes + 6 * (size_t)i, 24);
    Lbvh l;
    lbvh_build(l, b);
    if (morton) std::memcpy(morton, l.morton.data(), 4 * (size_t)n);
    if (order) std::memcpy(order, l.order.data(), 4 * (size_t)n);
    if (n > 1) {
        if (left) std::memcpy(left, l.left.data(), 4 * (size_t)(n - 1));
        if (right) std::memcpy(right, l.right.data(), 4 * (size_t)(n - 1));
        if (nodeboxes) std::memcpy(nodeboxes, l.nodeBox.data(), 24 * (size_t)(n - 1));
    }
    return n;
}

// binned-SAH BVH2 over n boxes (sah_build above, ranges halved from level medianLevel on); returns
// the number of levels
uint32_t orc_sah(const float* boxes, uint32_t n, uint32_t medianLevel, uint32_t* order, uint32_t* left, uint32_t* right, float* nodeboxes) {
    std::vector<Box> b(n);
    for (uint32_t i = 0; i < n; ++i) std::memcpy(&b[i], boxes + 6 * (size_t)i, 24);
    Lbvh l;
    const uint32_t levels = sah_build(l, b, medianLevel);
    if (order) std::memcpy(order, l.order.data(), 4 * (size_t)n);
    if (n > 1) {
        if (left) std::memcpy(left, l.left.data(), 4 * (size_t)(n - 1));
        if (right) std::memcpy(right, l.right.data(), 4 * (size_t)(n - 1));
        if (nodeboxes) std::memcpy(nodeboxes, l.nodeBox.data(), 24 * (size_t)(n - 1));
    }
    return levels;
}

orc_scene* orc_scene_create(const void* vertices, uint32_t nv, const uint32_t* indices, uint32_t ni, const void* materials, uint32_t nm,
                            const uint32_t* meshes, uint32_t nmesh, const void* instances, uint32_t ninst) {
    Scene* s = new Scene();
    s->vertices.assign((const Vertex*)vertices, (const Vertex*)vertices + nv);
    s->indices.assign(indices, indices + ni);
    s->materials.assign((const Material*)materials, (const Material*)materials + nm);
    s->blas.resize(nmesh);
    for (uint32_t b = 0; b < nmesh; ++b) {
        s->blas[b].vertexOffset = meshes[3 * b + 0];
        s->blas[b].indexOffset = meshes[3 * b + 1];
        s->blas[b].triCount = meshes[3 * b + 2];
        build_blas(*s, s->blas[b], false);
    }
    const Instance* in = (const Instance*)instances;
    s->inst.resize(ninst);
    for (uint32_t i = 0; i < ninst; ++i) {
        Inst& d = s->inst[i];
        std::memcpy(d.m, in[i].transform, 48);
        d.valid = affine_inverse(d.m, d.inv) && in[i].blas < nmesh && (in[i].mask & 0xFFu) != 0u;
        d.blas = in[i].blas < nmesh ? in[i].blas : 0;
        d.vOff = in[i].vertexBufferOffset;
        d.iOff = in[i].indexBufferOffset;
        d.mOff = in[i].materialBufferOffset;
    }
    build_tlas(*s);
    return (orc_scene*)s;
}

void orc_scene_destroy(orc_scene* s) { delete (Scene*)s; }

// replace vertex positions [first, first+n) and refit the given BLAS, then rebuild the TLAS
int orc_scene_refit(orc_scene* sc, uint32_t blas, const void* vertices, uint32_t first, uint32_t n) {
    Scene* s = (Scene*)sc;
    if (blas >= s->blas.size() || (size_t)first + n > s->vertices.size()) return -1;
    std::memcpy(&s->vertices[first], vertices, 32 * (size_t)n);
    build_blas(*s, s->blas[blas], true);
    build_tlas(*s);
    return 0;
}

int orc_scene_set_instances(orc_scene* sc, const void* instances, uint32_t ninst) {
    Scene* s = (Scene*)sc;
    const Instance* in = (const Instance*)instances;
    s->inst.resize(ninst);
    for (uint32_t i = 0; i < ninst; ++i) {
        Inst& d = s->inst[i];
        std::memcpy(d.m, in[i].transform, 48);
        d.valid = affine_inverse(d.m, d.inv) && in[i].blas < s->blas.size() && (in[i].mask & 0xFFu) != 0u;
        d.blas = in[i].blas < s->blas.size() ? in[i].blas : 0;
        d.vOff = in[i].vertexBufferOffset;
        d.iOff = in[i].indexBufferOffset;
        d.mOff = in[i].materialBufferOffset;
    }
    build_tlas(*s);
    return 0;
}

// BVH of one BLAS (blas < nmesh) or of the TLAS (blas == 0xFFFFFFFF)
int orc_bvh_info(orc_scene* sc, uint32_t blas, uint32_t* morton, uint32_t* order, uint32_t* left, uint32_t* right, float* nodeboxes) {
    Scene* s = (Scene*)sc;
    const Lbvh* l = nullptr;
    if (blas == 0xFFFFFFFFu) l = &s->tlas;
    else if (blas < s->blas.size()) l = &s->blas[blas].bvh;
    else return -1;
    uint32_t n = l->n;
    if (morton) std::memcpy(morton, l->morton.data(), 4 * (size_t)n);
    if (order) std::memcpy(order, l->order.data(), 4 * (size_t)n);
    if (n > 1) {
        if (left) std::memcpy(left, l->left.data(), 4 * (size_t)(n - 1));
        if (right) std::memcpy(right, l->right.data(), 4 * (size_t)(n - 1));
        if (nodeboxes) std::memcpy(nodeboxes, l->nodeBox.data(), 24 * (size_t)(n - 1));
    }
    return (int)n;
}

// instance inverse transforms (12 floats each), for parity of the TLAS set-up
int orc_instance_inverse(orc_scene* sc, float* out) {
    Scene* s = (Scene*)sc;
    for (size_t i = 0; i < s->inst.size(); ++i) std::memcpy(out + 12 * i, s->inst[i].inv, 48);
    return (int)s->inst.size();
}

// closest hit of n rays (8 floats each: o.xyz, tmin, d.xyz, tmax)
// hit_f: n x 3 (t, u, v); hit_i: n x 2 (instance, primitive), 0xFFFFFFFF when missed
int orc_trace(orc_scene* sc, const float* rays, uint32_t n, float* hit_f, uint32_t* hit_i, int brute, int nthreads) {
    const Scene* s = (const Scene*)sc;
    auto one = [&](uint32_t k) {
        const float* r = rays + 8 * (size_t)k;
        TraceStats st;
        Hit h = brute ? closest_hit_brute(*s, r, r + 4, r[3], r[7]) : closest_hit(*s, r, r + 4, r[3], r[7], st);
        if (h.hit) {
            hit_f[3 * k] = h.t; hit_f[3 * k + 1] = h.u; hit_f[3 * k + 2] = h.v;
            hit_i[2 * k] = h.inst; hit_i[2 * k + 1] = h.prim;
        } else {
            hit_f[3 * k] = hit_f[3 * k + 1] = hit_f[3 * k + 2] = 0.0f;
            hit_i[2 * k] = hit_i[2 * k + 1] = 0xFFFFFFFFu;
        }
    };
    const uint32_t chunk = 1024;
    uint32_t nchunks = (n + chunk - 1) / chunk;
    parallel_rows(0, nchunks, nthreads, [&](uint32_t c, int) {
        for (uint32_t k = c * chunk; k < std::min(n, (c + 1) * chunk); ++k) one(k);
    });
    return 0;
}

// raygen for rows row0, row0+row_step, ... < row1: writes base/normal/rough images (W*H*4 floats
// each, FP16-rounded values).  stats (6 x u64): primary, shadow, secondary, masked-miss traces, nodes, triangles.
int orc_render(orc_scene* sc, const void* ubo, uint32_t W, uint32_t H, uint32_t row0, uint32_t row1, uint32_t row_step, float* base,
               float* normal, float* rough, uint64_t* stats, int nthreads, int fp64) {
    const Scene* s = (const Scene*)sc;
    const Ubo& u = *(const Ubo*)ubo;
    if (row1 > H) row1 = H;
    if (row_step < 1) row_step = 1;
    int nt = nthreads < 1 ? 1 : nthreads;
    std::vector<Counters> cs(nt);
    uint32_t nrows = row1 > row0 ? (row1 - row0 + row_step - 1) / row_step : 0;
    parallel_rows(0, nrows, nt, [&](uint32_t k, int t) {
        uint32_t y = row0 + k * row_step;
        for (uint32_t x = 0; x < W; ++x) {
            float o[12];
            if (fp64) raygen_pixel<double>(*s, u, x, y, W, H, o, cs[t]);
            else raygen_pixel<float>(*s, u, x, y, W, H, o, cs[t]);
            size_t i = 4 * ((size_t)y * W + x);
            std::memcpy(base + i, o, 16);
            std::memcpy(normal + i, o + 4, 16);
            std::memcpy(rough + i, o + 8, 16);
        }
    });
    if (stats) {
        Counters tot;
        for (auto& c : cs) {
            tot.primary += c.primary; tot.shadow += c.shadow; tot.secondary += c.secondary;
            tot.masked += c.masked; tot.nodes += c.nodes; tot.tris += c.tris;
        }
        stats[0] = tot.primary; stats[1] = tot.shadow; stats[2] = tot.secondary;
        stats[3] = tot.masked; stats[4] = tot.nodes; stats[5] = tot.tris;
    }
    return 0;
}

// post passes of Raytracer::doRaytracing (raytracer.cpp:106-142) on the three G-buffer images.
// final_out: W*H*4.  debug (nullable): 4 images of W*H*4 -- roughTransitions, roughColorsA,
// roughColorsB, finalImage before FXAA.  When showAlpha is set, the images get .aaaa as in
// postprocess.comp:41-49 (normal/rough/base are modified in place).
int orc_post(const void* ubo, uint32_t W, uint32_t H, float* base, float* normal, float* rough, float* final_out, float* debug,
             int fxaa, int nthreads) {
    const Ubo& u = *(const Ubo*)ubo;
    Img ib(W, H), in(W, H), ir(W, H), tr(W, H), A(W, H), B(W, H), fin(W, H);
    std::memcpy(ib.px.data(), base, 16 * (size_t)W * H);
    std::memcpy(in.px.data(), normal, 16 * (size_t)W * H);
    std::memcpy(ir.px.data(), rough, 16 * (size_t)W * H);
    rough_passes(ir, in, tr, A, B, nthreads);
    postprocess(ib, A, u, fin);
    if (u.showAlpha) {
        for (Img* im : {&fin, &in, &ir, &ib, &A, &B})
            for (size_t p = 0; p < (size_t)W * H; ++p) {
                float a = im->px[4 * p + 3];
                im->px[4 * p] = im->px[4 * p + 1] = im->px[4 * p + 2] = a;
            }
        for (size_t p = 0; p < (size_t)W * H; ++p) tr.px[4 * p] = 1.0f;  // R8_SNORM .aaaa = 1
        std::memcpy(base, ib.px.data(), 16 * (size_t)W * H);
        std::memcpy(normal, in.px.data(), 16 * (size_t)W * H);
        std::memcpy(rough, ir.px.data(), 16 * (size_t)W * H);
    }
    if (debug) {
        size_t sz = 4 * (size_t)W * H;
        std::memcpy(debug, tr.px.data(), 4 * sz);
        std::memcpy(debug + sz, A.px.data(), 4 * sz);
        std::memcpy(debug + 2 * sz, B.px.data(), 4 * sz);
        std::memcpy(debug + 3 * sz, fin.px.data(), 4 * sz);
    }
    if (!fxaa) {
        std::memcpy(final_out, fin.px.data(), 16 * (size_t)W * H);
        return 0;
    }
    Fxaa f(fin);
    parallel_rows(0, H, nthreads, [&](uint32_t y, int) {
        for (uint32_t x = 0; x < W; ++x) {
            float o[4];
            f.pixel((int)x, (int)y, o);
            float* d = final_out + 4 * ((size_t)y * W + x);
            for (int k = 0; k < 4; ++k) d[k] = rh(o[k]);
        }
    });
    return 0;
}

// FP16 rounding helper exposed for tests
void orc_round_half(const float* in, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) out[i] = rh(in[i]);
}

}  // extern "C"
