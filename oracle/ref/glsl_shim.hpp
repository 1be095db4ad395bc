// glsl_shim.hpp -- just enough GLSL in C++ to compile Raygun's own shader sources on the host.
//
// TEST INFRASTRUCTURE ONLY (the reference-compiled checker).  The shader files themselves are not
// copied into this repository: oracle/ref/build.py reads them from the reference tree, applies a
// few mechanical rewrites a C++ compiler needs (drop #version/#extension, `inout T x` -> `T& x`,
// unsized buffer arrays -> pointers, drop the compute `layout(...) in;` line) into the ignored
// oracle/_ref/ folder, and compiles ref_shaders.cpp, which includes them inside namespaces that
// see this shim.
//
// Semantics follow the GLSL specification's definitions, with the same evaluation order and the
// same policies for GLSL-undefined cases as the oracle (rg_oracle.cpp P1-P9).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace rgsl {

typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;
struct ivec2;
struct uvec2;

// swizzle views (.xy, .xyz, .rgb of a vector of the same or larger size)
struct vec2v {
    float x, y;
    inline operator vec2() const;
};
struct vec3v {
    float x, y, z;
    inline operator vec3() const;
};
struct uvec2v {
    uint x, y;
    inline operator uvec2() const;
};

struct vec2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
        vec2v xy;
    };
    vec2() { x = y = 0.0f; }
    vec2(float a, float b) { x = a; y = b; }
    explicit vec2(float s) { x = y = s; }
    inline explicit vec2(const uvec2& u);
    inline explicit vec2(const ivec2& u);
};
struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        vec3v xyz;
        vec3v rgb;
        vec2v xy;
    };
    vec3() { x = y = z = 0.0f; }
    vec3(float a, float b, float c) { x = a; y = b; z = c; }
    explicit vec3(float s) { x = y = z = s; }
};
struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        vec3v xyz;
        vec3v rgb;
        vec2v xy;
    };
    vec4() { x = y = z = w = 0.0f; }
    vec4(float a_, float b_, float c_, float d_) { x = a_; y = b_; z = c_; w = d_; }
    explicit vec4(float s) { x = y = z = w = s; }
    vec4(const vec3& v, float s) { x = v.x; y = v.y; z = v.z; w = s; }
};
struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    inline explicit ivec2(const uvec2& u);
};
struct uvec2 {
    uint x, y;
    uvec2() : x(0), y(0) {}
    uvec2(uint a, uint b) : x(a), y(b) {}
};
struct uvec3 {
    union {
        struct { uint x, y, z; };
        uvec2v xy;
    };
    uvec3() { x = y = z = 0; }
    uvec3(uint a, uint b, uint c) { x = a; y = b; z = c; }
};

inline vec2v::operator vec2() const { return vec2(x, y); }
inline vec3v::operator vec3() const { return vec3(x, y, z); }
inline uvec2v::operator uvec2() const { return uvec2(x, y); }
inline vec2::vec2(const uvec2& u) { x = (float)u.x; y = (float)u.y; }
inline vec2::vec2(const ivec2& u) { x = (float)u.x; y = (float)u.y; }
inline ivec2::ivec2(const uvec2& u) : x((int)u.x), y((int)u.y) {}

// a loaded texel also offers .aaaa (postprocess.comp:41-49)
struct Texel : vec4 {
    vec4 aaaa;
    explicit Texel(const vec4& v) : vec4(v), aaaa(v.w) {}
};

// ---- arithmetic ------------------------------------------------------------------------------
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(const vec2& a, const vec2& b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator/(const vec2& a, float s) { return vec2(a.x / s, a.y / s); }
inline vec2 operator+(const vec2& a, float s) { return vec2(a.x + s, a.y + s); }
inline vec2 operator-(const vec2& a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2 operator+(const uvec2& a, const vec2& b) { return vec2(a) + b; }

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator-(float s, const vec3& a) { return vec3(s - a.x, s - a.y, s - a.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, const vec3& b) { a = a + b; return a; }
inline vec3& operator-=(vec3& a, const vec3& b) { a = a - b; return a; }
inline vec3& operator*=(vec3& a, const vec3& b) { a = a * b; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }

inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator-(const vec4& a, const vec4& b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator/(const vec4& a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline vec4& operator+=(vec4& a, const vec4& b) { a = a + b; return a; }

inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator-(const ivec2& a, const ivec2& b) { return ivec2(a.x - b.x, a.y - b.y); }

// ---- matrices (column-major) ----------------------------------------------------------------
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
struct mat4x3 {  // 4 columns of 3 rows (gl_ObjectToWorldEXT)
    vec3 c[4];
};
struct mat3 {
    vec3 c[3];
    explicit mat3(const mat4x3& m) { c[0] = m.c[0]; c[1] = m.c[1]; c[2] = m.c[2]; }
};
struct mat3x4 {  // 3 columns of 4 rows
    vec4 c[3];
    mat3x4(const vec4& a, const vec4& b, const vec4& d) { c[0] = a; c[1] = b; c[2] = d; }
    vec4& operator[](int i) { return c[i]; }
};
inline vec4 operator*(const mat4& m, const vec4& v) {
    float o[4];
    const float* cols[4] = {&m.c[0].x, &m.c[1].x, &m.c[2].x, &m.c[3].x};
    for (int r = 0; r < 4; ++r) o[r] = ((cols[0][r] * v.x + cols[1][r] * v.y) + cols[2][r] * v.z) + cols[3][r] * v.w;
    return vec4(o[0], o[1], o[2], o[3]);
}
inline vec3 operator*(const mat3& m, const vec3& v) {
    float o[3];
    const float* cols[3] = {&m.c[0].x, &m.c[1].x, &m.c[2].x};
    for (int r = 0; r < 3; ++r) o[r] = (cols[0][r] * v.x + cols[1][r] * v.y) + cols[2][r] * v.z;
    return vec3(o[0], o[1], o[2]);
}
inline mat3x4 operator/(const mat3x4& m, float s) { return mat3x4(m.c[0] / s, m.c[1] / s, m.c[2] / s); }

// ---- built-in functions (GLSL specification definitions) ------------------------------------
inline float abs(float x) { return std::fabs(x); }
inline float min(float a, float b) { return std::fmin(a, b); }  // P8
inline float max(float a, float b) { return std::fmax(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline vec3 clamp(const vec3& v, float lo, float hi) { return vec3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)); }
inline float floor(float x) { return std::floor(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float log(float x) { return std::log(x); }
// P2: an integer exponent up to 8 is a repeated multiply
inline float pow(float x, float y) {
    if (y == std::rint(y) && y >= 1.0f && y <= 8.0f) {
        float r = x;
        for (int k = 1; k < (int)y; ++k) r = r * x;
        return r;
    }
    return std::pow(x, y);
}
inline float mod(float x, float y) { return x - y * std::floor(x / y); }
// P1: a NaN weight (0/0 of r/(tr+r)) counts as 0
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, float a) {
    if (a != a) a = 0.0f;
    return vec3(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a));
}
inline float dot(float a, float b) { return a * b; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline float length(const vec4& v) { return std::sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline float distance(const vec4& a, const vec4& b) { return length(a - b); }
inline vec3 normalize(const vec3& v) {
    float l = std::sqrt(dot(v, v));
    return vec3(v.x / l, v.y / l, v.z / l);
}
inline vec3 reflect(const vec3& I, const vec3& N) {
    float k = 2.0f * dot(N, I);
    return I - N * k;
}
inline vec3 refract(const vec3& I, const vec3& N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return vec3(0.0f);
    float s = eta * d + std::sqrt(k);
    return I * eta - N * s;
}

// ---- images and samplers ----------------------------------------------------------------------
float round_half(float f);  // RGBA16F store rounding (P6), defined in ref_shaders.cpp

enum { FMT_RGBA16F = 0, FMT_R8_SNORM = 1 };
struct image2D {
    float* px = nullptr;  // RGBA float storage holding the format's representable values
    int W = 0, H = 0, fmt = FMT_RGBA16F;
};
struct sampler2D {
    const image2D* img = nullptr;
};
struct accelerationStructureEXT {};

inline ivec2 imageSize(const image2D& im) { return ivec2(im.W, im.H); }
inline Texel imageLoad(const image2D& im, const ivec2& p) {  // P4: out of bounds reads 0
    if (p.x < 0 || p.y < 0 || p.x >= im.W || p.y >= im.H) return Texel(vec4(0.0f));
    const float* q = im.px + 4 * ((size_t)p.y * im.W + p.x);
    return Texel(vec4(q[0], q[1], q[2], q[3]));
}
inline void imageStore(image2D& im, const ivec2& p, const vec4& v) {  // out-of-bounds stores are dropped
    if (p.x < 0 || p.y < 0 || p.x >= im.W || p.y >= im.H) return;
    float* q = im.px + 4 * ((size_t)p.y * im.W + p.x);
    if (im.fmt == FMT_R8_SNORM) {  // P5
        q[0] = std::rint(clamp(v.x, -1.0f, 1.0f) * 127.0f) / 127.0f;
        q[1] = 0.0f;
        q[2] = 0.0f;
        q[3] = 1.0f;
    } else {
        q[0] = round_half(v.x);
        q[1] = round_half(v.y);
        q[2] = round_half(v.z);
        q[3] = round_half(v.w);
    }
}
inline const float* texel(const image2D& im, int x, int y) {
    x = x < 0 ? 0 : (x >= im.W ? im.W - 1 : x);
    y = y < 0 ? 0 : (y >= im.H ? im.H - 1 : y);
    return im.px + 4 * ((size_t)y * im.W + x);
}
// P9: a coordinate equal to a texel centre ((i + 0.5) / size in FP32) samples that texel; any other
// coordinate is FP32 bilinear (x = u * size - 0.5, weights (1 - f, f)), clamped to the edge
inline void axis(float u, int size, int& i0, float& f) {
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
inline vec4 textureLod(const sampler2D& s, const vec2& uv, float) {
    const image2D& im = *s.img;
    int ix, iy;
    float ax, ay;
    axis(uv.x, im.W, ix, ax);
    axis(uv.y, im.H, iy, ay);
    const float *t00 = texel(im, ix, iy), *t10 = texel(im, ix + 1, iy), *t01 = texel(im, ix, iy + 1), *t11 = texel(im, ix + 1, iy + 1);
    float o[4];
    for (int k = 0; k < 4; ++k) {
        float top = t00[k] * (1.0f - ax) + t10[k] * ax;
        float bot = t01[k] * (1.0f - ax) + t11[k] * ax;
        o[k] = top * (1.0f - ay) + bot * ay;
    }
    return vec4(o[0], o[1], o[2], o[3]);
}
inline vec4 textureLodOffset(const sampler2D& s, const vec2& uv, float, const ivec2& off) {
    const image2D& im = *s.img;
    int ix = (int)std::floor(uv.x * (float)im.W), iy = (int)std::floor(uv.y * (float)im.H);
    const float* t = texel(im, ix + off.x, iy + off.y);
    return vec4(t[0], t[1], t[2], t[3]);
}

// ---- ray tracing --------------------------------------------------------------------------------
struct Invocation {  // built-in variables of one shader invocation
    uvec3 launchID, launchSize, globalID;
    vec3 worldO, worldD;
    float hitT = 0.0f;
    int customIndex = 0, primitiveID = 0;
    mat4x3 objectToWorld;
};
extern thread_local Invocation* g_inv;
const uint gl_RayFlagsOpaqueEXT = 1u;
// traceRayEXT: traversal (unless cullMask == 0), then closest-hit or miss shader `missIndex`
void trace_ray(uint cullMask, int missIndex, const vec3& o, float tmin, const vec3& d, float tmax);
inline void traceRayEXT(const accelerationStructureEXT&, uint, uint cullMask, int, int, int missIndex, const vec3& o, float tmin,
                        const vec3& d, float tmax, int) {
    trace_ray(cullMask, missIndex, o, tmin, d, tmax);
}

}  // namespace rgsl

// built-ins, qualifiers and storage classes of the shader sources
#define gl_LaunchIDEXT (rgsl::g_inv->launchID)
#define gl_LaunchSizeEXT (rgsl::g_inv->launchSize)
#define gl_GlobalInvocationID (rgsl::g_inv->globalID)
#define gl_WorldRayOriginEXT (rgsl::g_inv->worldO)
#define gl_WorldRayDirectionEXT (rgsl::g_inv->worldD)
#define gl_HitTEXT (rgsl::g_inv->hitT)
#define gl_InstanceCustomIndexEXT (rgsl::g_inv->customIndex)
#define gl_PrimitiveID (rgsl::g_inv->primitiveID)
#define gl_ObjectToWorldEXT (rgsl::g_inv->objectToWorld)
#define layout(...)
#define uniform struct
#define buffer struct
#define restrict
#define hitAttributeEXT thread_local
#define rayPayloadEXT thread_local
#define rayPayloadInEXT thread_local
// every shader shares ONE payload (payload.h:29-43): `payload` is a per-namespace pointer to it
#define payload (*rgref_payload)

#define RGSL_IMPORT                                                                                          \
    using namespace rgsl;                                                                                    \
    using rgsl::abs; using rgsl::min; using rgsl::max; using rgsl::clamp; using rgsl::floor; using rgsl::sqrt; \
    using rgsl::log; using rgsl::pow; using rgsl::mod; using rgsl::mix; using rgsl::dot; using rgsl::length;  \
    using rgsl::distance; using rgsl::normalize; using rgsl::reflect; using rgsl::refract
