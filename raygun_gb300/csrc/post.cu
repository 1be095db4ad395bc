// post.cu -- screen-space roughness approximation, postprocess composite and FXAA.
//
// Replaces the compute passes of Raytracer::doRaytracing (render/raytracer.cpp:106-142):
//   rough_prepare.comp:28-54, 10 x (rough_blur_h.comp, rough_blur_v.comp) = rough_blur.h:23-40,
//   postprocess.comp:28-50, fxaa.comp:29-36 with FXAA 3.11 PC quality preset 39 (fxaa.h:615-1136).
//
// The reference runs 22 full-screen dispatches with image barriers between them.  Here one kernel
// does prepare + all 20 blur passes + composite per 32x16 tile: the tile and a 10-pixel halo live
// in shared memory, so the intermediate roughColorsA/B images never touch HBM (a blur pass moves
// colour by one pixel, so 10 passes per axis need exactly 10 pixels of halo; the transition mask
// of the halo needs one more ring of the G-buffer).  Every store is rounded to the storage format
// of the reference image (RGBA16F, R8_SNORM for the transition mask) so the values match the
// reference's pass-by-pass evaluation.  Out-of-image loads read 0 as robust image access does.
// FXAA runs as a second kernel: its edge search reaches ~27 pixels, too far for a halo.
#include <atomic>

#include "rg_internal.cuh"

namespace rg {
namespace {

constexpr int TW = 32, TH = 16, HALO = 10;
constexpr int RW = TW + 2 * HALO, RH = TH + 2 * HALO;  // blur region
constexpr int GW = RW + 2, GH = RH + 2;                // G-buffer region (one more ring)
constexpr int kPostThreads = 256;

__device__ __forceinline__ float4 unpack_half4(uint2 v) {
    __half2 lo = *reinterpret_cast<__half2*>(&v.x), hi = *reinterpret_cast<__half2*>(&v.y);
    float2 a = __half22float2(lo), b = __half22float2(hi);
    return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ uint2 pack_half4(float a, float b, float c, float d) {
    __half2 lo = __floats2half2_rn(a, b), hi = __floats2half2_rn(c, d);
    return make_uint2(*reinterpret_cast<uint32_t*>(&lo), *reinterpret_cast<uint32_t*>(&hi));
}
__device__ __forceinline__ float rh(float x) { return __half2float(__float2half_rn(x)); }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float mixs(float x, float y, float a) { return x * (1.0f - a) + y * a; }

__device__ __forceinline__ float dist4(float4 a, float4 b) {
    float d0 = a.x - b.x, d1 = a.y - b.y, d2 = a.z - b.z, d3 = a.w - b.w;
    return sqrtf(((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3);
}

struct RoughSmem {
    uint2 rough[GH][GW];   // RGBA16F
    uint2 normal[GH][GW];
    float trans[RH][RW];
    __half col[2][3][RH][RW];  // ping-pong roughColorsA (0) / roughColorsB (1), rgb planes
};

__global__ void __launch_bounds__(kPostThreads) k_rough_post(const PostParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RoughSmem& S = *reinterpret_cast<RoughSmem*>(smem_raw);
    const int W = (int)P.W, H = (int)P.H;
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    const int gx0 = x0 - HALO - 1, gy0 = y0 - HALO - 1;
    // 1. G-buffer region (out-of-image = 0)
    for (int i = threadIdx.x; i < GW * GH; i += kPostThreads) {
        int ly = i / GW, lx = i - ly * GW;
        int x = gx0 + lx, y = gy0 + ly;
        uint2 r = make_uint2(0, 0), n = make_uint2(0, 0);
        if (x >= 0 && y >= 0 && x < W && y < H) {
            size_t pix = (size_t)y * W + x;
            r = __ldg(P.rough + pix);
            n = __ldg(P.normal + pix);
        }
        S.rough[ly][lx] = r;
        S.normal[ly][lx] = n;
    }
    __syncthreads();
    // 2. rough_prepare on the blur region: transition mask (R8_SNORM), A = B = rough
    for (int i = threadIdx.x; i < RW * RH; i += kPostThreads) {
        int ly = i / RW, lx = i - ly * RW;
        int gx = lx + 1, gy = ly + 1;
        int x = x0 - HALO + lx, y = y0 - HALO + ly;
        float4 r = unpack_half4(S.rough[gy][gx]);
        float t = 0.0f;
        if (x >= 0 && y >= 0 && x < W && y < H) {
            float4 ru = unpack_half4(S.rough[gy + 1][gx]), rd = unpack_half4(S.rough[gy - 1][gx]);
            float4 rl = unpack_half4(S.rough[gy][gx + 1]), rr = unpack_half4(S.rough[gy][gx - 1]);
            float4 n = unpack_half4(S.normal[gy][gx]);
            float4 nu = unpack_half4(S.normal[gy + 1][gx]), nd = unpack_half4(S.normal[gy - 1][gx]);
            float4 nl = unpack_half4(S.normal[gy][gx + 1]), nr = unpack_half4(S.normal[gy][gx - 1]);
            float uf = fminf(ru.w, r.w) * clampf(1.0f - dist4(nu, n) * 10.0f, 0.0f, 1.0f);
            float df = fminf(rd.w, r.w) * clampf(1.0f - dist4(nd, n) * 10.0f, 0.0f, 1.0f);
            float lf = fminf(rl.w, r.w) * clampf(1.0f - dist4(nl, n) * 10.0f, 0.0f, 1.0f);
            float rf = fminf(rr.w, r.w) * clampf(1.0f - dist4(nr, n) * 10.0f, 0.0f, 1.0f);
            float tt = fminf(fminf(fminf(uf, df), lf), rf);
            t = rintf(clampf(tt, -1.0f, 1.0f) * 127.0f) / 127.0f;
        }
        S.trans[ly][lx] = t;
        __half hr = __float2half_rn(r.x), hg = __float2half_rn(r.y), hb = __float2half_rn(r.z);
        S.col[0][0][ly][lx] = hr; S.col[0][1][ly][lx] = hg; S.col[0][2][ly][lx] = hb;
        S.col[1][0][ly][lx] = hr; S.col[1][1][ly][lx] = hg; S.col[1][2][ly][lx] = hb;
    }
    __syncthreads();
    // 3. 10 x (H: A -> B, V: B -> A); out-of-region neighbours read 0 (their error never reaches
    //    the tile: it moves one pixel per pass along the pass axis)
    for (int it = 0; it < 10; ++it) {
        for (int pass = 0; pass < 2; ++pass) {
            const int src = pass, dst = pass ^ 1;
            const int ox = pass == 0 ? 1 : 0, oy = pass == 0 ? 0 : 1;
            for (int i = threadIdx.x; i < RW * RH; i += kPostThreads) {
                int ly = i / RW, lx = i - ly * RW;
                float t = S.trans[ly][lx];
                if (t < 0.001f) continue;
                float w = (1.0f - t) - t;
                int ax = lx + ox, ay = ly + oy, bx = lx - ox, by = ly - oy;
                bool aok = ax < RW && ay < RH, bok = bx >= 0 && by >= 0;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    float c = __half2float(S.col[src][k][ly][lx]);
                    float a = aok ? __half2float(S.col[src][k][ay][ax]) : 0.0f;
                    float b = bok ? __half2float(S.col[src][k][by][bx]) : 0.0f;
                    S.col[dst][k][ly][lx] = __float2half_rn((c * w + a * t) + b * t);
                }
            }
            __syncthreads();
        }
    }
    // 4. postprocess.comp:28-50 on the tile
    for (int i = threadIdx.x; i < TW * TH; i += kPostThreads) {
        int ty = i / TW, tx = i - ty * TW;
        int x = x0 + tx, y = y0 + ty;
        if (x >= W || y >= H) continue;
        size_t pix = (size_t)y * W + x;
        int lx = tx + HALO, ly = ty + HALO;
        float4 b = unpack_half4(__ldg(P.base + pix));
        float r[3] = {__half2float(S.col[0][0][ly][lx]), __half2float(S.col[0][1][ly][lx]), __half2float(S.col[0][2][ly][lx])};
        float bb[3] = {b.x, b.y, b.z};
        float col[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) col[k] = clampf(mixs(bb[k], r[k], b.w), 0.0f, 1.0f);
        float luma = (col[0] * 0.299f + col[1] * 0.587f) + col[2] * 0.114f;
#pragma unroll
        for (int k = 0; k < 3; ++k) col[k] = mixs(col[k], P.fade[k], P.fade[3]);
        float ra = unpack_half4(S.rough[ly + 1][lx + 1]).w;
        if (P.showAlpha) {
            float l = rh(luma);
            P.finalImg[pix] = pack_half4(l, l, l, l);
        } else {
            P.finalImg[pix] = pack_half4(col[0], col[1], col[2], luma);
        }
        if (P.dbgTransition) P.dbgTransition[pix] = P.showAlpha ? 1.0f : S.trans[ly][lx];
        if (P.dbgA) {
            if (P.showAlpha) P.dbgA[pix] = pack_half4(ra, ra, ra, ra);
            else P.dbgA[pix] = pack_half4(r[0], r[1], r[2], ra);
        }
        if (P.dbgB) {
            float g[3] = {__half2float(S.col[1][0][ly][lx]), __half2float(S.col[1][1][ly][lx]), __half2float(S.col[1][2][ly][lx])};
            if (P.showAlpha) P.dbgB[pix] = pack_half4(ra, ra, ra, ra);
            else P.dbgB[pix] = pack_half4(g[0], g[1], g[2], ra);
        }
    }
}

// postprocess.comp:41-49: with showAlpha the G-buffer images become .aaaa (after the fused pass
// has consumed them)
__global__ void k_show_alpha(uint2* base, uint2* normal, uint2* rough, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint2* imgs[3] = {base, normal, rough};
    for (int k = 0; k < 3; ++k) {
        float a = unpack_half4(imgs[k][i]).w;
        imgs[k][i] = pack_half4(a, a, a, a);
    }
}

// ---- FXAA 3.11, PC quality, preset 39, green as luma --------------------------------------------
struct Tex {
    const uint2* img;
    int W, H;
    __device__ __forceinline__ float4 texel(int x, int y) const {
        x = min(max(x, 0), W - 1);
        y = min(max(y, 0), H - 1);
        return unpack_half4(__ldg(img + (size_t)y * W + x));
    }
    __device__ __forceinline__ float green(int x, int y) const {
        x = min(max(x, 0), W - 1);
        y = min(max(y, 0), H - 1);
        const __half* h = reinterpret_cast<const __half*>(img + (size_t)y * W + x);
        return __half2float(__ldg(h + 1));
    }
    // a coordinate equal to a texel centre ((i + 0.5) / size in FP32) samples that texel, as the
    // hardware's subtexel grid does; any other coordinate is FP32 bilinear x = u*size - 0.5 with
    // weights (1-f, f); clamp to edge
    __device__ __forceinline__ static void axis(float u, int size, int& i0, float& f) {
        int c = (int)floorf(u * (float)size);
        if (u == ((float)c + 0.5f) / (float)size) {
            i0 = c;
            f = 0.0f;
            return;
        }
        float fx = u * (float)size - 0.5f;
        float x0 = floorf(fx);
        f = fx - x0;
        i0 = (int)x0;
    }
    __device__ __forceinline__ void coords(float u, float v, int& ix, int& iy, float& ax, float& ay) const {
        axis(u, W, ix, ax);
        axis(v, H, iy, ay);
    }
    __device__ __forceinline__ float lumaAt(float u, float v) const {
        int ix, iy;
        float ax, ay;
        coords(u, v, ix, iy, ax, ay);
        float t00 = green(ix, iy), t10 = green(ix + 1, iy), t01 = green(ix, iy + 1), t11 = green(ix + 1, iy + 1);
        float top = t00 * (1.0f - ax) + t10 * ax;
        float bot = t01 * (1.0f - ax) + t11 * ax;
        return top * (1.0f - ay) + bot * ay;
    }
    __device__ __forceinline__ float4 bilinear(float u, float v) const {
        int ix, iy;
        float ax, ay;
        coords(u, v, ix, iy, ax, ay);
        float4 t00 = texel(ix, iy), t10 = texel(ix + 1, iy), t01 = texel(ix, iy + 1), t11 = texel(ix + 1, iy + 1);
        float4 o;
        float topx = t00.x * (1.0f - ax) + t10.x * ax, botx = t01.x * (1.0f - ax) + t11.x * ax;
        float topy = t00.y * (1.0f - ax) + t10.y * ax, boty = t01.y * (1.0f - ax) + t11.y * ax;
        float topz = t00.z * (1.0f - ax) + t10.z * ax, botz = t01.z * (1.0f - ax) + t11.z * ax;
        o.x = topx * (1.0f - ay) + botx * ay;
        o.y = topy * (1.0f - ay) + boty * ay;
        o.z = topz * (1.0f - ay) + botz * ay;
        o.w = 0.0f;
        return o;
    }
};

__device__ float4 fxaa_pixel(const Tex& T, int x, int y) {
    const float P_[12] = {1.0f, 1.0f, 1.0f, 1.0f, 1.0f, 1.5f, 2.0f, 2.0f, 2.0f, 2.0f, 4.0f, 8.0f};
    const float subpix = 1.0f, edgeThreshold = 0.063f, edgeThresholdMin = 0.0312f;
    const float rcpW = 1.0f / (float)T.W, rcpH = 1.0f / (float)T.H;
    float posMx = ((float)x + 0.5f) / (float)T.W;
    float posMy = ((float)y + 0.5f) / (float)T.H;
    float4 rgbyM = T.texel(x, y);
    float lumaM = rgbyM.y;
    float lumaS = T.green(x, y + 1), lumaE = T.green(x + 1, y), lumaN = T.green(x, y - 1), lumaW = T.green(x - 1, y);
    float maxSM = fmaxf(lumaS, lumaM), minSM = fminf(lumaS, lumaM);
    float maxESM = fmaxf(lumaE, maxSM), minESM = fminf(lumaE, minSM);
    float maxWN = fmaxf(lumaN, lumaW), minWN = fminf(lumaN, lumaW);
    float rangeMax = fmaxf(maxWN, maxESM), rangeMin = fminf(minWN, minESM);
    float rangeMaxScaled = rangeMax * edgeThreshold;
    float range = rangeMax - rangeMin;
    float rangeMaxClamped = fmaxf(edgeThresholdMin, rangeMaxScaled);
    if (range < rangeMaxClamped) return rgbyM;
    float lumaNW = T.green(x - 1, y - 1), lumaSE = T.green(x + 1, y + 1);
    float lumaNE = T.green(x + 1, y - 1), lumaSW = T.green(x - 1, y + 1);
    float lumaNS = lumaN + lumaS, lumaWE = lumaW + lumaE;
    float subpixRcpRange = 1.0f / range;
    float subpixNSWE = lumaNS + lumaWE;
    float edgeHorz1 = (-2.0f * lumaM) + lumaNS, edgeVert1 = (-2.0f * lumaM) + lumaWE;
    float lumaNESE = lumaNE + lumaSE, lumaNWNE = lumaNW + lumaNE;
    float edgeHorz2 = (-2.0f * lumaE) + lumaNESE, edgeVert2 = (-2.0f * lumaN) + lumaNWNE;
    float lumaNWSW = lumaNW + lumaSW, lumaSWSE = lumaSW + lumaSE;
    float edgeHorz4 = (fabsf(edgeHorz1) * 2.0f) + fabsf(edgeHorz2);
    float edgeVert4 = (fabsf(edgeVert1) * 2.0f) + fabsf(edgeVert2);
    float edgeHorz3 = (-2.0f * lumaW) + lumaNWSW, edgeVert3 = (-2.0f * lumaS) + lumaSWSE;
    float edgeHorz = fabsf(edgeHorz3) + edgeHorz4, edgeVert = fabsf(edgeVert3) + edgeVert4;
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
    bool pairN = fabsf(gradientN) >= fabsf(gradientS);
    float gradient = fmaxf(fabsf(gradientN), fabsf(gradientS));
    if (pairN) lengthSign = -lengthSign;
    float subpixC = clampf(fabsf(subpixB) * subpixRcpRange, 0.0f, 1.0f);
    float posBx = posMx, posBy = posMy;
    float offNPx = (!horzSpan) ? 0.0f : rcpW;
    float offNPy = (horzSpan) ? 0.0f : rcpH;
    if (!horzSpan) posBx = posBx + lengthSign * 0.5f;
    if (horzSpan) posBy = posBy + lengthSign * 0.5f;
    float posNx = posBx - offNPx * P_[0], posNy = posBy - offNPy * P_[0];
    float posPx = posBx + offNPx * P_[0], posPy = posBy + offNPy * P_[0];
    float subpixD = ((-2.0f) * subpixC) + 3.0f;
    float lumaEndN = T.lumaAt(posNx, posNy);
    float subpixE = subpixC * subpixC;
    float lumaEndP = T.lumaAt(posPx, posPy);
    if (!pairN) lumaNN = lumaSS;
    float gradientScaled = gradient * 1.0f / 4.0f;
    float lumaMM = lumaM - lumaNN * 0.5f;
    float subpixF = subpixD * subpixE;
    bool lumaMLTZero = lumaMM < 0.0f;
    lumaEndN = lumaEndN - lumaNN * 0.5f;
    lumaEndP = lumaEndP - lumaNN * 0.5f;
    bool doneN = fabsf(lumaEndN) >= gradientScaled;
    bool doneP = fabsf(lumaEndP) >= gradientScaled;
    if (!doneN) { posNx = posNx - offNPx * P_[1]; posNy = posNy - offNPy * P_[1]; }
    bool doneNP = (!doneN) || (!doneP);
    if (!doneP) { posPx = posPx + offNPx * P_[1]; posPy = posPy + offNPy * P_[1]; }
#pragma unroll
    for (int k = 2; k < 12; ++k) {
        if (!doneNP) break;
        if (!doneN) lumaEndN = T.lumaAt(posNx, posNy);
        if (!doneP) lumaEndP = T.lumaAt(posPx, posPy);
        if (!doneN) lumaEndN = lumaEndN - lumaNN * 0.5f;
        if (!doneP) lumaEndP = lumaEndP - lumaNN * 0.5f;
        doneN = fabsf(lumaEndN) >= gradientScaled;
        doneP = fabsf(lumaEndP) >= gradientScaled;
        if (!doneN) { posNx = posNx - offNPx * P_[k]; posNy = posNy - offNPy * P_[k]; }
        doneNP = (!doneN) || (!doneP);
        if (!doneP) { posPx = posPx + offNPx * P_[k]; posPy = posPy + offNPy * P_[k]; }
    }
    float dstN = posMx - posNx, dstP = posPx - posMx;
    if (!horzSpan) dstN = posMy - posNy;
    if (!horzSpan) dstP = posPy - posMy;
    bool goodSpanN = (lumaEndN < 0.0f) != lumaMLTZero;
    float spanLength = (dstP + dstN);
    bool goodSpanP = (lumaEndP < 0.0f) != lumaMLTZero;
    float spanLengthRcp = 1.0f / spanLength;
    bool directionN = dstN < dstP;
    float dst = fminf(dstN, dstP);
    bool goodSpan = directionN ? goodSpanN : goodSpanP;
    float subpixG = subpixF * subpixF;
    float pixelOffset = (dst * (-spanLengthRcp)) + 0.5f;
    float subpixH = subpixG * subpix;
    float pixelOffsetGood = goodSpan ? pixelOffset : 0.0f;
    float pixelOffsetSubpix = fmaxf(pixelOffsetGood, subpixH);
    if (!horzSpan) posMx = posMx + pixelOffsetSubpix * lengthSign;
    if (horzSpan) posMy = posMy + pixelOffsetSubpix * lengthSign;
    float4 o = T.bilinear(posMx, posMy);
    o.w = lumaM;
    return o;
}

__global__ void __launch_bounds__(256) k_fxaa(const PostParams P) {
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= (int)P.W || y >= (int)P.H) return;
    size_t pix = (size_t)y * P.W + x;
    Tex T{P.finalImg, (int)P.W, (int)P.H};
    float4 o;
    if (P.fxaa) {
        o = fxaa_pixel(T, x, y);
        uint2 hv = pack_half4(o.x, o.y, o.z, o.w);
        if (P.fxaaOut) P.fxaaOut[pix] = hv;
        o = unpack_half4(hv);
    } else {
        o = unpack_half4(__ldg(P.finalImg + pix));
    }
    P.framebuffer[pix] = o;
}

__global__ void k_f32_to_h16(const float4* __restrict__ in, uint2* __restrict__ out, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) {
        float4 v = in[i];
        out[i] = pack_half4(v.x, v.y, v.z, v.w);
    }
}
__global__ void k_h16_to_f32(const uint2* __restrict__ in, float4* __restrict__ out, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = unpack_half4(in[i]);
}
__global__ void k_r32_to_rgba(const float* __restrict__ in, float4* __restrict__ out, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float4(in[i], 0.0f, 0.0f, 1.0f);
}

}  // namespace

cudaError_t f32_to_h16(const float4* in, uint2* out, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_f32_to_h16<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, n);
    count_launch();
    return cudaGetLastError();
}
cudaError_t h16_to_f32(const uint2* in, float4* out, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_h16_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, n);
    count_launch();
    return cudaGetLastError();
}
cudaError_t r32_to_rgba(const float* in, float4* out, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_r32_to_rgba<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, out, n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_rough_post(const PostParams& p, cudaStream_t s) {
    static std::atomic<bool> attr{false};
    const int smem = (int)sizeof(RoughSmem);
    if (!attr.load(std::memory_order_acquire)) {
        cudaError_t e = cudaFuncSetAttribute(k_rough_post, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr.store(true, std::memory_order_release);
    }
    dim3 grid((p.W + TW - 1) / TW, (p.H + TH - 1) / TH);
    k_rough_post<<<grid, kPostThreads, smem, s>>>(p);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !p.showAlpha) return e;
    size_t n = (size_t)p.W * p.H;
    k_show_alpha<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(const_cast<uint2*>(p.base), const_cast<uint2*>(p.normal),
                                                            const_cast<uint2*>(p.rough), n);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_fxaa(const PostParams& p, cudaStream_t s) {
    dim3 grid((p.W + 15) / 16, (p.H + 15) / 16);
    k_fxaa<<<grid, 256, 0, s>>>(p);
    count_launch();
    return cudaGetLastError();
}

}  // namespace rg
