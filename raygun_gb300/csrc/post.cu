// post.cu -- screen-space roughness approximation, postprocess composite and FXAA.
//
// Replaces the compute passes of Raytracer::doRaytracing (render/raytracer.cpp:106-142):
//   rough_prepare.comp:28-54, 10 x (rough_blur_h.comp, rough_blur_v.comp) = rough_blur.h:23-40,
//   postprocess.comp:28-50, fxaa.comp:29-36 with FXAA 3.11 PC quality preset 39 (fxaa.h:615-1136).
//
// The reference runs 22 full-screen dispatches with image barriers between them.  Here one
// persistent kernel does prepare + all 20 blur passes + composite per 64x32 tile: the tile and a
// 10-pixel halo live in shared memory, so the intermediate roughColorsA/B images never touch HBM (a
// blur pass moves colour by one pixel, so 10 passes per axis need exactly 10 pixels of halo; the
// transition mask of the halo needs one more ring of the G-buffer).  Every store is rounded to the
// storage format of the reference image (RGBA16F, R8_SNORM for the transition mask) so the values
// match the reference's pass-by-pass evaluation.  Out-of-image loads read 0 as robust image access
// does.  FXAA runs as a second kernel: its edge search reaches ~27 pixels, too far for a halo.
//
// Per block (one per SM, 512 threads), tiles in turn:
//   * the rough and normal G-buffer region of the tile is staged by TMA (a 2-D tensor map of 8-byte
//     pixels; the out-of-image part is zero-filled by the copy), double-buffered: the next tile's
//     region lands while this tile blurs.  Images of odd width (row pitch not a multiple of 16 bytes)
//     are staged by plain loads into the same layout;
//   * only pixel pairs with a transition (t >= 0.001; a few percent of a game frame) are blurred: the
//     others keep their value, which both planes already hold.  They are listed once per tile;
//   * each blur pass computes only the region later passes still read -- the halo shrinks by one
//     pixel per pass along the pass's axis -- 30 pixel updates per output pixel instead of 73 when
//     every pixel has a transition;
//   * two horizontally adjacent pixels per thread (half2 loads and stores), FP32 arithmetic in the
//     reference's operation order, never contracted, so the values are the reference's;
//   * a tile whose transition mask is below 0.001 everywhere skips the blur (its colours stay).
#include <algorithm>
#include <atomic>
#include <cstring>

#include "rg_internal.cuh"
#include "rg_tma.cuh"

namespace rg {
namespace {

constexpr int TW = 64, TH = 32, HALO = 10;
constexpr int RW = TW + 2 * HALO, RH = TH + 2 * HALO;  // blur region 84 x 52 (tile at [10, 74) x [10, 42))
constexpr int SW = RW + 4, SH = RH + 2;                // staged G-buffer region 88 x 54: columns x0-12 .. x0+75
                                                       // (an even first column for the TMA), rows y0-11 .. y0+42
constexpr int CP = 2, CW = RW + 2 * CP;                // colour planes: 2 zero columns each side, 88 halves a row
#ifndef RG_POST_THREADS
#define RG_POST_THREADS 1024
#endif
constexpr int kPostThreads = RG_POST_THREADS;

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

// (c*w + a*t) + b*t of the reference's blur, each product and sum one IEEE round-to-nearest
// operation (the _rn intrinsics are never contracted into fused multiply-adds)
__device__ __forceinline__ float blur_mix(float c, float a, float b, float w, float t) {
    return __fadd_rn(__fadd_rn(__fmul_rn(c, w), __fmul_rn(a, t)), __fmul_rn(b, t));
}

struct RoughSmem {
    uint2 rough[2][SH][SW];     // staged G-buffer (RGBA16F), two stages: 38,016 B each, 128-byte multiples
    uint2 normal[2][SH][SW];
    __half col[2][3][RH][CW];   // ping-pong roughColorsA (0) / roughColorsB (1), rgb planes
    int8_t trans[RH][RW];       // roughTransitions as its R8_SNORM integer q (value q / 127)
    uint16_t active[RH * RW / 2];  // the pixel pairs with a transition: row * 64 + pair column
    float2 tw[256];                // per mask value q: t = q / 127 and w = (1 - t) - t (index q + 128)
    uint64_t mbar[2];
    uint32_t nActive;
};
static_assert(sizeof(uint2) * SH * SW % 128 == 0, "TMA destinations 128-byte aligned");

// one blur pass (rough_blur.h:23-40) over the active pixel pairs inside [xa, xb) x rows [ya, yb) of
// the blur region, src plane set -> the other; H: neighbours x -+ 1, V: y -+ 1.  out = (c*w + a*t) +
// b*t with a the +1 and b the -1 neighbour, w = (1 - t) - t; a pixel with t < 0.001 keeps its value
// (pairs of two such pixels are not in the list: both planes already hold their value).
template <bool H>
__device__ __forceinline__ void blur_pass(RoughSmem& S, int nActive, int src, int xa, int xb, int ya, int yb) {
    for (int i = threadIdx.x; i < nActive; i += kPostThreads) {
        const uint32_t e = S.active[i];
        const int ly = (int)(e >> 6), lx = 2 * (int)(e & 63u);
        if (lx < xa || lx >= xb || ly < ya || ly >= yb) continue;
        const char2 q = *reinterpret_cast<const char2*>(&S.trans[ly][lx]);
        const float2 tw0 = S.tw[q.x + 128], tw1 = S.tw[q.y + 128];
        const float t0 = tw0.x, t1 = tw1.x, w0 = tw0.y, w1 = tw1.y;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const __half2* row = reinterpret_cast<const __half2*>(&S.col[src][k][ly][CP + lx]);
            const __half2 c = row[0];
            float2 cf = __half22float2(c), af, bf;
            if (H) {
                const float l = __high2float(row[-1]), r = __low2float(row[1]);
                af = make_float2(cf.y, r);
                bf = make_float2(l, cf.x);
            } else {
                af = __half22float2(*reinterpret_cast<const __half2*>(&S.col[src][k][ly + 1][CP + lx]));
                bf = __half22float2(*reinterpret_cast<const __half2*>(&S.col[src][k][ly - 1][CP + lx]));
            }
            __half2 o = __floats2half2_rn(blur_mix(cf.x, af.x, bf.x, w0, t0), blur_mix(cf.y, af.y, bf.y, w1, t1));
            if (q.x <= 0) o = __halves2half2(__low2half(c), __high2half(o));
            if (q.y <= 0) o = __halves2half2(__low2half(o), __high2half(c));
            *reinterpret_cast<__half2*>(&S.col[src ^ 1][k][ly][CP + lx]) = o;
        }
    }
}

// the G-buffer region of tile (x0, y0) into stage st: TMA (thread 0 issues, completes on mbar[st])
// or plain loads by every thread (the caller synchronises)
__device__ __forceinline__ void stage_tile(RoughSmem& S, const PostParams& P, const CUtensorMap* mapRough, const CUtensorMap* mapNormal,
                                           bool tma, int st, int x0, int y0) {
    const int gx0 = x0 - HALO - 2, gy0 = y0 - HALO - 1;
    if (tma) {
        if (threadIdx.x == 0) {
            async_proxy_fence();  // the stage was last read through the generic proxy
            mbar_expect_tx(&S.mbar[st], 2u * (uint32_t)sizeof(S.rough[0]));
            tma_load_2d(&S.rough[st][0][0], mapRough, gx0, gy0, &S.mbar[st]);
            tma_load_2d(&S.normal[st][0][0], mapNormal, gx0, gy0, &S.mbar[st]);
        }
        return;
    }
    const int W = (int)P.W, H = (int)P.H;
    for (int i = threadIdx.x; i < SW * SH; i += kPostThreads) {
        const int ly = i / SW, lx = i - ly * SW;
        const int x = gx0 + lx, y = gy0 + ly;
        uint2 r = make_uint2(0, 0), n = make_uint2(0, 0);
        if (x >= 0 && y >= 0 && x < W && y < H) {
            const size_t pix = (size_t)y * W + x;
            r = __ldg(P.rough + pix);
            n = __ldg(P.normal + pix);
        }
        S.rough[st][ly][lx] = r;
        S.normal[st][ly][lx] = n;
    }
}

__global__ void __launch_bounds__(kPostThreads, 1) k_rough_post(const __grid_constant__ CUtensorMap mapRough,
                                                                const __grid_constant__ CUtensorMap mapNormal, const PostParams P,
                                                                int tma) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    RoughSmem& S = *reinterpret_cast<RoughSmem*>(smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127));
    const int W = (int)P.W, H = (int)P.H;
    const int tilesX = (W + TW - 1) / TW, nTiles = tilesX * ((H + TH - 1) / TH);
    if (threadIdx.x == 0) {
        mbar_init(&S.mbar[0], 1);
        mbar_init(&S.mbar[1], 1);
        mbar_init_fence();
        S.nActive = 0;
    }
    for (int q = threadIdx.x; q < 256; q += kPostThreads) {
        const float t = (float)(q - 128) / 127.0f;
        S.tw[q] = make_float2(t, (1.0f - t) - t);
    }
    for (int i = threadIdx.x; i < 2 * 3 * RH; i += kPostThreads) {  // the zero columns either side of each plane row
        __half* row = &S.col[0][0][0][0] + (size_t)i * CW;
        row[0] = row[1] = row[CW - 2] = row[CW - 1] = __float2half_rn(0.0f);
    }
    __syncthreads();
    int k = 0;
    if ((int)blockIdx.x < nTiles)
        stage_tile(S, P, &mapRough, &mapNormal, tma != 0, 0, (blockIdx.x % tilesX) * TW, (blockIdx.x / tilesX) * TH);
    for (int tile = blockIdx.x; tile < nTiles; tile += gridDim.x, ++k) {
        const int st = k & 1;
        const int x0 = (tile % tilesX) * TW, y0 = (tile / tilesX) * TH;
        if (tma) {
            const bool ok = mbar_wait(&S.mbar[st], (uint32_t)(k >> 1) & 1u, P.status, P.waitLimit);
            if (__syncthreads_or(!ok)) {  // the copy did not land: wait once more (bounded) for it, then give up
                if (threadIdx.x == 0) mbar_wait(&S.mbar[st], (uint32_t)(k >> 1) & 1u, nullptr);
                __syncthreads();
                return;
            }
        } else {
            __syncthreads();
        }
        // rough_prepare.comp:28-54 over the blur region: the transition mask, A = B = rough
        int busy = 0;
        for (int i = threadIdx.x; i < RW * RH; i += kPostThreads) {
            const int ly = i / RW, lx = i - ly * RW;
            const int sx = lx + 2, sy = ly + 1;
            const int x = x0 - HALO + lx, y = y0 - HALO + ly;
            const float4 r = unpack_half4(S.rough[st][sy][sx]);
            int q = 0;
            if (x >= 0 && y >= 0 && x < W && y < H) {
                const float4 ru = unpack_half4(S.rough[st][sy + 1][sx]), rd = unpack_half4(S.rough[st][sy - 1][sx]);
                const float4 rl = unpack_half4(S.rough[st][sy][sx + 1]), rr = unpack_half4(S.rough[st][sy][sx - 1]);
                const float4 n = unpack_half4(S.normal[st][sy][sx]);
                const float4 nu = unpack_half4(S.normal[st][sy + 1][sx]), nd = unpack_half4(S.normal[st][sy - 1][sx]);
                const float4 nl = unpack_half4(S.normal[st][sy][sx + 1]), nr = unpack_half4(S.normal[st][sy][sx - 1]);
                const float uf = fminf(ru.w, r.w) * clampf(1.0f - dist4(nu, n) * 10.0f, 0.0f, 1.0f);
                const float df = fminf(rd.w, r.w) * clampf(1.0f - dist4(nd, n) * 10.0f, 0.0f, 1.0f);
                const float lf = fminf(rl.w, r.w) * clampf(1.0f - dist4(nl, n) * 10.0f, 0.0f, 1.0f);
                const float rf = fminf(rr.w, r.w) * clampf(1.0f - dist4(nr, n) * 10.0f, 0.0f, 1.0f);
                const float tt = fminf(fminf(fminf(uf, df), lf), rf);
                q = (int)rintf(clampf(tt, -1.0f, 1.0f) * 127.0f);
            }
            S.trans[ly][lx] = (int8_t)q;
            busy |= q > 0;
            const __half hr = __float2half_rn(r.x), hg = __float2half_rn(r.y), hb = __float2half_rn(r.z);
            S.col[0][0][ly][CP + lx] = hr; S.col[0][1][ly][CP + lx] = hg; S.col[0][2][ly][CP + lx] = hb;
            S.col[1][0][ly][CP + lx] = hr; S.col[1][1][ly][CP + lx] = hg; S.col[1][2][ly][CP + lx] = hb;
        }
        busy = __syncthreads_or(busy);
        // the next tile's G-buffer into the other stage (its last reader, the previous tile's prepare, is done)
        const int next = tile + (int)gridDim.x;
        if (next < nTiles) stage_tile(S, P, &mapRough, &mapNormal, tma != 0, st ^ 1, (next % tilesX) * TW, (next / tilesX) * TH);
        // 10 x (H: A -> B, V: B -> A), each over the region the later passes read: after V_i the tile
        // plus j = 10 - i pixels a side; H_i computes that plus one row a side (rounded out to pairs)
        if (busy) {
            // the pairs with a transition (a few percent of a game frame's pixels), listed once per tile
            for (int pw = threadIdx.x & ~31; pw < RH * RW / 2; pw += kPostThreads) {  // warp-uniform trip count
                const int p = pw + (threadIdx.x & 31);
                const int ly = p / (RW / 2), pc = p - ly * (RW / 2);
                bool on = false;
                if (p < RH * RW / 2) {
                    const char2 q = *reinterpret_cast<const char2*>(&S.trans[ly][2 * pc]);
                    on = q.x > 0 || q.y > 0;
                }
                const unsigned m = __ballot_sync(0xFFFFFFFFu, on);
                uint32_t base = 0;
                if ((threadIdx.x & 31) == 0 && m) base = atomicAdd(&S.nActive, (uint32_t)__popc(m));
                base = __shfl_sync(0xFFFFFFFFu, base, 0);
                if (on) S.active[base + __popc(m & ((1u << (threadIdx.x & 31)) - 1u))] = (uint16_t)(ly * 64 + pc);
            }
            __syncthreads();
            const int nActive = (int)S.nActive;
            for (int j = 9; j >= 0; --j) {
                const int xa = (HALO - j) & ~1, xb = (HALO + TW + j + 1) & ~1;
                blur_pass<true>(S, nActive, 0, xa, xb, HALO - j - 1, HALO + TH + j + 1);
                __syncthreads();
                blur_pass<false>(S, nActive, 1, xa, xb, HALO - j, HALO + TH + j);
                __syncthreads();
            }
            if (threadIdx.x == 0) S.nActive = 0;  // read by every thread above; the next tile's list starts empty
        }
        // postprocess.comp:28-50 on the tile
        for (int i = threadIdx.x; i < TW * TH; i += kPostThreads) {
            const int ty = i / TW, tx = i - ty * TW;
            const int x = x0 + tx, y = y0 + ty;
            if (x >= W || y >= H) continue;
            const size_t pix = (size_t)y * W + x;
            const int lx = tx + HALO, ly = ty + HALO;
            const float4 b = unpack_half4(__ldg(P.base + pix));
            const float r[3] = {__half2float(S.col[0][0][ly][CP + lx]), __half2float(S.col[0][1][ly][CP + lx]),
                                __half2float(S.col[0][2][ly][CP + lx])};
            const float bb[3] = {b.x, b.y, b.z};
            float col[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) col[c] = clampf(mixs(bb[c], r[c], b.w), 0.0f, 1.0f);
            const float luma = (col[0] * 0.299f + col[1] * 0.587f) + col[2] * 0.114f;
#pragma unroll
            for (int c = 0; c < 3; ++c) col[c] = mixs(col[c], P.fade[c], P.fade[3]);
            if (P.showAlpha) {
                const float l = rh(luma);
                P.finalImg[pix] = pack_half4(l, l, l, l);
            } else {
                P.finalImg[pix] = pack_half4(col[0], col[1], col[2], luma);
            }
            if (P.dbgTransition) P.dbgTransition[pix] = P.showAlpha ? 1.0f : (float)S.trans[ly][lx] / 127.0f;
            if (P.dbgA || P.dbgB) {
                const float ra = unpack_half4(S.rough[st][ly + 1][lx + 2]).w;
                if (P.dbgA) {
                    if (P.showAlpha) P.dbgA[pix] = pack_half4(ra, ra, ra, ra);
                    else P.dbgA[pix] = pack_half4(r[0], r[1], r[2], ra);
                }
                if (P.dbgB) {
                    const float g[3] = {__half2float(S.col[1][0][ly][CP + lx]), __half2float(S.col[1][1][ly][CP + lx]),
                                        __half2float(S.col[1][2][ly][CP + lx])};
                    if (P.showAlpha) P.dbgB[pix] = pack_half4(ra, ra, ra, ra);
                    else P.dbgB[pix] = pack_half4(g[0], g[1], g[2], ra);
                }
            }
        }
        __syncthreads();  // the colour planes and the mask are rewritten by the next tile
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

// tensor map of an RGBA16F image as a W x H array of 8-byte pixels, boxes of the staged region;
// false when the image cannot be a TMA source (row pitch not a multiple of 16 bytes, unaligned base)
static bool image_map(CUtensorMap* map, const uint2* img, uint32_t W, uint32_t H) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc || (W & 1u) || (reinterpret_cast<uintptr_t>(img) & 15u)) return false;
    const cuuint64_t dims[2] = {W, H};
    const cuuint64_t strides[1] = {(cuuint64_t)W * 8};
    const cuuint32_t box[2] = {(cuuint32_t)SW, (cuuint32_t)SH};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<uint2*>(img), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_rough_post(const PostParams& p, cudaStream_t s) {
    static std::atomic<int> gridCache{0};
    const int smem = (int)sizeof(RoughSmem) + 128;
    int grid = gridCache.load(std::memory_order_acquire);
    if (!grid) {
        cudaError_t e = cudaFuncSetAttribute(k_rough_post, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = sms;
        gridCache.store(grid, std::memory_order_release);
    }
    CUtensorMap mr, mn;
    std::memset(&mr, 0, sizeof(mr));
    std::memset(&mn, 0, sizeof(mn));
    const bool tma = image_map(&mr, p.rough, p.W, p.H) && image_map(&mn, p.normal, p.W, p.H);
    const int tiles = (int)(((p.W + TW - 1) / TW) * ((p.H + TH - 1) / TH));
    k_rough_post<<<std::min(grid, tiles), kPostThreads, smem, s>>>(mr, mn, p, tma ? 1 : 0);
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
