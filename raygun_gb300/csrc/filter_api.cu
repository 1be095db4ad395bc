// filter_api.cu -- the learned roughness filter's host side: parameters (FP32 master copy, Adam
// state), packed BF16 weights, activation buffers, and the rg_filter_* C ABI (include/rgcuda.h).
// The kernels are in filter.cu.
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "rg_internal.cuh"

using namespace rg;

namespace {

// layer shapes: real channel counts and the padded ones the kernels run on
constexpr int kL = 5;
constexpr int kCinR[kL] = {12, 32, 64, 64, 32}, kCoutR[kL] = {32, 64, 64, 32, 3};
constexpr int kCin[kL] = {16, 32, 64, 64, 32}, kCout[kL] = {32, 64, 64, 32, 16};

constexpr int param_count() {
    int n = 0;
    for (int l = 0; l < kL; ++l) n += kCoutR[l] * kCinR[l] * 9 + kCoutR[l];
    return n;
}
static_assert(param_count() == RG_FILTER_PARAMS, "parameter count");

#define TRY_F(expr)                \
    do {                           \
        rg_status s_ = (expr);     \
        if (s_ != RG_OK) return s_; \
    } while (0)

struct Dev {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

struct rg_filter {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int offW[kL], offB[kL];
    Dev params, grads, m, v, wf[kL], wt[kL], bias[kL], status;
    Dev x0, y1, y2, y3, y4, x5, out, g5, gx5, gp4, gp3, gp2, gp1, target, dwPartial, bPartial, lossPartial;
    size_t actPixels = 0;
    uint64_t steps = 0;
    bool packed = false;
};

namespace {

rg_status ffail(rg_filter* f, rg_status code, const std::string& m) {
    if (f) f->err = m;
    return code;
}

#define FCK(call)                                                                                            \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess)                                                                               \
            return ffail(f, e_ == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA,            \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                                \
    } while (0)

// packed BF16 weights (forward, and transposed / flipped for the data gradient) and padded biases
rg_status refresh_weights(rg_filter* f) {
    const float* P = f->params.as<float>();
    for (int l = 0; l < kL; ++l) {
        FCK(filter_pack(P + f->offW[l], kCoutR[l], kCinR[l], kCin[l], kCout[l], 0, f->wf[l].p, f->stream));
        if (l > 0) FCK(filter_pack(P + f->offW[l], kCoutR[l], kCinR[l], kCout[l], kCin[l], 1, f->wt[l].p, f->stream));
        FCK(filter_bias_pad(P + f->offB[l], kCoutR[l], kCout[l], f->bias[l].as<float>(), f->stream));
    }
    f->packed = true;
    return RG_OK;
}

rg_status ensure_activations(rg_filter* f, size_t P, bool training) {
    FCK(f->out.ensure(16 * P));
    FCK(f->y1.ensure(2 * 32 * P));
    FCK(f->y2.ensure(2 * 64 * P));
    FCK(f->y3.ensure(2 * 64 * P));
    FCK(f->y4.ensure(2 * 32 * P));
    FCK(f->x5.ensure(2 * 32 * P));
    if (training) {
        FCK(f->g5.ensure(2 * 16 * P));
        FCK(f->gx5.ensure(2 * 32 * P));
        FCK(f->gp4.ensure(2 * 32 * P));
        FCK(f->gp3.ensure(2 * 64 * P));
        FCK(f->gp2.ensure(2 * 64 * P));
        FCK(f->gp1.ensure(2 * 32 * P));
    }
    return RG_OK;
}

// training: keep layer 4's own activations (its ReLU mask in the backward pass); inference writes
// only their sum with the skip, x5
// status: where a wait that gives up is reported (nullptr: the filter's own status word)
rg_status forward(rg_filter* f, const __nv_bfloat16* x0, int B, int H, int W, bool training, int* status = nullptr) {
    if (!f->packed) TRY_F(refresh_weights(f));
    FilterConvArgs a;
    std::memset(&a, 0, sizeof a);
    a.B = B;
    a.H = H;
    a.W = W;
    a.status = status ? status : f->status.as<int>();
    using bf = __nv_bfloat16;
    const bf* w[kL];
    for (int l = 0; l < kL; ++l) w[l] = f->wf[l].as<bf>();
    // layers 1-4: conv + bias + ReLU; layer 4 also writes x5 = y4 + y1 (the skip)
    bf* outs[4] = {f->y1.as<bf>(), f->y2.as<bf>(), f->y3.as<bf>(), f->y4.as<bf>()};
    const bf* in = x0;
    for (int l = 0; l < 4; ++l) {
        FilterConvArgs c = a;
        c.x = in;
        c.w = w[l];
        c.bias = f->bias[l].as<float>();
        c.relu = 1;
        c.y = outs[l];
        if (l == 3) {
            c.add = f->y1.as<bf>();
            c.ya = f->x5.as<bf>();
            if (!training) c.y = nullptr;
        }
        FCK(filter_conv(kCin[l], kCout[l], c, f->stream));
        in = outs[l];
    }
    // layer 5 on x5, linear, FP32 prediction
    FilterConvArgs c = a;
    c.x = f->x5.as<bf>();
    c.w = w[4];
    c.bias = f->bias[4].as<float>();
    c.yf = f->out.as<float>();
    FCK(filter_conv(kCin[4], kCout[4], c, f->stream));
    return RG_OK;
}

}  // namespace

namespace rg {

cudaError_t filter_frame(rg_filter* f, const uint2* base, const uint2* normal, const uint2* rough, uint32_t W, uint32_t H, float samples,
                         const float fade[4], int showAlpha, uint2* finalImg, int* status, cudaStream_t s) {
    const size_t P = (size_t)W * H;
    cudaError_t e0 = cudaStreamSynchronize(f->stream);  // parameter updates issued on the filter's stream
    if (e0 != cudaSuccess) return e0;
    cudaStream_t saved = f->stream;
    f->stream = s;
    cudaError_t e = f->x0.ensure(2 * 16 * P);
    if (e == cudaSuccess && ensure_activations(f, P, false) != RG_OK) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = filter_gbuffer(base, normal, rough, P, samples, f->x0.p, s);
    if (e == cudaSuccess && forward(f, f->x0.as<__nv_bfloat16>(), 1, (int)H, (int)W, false, status) != RG_OK) e = cudaErrorUnknown;
    if (e == cudaSuccess) e = filter_composite(base, f->out.as<float4>(), P, fade, showAlpha, finalImg, s);
    f->stream = saved;
    return e;
}

const float4* filter_prediction(const rg_filter* f) { return static_cast<const float4*>(f->out.p); }

}  // namespace rg

extern "C" {

rg_status rg_filter_create(rg_ctx* ctx, uint64_t seed, rg_filter** out) {
    if (!ctx || !out) return RG_ERR_INVALID_ARG;
    *out = nullptr;
    void* s = nullptr;
    if (rg_get_stream(ctx, &s) != RG_OK) return RG_ERR_INVALID_ARG;  // the context's device is current
    rg_filter* f = new rg_filter();
    cudaGetDevice(&f->device);
    // its own stream: the filter may outlive the context it was created with; frames of a context
    // run it on the context's stream (filter_frame)
    if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete f;
        return RG_ERR_CUDA;
    }
    int off = 0;
    for (int l = 0; l < kL; ++l) {
        f->offW[l] = off;
        off += kCoutR[l] * kCinR[l] * 9;
        f->offB[l] = off;
        off += kCoutR[l];
    }
    // He-normal weights (std = sqrt(2 / fan_in)), zero biases
    std::vector<float> h(RG_FILTER_PARAMS, 0.0f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < kL; ++l) {
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (9.0f * kCinR[l])) * (l == kL - 1 ? 0.5f : 1.0f));
        for (int i = 0; i < kCoutR[l] * kCinR[l] * 9; ++i) h[f->offW[l] + i] = nd(rng);
    }
    const size_t pb = sizeof(float) * RG_FILTER_PARAMS;
    cudaError_t e = f->params.ensure(pb);
    if (e == cudaSuccess) e = f->grads.ensure(pb);
    if (e == cudaSuccess) e = f->m.ensure(pb);
    if (e == cudaSuccess) e = f->v.ensure(pb);
    if (e == cudaSuccess) e = f->status.ensure(16);
    for (int l = 0; l < kL && e == cudaSuccess; ++l) {
        e = f->wf[l].ensure(2ull * 9 * kCin[l] * kCout[l]);
        if (e == cudaSuccess) e = f->wt[l].ensure(2ull * 9 * kCin[l] * kCout[l]);
        if (e == cudaSuccess) e = f->bias[l].ensure(64 * sizeof(float));
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(f->params.p, h.data(), pb, cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->m.p, 0, pb, f->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->v.p, 0, pb, f->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->grads.p, 0, pb, f->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->status.p, 0, 16, f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) {
        rg_filter_destroy(f);
        return e == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA;
    }
    *out = f;
    return RG_OK;
}

rg_status rg_filter_destroy(rg_filter* f) {
    if (!f) return RG_ERR_INVALID_ARG;
    cudaSetDevice(f->device);
    if (f->stream) cudaStreamSynchronize(f->stream);
    Dev* all[] = {&f->params, &f->grads, &f->m, &f->v, &f->status, &f->x0, &f->y1, &f->y2, &f->y3, &f->y4, &f->x5, &f->out, &f->g5, &f->gx5,
                  &f->gp4, &f->gp3, &f->gp2, &f->gp1, &f->target, &f->dwPartial, &f->bPartial, &f->lossPartial};
    for (Dev* d : all) d->release();
    for (int l = 0; l < kL; ++l) {
        f->wf[l].release();
        f->wt[l].release();
        f->bias[l].release();
    }
    if (f->stream) cudaStreamDestroy(f->stream);
    delete f;
    return RG_OK;
}

const char* rg_filter_last_error(const rg_filter* f) { return f ? f->err.c_str() : "null filter"; }

rg_status rg_filter_get_params(rg_filter* f, float* host, uint32_t n) {
    if (!f || !host || n != RG_FILTER_PARAMS) return ffail(f, RG_ERR_INVALID_ARG, "expected RG_FILTER_PARAMS floats");
    FCK(cudaSetDevice(f->device));
    FCK(cudaMemcpyAsync(host, f->params.p, sizeof(float) * n, cudaMemcpyDeviceToHost, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    return RG_OK;
}

rg_status rg_filter_get_grads(rg_filter* f, float* host, uint32_t n) {
    if (!f || !host || n != RG_FILTER_PARAMS) return ffail(f, RG_ERR_INVALID_ARG, "expected RG_FILTER_PARAMS floats");
    FCK(cudaSetDevice(f->device));
    FCK(cudaMemcpyAsync(host, f->grads.p, sizeof(float) * n, cudaMemcpyDeviceToHost, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    return RG_OK;
}

rg_status rg_filter_set_params(rg_filter* f, const float* host, uint32_t n) {
    if (!f || !host || n != RG_FILTER_PARAMS) return ffail(f, RG_ERR_INVALID_ARG, "expected RG_FILTER_PARAMS floats");
    FCK(cudaSetDevice(f->device));
    FCK(cudaMemcpyAsync(f->params.p, host, sizeof(float) * n, cudaMemcpyHostToDevice, f->stream));
    FCK(cudaMemsetAsync(f->m.p, 0, sizeof(float) * n, f->stream));
    FCK(cudaMemsetAsync(f->v.p, 0, sizeof(float) * n, f->stream));
    f->steps = 0;
    return refresh_weights(f);
}

rg_status rg_filter_forward(rg_filter* f, const void* d_input, uint32_t B, uint32_t H, uint32_t W, float* d_out) {
    if (!f || !d_input || !d_out || !B || !H || !W) return ffail(f, RG_ERR_INVALID_ARG, "bad filter forward arguments");
    FCK(cudaSetDevice(f->device));
    const size_t P = (size_t)B * H * W;
    TRY_F(ensure_activations(f, P, false));
    TRY_F(forward(f, static_cast<const __nv_bfloat16*>(d_input), (int)B, (int)H, (int)W, false));
    FCK(cudaMemcpyAsync(d_out, f->out.p, 16 * P, cudaMemcpyDeviceToDevice, f->stream));
    int st = 0;
    FCK(cudaMemcpyAsync(&st, f->status.p, sizeof(int), cudaMemcpyDeviceToHost, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    if (st) return ffail(f, RG_ERR_CUDA, "tensor-core completion wait gave up");
    return RG_OK;
}

rg_status rg_filter_train_step(rg_filter* f, const void* d_input, const float* d_target, uint32_t B, uint32_t H, uint32_t W, float lr,
                               float* loss_out) {
    if (!f || !d_input || !d_target || !B || !H || !W) return ffail(f, RG_ERR_INVALID_ARG, "bad filter training arguments");
    FCK(cudaSetDevice(f->device));
    using bf = __nv_bfloat16;
    const size_t P = (size_t)B * H * W;
    TRY_F(ensure_activations(f, P, true));
    const int ctas = filter_dw_ctas(), lossBlocks = 512, biasBlocks = 256;
    FCK(f->dwPartial.ensure(sizeof(float) * (size_t)ctas * 64 * 9 * 64));
    FCK(f->bPartial.ensure(sizeof(float) * biasBlocks * 64));
    FCK(f->lossPartial.ensure(sizeof(float) * lossBlocks));
    const bf* x0 = static_cast<const bf*>(d_input);
    TRY_F(forward(f, x0, (int)B, (int)H, (int)W, true));
    FCK(filter_loss(f->out.as<float4>(), reinterpret_cast<const float4*>(d_target), P, 1.0f / (3.0f * (float)P), f->g5.p,
                    f->lossPartial.as<float>(), lossBlocks, f->stream));
    float* G = f->grads.as<float>();
    int* st = f->status.as<int>();
    auto dW = [&](int l, const void* x, const void* x2, const void* g) -> rg_status {
        FCK(filter_dw(kCin[l], kCout[l], x, x2, g, (int)B, (int)H, (int)W, f->dwPartial.as<float>(), ctas, st, f->stream));
        FCK(filter_dw_reduce(f->dwPartial.as<float>(), ctas, kCout[l], kCin[l], kCoutR[l], kCinR[l], G + f->offW[l], f->stream));
        FCK(filter_bias_grad(g, P, kCout[l], kCoutR[l], f->bPartial.as<float>(), biasBlocks, G + f->offB[l], f->stream));
        return RG_OK;
    };
    FilterConvArgs a;
    std::memset(&a, 0, sizeof a);
    a.B = (int)B;
    a.H = (int)H;
    a.W = (int)W;
    a.status = st;
    // layer 5 (input x5 = y4 + y1)
    TRY_F(dW(4, f->x5.p, nullptr, f->g5.p));
    {
        FilterConvArgs c = a;  // gx5 (kept for the skip), gp4 = gx5 where y4 > 0
        c.x = f->g5.as<bf>();
        c.w = f->wt[4].as<bf>();
        c.y = f->gx5.as<bf>();
        c.ym = f->gp4.as<bf>();
        c.mask = f->y4.as<bf>();
        FCK(filter_conv(kCout[4], kCin[4], c, f->stream));
    }
    TRY_F(dW(3, f->y3.p, nullptr, f->gp4.p));
    {
        FilterConvArgs c = a;
        c.x = f->gp4.as<bf>();
        c.w = f->wt[3].as<bf>();
        c.ym = f->gp3.as<bf>();
        c.mask = f->y3.as<bf>();
        FCK(filter_conv(kCout[3], kCin[3], c, f->stream));
    }
    TRY_F(dW(2, f->y2.p, nullptr, f->gp3.p));
    {
        FilterConvArgs c = a;
        c.x = f->gp3.as<bf>();
        c.w = f->wt[2].as<bf>();
        c.ym = f->gp2.as<bf>();
        c.mask = f->y2.as<bf>();
        FCK(filter_conv(kCout[2], kCin[2], c, f->stream));
    }
    TRY_F(dW(1, f->y1.p, nullptr, f->gp2.p));
    {
        FilterConvArgs c = a;  // through layer 2, plus the skip's gradient, masked by y1
        c.x = f->gp2.as<bf>();
        c.w = f->wt[1].as<bf>();
        c.add = f->gx5.as<bf>();
        c.ym = f->gp1.as<bf>();
        c.mask = f->y1.as<bf>();
        FCK(filter_conv(kCout[1], kCin[1], c, f->stream));
    }
    TRY_F(dW(0, x0, nullptr, f->gp1.p));
    // Adam
    f->steps++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)f->steps), c2 = 1.0f - std::pow(b2, (float)f->steps);
    if (lr > 0.0f) {
        FCK(filter_adam(f->params.as<float>(), G, f->m.as<float>(), f->v.as<float>(), RG_FILTER_PARAMS, lr, b1, b2, 1e-8f, c1, c2,
                        f->stream));
        TRY_F(refresh_weights(f));
    }
    std::vector<float> lp(lossBlocks);
    FCK(cudaMemcpyAsync(lp.data(), f->lossPartial.p, sizeof(float) * lossBlocks, cudaMemcpyDeviceToHost, f->stream));
    int status = 0;
    FCK(cudaMemcpyAsync(&status, st, sizeof(int), cudaMemcpyDeviceToHost, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    if (status) return ffail(f, RG_ERR_CUDA, "tensor-core completion wait gave up");
    double loss = 0.0;
    for (float x : lp) loss += x;
    if (loss_out) *loss_out = (float)(loss / (3.0 * (double)P));
    return RG_OK;
}

}  // extern "C"
