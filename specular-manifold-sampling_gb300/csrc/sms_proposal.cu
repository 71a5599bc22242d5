// sms_proposal.cu -- host side of the learned seed proposal (sms_proposal_*).
//
// No counterpart in the reference (its walks are seeded uniformly,
// manifold_ss.cpp:223).  A proposal owns one network (FP32 master weights,
// Adam moments, BF16 copies), a device-resident training set filled by the
// solver itself (ss_collect_kernel) and the activation buffers of training.
// Training steps are captured once into a CUDA graph and replayed; the step
// counter, the batch draw and the loss ring live on the device, so replays
// need no host work per step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sms_gb300.h"
#include "sms_device.cuh"
#include "sms_kernels.h"

using namespace sms;

struct sms_proposal {
    sms_ctx *ctx = nullptr;
    int device = 0;
    int shape = -1;
    mlp::SeedFrame frame{};
    mlp::MlpDev net{};
    void *block = nullptr;       // parameters, moments, copies, counters
    float *data = nullptr;       // kDataRows x cap training pairs (features, uv, weight)
    uint32_t cap = 0;
    unsigned *fill = nullptr;    // device: pairs appended (may exceed cap)
    uint32_t n_data = 0;
    double *moments = nullptr;   // 2 kIn
    void *act = nullptr;         // hT and dzT for act_batch
    int act_batch = 0;
    // cached graph of kGraphSteps training steps
    cudaGraphExec_t graph = nullptr;
    int graph_batch = 0;
    float graph_lr = 0.f;
    uint32_t graph_n = 0;
    uint64_t graph_version = 0;
    uint64_t version = 1;        // bumped whenever captured kernel arguments change
};

namespace {

constexpr int kGraphSteps = 50;

sms_status fail(sms_status st, const std::string &msg) { return (sms_status)set_last_error_impl((int)st, msg.c_str()); }
sms_status cuda_fail(cudaError_t e, const char *what) {
    return fail(SMS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define PTRY(expr)                                       \
    do {                                                 \
        cudaError_t e_ = (expr);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr); \
    } while (0)

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

bool live(sms_proposal *p, CtxView &v) { return p && p->ctx && ctx_view(p->ctx, v); }

// Initial parameters: uniform He-style weights (bound sqrt(6 / fan_in)), zero
// hidden biases; the output layer starts near a broad mixture: small weights,
// equal logits, means spread over the uv square, sigma about 0.1.
void init_params(std::vector<float> &P, uint64_t seed) {
    P.assign(mlp::kParams, 0.f);
    Pcg32 rng;
    rng.seed(seed, 0x5eedull);
    for (int l = 0; l < mlp::kLayers; ++l) {
        const int K = mlp::layer_in(l), N = mlp::layer_out(l);
        const int fan_in = l == 0 ? mlp::kInEnc : K;
        float bound = std::sqrt(6.f / (float)fan_in);
        if (l == mlp::kLayers - 1) bound *= 0.1f;
        for (int r = 0; r < N; ++r)
            for (int c = 0; c < K; ++c)
                P[mlp::w_off(l) + r * K + c] =
                    c < (l == 0 ? mlp::kInEnc : K) ? (2.f * rng.next_f32() - 1.f) * bound : 0.f;
    }
    float *bo = &P[mlp::b_off(mlp::kLayers - 1)];
    const float s0 = (std::log(0.1f) - mlp::kLsMin) / (mlp::kLsMax - mlp::kLsMin);
    for (int k = 0; k < mlp::kComp; ++k) {
        bo[8 + 2 * k] = 0.1f + 0.8f * rng.next_f32();
        bo[9 + 2 * k] = 0.1f + 0.8f * rng.next_f32();
        bo[24 + 2 * k] = bo[25 + 2 * k] = std::log(s0 / (1.f - s0));
    }
}

sms_status ensure_act(sms_proposal *p, int batch, cudaStream_t s) {
    if (p->act_batch >= batch) return SMS_OK;
    if (p->act) {
        PTRY(cudaStreamSynchronize(s));
        cudaFree(p->act);
        p->act = nullptr;
        p->act_batch = 0;
    }
    const size_t hb = align256((size_t)mlp::kHRows * batch * 2), db = (size_t)mlp::kDzRows * batch * 2;
    PTRY(cudaMalloc(&p->act, hb + db));
    p->act_batch = batch;
    p->net.hT = reinterpret_cast<__nv_bfloat16 *>(p->act);
    p->net.dzT = reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(p->act) + hb);
    p->version++;
    return SMS_OK;
}

sms_status drop_graph(sms_proposal *p) {
    if (p->graph) cudaGraphExecDestroy(p->graph);
    p->graph = nullptr;
    return SMS_OK;
}

}  // namespace

// ----------------------------------------------------- library-internal API
sms_ctx *proposal_ctx(sms_proposal *p) { return p ? p->ctx : nullptr; }

bool proposal_seed_desc(sms_proposal *p, mlp::SeedProposal &out) {
    if (!p || !p->ctx) return false;
    out.shape = p->shape;
    out.frame = p->frame;
    out.net = p->net;
    return true;
}

void proposal_detach(sms_proposal *p) {
    if (!p) return;
    drop_graph(p);
    p->ctx = nullptr;
}

// ---------------------------------------------------------------- C ABI
extern "C" sms_status sms_proposal_create(sms_ctx *ctx, int32_t caster, uint64_t init_seed, uint32_t capacity,
                                          sms_proposal **out) {
    if (!out) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_create: null output");
    *out = nullptr;
    CtxView v;
    if (!ctx || !ctx_view(ctx, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_create: null context");
    bool is_caster = false;
    for (int i = 0; i < v.scene->n_casters_ss; ++i) is_caster |= v.scene->casters_ss[i] == caster;
    if (caster < 0 || caster >= v.n_shapes || !is_caster)
        return fail(SMS_ERR_INVALID_ARG, "sms_proposal_create: shape is not a single-scatter caster");
    if (capacity == 0 || capacity > (1u << 28))
        return fail(SMS_ERR_INVALID_ARG, "sms_proposal_create: capacity must lie in [1, 2^28]");
    PTRY(cudaSetDevice(v.device));
    {
        cudaError_t e = mlp::configure_kernels();
        if (e != cudaSuccess) return cuda_fail(e, "configure proposal kernels");
    }
    sms_proposal *p = new sms_proposal();
    p->ctx = ctx;
    p->device = v.device;
    p->shape = caster;
    p->frame = v.frames[caster];
    p->net.frame = p->frame;
    p->cap = capacity;
    // one block: params, grad, m, v | bias | loss | step, fill | wbf | moments
    const size_t pb = align256((size_t)mlp::kParams * 4);
    const size_t off_bias = 4 * pb, off_loss = off_bias + align256(mlp::kLayers * 64 * 4);
    const size_t off_step = off_loss + align256(mlp::kLossHist * 4), off_wbf = off_step + 256;
    const size_t off_mom = off_wbf + align256((size_t)mlp::kWeightsAll * 2);
    const size_t total = off_mom + align256(2 * mlp::kIn * sizeof(double));
    sms_status st = SMS_OK;
    do {
        cudaError_t e = cudaMalloc(&p->block, total);
        if (e != cudaSuccess) { st = cuda_fail(e, "cudaMalloc(proposal)"); break; }
        e = cudaMalloc(&p->data, (size_t)mlp::kDataRows * capacity * sizeof(float));
        if (e != cudaSuccess) { st = cuda_fail(e, "cudaMalloc(proposal training set)"); break; }
        char *b = reinterpret_cast<char *>(p->block);
        p->net.params = reinterpret_cast<float *>(b);
        p->net.grad = reinterpret_cast<float *>(b + pb);
        p->net.adam_m = reinterpret_cast<float *>(b + 2 * pb);
        p->net.adam_v = reinterpret_cast<float *>(b + 3 * pb);
        p->net.bias = reinterpret_cast<float *>(b + off_bias);
        p->net.loss = reinterpret_cast<float *>(b + off_loss);
        p->net.step = reinterpret_cast<uint32_t *>(b + off_step);
        p->fill = reinterpret_cast<unsigned *>(b + off_step + 4);
        p->net.wbf = reinterpret_cast<__nv_bfloat16 *>(b + off_wbf);
        p->moments = reinterpret_cast<double *>(b + off_mom);
        for (int k = 0; k < mlp::kIn; ++k) { p->net.shift[k] = 0.f; p->net.scale[k] = 1.f; }
        p->net.sigma_scale = 1.f;
        p->net.weighted = 1;
        e = cudaMemsetAsync(p->block, 0, total, v.stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "cudaMemset(proposal)"); break; }
        std::vector<float> P;
        init_params(P, init_seed);
        e = cudaMemcpyAsync(p->net.params, P.data(), P.size() * 4, cudaMemcpyHostToDevice, v.stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "upload proposal parameters"); break; }
        e = mlp::launch_sync(p->net, v.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "initialise proposal"); break; }
    } while (0);
    if (st != SMS_OK) {
        if (p->data) cudaFree(p->data);
        if (p->block) cudaFree(p->block);
        delete p;
        return st;
    }
    ctx_register_proposal(ctx, p);
    *out = p;
    return SMS_OK;
}

extern "C" sms_status sms_proposal_destroy(sms_proposal *p) {
    if (!p) return SMS_OK;
    cudaSetDevice(p->device);
    if (p->ctx) {
        CtxView v;
        if (ctx_view(p->ctx, v)) cudaStreamSynchronize(v.stream);
        ctx_forget_proposal(p->ctx, p);
    }
    drop_graph(p);
    if (p->act) cudaFree(p->act);
    if (p->data) cudaFree(p->data);
    if (p->block) cudaFree(p->block);
    delete p;
    return SMS_OK;
}

extern "C" sms_status sms_proposal_collect(sms_proposal *p, const float *q, uint32_t n, uint64_t seed,
                                           uint64_t stream_offset, int32_t walks_per_query, uint32_t *total) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_collect: proposal without context");
    if (n && !q) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_collect: null queries");
    if (walks_per_query < 0 || walks_per_query > 4096)
        return fail(SMS_ERR_INVALID_ARG, "sms_proposal_collect: walks_per_query must lie in [0, 4096]");
    PTRY(cudaSetDevice(v.device));
    PTRY(launch_ss_collect(*v.scene, v.solver, p->shape, q, n, seed, stream_offset, walks_per_query, p->frame,
                           p->data, p->cap, p->fill, v.counters, v.timer, v.stream));
    unsigned filled = 0;
    PTRY(cudaMemcpyAsync(&filled, p->fill, sizeof(unsigned), cudaMemcpyDeviceToHost, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    p->n_data = std::min<uint32_t>(filled, p->cap);
    p->version++;
    if (total) *total = p->n_data;
    return SMS_OK;
}

extern "C" sms_status sms_proposal_set_data(sms_proposal *p, const float *feat, const float *uv, const float *weight,
                                            uint32_t n) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_set_data: proposal without context");
    if (n && (!feat || !uv)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_set_data: null array");
    if (n > p->cap) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_set_data: more pairs than the capacity");
    PTRY(cudaSetDevice(v.device));
    std::vector<float> ones;
    if (!weight) {
        ones.assign(n, 1.f);
        weight = ones.data();
    }
    for (int k = 0; k < mlp::kDataRows && n; ++k) {
        const float *src = k < mlp::kIn ? feat + (size_t)k * n
                         : k < mlp::kIn + 2 ? uv + (size_t)(k - mlp::kIn) * n : weight;
        PTRY(cudaMemcpyAsync(p->data + (size_t)k * p->cap, src, (size_t)n * 4, cudaMemcpyHostToDevice, v.stream));
    }
    unsigned f = n;
    PTRY(cudaMemcpyAsync(p->fill, &f, sizeof(unsigned), cudaMemcpyHostToDevice, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    p->n_data = n;
    p->version++;
    return SMS_OK;
}

extern "C" sms_status sms_proposal_get_data(sms_proposal *p, float *feat, float *uv, float *weight, uint32_t cap,
                                            uint32_t *n) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_get_data: proposal without context");
    if (!n) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_get_data: null count");
    *n = p->n_data;
    const uint32_t m = std::min(cap, p->n_data);
    if (m && (!feat || !uv)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_get_data: null array");
    PTRY(cudaSetDevice(v.device));
    for (int k = 0; k < mlp::kDataRows && m; ++k) {
        float *dst = k < mlp::kIn ? feat + (size_t)k * m
                   : k < mlp::kIn + 2 ? uv + (size_t)(k - mlp::kIn) * m : weight;
        if (!dst) continue;
        PTRY(cudaMemcpyAsync(dst, p->data + (size_t)k * p->cap, (size_t)m * 4, cudaMemcpyDeviceToHost, v.stream));
    }
    PTRY(cudaStreamSynchronize(v.stream));
    return SMS_OK;
}

extern "C" sms_status sms_proposal_normalize(sms_proposal *p) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_normalize: proposal without context");
    if (p->n_data == 0) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_normalize: empty training set");
    PTRY(cudaSetDevice(v.device));
    PTRY(cudaMemsetAsync(p->moments, 0, 2 * mlp::kIn * sizeof(double), v.stream));
    PTRY(mlp::launch_feature_moments(p->data, p->cap, p->n_data, p->moments, v.stream));
    double h[2 * mlp::kIn];
    PTRY(cudaMemcpyAsync(h, p->moments, sizeof(h), cudaMemcpyDeviceToHost, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    for (int k = 0; k < mlp::kIn; ++k) {
        const double mean = h[k] / p->n_data;
        const double var = std::max(0.0, h[mlp::kIn + k] / p->n_data - mean * mean);
        const double sd = std::sqrt(var);
        p->net.shift[k] = (float)mean;
        p->net.scale[k] = sd > 1e-6 * std::max(1.0, std::fabs(mean)) ? (float)(1.0 / sd) : 0.f;
    }
    p->version++;
    return SMS_OK;
}

extern "C" sms_status sms_proposal_train(sms_proposal *p, int32_t steps, int32_t batch, float lr, float *mean_loss) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_train: proposal without context");
    if (steps < 0) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_train: negative step count");
    if (batch < 16 || batch > mlp::kMaxBatch || batch % 16)
        return fail(SMS_ERR_INVALID_ARG, "sms_proposal_train: batch must be a multiple of 16 in [16, 65536]");
    if (!(lr > 0.f) || !std::isfinite(lr)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_train: bad learning rate");
    if (p->n_data == 0) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_train: empty training set");
    PTRY(cudaSetDevice(v.device));
    if (sms_status st = ensure_act(p, batch, v.stream)) return st;
    const float *feat = p->data, *uv = p->data + (size_t)mlp::kIn * p->cap;
    uint32_t start = 0;
    PTRY(cudaMemcpyAsync(&start, p->net.step, 4, cudaMemcpyDeviceToHost, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    if (steps >= kGraphSteps) {
        if (!p->graph || p->graph_batch != batch || p->graph_lr != lr || p->graph_n != p->n_data ||
            p->graph_version != p->version) {
            drop_graph(p);
            cudaGraph_t g = nullptr;
            PTRY(cudaStreamBeginCapture(v.stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            for (int i = 0; i < kGraphSteps && e == cudaSuccess; ++i)
                e = mlp::launch_train_step(p->net, feat, uv, p->cap, p->n_data, batch, lr, true, true, v.stream);
            cudaError_t e2 = cudaStreamEndCapture(v.stream, &g);
            if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(e, "capture training steps"); }
            if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&p->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { p->graph = nullptr; return cuda_fail(e, "cudaGraphInstantiate"); }
            p->graph_batch = batch;
            p->graph_lr = lr;
            p->graph_n = p->n_data;
            p->graph_version = p->version;
        }
        for (int i = 0; i + kGraphSteps <= steps; i += kGraphSteps) PTRY(cudaGraphLaunch(p->graph, v.stream));
    }
    const int eager = steps >= kGraphSteps ? steps % kGraphSteps : steps;
    for (int i = 0; i < eager; ++i)
        PTRY(mlp::launch_train_step(p->net, feat, uv, p->cap, p->n_data, batch, lr, true, true, v.stream));
    float ring[mlp::kLossHist];
    uint32_t end = 0;
    PTRY(cudaMemcpyAsync(ring, p->net.loss, sizeof(ring), cudaMemcpyDeviceToHost, v.stream));
    PTRY(cudaMemcpyAsync(&end, p->net.step, 4, cudaMemcpyDeviceToHost, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    if (end - start != (uint32_t)steps) return fail(SMS_ERR_CUDA, "sms_proposal_train: step counter mismatch");
    if (mean_loss) {
        const int k = std::min<int>(steps, mlp::kLossHist - 1);
        double s = 0.0;
        for (int i = 1; i <= k; ++i) s += ring[(end - (uint32_t)i) % mlp::kLossHist];
        *mean_loss = k ? (float)(s / k) : NAN;
    }
    return SMS_OK;
}

extern "C" sms_status sms_proposal_loss_grad(sms_proposal *p, int32_t batch, float *loss, float *grad) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_loss_grad: proposal without context");
    if (batch < 16 || batch > mlp::kMaxBatch || batch % 16 || (uint32_t)batch > p->n_data)
        return fail(SMS_ERR_INVALID_ARG,
                    "sms_proposal_loss_grad: batch must be a multiple of 16 and at most the training set");
    PTRY(cudaSetDevice(v.device));
    if (sms_status st = ensure_act(p, batch, v.stream)) return st;
    uint32_t step = 0;
    PTRY(cudaMemcpyAsync(&step, p->net.step, 4, cudaMemcpyDeviceToHost, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    float *slot = p->net.loss + step % mlp::kLossHist;
    PTRY(cudaMemsetAsync(slot, 0, 4, v.stream));
    PTRY(cudaMemsetAsync(p->net.grad, 0, (size_t)mlp::kParams * 4, v.stream));
    PTRY(mlp::launch_train_step(p->net, p->data, p->data + (size_t)mlp::kIn * p->cap, p->cap, p->n_data, batch, 0.f,
                                false, false, v.stream));
    float l = 0.f;
    PTRY(cudaMemcpyAsync(&l, slot, 4, cudaMemcpyDeviceToHost, v.stream));
    if (grad) PTRY(cudaMemcpyAsync(grad, p->net.grad, (size_t)mlp::kParams * 4, cudaMemcpyDeviceToHost, v.stream));
    PTRY(cudaMemsetAsync(p->net.grad, 0, (size_t)mlp::kParams * 4, v.stream));
    PTRY(cudaMemsetAsync(slot, 0, 4, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    if (loss) *loss = l;
    return SMS_OK;
}

extern "C" sms_status sms_proposal_get_state(sms_proposal *p, float *params, float *adam_m, float *adam_v,
                                             float *norm, uint32_t *step) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_get_state: proposal without context");
    PTRY(cudaSetDevice(v.device));
    const size_t b = (size_t)mlp::kParams * 4;
    if (params) PTRY(cudaMemcpyAsync(params, p->net.params, b, cudaMemcpyDeviceToHost, v.stream));
    if (adam_m) PTRY(cudaMemcpyAsync(adam_m, p->net.adam_m, b, cudaMemcpyDeviceToHost, v.stream));
    if (adam_v) PTRY(cudaMemcpyAsync(adam_v, p->net.adam_v, b, cudaMemcpyDeviceToHost, v.stream));
    if (step) PTRY(cudaMemcpyAsync(step, p->net.step, 4, cudaMemcpyDeviceToHost, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    if (norm)
        for (int k = 0; k < mlp::kIn; ++k) { norm[k] = p->net.shift[k]; norm[mlp::kIn + k] = p->net.scale[k]; }
    return SMS_OK;
}

extern "C" sms_status sms_proposal_set_state(sms_proposal *p, const float *params, const float *adam_m,
                                             const float *adam_v, const float *norm, uint32_t step) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_set_state: proposal without context");
    if (!params) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_set_state: null parameters");
    PTRY(cudaSetDevice(v.device));
    const size_t b = (size_t)mlp::kParams * 4;
    PTRY(cudaMemcpyAsync(p->net.params, params, b, cudaMemcpyHostToDevice, v.stream));
    if (adam_m) PTRY(cudaMemcpyAsync(p->net.adam_m, adam_m, b, cudaMemcpyHostToDevice, v.stream));
    else PTRY(cudaMemsetAsync(p->net.adam_m, 0, b, v.stream));
    if (adam_v) PTRY(cudaMemcpyAsync(p->net.adam_v, adam_v, b, cudaMemcpyHostToDevice, v.stream));
    else PTRY(cudaMemsetAsync(p->net.adam_v, 0, b, v.stream));
    PTRY(cudaMemsetAsync(p->net.grad, 0, b, v.stream));
    PTRY(cudaMemsetAsync(p->net.loss, 0, mlp::kLossHist * 4, v.stream));
    PTRY(cudaMemcpyAsync(p->net.step, &step, 4, cudaMemcpyHostToDevice, v.stream));
    PTRY(mlp::launch_sync(p->net, v.stream));
    PTRY(cudaStreamSynchronize(v.stream));
    if (norm)
        for (int k = 0; k < mlp::kIn; ++k) { p->net.shift[k] = norm[k]; p->net.scale[k] = norm[mlp::kIn + k]; }
    p->version++;
    return SMS_OK;
}

extern "C" sms_status sms_proposal_set_options(sms_proposal *p, float sigma_scale, int32_t weighted) {
    if (!p) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_set_options: null proposal");
    if (!(sigma_scale > 0.f) || !std::isfinite(sigma_scale))
        return fail(SMS_ERR_INVALID_ARG, "sms_proposal_set_options: sigma_scale must be positive");
    p->net.sigma_scale = sigma_scale;
    p->net.weighted = weighted != 0;
    p->version++;
    return SMS_OK;
}

extern "C" sms_status sms_proposal_frame(sms_proposal *p, float frame[10]) {
    if (!p || !frame) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_frame: null argument");
    frame[0] = (float)p->frame.kind;
    for (int k = 0; k < 3; ++k) {
        frame[1 + k] = p->frame.org[k];
        frame[4 + k] = p->frame.ax_u[k];
        frame[7 + k] = p->frame.ax_v[k];
    }
    return SMS_OK;
}

extern "C" sms_status sms_proposal_eval(sms_proposal *p, const float *feat, uint32_t n, int32_t mixture, float *out) {
    CtxView v;
    if (!live(p, v)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_eval: proposal without context");
    if (n && (!feat || !out)) return fail(SMS_ERR_INVALID_ARG, "sms_proposal_eval: null array");
    if (n == 0) return SMS_OK;
    PTRY(cudaSetDevice(v.device));
    void *buf = nullptr;
    const size_t fb = (size_t)mlp::kIn * n * 4, ob = (size_t)mlp::kGmmParams * n * 4;
    PTRY(cudaMalloc(&buf, fb + ob));
    float *df = reinterpret_cast<float *>(buf), *dout = reinterpret_cast<float *>(reinterpret_cast<char *>(buf) + fb);
    cudaError_t e = cudaMemcpyAsync(df, feat, fb, cudaMemcpyHostToDevice, v.stream);
    if (e == cudaSuccess) e = mlp::launch_forward(p->net, df, n, dout, mixture != 0, v.num_sms, v.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, ob, cudaMemcpyDeviceToHost, v.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "sms_proposal_eval");
    return SMS_OK;
}
