// sms_mlp.cu -- training and inference kernels of the learned seed proposal.
//
// No counterpart in the reference, which seeds Newton walks uniformly on the
// specular shape (manifold_ss.cpp:223, Shape::sample_position).  The network
// maps a query's features (shading point, light sample, shading normal) to an
// 8-component diagonal Gaussian mixture over the caster's uv frame; the
// estimator mixes it with the uniform seeding (sms_mlp.cuh, proposal_seed).
//
// Network: 9 (padded to 16) -> 64 -> 64 -> 64 -> 64 -> 48 (40 used), SiLU
// between layers, BF16 weights and activations, FP32 accumulation on the
// tensor cores (mma.m16n8k16), FP32 master weights and Adam moments.
//
// One optimizer step is four launches:
//   mlp_train_fb_kernel  forward, mixture NLL and its gradient, backward
//                        through all layers (register-resident per warp);
//                        writes the transposed layer inputs h^T and
//                        pre-activation gradients dz^T, accumulates bias
//                        gradients and the batch loss
//   mlp_wgrad_kernel     dW_l = dz_l^T h_l on the tensor cores, one warp per
//                        (16x8 tile, batch chunk)
//   mlp_adam_kernel      Adam on the master copy, refreshes both BF16 copies
//   mlp_step_kernel      advances the device step counter
#include <algorithm>

#include "sms_mlp.cuh"

namespace sms {
namespace mlp {

constexpr int kZsFloats = 4 * 8 * 4 * 32;   // per warp: hidden pre-activations
// per warp: the staged input tile (16 x kXLd bf16), reused for the output
// rows (16 x kOutPad floats)
constexpr int kStageFloats = 16 * kXLd / 2;
static_assert(kStageFloats >= 16 * kOutPad, "stage holds the output rows");

// lowbias32 integer hash (C. Wellons, "Prospecting for hash functions").
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// Negative log-likelihood of (u, v) (relative to the anchor) under the
// mixture of raw outputs o[40] and its gradient with respect to o (go[0..47],
// padded columns zero).
__device__ float mixture_nll(const float *o, float u, float v, float *go) {
    float mx = o[0];
    #pragma unroll
    for (int k = 1; k < kComp; ++k) mx = fmaxf(mx, o[k]);
    float se = 0.f;
    #pragma unroll
    for (int k = 0; k < kComp; ++k) se += __expf(o[k] - mx);
    const float logz = mx + __logf(se);
    float lp[kComp], lmax = -INFINITY;
    #pragma unroll
    for (int k = 0; k < kComp; ++k) {
        const float lsx = log_sigma(o[24 + 2 * k]), lsy = log_sigma(o[25 + 2 * k]);
        const float dx = (u - o[8 + 2 * k]) * __expf(-lsx), dy = (v - o[9 + 2 * k]) * __expf(-lsy);
        lp[k] = (o[k] - logz) - 1.8378770664093453f - lsx - lsy - 0.5f * (dx * dx + dy * dy);
        lmax = fmaxf(lmax, lp[k]);
    }
    float s = 0.f;
    #pragma unroll
    for (int k = 0; k < kComp; ++k) s += __expf(lp[k] - lmax);
    const float logp = lmax + __logf(s);
    #pragma unroll
    for (int k = 0; k < kComp; ++k) {
        const float r = __expf(lp[k] - logp);   // responsibility
        go[k] = __expf(o[k] - logz) - r;
        #pragma unroll
        for (int d = 0; d < 2; ++d) {
            const float raw = o[24 + 2 * k + d];
            const float sg = sigmoid(raw);
            const float ls = kLsMin + (kLsMax - kLsMin) * sg;
            const float iv = __expf(-2.f * ls);
            const float e = (d == 0 ? u : v) - o[8 + 2 * k + d];
            go[8 + 2 * k + d] = -r * e * iv;
            go[24 + 2 * k + d] = r * (1.f - e * e * iv) * (kLsMax - kLsMin) * sg * (1.f - sg);
        }
    }
    #pragma unroll
    for (int c = kGmmParams; c < kOutPad; ++c) go[c] = 0.f;
    return -logp;
}

// ------------------------------------------------------------------ inference
__global__ void __launch_bounds__(128) mlp_forward_kernel(MlpDev m, const float *__restrict__ feat, uint32_t n,
                                                          float *__restrict__ out, int mixture) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
    float *stage = reinterpret_cast<float *>(smem_raw + (size_t)kWeightsFwd * 2) + (threadIdx.x / 32) * kStageFloats;
    stage_weights(m.wbf, sw, kWeightsFwd);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t wpb = blockDim.x / 32;
    for (uint32_t w = blockIdx.x * wpb + threadIdx.x / 32; (size_t)w * 16 < n; w += gridDim.x * wpb) {
        const uint32_t b0 = w * 16;
        float xn[kIn];
        #pragma unroll
        for (int k = 0; k < kIn; ++k) {
            const uint32_t row = b0 + (uint32_t)(lane & 15);
            xn[k] = row < n ? (__ldg(feat + (size_t)k * n + row) - m.shift[k]) * m.scale[k] : 0.f;
        }
        __nv_bfloat16 *sx = reinterpret_cast<__nv_bfloat16 *>(stage);
        stage_inputs(xn, sx);
        float o[6][4];
        forward<false>(m, sw, sx, o);
        __syncwarp();
        stage_outputs(o, stage);
        __syncwarp();
        if (lane < 16 && b0 + lane < n) {
            const float *row = stage + lane * kOutPad;
            if (mixture) {
                const uint32_t r = b0 + lane;
                auto F = [&](int k) { return __ldg(feat + (size_t)k * n + r); };
                float au, av;
                anchor_uv(m.frame, mk(F(0), F(1), F(2)), mk(F(3), F(4), F(5)), au, av);
                mixture_from_raw(row, out + r, n, au, av, m.sigma_scale);
            } else {
                for (int c = 0; c < kGmmParams; ++c) out[(size_t)c * n + b0 + lane] = row[c];
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ training
__global__ void __launch_bounds__(128) mlp_train_fb_kernel(MlpDev m, const float *__restrict__ feat,
                                                           const float *__restrict__ uv, size_t ld, uint32_t n_data,
                                                           int batch, int shuffle) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
    float *zs = reinterpret_cast<float *>(smem_raw + (size_t)kWeightsAll * 2) + (threadIdx.x / 32) * kZsFloats;
    float *stage = reinterpret_cast<float *>(smem_raw + (size_t)kWeightsAll * 2) + 4 * kZsFloats +
                   (threadIdx.x / 32) * kStageFloats;
    stage_weights(m.wbf, sw, kWeightsAll);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int b0 = (blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32) * 16;
    if (b0 >= batch) return;   // whole warps only (batch is a multiple of 16)
    const uint32_t step = *m.step;
    auto row_of = [&](int r) -> uint32_t {
        const uint32_t b = (uint32_t)(b0 + r);
        return shuffle ? hash32(step * 0x9E3779B9u ^ hash32(b)) % n_data : b % n_data;
    };
    float xn[kIn];
    {
        const uint32_t r = row_of(lane & 15);
        #pragma unroll
        for (int k = 0; k < kIn; ++k) xn[k] = (__ldg(feat + (size_t)k * ld + r) - m.shift[k]) * m.scale[k];
    }
    __nv_bfloat16 *sx = reinterpret_cast<__nv_bfloat16 *>(stage);
    stage_inputs(xn, sx);
    float o[6][4];
    forward<true>(m, sw, sx, o, zs, batch, b0);
    __syncwarp();
    stage_outputs(o, stage);
    __syncwarp();
    float loss = 0.f;
    if (lane < 16) {
        float oo[kOutPad], go[kOutPad];
        #pragma unroll
        for (int c = 0; c < kOutPad; ++c) oo[c] = stage[lane * kOutPad + c];
        const uint32_t r = row_of(lane);
        auto F = [&](int k) { return __ldg(feat + (size_t)k * ld + r); };
        float au, av;
        anchor_uv(m.frame, mk(F(0), F(1), F(2)), mk(F(3), F(4), F(5)), au, av);
        loss = mixture_nll(oo, __ldg(uv + r) - au, __ldg(uv + ld + r) - av, go);
        // the loss is the batch mean of (weighted) NLLs
        const float inv_b = (m.weighted ? __ldg(uv + 2 * ld + r) : 1.f) / (float)batch;
        #pragma unroll
        for (int c = 0; c < kOutPad; ++c) stage[lane * kOutPad + c] = go[c] * inv_b;
        loss *= inv_b;
    }
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
    if (lane == 0) atomicAdd(m.loss + step % kLossHist, loss);
    __syncwarp();
    float dz[8][4];
    #pragma unroll
    for (int nt = 0; nt < 6; ++nt) {
        const int c = nt * 8 + 2 * t;
        dz[nt][0] = stage[g * kOutPad + c];
        dz[nt][1] = stage[g * kOutPad + c + 1];
        dz[nt][2] = stage[(g + 8) * kOutPad + c];
        dz[nt][3] = stage[(g + 8) * kOutPad + c + 1];
    }
    #pragma unroll
    for (int l = kLayers - 1; l >= 0; --l) {
        const int NT = layer_out(l) / 8;
        // transposed dz of layer l (weight gradient operand) and bias gradient
        __nv_bfloat16 *dst = m.dzT + (size_t)dz_row(l) * batch + b0;
        #pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int c = nt * 8 + 2 * t;
            dst[(size_t)c * batch + g] = __float2bfloat16(dz[nt][0]);
            dst[(size_t)(c + 1) * batch + g] = __float2bfloat16(dz[nt][1]);
            dst[(size_t)c * batch + g + 8] = __float2bfloat16(dz[nt][2]);
            dst[(size_t)(c + 1) * batch + g + 8] = __float2bfloat16(dz[nt][3]);
            float s0 = dz[nt][0] + dz[nt][2], s1 = dz[nt][1] + dz[nt][3];
            #pragma unroll
            for (int off = 4; off < 32; off <<= 1) {
                s0 += __shfl_xor_sync(0xffffffffu, s0, off);
                s1 += __shfl_xor_sync(0xffffffffu, s1, off);
            }
            if (g == 0) {
                atomicAdd(m.grad + b_off(l) + c, s0);
                atomicAdd(m.grad + b_off(l) + c + 1, s1);
            }
        }
        if (l == 0) break;
        // dH_{l-1} = dZ_l W_l: A = dZ (bf16), B from the [in][out] copy
        uint32_t da[4][4];
        #pragma unroll
        for (int kt = 0; kt < NT / 2; ++kt) {
            da[kt][0] = pack_bf16(dz[2 * kt][0], dz[2 * kt][1]);
            da[kt][1] = pack_bf16(dz[2 * kt][2], dz[2 * kt][3]);
            da[kt][2] = pack_bf16(dz[2 * kt + 1][0], dz[2 * kt + 1][1]);
            da[kt][3] = pack_bf16(dz[2 * kt + 1][2], dz[2 * kt + 1][3]);
        }
        const __nv_bfloat16 *Wb = sw + smb_off(l);
        const int ldb = layer_out(l) + kPadK;
        const float *zp = zs + ((l - 1) * 8 * 4) * 32 + lane;
        #pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            float dh[4] = {0.f, 0.f, 0.f, 0.f};
            #pragma unroll
            for (int kt = 0; kt < NT / 2; ++kt) {
                const __nv_bfloat16 *wp = Wb + (nt * 8 + g) * ldb + kt * 16 + 2 * t;
                mma16816(dh, da[kt], *reinterpret_cast<const uint32_t *>(wp),
                         *reinterpret_cast<const uint32_t *>(wp + 8));
            }
            #pragma unroll
            for (int i = 0; i < 4; ++i) dz[nt][i] = dh[i] * dsilu(zp[(nt * 4 + i) * 32]);
        }
    }
}

// dW_l[o][i] += sum_b dz_l[b][o] h_l[b][i] over one batch chunk; one warp per
// (layer, 16x8 output tile, chunk).  A = dz^T rows, B = h^T rows: both read as
// contiguous bf16 pairs along the batch.
__global__ void __launch_bounds__(128) mlp_wgrad_kernel(MlpDev m, int batch, int chunk) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int wid = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int chunks = batch / chunk;
    int tile = wid / chunks;
    const int ch = wid % chunks;
    int l = 0;
    for (; l < kLayers; ++l) {
        const int tl = (layer_out(l) / 16) * (layer_in(l) / 8);
        if (tile < tl) break;
        tile -= tl;
    }
    if (l >= kLayers) return;
    const int K = layer_in(l);
    const int mt = tile / (K / 8), nt = tile % (K / 8);
    const __nv_bfloat16 *dz = m.dzT + (size_t)dz_row(l) * batch;
    const __nv_bfloat16 *h = m.hT + (size_t)h_row(l) * batch;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int bb = ch * chunk; bb < (ch + 1) * chunk; bb += 16) {
        const __nv_bfloat16 *ar = dz + (size_t)(mt * 16 + g) * batch + bb + 2 * t;
        const __nv_bfloat16 *ar8 = ar + (size_t)8 * batch;
        const uint32_t a[4] = {*reinterpret_cast<const uint32_t *>(ar), *reinterpret_cast<const uint32_t *>(ar8),
                               *reinterpret_cast<const uint32_t *>(ar + 8),
                               *reinterpret_cast<const uint32_t *>(ar8 + 8)};
        const __nv_bfloat16 *br = h + (size_t)(nt * 8 + g) * batch + bb + 2 * t;
        mma16816(acc, a, *reinterpret_cast<const uint32_t *>(br), *reinterpret_cast<const uint32_t *>(br + 8));
    }
    float *gw = m.grad + w_off(l);
    const int r0 = mt * 16 + g, c0 = nt * 8 + 2 * t;
    atomicAdd(gw + r0 * K + c0, acc[0]);
    atomicAdd(gw + r0 * K + c0 + 1, acc[1]);
    atomicAdd(gw + (r0 + 8) * K + c0, acc[2]);
    atomicAdd(gw + (r0 + 8) * K + c0 + 1, acc[3]);
}

// Store parameter i (FP32) into the BF16 copies / bias table.  Padded input
// columns (>= kInEnc) of the first layer stay zero.
__device__ __forceinline__ float publish(const MlpDev &m, int i, float p) {
    int l = 0;
    while (l + 1 < kLayers && i >= w_off(l + 1)) ++l;
    const int j = i - w_off(l), K = layer_in(l), N = layer_out(l);
    if (j < N * K) {
        const int r = j / K, c = j % K;
        if (l == 0 && c >= kInEnc) p = 0.f;
        m.wbf[smf_off(l) + r * (K + kPadK) + c] = __float2bfloat16(p);
        m.wbf[smb_off(l) + c * (N + kPadK) + r] = __float2bfloat16(p);
    } else {
        m.bias[l * 64 + (j - N * K)] = p;
    }
    return p;
}

__global__ void mlp_adam_kernel(MlpDev m, float lr) {
    constexpr float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float tstep = (float)(*m.step + 1u);
    const float c1 = 1.f - powf(b1, tstep), c2 = 1.f - powf(b2, tstep);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
        const float gv = m.grad[i];
        const float mo = b1 * m.adam_m[i] + (1.f - b1) * gv;
        const float vo = b2 * m.adam_v[i] + (1.f - b2) * gv * gv;
        m.adam_m[i] = mo;
        m.adam_v[i] = vo;
        m.params[i] = publish(m, i, m.params[i] - lr * (mo / c1) / (sqrtf(vo / c2) + eps));
        m.grad[i] = 0.f;
    }
}

__global__ void mlp_step_kernel(MlpDev m) {
    const uint32_t s = *m.step + 1u;
    m.loss[s % kLossHist] = 0.f;
    *m.step = s;
}

__global__ void mlp_sync_kernel(MlpDev m) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x)
        m.params[i] = publish(m, i, m.params[i]);
}

__global__ void feature_moments_kernel(const float *__restrict__ feat, size_t ld, uint32_t n, double *out) {
    __shared__ double part[2 * kIn];
    if (threadIdx.x < 2 * kIn) part[threadIdx.x] = 0.0;
    __syncthreads();
    double s[kIn], q[kIn];
    #pragma unroll
    for (int k = 0; k < kIn; ++k) { s[k] = 0.0; q[k] = 0.0; }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        #pragma unroll
        for (int k = 0; k < kIn; ++k) {
            const double f = feat[(size_t)k * ld + i];
            s[k] += f;
            q[k] += f * f;
        }
    }
    #pragma unroll
    for (int k = 0; k < kIn; ++k) {
        atomicAdd(&part[k], s[k]);
        atomicAdd(&part[kIn + k], q[k]);
    }
    __syncthreads();
    if (threadIdx.x < 2 * kIn) atomicAdd(out + threadIdx.x, part[threadIdx.x]);
}

// ---------------------------------------------------------------- launchers
size_t smem_forward() { return (size_t)kWeightsFwd * 2 + (size_t)4 * kStageFloats * 4; }
size_t smem_train() { return (size_t)kWeightsAll * 2 + (size_t)4 * (kZsFloats + kStageFloats) * 4; }
size_t smem_seed_fused() { return (size_t)kWeightsFwd * 2 + (size_t)4 * (32 * kIn + kStageFloats) * 4; }

cudaError_t configure_kernels() {
    cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_forward());
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(mlp_train_fb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_train());
}

cudaError_t launch_sync(const MlpDev &m, cudaStream_t s) {
    mlp_sync_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(m);
    return cudaGetLastError();
}

cudaError_t launch_forward(const MlpDev &m, const float *feat, uint32_t n, float *out, bool mixture, int num_sms,
                           cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t warps = (n + 15) / 16;
    const uint32_t blocks = std::min<uint32_t>((warps + 3) / 4, (uint32_t)num_sms * 4);
    mlp_forward_kernel<<<blocks, 128, smem_forward(), s>>>(m, feat, n, out, mixture ? 1 : 0);
    return cudaGetLastError();
}

static int wgrad_chunk(int batch) {
    for (int c = 1024; c > 16; c >>= 1)
        if (batch % c == 0) return c;
    return 16;
}

cudaError_t launch_train_step(const MlpDev &m, const float *feat, const float *uv, size_t ld, uint32_t n_data,
                              int batch, float lr, bool shuffle, bool update, cudaStream_t s) {
    const int warps = batch / 16;
    mlp_train_fb_kernel<<<(warps + 3) / 4, 128, smem_train(), s>>>(m, feat, uv, ld, n_data, batch, shuffle ? 1 : 0);
    int tiles = 0;
    for (int l = 0; l < kLayers; ++l) tiles += (layer_out(l) / 16) * (layer_in(l) / 8);
    const int chunk = wgrad_chunk(batch);
    const int wg_warps = tiles * (batch / chunk);
    mlp_wgrad_kernel<<<(wg_warps + 3) / 4, 128, 0, s>>>(m, batch, chunk);
    if (update) {
        mlp_adam_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(m, lr);
        mlp_step_kernel<<<1, 1, 0, s>>>(m);
    }
    return cudaGetLastError();
}

cudaError_t launch_feature_moments(const float *feat, size_t ld, uint32_t n, double *out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 512u);
    feature_moments_kernel<<<blocks, 256, 0, s>>>(feat, ld, n, out);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace sms
