// sms_mlp.h -- host-visible layout of the learned seed proposal (network
// parameters, training buffers, seeding frame) and its kernel launchers.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sms {
namespace mlp {

constexpr int kIn = 9;          // shading point, light sample, shading normal
// The first layer sees each normalised feature f and sin / cos (pi 2^j f),
// j < kEncFreq (a frequency encoding: a plain MLP on raw coordinates cannot
// follow how fast solutions move with the shading point under a wavy
// caster), zero-padded to six k-tiles.
constexpr int kEncFreq = 4;
constexpr int kInEnc = kIn * (1 + 2 * kEncFreq);   // 81
constexpr int kInPad = 96;
constexpr int kXLd = kInPad + 8;                   // staged input row (bf16)
constexpr int kHidden = 64;
constexpr int kLayers = 5;      // 4 hidden layers + output layer
constexpr int kComp = 8;        // mixture components
constexpr int kGmmParams = 40;  // 8 logits, 8 x 2 means, 8 x 2 log-sigma logits
constexpr int kOutPad = 48;     // output layer width (multiple of 16)
// Log-sigma of a component is kLsMin + (kLsMax - kLsMin) * sigmoid(raw).
constexpr float kLsMin = -7.f;
constexpr float kLsMax = 0.f;
constexpr int kDataRows = kIn + 3;   // training pair: features, uv, weight
constexpr int kLossHist = 256;  // per-step loss ring
constexpr int kMaxBatch = 65536;

__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? kInPad : kHidden; }
__host__ __device__ constexpr int layer_out(int l) { return l == kLayers - 1 ? kOutPad : kHidden; }
// FP32 master parameters: W_l [out][in] then b_l [out], layer after layer.
__host__ __device__ constexpr int w_off(int l) {
    int o = 0;
    for (int i = 0; i < l; ++i) o += layer_out(i) * layer_in(i) + layer_out(i);
    return o;
}
__host__ __device__ constexpr int b_off(int l) { return w_off(l) + layer_out(l) * layer_in(l); }
constexpr int kParams = w_off(kLayers);
static_assert(kParams == 21808, "parameter count");
// BF16 weight copies: forward [out][in + pad] for all layers, then backward
// [in][out + pad]; rows padded by 8 elements against shared-memory bank
// conflicts of the fragment loads.
constexpr int kPadK = 8;
__host__ __device__ constexpr int smf_off(int l) {
    int o = 0;
    for (int i = 0; i < l; ++i) o += layer_out(i) * (layer_in(i) + kPadK);
    return o;
}
__host__ __device__ constexpr int smb_off(int l) {
    int o = smf_off(kLayers);
    for (int i = 0; i < l; ++i) o += layer_in(i) * (layer_out(i) + kPadK);
    return o;
}
constexpr int kWeightsFwd = smf_off(kLayers);  // bf16 elements of the forward copy
constexpr int kWeightsAll = smb_off(kLayers);  // both copies
// Rows of the transposed training activations: layer inputs and
// pre-activation gradients, [row][batch] bf16.
__host__ __device__ constexpr int h_row(int l) { return l == 0 ? 0 : kInPad + (l - 1) * kHidden; }
__host__ __device__ constexpr int dz_row(int l) { return l * kHidden; }
constexpr int kHRows = h_row(kLayers);
constexpr int kDzRows = dz_row(kLayers);

// Where a seed drawn in uv lands on the specular shape.
//  kind 0 (mesh): seed = org + u ax_u + v ax_v over the caster's bounding
//                 box (the two widest axes; org on the mid-plane of the third)
//  kind 1 (sphere): seed = org + r (sin(pi u) cos(2 pi v), sin(pi u) sin(2 pi v), cos(pi u)), r = ax_u[0]
struct SeedFrame {
    int kind;
    float org[3];
    float ax_u[3];
    float ax_v[3];
};

// Device state of one network.  The mixture means are offsets from an
// anchor uv computed in FP32 from the raw features and the caster's frame
// (sms_mlp.cuh, anchor_uv), so the BF16 network only regresses the small
// displacement of a solution from the straight light path, not absolute
// coordinates.
struct MlpDev {
    float *params;          // kParams FP32 master copy
    float *grad;            // kParams, cleared by the Adam kernel
    float *adam_m, *adam_v; // kParams each
    __nv_bfloat16 *wbf;     // kWeightsAll
    float *bias;            // [kLayers][64] FP32 biases read by the forward pass
    uint32_t *step;         // optimizer steps taken
    float *loss;            // kLossHist mean batch losses, slot step % kLossHist
    __nv_bfloat16 *hT;      // kHRows x batch
    __nv_bfloat16 *dzT;     // kDzRows x batch
    float shift[kIn];       // input normalisation: (f - shift) * scale
    float scale[kIn];
    SeedFrame frame;        // anchor of the mixture means
    float sigma_scale;      // seeding sharpness: sigmas of the processed mixture x this
    int weighted;           // training loss weighted by the pairs' contribution shares
};

// A learned proposal bound to a context for the unbiased single-scatter
// estimator: one caster shape, its seeding frame, the network and the
// per-query mixture scratch (kGmmParams x n: cdf[8], mean[8][2], sigma[8][2]).
struct SeedProposal {
    int shape;          // caster shape id the proposal seeds; -1 = none
    float defensive;    // probability of the uniform seeding
    SeedFrame frame;
    MlpDev net;
    float *gmm;
};

size_t smem_forward();
size_t smem_train();
size_t smem_seed_fused();
cudaError_t configure_kernels();
cudaError_t launch_sync(const MlpDev &m, cudaStream_t s);
// Raw network outputs (kGmmParams x n) or the processed mixture (same shape).
cudaError_t launch_forward(const MlpDev &m, const float *feat, uint32_t n, float *out, bool mixture, int num_sms,
                           cudaStream_t s);
// One optimizer step over a batch drawn (with replacement) from the data set
// (feat: kIn rows, then uv: 2 rows and weight: 1 row, row stride ld, n_data
// pairs); shuffle=false takes rows 0..batch-1; update=false stops after the
// gradient.
cudaError_t launch_train_step(const MlpDev &m, const float *feat, const float *uv, size_t ld, uint32_t n_data,
                              int batch, float lr, bool shuffle, bool update, cudaStream_t s);
// Per-feature sums and sums of squares (2 kIn doubles, accumulated).
cudaError_t launch_feature_moments(const float *feat, size_t ld, uint32_t n, double *out, cudaStream_t s);

}  // namespace mlp
}  // namespace sms
