// sms_mlp.cuh -- device side of the learned seed proposal: the warp-level
// BF16 tensor-core forward pass, the mixture transform and seed sampling.
//
// A warp carries 16 samples (one m16 tile) through all layers in registers:
// the FP32 accumulator fragment of n-tiles (2k, 2k+1) of mma.m16n8k16 is, once
// rounded to BF16 and paired, exactly the A fragment of k-tile k of the next
// layer, so hidden activations never leave the register file.
#pragma once
#include <cuda_bf16.h>

#include "sms_device.cuh"
#include "sms_mlp.h"

namespace sms {
namespace mlp {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ float2 unpack_bf16(uint32_t u) {
    __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162 *>(&u);
    return __bfloat1622float2(v);
}

// D += A (16x16 bf16, row-major) * B (16x8 bf16, column-major), FP32 accumulate.
__device__ __forceinline__ void mma16816(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float sigmoid(float z) { return 1.f / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid(z); }
__device__ __forceinline__ float dsilu(float z) {
    float s = sigmoid(z);
    return s * (1.f + z * (1.f - s));
}

// Copy bf16 weights (first `elems` elements) to shared memory; 16-byte moves.
__device__ __forceinline__ void stage_weights(const __nv_bfloat16 *__restrict__ src, __nv_bfloat16 *dst, int elems) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (int i = threadIdx.x; i < elems / 8; i += blockDim.x) d4[i] = __ldg(s4 + i);
}

// Stage the encoded inputs of a 16-row tile as bf16 rows of kXLd elements:
// lanes 0..15 each write the row of their own normalised features xn (the
// other lanes' xn is ignored).  Columns: xn[0..8], then per feature sin
// (pi 2^j xn), j < kEncFreq, and cos (pi 2^j xn), then zeros.
__device__ __forceinline__ void stage_inputs(const float xn[kIn], __nv_bfloat16 *sx) {
    const int lane = threadIdx.x & 31;
    if (lane < 16) {
        __nv_bfloat16 *row = sx + lane * kXLd;
        #pragma unroll
        for (int f = 0; f < kIn; ++f) {
            row[f] = __float2bfloat16(xn[f]);
            #pragma unroll
            for (int j = 0; j < kEncFreq; ++j) {
                float sn, cs;
                sincospif(xn[f] * (float)(1 << j), &sn, &cs);
                row[kIn + f * 2 * kEncFreq + j] = __float2bfloat16(sn);
                row[kIn + f * 2 * kEncFreq + kEncFreq + j] = __float2bfloat16(cs);
            }
        }
        #pragma unroll
        for (int c = kInEnc; c < kInPad; ++c) row[c] = __float2bfloat16(0.f);
    }
    __syncwarp();
}

// Forward pass of one warp's 16 samples.  sw: forward weight copy in shared
// memory; sx: the staged input tile.  out: accumulators of the output layer
// (6 n-tiles).  When kTrain, the layer inputs are written transposed to hT
// ([row][batch]) and the hidden pre-activations to zs (per warp,
// [layer][ntile][4][32] floats).
template <bool kTrain>
__device__ __forceinline__ void forward(const MlpDev &m, const __nv_bfloat16 *sw, const __nv_bfloat16 *sx,
                                        float out[6][4], float *zs = nullptr, int batch = 0, int b0 = 0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    if (kTrain) {
        // layer-0 input, transposed
        for (int i = lane; i < kInPad * 16; i += 32) {
            const int c = i >> 4, r = i & 15;
            m.hT[(size_t)c * batch + b0 + r] = sx[r * kXLd + c];
        }
    }
    uint32_t a[4][4];
    #pragma unroll
    for (int l = 0; l < kLayers; ++l) {
        const int NT = layer_out(l) / 8, ld = layer_in(l) + kPadK;
        const __nv_bfloat16 *W = sw + smf_off(l);
        if (kTrain && l > 0) {
            __nv_bfloat16 *dst = m.hT + (size_t)h_row(l) * batch + b0;
            #pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                const int k0 = kt * 16 + 2 * t;
                const float2 v0 = unpack_bf16(a[kt][0]), v1 = unpack_bf16(a[kt][1]);
                const float2 v2 = unpack_bf16(a[kt][2]), v3 = unpack_bf16(a[kt][3]);
                dst[(size_t)k0 * batch + g] = __float2bfloat16(v0.x);
                dst[(size_t)(k0 + 1) * batch + g] = __float2bfloat16(v0.y);
                dst[(size_t)k0 * batch + g + 8] = __float2bfloat16(v1.x);
                dst[(size_t)(k0 + 1) * batch + g + 8] = __float2bfloat16(v1.y);
                dst[(size_t)(k0 + 8) * batch + g] = __float2bfloat16(v2.x);
                dst[(size_t)(k0 + 9) * batch + g] = __float2bfloat16(v2.y);
                dst[(size_t)(k0 + 8) * batch + g + 8] = __float2bfloat16(v3.x);
                dst[(size_t)(k0 + 9) * batch + g + 8] = __float2bfloat16(v3.y);
            }
        }
        float acc[8][4];
        #pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const float bb0 = m.bias[l * 64 + nt * 8 + 2 * t], bb1 = m.bias[l * 64 + nt * 8 + 2 * t + 1];
            acc[nt][0] = bb0; acc[nt][1] = bb1; acc[nt][2] = bb0; acc[nt][3] = bb1;
        }
        if (l == 0) {
            // A fragments straight from the staged rows, one k-tile at a time
            #pragma unroll
            for (int kt = 0; kt < kInPad / 16; ++kt) {
                const __nv_bfloat16 *xp = sx + g * kXLd + kt * 16 + 2 * t;
                const uint32_t a0[4] = {*reinterpret_cast<const uint32_t *>(xp),
                                        *reinterpret_cast<const uint32_t *>(xp + 8 * kXLd),
                                        *reinterpret_cast<const uint32_t *>(xp + 8),
                                        *reinterpret_cast<const uint32_t *>(xp + 8 * kXLd + 8)};
                #pragma unroll
                for (int nt = 0; nt < NT; ++nt) {
                    const __nv_bfloat16 *wp = W + (nt * 8 + g) * ld + kt * 16 + 2 * t;
                    mma16816(acc[nt], a0, *reinterpret_cast<const uint32_t *>(wp),
                             *reinterpret_cast<const uint32_t *>(wp + 8));
                }
            }
        } else {
            #pragma unroll
            for (int nt = 0; nt < NT; ++nt)
                #pragma unroll
                for (int kt = 0; kt < 4; ++kt) {
                    const __nv_bfloat16 *wp = W + (nt * 8 + g) * ld + kt * 16 + 2 * t;
                    mma16816(acc[nt], a[kt], *reinterpret_cast<const uint32_t *>(wp),
                             *reinterpret_cast<const uint32_t *>(wp + 8));
                }
        }
        if (l == kLayers - 1) {
            #pragma unroll
            for (int nt = 0; nt < 6; ++nt)
                #pragma unroll
                for (int i = 0; i < 4; ++i) out[nt][i] = acc[nt][i];
        } else {
            #pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                if (kTrain) {
                    float *zp = zs + ((l * 8 + nt) * 4) * 32 + lane;
                    #pragma unroll
                    for (int i = 0; i < 4; ++i) zp[i * 32] = acc[nt][i];
                }
                #pragma unroll
                for (int i = 0; i < 4; ++i) acc[nt][i] = silu(acc[nt][i]);
            }
            #pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                a[kt][0] = pack_bf16(acc[2 * kt][0], acc[2 * kt][1]);
                a[kt][1] = pack_bf16(acc[2 * kt][2], acc[2 * kt][3]);
                a[kt][2] = pack_bf16(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
                a[kt][3] = pack_bf16(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
            }
        }
    }
}

// Write the output accumulators as rows of `stage` ([16][kOutPad] floats).
__device__ __forceinline__ void stage_outputs(const float o[6][4], float *stage) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    #pragma unroll
    for (int nt = 0; nt < 6; ++nt) {
        const int c = nt * 8 + 2 * t;
        stage[g * kOutPad + c] = o[nt][0];
        stage[g * kOutPad + c + 1] = o[nt][1];
        stage[(g + 8) * kOutPad + c] = o[nt][2];
        stage[(g + 8) * kOutPad + c + 1] = o[nt][3];
    }
}

__device__ __forceinline__ float log_sigma(float raw) { return kLsMin + (kLsMax - kLsMin) * sigmoid(raw); }

// Raw outputs o[0..39] -> mixture (cdf[8], mean[16], sigma[16]) written with
// stride `stride` (SoA of a query batch); means are anchor + offset, sigmas
// are scaled by sigma_scale (seeding sharpness).
__device__ __forceinline__ void mixture_from_raw(const float *o, float *dst, size_t stride, float au, float av,
                                                 float sigma_scale) {
    float mx = o[0];
    #pragma unroll
    for (int k = 1; k < kComp; ++k) mx = fmaxf(mx, o[k]);
    float w[kComp], s = 0.f;
    #pragma unroll
    for (int k = 0; k < kComp; ++k) { w[k] = __expf(o[k] - mx); s += w[k]; }
    const float inv = 1.f / s;
    float c = 0.f;
    #pragma unroll
    for (int k = 0; k < kComp; ++k) {
        c += w[k] * inv;
        dst[(size_t)k * stride] = k == kComp - 1 ? 1.f : c;
    }
    #pragma unroll
    for (int k = 0; k < 2 * kComp; ++k) {
        dst[(size_t)(8 + k) * stride] = o[8 + k] + ((k & 1) ? av : au);
        dst[(size_t)(24 + k) * stride] = sigma_scale * __expf(log_sigma(o[24 + k]));
    }
}

// uv -> seed point on the frame.
__device__ __forceinline__ f3 frame_point(const SeedFrame &fr, float u, float v) {
    const f3 o = mk(fr.org[0], fr.org[1], fr.org[2]);
    if (fr.kind == 1) {
        float st, ct, sp, cp;
        sincospif(u, &st, &ct);
        sincospif(2.f * v, &sp, &cp);
        return o + mk(st * cp, st * sp, ct) * fr.ax_u[0];
    }
    return o + mk(fr.ax_u[0], fr.ax_u[1], fr.ax_u[2]) * u + mk(fr.ax_v[0], fr.ax_v[1], fr.ax_v[2]) * v;
}

// point on the shape -> uv (inverse of frame_point).
__device__ __forceinline__ void frame_uv(const SeedFrame &fr, f3 p, float &u, float &v) {
    const f3 d = p - mk(fr.org[0], fr.org[1], fr.org[2]);
    if (fr.kind == 1) {
        const float r = fr.ax_u[0];
        const float z = fminf(1.f, fmaxf(-1.f, d.z / r));
        u = acosf(z) * kInvPi;
        float ph = atan2f(d.y, d.x);
        if (ph < 0.f) ph += 2.f * kPi;
        v = ph * (0.5f * kInvPi);
        return;
    }
    const f3 au = mk(fr.ax_u[0], fr.ax_u[1], fr.ax_u[2]), av = mk(fr.ax_v[0], fr.ax_v[1], fr.ax_v[2]);
    u = dot(d, au) / dot(au, au);
    v = dot(d, av) / dot(av, av);
}

// Anchor of the mixture means for shading point x and light sample lp: the
// uv where the straight segment x -> lp meets the frame's plane (box frames;
// clamped to [-1, 2]^2), or the uv of the sphere point along the bisector of
// the directions from the centre to x and to lp (sphere frames).
__device__ __forceinline__ void anchor_uv(const SeedFrame &fr, f3 x, f3 lp, float &u, float &v) {
    const f3 o = mk(fr.org[0], fr.org[1], fr.org[2]);
    if (fr.kind == 1) {
        const f3 a = normalize(x - o), b = normalize(lp - o), h = a + b;
        const float l2 = dot(h, h);
        const f3 d = l2 > 1e-12f ? h * (1.f / sqrtf(l2)) : a;
        frame_uv(fr, o + d * fr.ax_u[0], u, v);
        return;
    }
    const f3 au = mk(fr.ax_u[0], fr.ax_u[1], fr.ax_u[2]), av = mk(fr.ax_v[0], fr.ax_v[1], fr.ax_v[2]);
    const f3 nrm = cross(au, av), d = lp - x;
    const float den = dot(d, nrm);
    const float t = fabsf(den) > 1e-12f * sqrtf(dot(d, d) * dot(nrm, nrm)) ? dot(o - x, nrm) / den : 0.5f;
    frame_uv(fr, x + d * t, u, v);
    u = fminf(2.f, fmaxf(-1.f, u));
    v = fminf(2.f, fmaxf(-1.f, v));
}

// Seed of one walk under the proposal: three uniform draws (component or
// defensive choice, then a 2D sample).  With probability `defensive` the
// shape's uniform seeding (the reference's sample_position); otherwise a
// Gaussian draw (Box-Muller) from the chosen component of the query's
// mixture (gmm: kGmmParams rows with row stride n).
__device__ __forceinline__ f3 proposal_seed(const DevScene &sc, const SeedProposal &pr, const DevShape &shape, const float *gmm,
                       size_t n, float u_sel, float u1, float u2) {
    if (u_sel < pr.defensive) return sample_position(sc, shape, u1, u2);
    const float us = (u_sel - pr.defensive) / (1.f - pr.defensive);
    int k = 0;
    while (k < kComp - 1 && us >= sms_ldg(gmm + (size_t)k * n)) ++k;
    const float r = sqrtf(-2.f * logf(1.f - u1));
    float sn, cs;
    sincospif(2.f * u2, &sn, &cs);
    const float u = sms_ldg(gmm + (size_t)(8 + 2 * k) * n) + sms_ldg(gmm + (size_t)(24 + 2 * k) * n) * (r * cs);
    const float v = sms_ldg(gmm + (size_t)(9 + 2 * k) * n) + sms_ldg(gmm + (size_t)(25 + 2 * k) * n) * (r * sn);
    return frame_point(pr.frame, u, v);
}

}  // namespace mlp
}  // namespace sms
