// sms_ms.cu -- multi-scatter entry points: dispatch on the chain length K and
// on normal-mapped or rough chain shapes to the launchers of sms_ms_kernels.cuh
// (instantiated in sms_ms_k{1..4}.cu, sms_ms_nm_k{1..4}.cu and
// sms_ms_rough_k{1..4}.cu).
#include "sms_device.cuh"
#include "sms_kernels.h"

namespace sms {

template <int K, bool kNM>
cudaError_t ms_walk_k(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q, const float *w,
                      uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s);
template <int K, bool kNM, bool kRough = false>
cudaError_t ms_connect_k(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                         uint64_t stream_off, float *value, int *count, int *walks, DevCounters *ctr,
                         const SsScratch &scr, int *tmpl, int num_sms, int bps, PhaseTimer *tm, cudaStream_t s);
template <int K, bool kNM>
cudaError_t ms_mnee_check_k(const DevScene &sc, const SolverCfg &cfg, const float *rec, const float *stage,
                            const int *want, float *L, uint32_t n, uint32_t stride, DevCounters *ctr,
                            cudaStream_t s);

// One launcher per (K, kNM): K from the chain length, kNM from the scene.
template <bool kNM>
static cudaError_t mnee_check_nm(const DevScene &sc, const SolverCfg &cfg, int bounces, const float *rec,
                                 const float *stage, const int *want, float *L, uint32_t n, uint32_t stride,
                                 DevCounters *ctr, cudaStream_t s) {
    switch (bounces) {
    case 1: return ms_mnee_check_k<1, kNM>(sc, cfg, rec, stage, want, L, n, stride, ctr, s);
    case 2: return ms_mnee_check_k<2, kNM>(sc, cfg, rec, stage, want, L, n, stride, ctr, s);
    case 3: return ms_mnee_check_k<3, kNM>(sc, cfg, rec, stage, want, L, n, stride, ctr, s);
    case 4: return ms_mnee_check_k<4, kNM>(sc, cfg, rec, stage, want, L, n, stride, ctr, s);
    default: return cudaErrorInvalidValue;
    }
}

template <bool kNM>
static cudaError_t walk_nm(const DevScene &sc, const SolverCfg &cfg, int bounces, int caster, const float *q,
                           const float *w, uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s) {
    switch (bounces) {
    case 1: return ms_walk_k<1, kNM>(sc, cfg, caster, q, w, n, out, ctr, tm, s);
    case 2: return ms_walk_k<2, kNM>(sc, cfg, caster, q, w, n, out, ctr, tm, s);
    case 3: return ms_walk_k<3, kNM>(sc, cfg, caster, q, w, n, out, ctr, tm, s);
    case 4: return ms_walk_k<4, kNM>(sc, cfg, caster, q, w, n, out, ctr, tm, s);
    default: return cudaErrorInvalidValue;
    }
}

template <bool kNM, bool kRough = false>
static cudaError_t connect_nm(const DevScene &sc, const SolverCfg &cfg, int bounces, const float *q, uint32_t n,
                              uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                              DevCounters *ctr, const SsScratch &scr, int *tmpl, int num_sms, int bps,
                              PhaseTimer *tm, cudaStream_t s) {
    switch (bounces) {
    case 1:
        return ms_connect_k<1, kNM, kRough>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl,
                                             num_sms, bps, tm, s);
    case 2:
        return ms_connect_k<2, kNM, kRough>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl,
                                             num_sms, bps, tm, s);
    case 3:
        return ms_connect_k<3, kNM, kRough>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl,
                                             num_sms, bps, tm, s);
    case 4:
        return ms_connect_k<4, kNM, kRough>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl,
                                             num_sms, bps, tm, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_ms_mnee_check(const DevScene &sc, const SolverCfg &cfg, int bounces, const float *rec,
                                 const float *stage, const int *want, float *L, uint32_t n, uint32_t stride,
                                 DevCounters *ctr, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    return sc.ms_nm ? mnee_check_nm<true>(sc, cfg, bounces, rec, stage, want, L, n, stride, ctr, s)
                    : mnee_check_nm<false>(sc, cfg, bounces, rec, stage, want, L, n, stride, ctr, s);
}

cudaError_t launch_ms_walk(const DevScene &sc, const SolverCfg &cfg, int bounces, int caster, const float *q,
                           const float *w, uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    return sc.ms_nm ? walk_nm<true>(sc, cfg, bounces, caster, q, w, n, out, ctr, tm, s)
                    : walk_nm<false>(sc, cfg, bounces, caster, q, w, n, out, ctr, tm, s);
}

cudaError_t launch_ms_connect(const DevScene &sc, const SolverCfg &cfg, int bounces, const float *q, uint32_t n,
                              uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                              DevCounters *ctr, const SsScratch &scr, int *tmpl, int num_sms, int blocks_per_sm,
                              PhaseTimer *tm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (sc.n_casters_ms == 0) {
        cudaError_t e = cudaMemsetAsync(value, 0, 3 * (size_t)n * sizeof(float), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, (size_t)n * sizeof(int), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(walks, 0, (size_t)n * sizeof(int), s);
        return e;
    }
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : 16;
    if (sc.ms_rough) {
        // rough chain shapes (offset normals); the host refuses rough + normal-mapped
        if (sc.ms_nm) return cudaErrorNotSupported;
        return connect_nm<false, true>(sc, cfg, bounces, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl,
                                       num_sms, bps, tm, s);
    }
    return sc.ms_nm ? connect_nm<true>(sc, cfg, bounces, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl,
                                       num_sms, bps, tm, s)
                    : connect_nm<false>(sc, cfg, bounces, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl,
                                        num_sms, bps, tm, s);
}

}  // namespace sms
