// sms_ms.cu -- multi-scatter entry points: dispatch on the chain length K to
// the per-K launchers of sms_ms_kernels.cuh (instantiated in sms_ms_k1.cu ..
// sms_ms_k4.cu).
#include "sms_device.cuh"
#include "sms_kernels.h"

namespace sms {

template <int K>
cudaError_t ms_walk_k(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q, const float *w,
                      uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s);
template <int K>
cudaError_t ms_connect_k(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                         uint64_t stream_off, float *value, int *count, int *walks, DevCounters *ctr,
                         const SsScratch &scr, int *tmpl, int num_sms, int bps, PhaseTimer *tm, cudaStream_t s);
template <int K>
cudaError_t ms_mnee_check_k(const DevScene &sc, const SolverCfg &cfg, const float *rec, const float *stage,
                            const int *want, float *L, uint32_t n, uint32_t stride, DevCounters *ctr,
                            cudaStream_t s);

cudaError_t launch_ms_mnee_check(const DevScene &sc, const SolverCfg &cfg, int bounces, const float *rec,
                                 const float *stage, const int *want, float *L, uint32_t n, uint32_t stride,
                                 DevCounters *ctr, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    switch (bounces) {
    case 1: return ms_mnee_check_k<1>(sc, cfg, rec, stage, want, L, n, stride, ctr, s);
    case 2: return ms_mnee_check_k<2>(sc, cfg, rec, stage, want, L, n, stride, ctr, s);
    case 3: return ms_mnee_check_k<3>(sc, cfg, rec, stage, want, L, n, stride, ctr, s);
    case 4: return ms_mnee_check_k<4>(sc, cfg, rec, stage, want, L, n, stride, ctr, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_ms_walk(const DevScene &sc, const SolverCfg &cfg, int bounces, int caster, const float *q,
                           const float *w, uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    switch (bounces) {
    case 1: return ms_walk_k<1>(sc, cfg, caster, q, w, n, out, ctr, tm, s);
    case 2: return ms_walk_k<2>(sc, cfg, caster, q, w, n, out, ctr, tm, s);
    case 3: return ms_walk_k<3>(sc, cfg, caster, q, w, n, out, ctr, tm, s);
    case 4: return ms_walk_k<4>(sc, cfg, caster, q, w, n, out, ctr, tm, s);
    default: return cudaErrorInvalidValue;
    }
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
    switch (bounces) {
    case 1: return ms_connect_k<1>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl, num_sms, bps, tm, s);
    case 2: return ms_connect_k<2>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl, num_sms, bps, tm, s);
    case 3: return ms_connect_k<3>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl, num_sms, bps, tm, s);
    case 4: return ms_connect_k<4>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, scr, tmpl, num_sms, bps, tm, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace sms
