// sms_ms_k3.cu -- multi-scatter kernels for chains of 3 specular vertices,
// chain shapes without the normal map.
#include "sms_ms_kernels.cuh"

namespace sms {

template cudaError_t ms_walk_k<3, false>(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q,
                                    const float *w, uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm,
                                    cudaStream_t s);
template cudaError_t ms_connect_k<3, false>(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n,
                                       uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                                       DevCounters *ctr, const SsScratch &scr, int *tmpl, int num_sms, int bps,
                                       PhaseTimer *tm, cudaStream_t s);
template cudaError_t ms_mnee_check_k<3, false>(const DevScene &sc, const SolverCfg &cfg, const float *rec,
                                          const float *stage, const int *want, float *L, uint32_t n,
                                          uint32_t stride, DevCounters *ctr, cudaStream_t s);

}  // namespace sms
