// sms_ms_rough_k1.cu -- multi-scatter estimators for chains of 1 specular
// vertices with rough (alpha > 0) chain shapes: offset normals per vertex.
#include "sms_ms_kernels.cuh"

namespace sms {

template cudaError_t ms_connect_k<1, false, true>(const DevScene &sc, const SolverCfg &cfg, const float *q,
                                                uint32_t n, uint64_t seed, uint64_t stream_off, float *value,
                                                int *count, int *walks, DevCounters *ctr, const SsScratch &scr,
                                                int *tmpl, int num_sms, int bps, PhaseTimer *tm, cudaStream_t s);

}  // namespace sms
