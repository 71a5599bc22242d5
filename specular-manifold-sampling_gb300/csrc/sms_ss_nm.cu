// sms_ss_nm.cu -- single-scatter estimator kernels for normal-mapped casters
// (manifold vertices with the normal map's frame, optionally rough and with
// the two-stage solver of manifold_ss.cpp:253-270).  Uniform seeding only.
#include "sms_ss_kernels.cuh"

namespace sms {

cudaError_t launch_ss_biased_nm(int var, const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n,
                                uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                                DevCounters *ctr, int num_sms, int bps, PhaseTimer *tm, cudaStream_t s) {
    switch (var) {
        case 4: return ss_biased_launch<4>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, num_sms, bps, tm, s);
        case 5: return ss_biased_launch<5>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, num_sms, bps, tm, s);
        case 6: return ss_biased_launch<6>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, num_sms, bps, tm, s);
        default: return ss_biased_launch<7>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, num_sms, bps, tm, s);
    }
}

cudaError_t launch_ss_caster_nm(int var, const DevScene &sc, const SolverCfg &cfg, int c, const float *q, uint32_t n,
                                uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                                DevCounters *ctr, const SsScratch &scr, int num_sms, int bps, PhaseTimer *tm,
                                cudaStream_t s, int trial_group) {
    switch (var) {
        case 4:
            return ss_caster_launch<4, false>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, ctr, scr,
                                              num_sms, bps, tm, s, nullptr, trial_group);
        case 5:
            return ss_caster_launch<5, false>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, ctr, scr,
                                              num_sms, bps, tm, s, nullptr, trial_group);
        case 6:
            return ss_caster_launch<6, false>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, ctr, scr,
                                              num_sms, bps, tm, s, nullptr, trial_group);
        default:
            return ss_caster_launch<7, false>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, ctr, scr,
                                              num_sms, bps, tm, s, nullptr, trial_group);
    }
}

}  // namespace sms
