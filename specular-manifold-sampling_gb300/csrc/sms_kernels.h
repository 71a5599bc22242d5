// sms_kernels.h -- interface between the host library and the CUDA kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sms {

struct DevScene;
struct DevCounters;

// Solver parameters the kernels read (a subset of sms_config, already
// validated by the host).
struct SolverCfg {
    int biased;
    int halfvector;
    int max_iterations;
    int max_trials;
    float solver_threshold;
    float uniqueness_threshold;
    float step_scale;
};

// Unique-solution capacity per query of the biased estimator (per lane, in
// local memory).  More unique solutions than this set an error flag.
constexpr int kMaxSolutions = 64;
// Bernoulli trials are unbounded in the reference when max_trials <= 0
// (manifold_ss.cpp:127); the device loop stops here and flags the query.
constexpr int kTrialHardLimit = 1 << 22;

cudaError_t launch_ss_walk(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q,
                           const float *w, uint32_t n, float *out, DevCounters *ctr, cudaStream_t s);
cudaError_t launch_ss_connect(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n,
                              uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                              DevCounters *ctr, int blocks, cudaStream_t s);
int ss_connect_max_blocks_per_sm();

}  // namespace sms
