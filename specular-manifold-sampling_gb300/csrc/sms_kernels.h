// sms_kernels.h -- interface between the host library and the CUDA kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sms_gb300.h"
#include "sms_mlp.h"

namespace sms {

struct DevScene;
struct DevCounters;

// Optional per-phase CUDA-event timing (host side, sms_host.cu).  Both calls
// are no-ops when tm is null or profiling is off.
struct PhaseTimer;
void phase_begin(PhaseTimer *tm, int phase, cudaStream_t s);
void phase_end(PhaseTimer *tm, cudaStream_t s);

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
    int mnee_init;      // seed along the straight path (manifold_ss.cpp:229-241)
    int twostage;       // two-stage solver on normal-mapped casters (manifold_ss.cpp:253-270)
    // Optional per-query random-number stream table: query i draws from stream
    // streams[i] instead of stream_off + i (the path tracer keys each query by
    // its path and bounce, so that results do not depend on which paths of a
    // wavefront reached a receiver or on how the queries were batched).
    const uint64_t *streams;
    // Queries a lane group of the Bernoulli-trial kernel claims from the work
    // queue per atomic (1: one at a time).
    int queue_chunk;
};

// Unique-solution capacity per query of the biased estimator (shared memory
// per lane group).  More unique solutions than this set an error flag.
constexpr int kMaxSolutions = 64;
// Bernoulli trials are unbounded in the reference when max_trials <= 0
// (manifold_ss.cpp:127); the device loop stops here and flags the query.
constexpr int kTrialHardLimit = 1 << 16;
// Rows of the per-walk outputs (sms_ss_walk_batch, sms_ms_walk_batch).
constexpr int kWalkOutFields = 11;
constexpr int kMsWalkOutFields = 9;
constexpr int kGlintWalkOutFields = 6;
constexpr int kGlintQueryFields = 21;
constexpr int kGlintWalkInFields = 5;
// Longest specular chain of the multi-scatter kernels.
constexpr int kMaxBounces = 4;

// Per-query scratch of the unbiased estimator (device memory, n entries):
// stream position after the walks done so far, first-walk direction and
// contribution, and the queue of queries that need Bernoulli trials.
struct SsScratch {
    uint32_t *pos;    // n
    float *dir0;      // 3 x n
    float *val;       // 3 x n
    uint32_t *list;   // n
};
// Bytes of SsScratch for n queries.
inline size_t ss_scratch_bytes(uint32_t n) { return (size_t)n * (4 + 12 + 12 + 4); }

// Largest shared-memory treelet of the trial kernel: 384 node records (24 KB
// per block; 8 resident blocks of 128 threads stay within 227 KB per SM).
constexpr int kMaxTreeletNodes = 384;

cudaError_t launch_ss_walk(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q,
                           const float *w, uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm,
                           cudaStream_t s);
cudaError_t launch_ss_connect(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n,
                              uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                              DevCounters *ctr, const SsScratch &scr, int num_sms, int blocks_per_sm,
                              PhaseTimer *tm, cudaStream_t s, const mlp::SeedProposal *prop = nullptr,
                              int trial_group = 0, uint32_t treelet = 0);
// The proposal network for every query of a batch (ss_proposal_kernel).
cudaError_t launch_ss_proposal(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                               uint64_t stream_off, const mlp::SeedProposal &pr, int num_sms, cudaStream_t s);
// The unbiased-MNEE test of path_sms_ms for a wavefront (ms_mnee_check_kernel).
cudaError_t launch_ms_mnee_check(const DevScene &sc, const SolverCfg &cfg, int bounces, const float *rec,
                                 const float *stage, const int *want, float *L, uint32_t n, uint32_t stride,
                                 DevCounters *ctr, cudaStream_t s);
// Normal-mapped caster variants (sms_ss_nm.cu), var = the caster variant bits.
cudaError_t launch_ss_biased_nm(int var, const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n,
                                uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                                DevCounters *ctr, int num_sms, int bps, PhaseTimer *tm, cudaStream_t s);
cudaError_t launch_ss_caster_nm(int var, const DevScene &sc, const SolverCfg &cfg, int c, const float *q, uint32_t n,
                                uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                                DevCounters *ctr, const SsScratch &scr, int num_sms, int bps, PhaseTimer *tm,
                                cudaStream_t s, int trial_group);
// Training pairs for a learned proposal (see ss_collect_kernel).
cudaError_t launch_ss_collect(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q, uint32_t n,
                              uint64_t seed, uint64_t stream_off, int per_query, const mlp::SeedFrame &fr,
                              float *data, uint32_t cap, unsigned *fill, DevCounters *ctr, PhaseTimer *tm,
                              cudaStream_t s);

cudaError_t launch_ms_walk(const DevScene &sc, const SolverCfg &cfg, int bounces, int caster, const float *q,
                           const float *w, uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s);
cudaError_t launch_ms_connect(const DevScene &sc, const SolverCfg &cfg, int bounces, const float *q, uint32_t n,
                              uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                              DevCounters *ctr, const SsScratch &scr, int *tmpl, int num_sms, int blocks_per_sm,
                              PhaseTimer *tm, cudaStream_t s);

cudaError_t launch_glint_walk(const DevScene &sc, const SolverCfg &cfg, const float *q, const float *w, uint32_t n,
                              float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s);
cudaError_t launch_glint_connect(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                                 uint64_t stream_off, float *value, int *count, int *walks, DevCounters *ctr,
                                 const SsScratch &scr, int num_sms, int blocks_per_sm, PhaseTimer *tm, cudaStream_t s);

// LEAN mip pyramid of the slope map: `levels` levels, level l at out + offsets[l].
cudaError_t launch_lean_build(const DevScene &sc, float *out, const uint32_t *offsets, int levels, cudaStream_t s);

// Read-only view of a context for entry points defined outside sms_host.cu.
struct CtxView {
    int device;
    cudaStream_t stream;
    const DevScene *scene;
    SolverCfg solver;
    DevCounters *counters;
    int num_sms;
    int blocks_per_sm;
    PhaseTimer *timer;
    const mlp::SeedFrame *frames;   // learned-proposal uv frame per shape
    int n_shapes;
    bool proposal_bound;            // a learned proposal seeds the SS estimator
    int trial_group;                // lanes per query of the trial kernel (0: auto)
    int bounces;                    // multi-scatter chain length (sms_config::bounces)
    int bsdf_strategy_only, sms_strategy_only;   // glints MIS switches (sms_config)
    bool nm_rough;                  // the normal-mapped shape is rough (alpha > 0)
};

}  // namespace sms

// Context accessors implemented in sms_host.cu.
struct sms_ctx;
bool ctx_view(sms_ctx *c, sms::CtxView &out);
// Replace the context's config by *in (validated), returning the old one in
// *old when old is not null; false if *in is invalid.
bool ctx_swap_config(sms_ctx *c, const sms_config *in, sms_config *old);
// Connection entry points shared with the path tracer (sms_render.cu): as
// sms_ss_connect_batch_device / sms_ms_connect_batch_device, with an optional
// per-query stream table (SolverCfg::streams).
sms_status ctx_ss_connect(sms_ctx *c, const float *q, uint32_t n, uint64_t seed, uint64_t stream_off,
                          const uint64_t *streams, sms_result *out);
// Configuration checks of a single-scatter connection (max_trials bound, learned
// proposal, two-stage solver and normal maps), shared by every single-scatter
// connection entry point.  may_allocate false: report a missing LEAN pyramid
// instead of building it.
sms_status ctx_ss_check(sms_ctx *c, bool may_allocate);
sms_status ctx_ms_connect(sms_ctx *c, const float *q, uint32_t n, uint64_t seed, uint64_t stream_off,
                          const uint64_t *streams, sms_result *out);
sms_status ctx_glint_connect(sms_ctx *c, const float *q, uint32_t n, uint64_t seed, uint64_t stream_off,
                             const uint64_t *streams, sms_result *out);
// Checks the glints scene, then builds the LEAN pyramid (ctx_build_lean).
sms_status ctx_ensure_lean(sms_ctx *c);
// Samples per pixel of the context's last render (sms_render_spp_done).
void ctx_set_render_spp(sms_ctx *c, uint32_t spp);
// Builds the LEAN pyramid of the scene's normal map on first use (the
// context's scene view then carries it).
sms_status ctx_build_lean(sms_ctx *c);
// Reads and clears the device error flags of a context (synchronizes its
// stream); SMS_ERR_DEVICE_LIMIT with the reasons when any was set.
sms_status ctx_check_device_error(sms_ctx *c);
// Records msg as sms_last_error() for this thread and returns st.
int set_last_error_impl(int st, const char *msg);

// Learned proposals (sms_proposal.cu) and the context that binds them.
struct sms_proposal;
sms_ctx *proposal_ctx(sms_proposal *p);
// Shape, frame and network of a proposal (defensive and gmm left to the caller).
bool proposal_seed_desc(sms_proposal *p, sms::mlp::SeedProposal &out);
// The context is going away: the proposal keeps working for nothing but destroy.
void proposal_detach(sms_proposal *p);
// A proposal was made on / is going away from a context (which detaches all
// of its proposals when it is destroyed first).
void ctx_register_proposal(sms_ctx *c, sms_proposal *p);
void ctx_forget_proposal(sms_ctx *c, sms_proposal *p);
