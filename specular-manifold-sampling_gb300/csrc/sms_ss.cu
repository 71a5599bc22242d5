// sms_ss.cu -- single-scatter SMS kernels for sm_103a.
//
// Reference: SpecularManifoldSingleScatter (src/librender/manifold_ss.cpp):
//   specular_manifold_sampling :28-201, sample_path :203-279,
//   evaluate_path_contribution :281-327, newton_solver :329-405.
//
// Random-number layout.  Query i draws from one PCG32 stream (seed, stream
// offset + i) in the reference's order: 3 draws for the emitter sample
// (manifold.h:204-260: next_1d + next_2d), then exactly 2 draws per walk
// (sample_path's next_2d for the seed; smooth casters draw nothing else).  Walk
// m of a query therefore starts at stream position 3 + 2m, and PCG32 jump-ahead
// lets lanes run the walks of one query side by side while reproducing the
// reference's sequential draws exactly.
//
// Kernels
//   ss_walk_kernel      one lane per walk (the per-walk harness, p_start).
//   ss_biased_kernel    biased estimator (:142-197): a group of G lanes (16 or
//                       32) per query, one walk per lane, then the walk-ordered
//                       deduplication by warp shuffles.
//   ss_first_kernel     unbiased estimator, part 1: one lane per query runs the
//                       first walk, the light visibility test and the
//                       contribution; queries that need Bernoulli trials are
//                       appended to a device work queue.
//   ss_trials_kernel    unbiased estimator, part 2 (:111-135): persistent warps
//                       take queries from the queue and run the Bernoulli
//                       trials 32 at a time (lane = trial); the first success is
//                       found by ballot, so one query's trials never serialize
//                       on a single lane.
#include <algorithm>

#include "sms_device.cuh"
#include "sms_estimator.cuh"
#include "sms_kernels.h"
#include "sms_mlp.cuh"
#include "sms_ss_kernels.cuh"

namespace sms {

// ------------------------------------------------------------ walk kernel
// kTwo: two-stage solver, slope sample in walk_in rows 8-9.
template <bool kTwo>
__global__ void __launch_bounds__(128) ss_walk_kernel(DevScene sc, SolverCfg cfg, int caster,
                                                      const float *__restrict__ q, const float *__restrict__ w,
                                                      uint32_t n, float *__restrict__ out, DevCounters *ctr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    LaneStats st;
    uint32_t err = 0;
    if (i < n) {
        auto Q = [&](int k) { return __ldg(q + (size_t)k * n + i); };
        auto W = [&](int k) { return __ldg(w + (size_t)k * n + i); };
        f3 x = mk(Q(0), Q(1), Q(2));
        f3 lp = mk(W(0), W(1), W(2));
        f3 ps = mk(W(3), W(4), W(5));
        f3 seed = sample_position(sc, sc.shapes[caster], W(6), W(7));
        if (ps.x != 0.f || ps.y != 0.f || ps.z != 0.f) seed = ps;
        Vtx v;
        int it = 0;
        f3 pi = splat(0.f);
        const float g0 = kTwo ? W(8) : 0.f, g1 = kTwo ? W(9) : 0.f;
        bool ok = ss_walk<false, kTwo, true>(sc, cfg, caster, x, lp, seed, v, it, err, st, &pi, mk(0.f, 0.f, 1.f), g0,
                                             g1);
        float res[kWalkOutFields] = {ok ? 1.f : 0.f, (float)it, 0.f, 0.f, 0.f, pi.x, pi.y, pi.z, 0.f, 0.f, 0.f};
        if (ok) {
            res[2] = v.p.x; res[3] = v.p.y; res[4] = v.p.z;
            res[8] = v.n.x; res[9] = v.n.y; res[10] = v.n.z;
        }
        #pragma unroll
        for (int k = 0; k < kWalkOutFields; ++k) out[(size_t)k * n + i] = res[k];
    }
    flush_stats(st, ctr, err, kPhaseSsWalk);
}

// ------------------------------------------ learned proposal: inference
// The proposal network for every query of a batch, before its first walk:
// each warp takes 32 queries, draws their emitter samples (the same 3 draws
// the estimator makes), evaluates the network on the tensor cores (weights
// staged once per block in shared memory) and stores each query's mixture
// (cdf, means, sigmas) for the first-walk and trial kernels.  Kept apart from
// the first-walk kernel so that kernel keeps the walk kernels' occupancy (the
// network needs 168 registers and 66 KB of shared memory per block).
__global__ void __launch_bounds__(128, 3) ss_proposal_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ qs,
                                                             uint32_t n, uint64_t seed, uint64_t stream_off,
                                                             mlp::SeedProposal pr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kStage = 16 * mlp::kXLd / 2;   // floats: input tile, then output rows
    __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
    float *feats = reinterpret_cast<float *>(smem_raw + (size_t)mlp::kWeightsFwd * 2) +
                   (threadIdx.x / 32) * (32 * mlp::kIn + kStage);
    float *stage = feats + 32 * mlp::kIn;
    mlp::stage_weights(pr.net.wbf, sw, mlp::kWeightsFwd);
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    const uint32_t wpb = blockDim.x / 32;
    for (uint32_t w = blockIdx.x * wpb + threadIdx.x / 32; (size_t)w * 32 < n; w += gridDim.x * wpb) {
        const uint32_t qi = w * 32 + lane;
        const bool active = qi < n;
        f3 fx = splat(0.f), fl = splat(0.f), fn = splat(0.f);
        if (active) {
            const Query Q = load_query(qs, n, qi);
            Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
            Light L;
            fx = Q.x;
            fn = Q.n;
            if (sample_emitter(sc, sc.emitters_ss, sc.n_emitters_ss, rng, Q.x, L)) fl = L.p;
        }
        // this lane's normalised features: shading point, light sample, normal
        const float fv[mlp::kIn] = {fx.x, fx.y, fx.z, fl.x, fl.y, fl.z, fn.x, fn.y, fn.z};
        #pragma unroll
        for (int k = 0; k < mlp::kIn; ++k) feats[lane * mlp::kIn + k] = (fv[k] - pr.net.shift[k]) * pr.net.scale[k];
        __syncwarp();
        #pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            float xn[mlp::kIn];
            #pragma unroll
            for (int k = 0; k < mlp::kIn; ++k) xn[k] = feats[(h * 16 + (lane & 15)) * mlp::kIn + k];
            __nv_bfloat16 *sx = reinterpret_cast<__nv_bfloat16 *>(stage);
            mlp::stage_inputs(xn, sx);
            float o[6][4];
            mlp::forward<false>(pr.net, sw, sx, o);
            __syncwarp();
            mlp::stage_outputs(o, stage);
            __syncwarp();
            if ((int)(lane >> 4) == h && active) {
                float au, av;
                mlp::anchor_uv(pr.net.frame, fx, fl, au, av);
                mlp::mixture_from_raw(stage + (lane & 15) * mlp::kOutPad, pr.gmm + qi, n, au, av,
                                      pr.net.sigma_scale);
            }
            __syncwarp();
        }
    }
}

// ------------------------------------------------- learned proposal: data
// Training pairs for the proposal from the uniform-seed solver: per query the
// emitter sample (3 draws) and `per_query` uniform-seeded walks (2 draws each,
// the biased estimator's layout).  Every distinct solution a query's walks
// converge to (directions compared with the uniqueness threshold, as the
// biased estimator does, manifold_ss.cpp:170-178) that the light sees becomes
// one pair: features (shading point, light sample, shading normal), the
// solution's uv in the proposal frame, and a weight = its share of the
// query's total contribution (diffuse BSDF x specular path contribution, mean
// of RGB).  Keeping each solution once, however often the uniform seeds found
// it, spreads the learned mixture over all of a query's solutions; the weight
// (used by weighted training) moves the mixture mass towards p_k ~ f_k, which
// minimises the Bernoulli estimator's variance sum_k f_k^2 (2 - p_k) / p_k for
// a given total success probability.
constexpr int kCollectUnique = 16;

__global__ void __launch_bounds__(128) ss_collect_kernel(DevScene sc, SolverCfg cfg, int caster,
                                                         const float *__restrict__ qs, uint32_t n, uint64_t seed,
                                                         uint64_t stream_off, int per_query, mlp::SeedFrame fr,
                                                         float *__restrict__ data, uint32_t cap, unsigned *fill,
                                                         DevCounters *ctr) {
    const uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31;
    LaneStats st;
    uint32_t err = 0;
    Query Q;
    Pcg32 rng;
    Light L;
    bool have_light = false;
    if (qi < n) {
        Q = load_query(qs, n, qi);
        rng = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
        have_light = sample_emitter(sc, sc.emitters_ss, sc.n_emitters_ss, rng, Q.x, L);
    }
    f3 seen[kCollectUnique];     // directions of the solutions kept so far
    float kuv[kCollectUnique][2], kf[kCollectUnique];
    int n_seen = 0;
    float fsum = 0.f;
    for (int m = 0; m < per_query && have_light; ++m) {
        Vtx v;
        const float sx = rng.next_f32(), sy = rng.next_f32();
        f3 sp = sample_position(sc, sc.shapes[caster], sx, sy);
        int it;
        bool ok = ss_walk(sc, cfg, caster, Q.x, L.p, sp, v, it, err, st);
        st.walks++;
        st.newton += (unsigned)it;
        if (ok) st.succ++; else st.fail++;
        if (!ok || n_seen >= kCollectUnique) continue;
        const f3 dir = normalize(v.p - Q.x);
        bool dup = false;
        for (int j = 0; j < n_seen; ++j)
            if (fabsf(dot(dir, seen[j]) - 1.f) < cfg.uniqueness_threshold) dup = true;
        if (dup || !visible(sc, L.p, v.p, err, st)) continue;
        const f3 c = receiver_eval(sc, Q, dir, err) * contribution(sc, Q.x, L, v, err, st);
        seen[n_seen] = dir;
        mlp::frame_uv(fr, v.p, kuv[n_seen][0], kuv[n_seen][1]);
        kf[n_seen] = fmaxf(0.f, (c.x + c.y + c.z) * (1.f / 3.f));
        fsum += kf[n_seen];
        n_seen++;
    }
    // warp-aggregated append of every lane's solutions
    int incl = n_seen;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, off);
        if ((int)lane >= off) incl += y;
    }
    unsigned base = 0;
    if (lane == 31 && incl) base = atomicAdd(fill, (unsigned)incl);
    base = __shfl_sync(0xffffffffu, base, 31) + (unsigned)(incl - n_seen);
    for (int j = 0; j < n_seen; ++j) {
        const unsigned idx = base + (unsigned)j;
        if (idx >= cap) break;
        const float w = fsum > 0.f ? kf[j] / fsum : 1.f / (float)n_seen;
        const float rec[mlp::kDataRows] = {Q.x.x, Q.x.y, Q.x.z, L.p.x, L.p.y, L.p.z, Q.n.x, Q.n.y, Q.n.z,
                                           kuv[j][0], kuv[j][1], w};
        #pragma unroll
        for (int k = 0; k < mlp::kDataRows; ++k) data[(size_t)k * cap + idx] = rec[k];
    }
    flush_stats(st, ctr, err, kPhaseSsWalk);
}

// ---------------------------------------------------------------- launchers
cudaError_t launch_ss_walk(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q, const float *w,
                           uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    phase_begin(tm, kPhaseSsWalk, s);
    auto walk = cfg.twostage ? ss_walk_kernel<true> : ss_walk_kernel<false>;
    walk<<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, caster, q, w, n, out, ctr);
    phase_end(tm, s);
    return cudaGetLastError();
}

cudaError_t launch_ss_proposal(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                               uint64_t stream_off, const mlp::SeedProposal &pr, int num_sms, cudaStream_t s) {
    const size_t smem = mlp::smem_seed_fused();
    cudaError_t e = cudaFuncSetAttribute(ss_proposal_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const uint32_t pblocks = std::min<uint32_t>((n + 127) / 128, (uint32_t)num_sms * 3);
    ss_proposal_kernel<<<pblocks, 128, smem, s>>>(sc, cfg, q, n, seed, stream_off, pr);
    return cudaGetLastError();
}

// Caster variant bits (sms_ss_kernels.cuh) of caster c, or of all casters.
static int ss_variant(const DevScene &sc, const SolverCfg &cfg, int c) {
    const uint32_t mask = c < 0 ? ~0u : (1u << c);
    int var = (sc.casters_ss_rough & mask) ? 1 : 0;
    if (sc.casters_ss_nm & mask) var |= 4 | (cfg.twostage ? 2 : 0);
    return var;
}

cudaError_t launch_ss_connect(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                              uint64_t stream_off, float *value, int *count, int *walks, DevCounters *ctr,
                              const SsScratch &scr, int num_sms, int blocks_per_sm, PhaseTimer *tm,
                              cudaStream_t s, const mlp::SeedProposal *prop, int trial_group, uint32_t treelet) {
    if (n == 0) return cudaSuccess;
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : 16;
    if (cfg.biased) {
        const int var = ss_variant(sc, cfg, -1);
        if (var & 4)
            return launch_ss_biased_nm(var, sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, num_sms, bps,
                                       tm, s);
        return var ? ss_biased_launch<1>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, num_sms, bps, tm, s)
                   : ss_biased_launch<0>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr, num_sms, bps, tm,
                                         s);
    }
    if (sc.n_casters_ss == 0) {
        // no caster: every query gets zero (manifold_ss.cpp:53-55)
        cudaError_t e = cudaMemsetAsync(value, 0, 3 * (size_t)n * sizeof(float), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, (size_t)n * sizeof(int), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(walks, 0, (size_t)n * sizeof(int), s);
        return e;
    }
    for (int c = 0; c < sc.n_casters_ss; ++c) {
        cudaError_t e = cudaMemsetAsync(&ctr->trial_count, 0, 2 * sizeof(unsigned), s);
        if (e != cudaSuccess) return e;
        const int var = ss_variant(sc, cfg, c);
        if (var & 4)
            e = launch_ss_caster_nm(var, sc, cfg, c, q, n, seed, stream_off, value, count, walks, ctr, scr, num_sms,
                                    bps, tm, s, trial_group);
        else if (var)
            e = ss_caster_launch<1, true>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, ctr, scr, num_sms,
                                          bps, tm, s, prop, trial_group, treelet);
        else
            e = ss_caster_launch<0, true>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, ctr, scr, num_sms,
                                          bps, tm, s, prop, trial_group, treelet);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_ss_collect(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q, uint32_t n,
                              uint64_t seed, uint64_t stream_off, int per_query, const mlp::SeedFrame &fr,
                              float *data, uint32_t cap, unsigned *fill, DevCounters *ctr, PhaseTimer *tm,
                              cudaStream_t s) {
    if (n == 0 || per_query <= 0) return cudaSuccess;
    phase_begin(tm, kPhaseSsWalk, s);
    ss_collect_kernel<<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, caster, q, n, seed, stream_off, per_query, fr, data,
                                                      cap, fill, ctr);
    phase_end(tm, s);
    return cudaGetLastError();
}

}  // namespace sms
