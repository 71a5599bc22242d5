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

namespace sms {

// ------------------------------------------------------------ walk kernel
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
        bool ok = ss_walk(sc, cfg, caster, x, lp, seed, v, it, err, st, &pi);
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

// ------------------------------------------------------ biased estimator
// Group of G lanes per query; walk m of caster c sits at stream position
// 3 + 2 (c M + m).  Contributions are summed in walk order over the first
// occurrences of each solution direction, exactly as manifold_ss.cpp:146-196.
template <int G, bool kRough>
__global__ void __launch_bounds__(128, 4) ss_biased_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ qs,
                                                        uint32_t n, uint64_t seed, uint64_t stream_off,
                                                        float *__restrict__ value, int *__restrict__ count,
                                                        int *__restrict__ walks, DevCounters *ctr) {
    constexpr int kGroupsPerBlock = 128 / G;
    __shared__ f3 rec[kGroupsPerBlock][kMaxSolutions];
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31;
    const int gl = (int)(threadIdx.x % G);             // lane within group
    const int gib = (int)(threadIdx.x / G);            // group within block
    const int gbase = (int)(lane & ~(unsigned)(G - 1));
    const unsigned gmask = (G == 32) ? full : (((1u << G) - 1u) << gbase);
    LaneStats st;
    uint32_t err = 0;
    const int M = cfg.max_trials > 0 ? cfg.max_trials : 0;
    const uint32_t groups_total = gridDim.x * kGroupsPerBlock;
    // every group of the grid runs the same number of rounds (full-warp syncs)
    const uint32_t rounds = (n + groups_total - 1) / groups_total;
    for (uint32_t r = 0; r < rounds; ++r) {
        uint32_t qi = (r * gridDim.x + blockIdx.x) * kGroupsPerBlock + gib;
        bool live = qi < n;
        Query Q{};
        Light L{};
        bool have_light = false;
        if (live) {
            Q = load_query(qs, n, qi);
            Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
            have_light = sample_emitter(sc, sc.emitters_ss, sc.n_emitters_ss, rng, Q.x, L);
        }
        bool work = live && have_light && sc.n_casters_ss > 0;
        if (work && gl == 0) st.conns++;
        f3 acc = splat(0.f);
        int n_unique = 0;
        uint64_t cpos = 3u;   // stream position of the caster's first draw
        for (int c = 0; c < sc.n_casters_ss; ++c) {
            int caster = sc.casters_ss[c];
            const DevShape &cs = sc.shapes[caster];
            float p_off = 1.f;
            f3 no = mk(0.f, 0.f, 1.f);
            if (kRough && work && cs.alpha > 0.f) {
                Pcg32 r0 = query_rng(seed, query_stream(cfg, stream_off, qi), cpos);
                no = caster_offset(cs, r0, p_off);
            }
            const uint64_t wpos = cpos + caster_draws(cs);
            int nrec = 0;
            f3 cur = splat(0.f);
            for (int m0 = 0; m0 < M; m0 += G) {
                int m = m0 + gl;
                bool cand = false;
                f3 dir = splat(0.f), contrib = splat(0.f);
                if (work && m < M) {
                    Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), wpos + 2u * (uint64_t)m);
                    float sx = rng.next_f32(), sy = rng.next_f32();
                    f3 sp = sample_position(sc, cs, sx, sy);
                    Vtx v;
                    int it;
                    bool ok = ss_walk<kRough>(sc, cfg, caster, Q.x, L.p, sp, v, it, err, st, nullptr, no);
                    st.walks++;
                    st.newton += (unsigned)it;
                    if (ok) {
                        st.succ++;
                        if (visible(sc, L.p, v.p, err, st)) {
                            cand = true;
                            dir = normalize(v.p - Q.x);
                            // evaluated for every visible solution; only first
                            // occurrences are kept below
                            contrib = diffuse_eval(Q, dir) * contribution(sc, Q.x, L, v, err, st);
                        }
                    } else {
                        st.fail++;
                    }
                }
                // walk-ordered deduplication within the group
                for (int k = 0; k < G; ++k) {
                    const int src = gbase + k;
                    bool ck = __shfl_sync(full, cand, src);
                    f3 dk = mk(__shfl_sync(full, dir.x, src), __shfl_sync(full, dir.y, src),
                               __shfl_sync(full, dir.z, src));
                    f3 vk = mk(__shfl_sync(full, contrib.x, src), __shfl_sync(full, contrib.y, src),
                               __shfl_sync(full, contrib.z, src));
                    bool dup = false;
                    if (ck)
                        for (int j = gl; j < nrec; j += G)
                            if (fabsf(dot(dk, rec[gib][j]) - 1.f) < cfg.uniqueness_threshold) dup = true;
                    unsigned anydup = __ballot_sync(full, dup) & gmask;
                    __syncwarp();
                    if (ck && !anydup) {
                        if (nrec < kMaxSolutions) {
                            if (gl == 0) rec[gib][nrec] = dk;
                            nrec++;
                            cur = cur + vk;
                        } else {
                            err |= kErrSolutionOverflow;
                        }
                    }
                    __syncwarp();
                }
            }
            acc = kRough ? acc + cur * (1.f / p_off) : acc + cur;
            n_unique += nrec;
            cpos = wpos + 2u * (uint64_t)M;
        }
        if (live && gl == 0) {
            value[qi] = acc.x;
            value[(size_t)n + qi] = acc.y;
            value[2 * (size_t)n + qi] = acc.z;
            count[qi] = n_unique;
            walks[qi] = work ? M * sc.n_casters_ss : 0;
        }
    }
    flush_stats(st, ctr, err, kPhaseSsBiased);
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

// --------------------------------------------------- unbiased: first walks
// kLearned: seeds come from the query's learned mixture (three draws per walk,
// mlp::proposal_seed, mixture from ss_proposal_kernel) instead of two-draw
// uniform seeding.
template <bool kLearned, bool kRough>
__global__ void __launch_bounds__(128, 8) ss_first_kernel(DevScene sc, SolverCfg cfg, int c, const float *__restrict__ qs,
                                                       uint32_t n, uint64_t seed, uint64_t stream_off,
                                                       float *__restrict__ value, int *__restrict__ count,
                                                       int *__restrict__ walks, SsScratch scr, DevCounters *ctr,
                                                       mlp::SeedProposal pr) {
    const uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = qi < n;
    const unsigned lane = threadIdx.x & 31;
    LaneStats st;
    uint32_t err = 0;
    bool enqueue = false;
    Query Q;
    Pcg32 rng;
    Light L;
    bool have_light = false;
    if (active) {
        Q = load_query(qs, n, qi);
        rng = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
        have_light = sample_emitter(sc, sc.emitters_ss, sc.n_emitters_ss, rng, Q.x, L);
    }
    if (active) {
        uint32_t pos = 3u;
        f3 acc = splat(0.f);
        int nw = 0;
        if (c == 0) {
            if (have_light) st.conns++;
        } else {
            pos = scr.pos[qi];
            acc = mk(value[qi], value[(size_t)n + qi], value[2 * (size_t)n + qi]);
            nw = walks[qi];
        }
        if (have_light) {
            const int caster = sc.casters_ss[c];
            rng.advance(pos - 3u);
            float p_off = 1.f;
            f3 no = mk(0.f, 0.f, 1.f);
            if (kRough) {
                no = caster_offset(sc.shapes[caster], rng, p_off);
                pos += caster_draws(sc.shapes[caster]);
            }
            f3 sp;
            if constexpr (kLearned) {
                const float us = rng.next_f32(), sx = rng.next_f32(), sy = rng.next_f32();
                pos += 3u;
                sp = mlp::proposal_seed(sc, pr, sc.shapes[caster], pr.gmm + qi, n, us, sx, sy);
            } else {
                const float sx = rng.next_f32(), sy = rng.next_f32();
                pos += 2u;
                sp = sample_position(sc, sc.shapes[caster], sx, sy);
            }
            Vtx v;
            int it;
            bool ok = ss_walk<kRough>(sc, cfg, caster, Q.x, L.p, sp, v, it, err, st, nullptr, no);
            st.walks++;
            st.newton += (unsigned)it;
            nw++;
            if (ok) {
                st.succ++;
                if (visible(sc, L.p, v.p, err, st)) {
                    f3 dir = normalize(v.p - Q.x);
                    f3 spec = contribution(sc, Q.x, L, v, err, st);
                    // the caster's estimate is divided by the offset density (manifold_ss.cpp:199)
                    f3 val = kRough ? diffuse_eval(Q, dir) * spec * (1.f / p_off) : diffuse_eval(Q, dir) * spec;
                    scr.dir0[qi] = dir.x; scr.dir0[(size_t)n + qi] = dir.y; scr.dir0[2 * (size_t)n + qi] = dir.z;
                    scr.val[qi] = val.x; scr.val[(size_t)n + qi] = val.y; scr.val[2 * (size_t)n + qi] = val.z;
                    enqueue = true;
                }
            } else {
                st.fail++;
            }
        }
        scr.pos[qi] = pos;
        value[qi] = acc.x;
        value[(size_t)n + qi] = acc.y;
        value[2 * (size_t)n + qi] = acc.z;
        count[qi] = 0;
        walks[qi] = nw;
    }
    // warp-aggregated append to the trial queue
    unsigned want = __ballot_sync(0xffffffffu, enqueue);
    if (want) {
        unsigned leader = __ffs(want) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&ctr->trial_count, (unsigned)__popc(want));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (enqueue) scr.list[base + __popc(want & ((1u << lane) - 1u))] = qi;
    }
    flush_stats(st, ctr, err, kPhaseSsFirst);
}

// ------------------------------------------------ unbiased: Bernoulli trials
// Persistent warps split into groups of G lanes; each group takes queries
// from the queue and runs their Bernoulli trials G at a time (lane = trial).
// For query q with first-walk direction dir0 the trials are t = 1, 2, ...;
// trial t draws stream positions pos + S(t-1) .. (S = 2 draws per walk, 3 with
// a learned proposal), so the first success -- found by ballot -- is exactly
// the reference's sequential trial count (manifold_ss.cpp:115-135) whatever
// G is.  G = 32 suits uniform seeding (tens of trials per query); a learned
// proposal succeeds within a few trials and runs G = 8 (four queries per warp)
// to cut the speculative walks past the first success.  Every trial redraws
// its seed from the same per-query proposal as the first walk, so the count
// still estimates the inverse probability of reaching dir0.
//
// All lanes run one warp-uniform loop: groups whose query finished fetch the
// next one at the top, so every ballot and shuffle has the whole warp.
template <bool kLearned, int G, bool kRough>
__global__ void __launch_bounds__(128, 8) ss_trials_kernel(DevScene sc, SolverCfg cfg, int c, const float *__restrict__ qs,
                                                        uint32_t n, uint64_t seed, uint64_t stream_off,
                                                        float *__restrict__ value, int *__restrict__ count,
                                                        int *__restrict__ walks, SsScratch scr, DevCounters *ctr,
                                                        mlp::SeedProposal pr) {
    static_assert(G == 8 || G == 16 || G == 32, "group size");
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31;
    const unsigned gbase = lane & ~(unsigned)(G - 1), gl = lane - gbase;
    const unsigned gmask = (G == 32) ? full : (((1u << G) - 1u) << gbase);
    constexpr uint32_t kStride = kLearned ? 3u : 2u;
    LaneStats st;
    uint32_t err = 0;
    const int cap = cfg.max_trials > 0 ? cfg.max_trials : kTrialHardLimit;
    const int caster = sc.casters_ss[c];
    const unsigned n_list = *(volatile unsigned *)&ctr->trial_count;
    // per-group state (replicated on the group's lanes)
    bool have = false, drained = false;
    uint32_t qi = 0, pos = 0;
    int t0 = 1;
    Query Q;
    Light L;
    Pcg32 base;
    f3 dir0 = splat(0.f);
    f3 no = mk(0.f, 0.f, 1.f);
    const DevShape &cshape = sc.shapes[caster];
    while (true) {
        // groups without a query take the next one
        const bool need = !have && !drained;
        unsigned idx = 0;
        if (need && gl == 0) idx = atomicAdd(&ctr->trial_head, 1u);
        idx = __shfl_sync(full, idx, gbase);
        if (need) {
            if (idx < n_list) {
                have = true;
                qi = scr.list[idx];
                Q = load_query(qs, n, qi);
                base = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
                sample_emitter(sc, sc.emitters_ss, sc.n_emitters_ss, base, Q.x, L);   // base sits at position 3
                pos = scr.pos[qi];
                dir0 = mk(scr.dir0[qi], scr.dir0[(size_t)n + qi], scr.dir0[2 * (size_t)n + qi]);
                t0 = 1;
                if (kRough) {
                    // the offset normal drawn before the first walk
                    Pcg32 r0 = base;
                    r0.advance((uint64_t)(pos - 3u - kStride - 2u));
                    float p_off;
                    no = caster_offset(cshape, r0, p_off);
                }
            } else {
                drained = true;
            }
        }
        if (__ballot_sync(full, have) == 0u) break;
        const int t = t0 + (int)gl;
        bool succ = false;
        int it = 0;
        if (have && t <= cap) {
            Pcg32 rng = base;
            rng.advance((uint64_t)(pos - 3u) + kStride * (uint64_t)(t - 1));
            f3 sp;
            if constexpr (kLearned) {
                const float us = rng.next_f32(), sx = rng.next_f32(), sy = rng.next_f32();
                sp = mlp::proposal_seed(sc, pr, sc.shapes[caster], pr.gmm + qi, n, us, sx, sy);
            } else {
                const float sx = rng.next_f32(), sy = rng.next_f32();
                sp = sample_position(sc, sc.shapes[caster], sx, sy);
            }
            Vtx v;
            succ = ss_walk<kRough>(sc, cfg, caster, Q.x, L.p, sp, v, it, err, st, nullptr, no) &&
                   fabsf(dot(dir0, normalize(v.p - Q.x)) - 1.f) < cfg.uniqueness_threshold;
        }
        const unsigned b = (__ballot_sync(full, succ) & gmask) >> gbase;
        const int f = b ? t0 + __ffs(b) - 1 : 0x7fffffff;
        if (have && t <= cap) {
            // trials up to the first success are the reference's walks; the
            // rest of the chunk is speculative work
            if (t <= f) { st.walks++; st.newton += (unsigned)it; }
            else st.spec++;
        }
        if (have && (b || t0 + G > cap)) {
            if (gl == 0) {
                float inv_prob;
                int iterations, trial_walks;
                if (b) {
                    iterations = f;
                    inv_prob = (float)f;
                    trial_walks = f;
                } else {
                    iterations = cap + 1;
                    inv_prob = 0.f;
                    trial_walks = cap;
                    if (cfg.max_trials <= 0) err |= kErrTrialLimit;
                }
                f3 val = mk(scr.val[qi], scr.val[(size_t)n + qi], scr.val[2 * (size_t)n + qi]);
                f3 cur = val * inv_prob;
                value[qi] += cur.x;
                value[(size_t)n + qi] += cur.y;
                value[2 * (size_t)n + qi] += cur.z;
                count[qi] = b ? iterations : -1;
                walks[qi] += trial_walks;
                scr.pos[qi] = pos + kStride * (uint32_t)trial_walks;
                st.calls++;
                st.iters += (unsigned long long)iterations;
                st.imax = max(st.imax, (unsigned long long)iterations);
            }
            have = false;
        } else if (have) {
            t0 += G;
        }
    }
    flush_stats(st, ctr, err, kPhaseSsTrials);
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
        const f3 c = diffuse_eval(Q, dir) * contribution(sc, Q.x, L, v, err, st);
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
    ss_walk_kernel<<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, caster, q, w, n, out, ctr);
    phase_end(tm, s);
    return cudaGetLastError();
}

cudaError_t launch_ss_connect(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                              uint64_t stream_off, float *value, int *count, int *walks, DevCounters *ctr,
                              const SsScratch &scr, int num_sms, int blocks_per_sm, PhaseTimer *tm,
                              cudaStream_t s, const mlp::SeedProposal *prop, int trial_group) {
    if (n == 0) return cudaSuccess;
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : 16;
    if (cfg.biased) {
        const int G = cfg.max_trials <= 16 ? 16 : 32;
        const uint32_t groups_per_block = 128 / G;
        uint32_t blocks_needed = (n + groups_per_block - 1) / groups_per_block;
        uint32_t blocks = std::min<uint32_t>(blocks_needed, (uint32_t)(num_sms * bps));
        phase_begin(tm, kPhaseSsBiased, s);
        auto biased = sc.casters_ss_rough ? (G == 16 ? ss_biased_kernel<16, true> : ss_biased_kernel<32, true>)
                                          : (G == 16 ? ss_biased_kernel<16, false> : ss_biased_kernel<32, false>);
        biased<<<blocks, 128, 0, s>>>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr);
        phase_end(tm, s);
        return cudaGetLastError();
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
        const bool learned = prop && prop->shape == sc.casters_ss[c];
        const bool rough = (sc.casters_ss_rough >> c) & 1u;
        const mlp::SeedProposal pr = learned ? *prop : mlp::SeedProposal{};
        phase_begin(tm, kPhaseSsFirst, s);
        if (learned) {
            const size_t smem = mlp::smem_seed_fused();
            e = cudaFuncSetAttribute(ss_proposal_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            const uint32_t pblocks = std::min<uint32_t>((n + 127) / 128, (uint32_t)num_sms * 3);
            ss_proposal_kernel<<<pblocks, 128, smem, s>>>(sc, cfg, q, n, seed, stream_off, pr);
            auto first = rough ? ss_first_kernel<true, true> : ss_first_kernel<true, false>;
            first<<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, scr, ctr,
                                                  pr);
        } else {
            auto first = rough ? ss_first_kernel<false, true> : ss_first_kernel<false, false>;
            first<<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, scr, ctr,
                                                  pr);
        }
        phase_end(tm, s);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        phase_begin(tm, kPhaseSsTrials, s);
        const int group = trial_group > 0 ? trial_group : (learned ? 8 : 32);
        auto trials =
            rough ? (learned ? (group == 8    ? ss_trials_kernel<true, 8, true>
                                : group == 16 ? ss_trials_kernel<true, 16, true>
                                              : ss_trials_kernel<true, 32, true>)
                             : (group == 8    ? ss_trials_kernel<false, 8, true>
                                : group == 16 ? ss_trials_kernel<false, 16, true>
                                              : ss_trials_kernel<false, 32, true>))
                  : (learned ? (group == 8    ? ss_trials_kernel<true, 8, false>
                                : group == 16 ? ss_trials_kernel<true, 16, false>
                                              : ss_trials_kernel<true, 32, false>)
                             : (group == 8    ? ss_trials_kernel<false, 8, false>
                                : group == 16 ? ss_trials_kernel<false, 16, false>
                                              : ss_trials_kernel<false, 32, false>));
        trials<<<num_sms * bps, 128, 0, s>>>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, scr, ctr, pr);
        phase_end(tm, s);
        e = cudaGetLastError();
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
