// sms_ss_kernels.cuh -- the single-scatter estimator kernels (biased, unbiased
// first walks, Bernoulli trials) and their per-caster launchers, templated on
// the caster variant kVar: bit 0 rough (offset normals), bit 1 two-stage
// solver, bit 2 normal-mapped manifold vertices.  sms_ss.cu instantiates the
// plain and rough variants, sms_ss_nm.cu the normal-mapped ones, so neither
// translation unit carries all of them.
//
// Random-number layout: query i owns stream (seed, stream) -- 3 numbers for
// the emitter sample, then per caster its offset normal (2, rough casters)
// and per walk the seed (2; 3 with a learned proposal) and, with the
// two-stage solver, the slope of its smoothed first solve (2, drawn for every
// walk so that walk m always starts at the same position).
#pragma once
#include <algorithm>

#include "sms_device.cuh"
#include "sms_estimator.cuh"
#include "sms_kernels.h"
#include "sms_mlp.cuh"

namespace sms {

// Resident blocks per SM the first-walk and trial kernels are compiled for
// (128 threads each): 9 gives 56 registers per thread, the measured optimum of
// the latency-bound walks (the headline step at 4 / 6 / 7 / 8 / 10 blocks:
// 62.4 / 53.3 / 50.6 / 49.7 / 57.8 ms; with the current traversal loop 8 and
// 9 blocks: 42.9 and 42.1 ms).
#ifndef SMS_SS_WALK_MIN_BLOCKS
#define SMS_SS_WALK_MIN_BLOCKS 9
#endif

// ------------------------------------------------------ biased estimator
// Group of G lanes per query; walk m of caster c sits at stream position
// 3 + 2 (c M + m).  Contributions are summed in walk order over the first
// occurrences of each solution direction, exactly as manifold_ss.cpp:146-196.
template <int G, int kVar>
__global__ void __launch_bounds__(128, 4) ss_biased_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ qs,
                                                        uint32_t n, uint64_t seed, uint64_t stream_off,
                                                        float *__restrict__ value, int *__restrict__ count,
                                                        int *__restrict__ walks, DevCounters *ctr) {
    constexpr bool kRough = (kVar & 1) != 0, kTwo = (kVar & 2) != 0, kNM = (kVar & 4) != 0;
    constexpr uint32_t kWalk = kTwo ? 4u : 2u;   // numbers per walk: seed position (+ two-stage slope)
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
                    Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), wpos + kWalk * (uint64_t)m);
                    float sx = rng.next_f32(), sy = rng.next_f32();
                    f3 sp = sample_position(sc, cs, sx, sy);
                    float g0 = 0.f, g1 = 0.f;
                    if (kTwo) { g0 = rng.next_f32(); g1 = rng.next_f32(); }
                    Vtx v;
                    int it;
                    bool ok = ss_walk<kRough, kTwo, kNM>(sc, cfg, caster, Q.x, L.p, sp, v, it, err, st, nullptr, no,
                                                         g0, g1);
                    st.walks++;
                    st.newton += (unsigned)it;
                    if (ok) {
                        st.succ++;
                        if (visible(sc, L.p, v.p, err, st)) {
                            cand = true;
                            dir = normalize(v.p - Q.x);
                            // evaluated for every visible solution; only first
                            // occurrences are kept below
                            contrib = receiver_eval(sc, Q, dir, err) * contribution<kNM>(sc, Q.x, L, v, err, st);
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
            cpos = wpos + kWalk * (uint64_t)M;
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

// --------------------------------------------------- unbiased: first walks
// kLearned: seeds come from the query's learned mixture (three draws per walk,
// mlp::proposal_seed, mixture from ss_proposal_kernel) instead of two-draw
// uniform seeding.
template <bool kLearned, int kVar>
__global__ void __launch_bounds__(128, SMS_SS_WALK_MIN_BLOCKS) ss_first_kernel(DevScene sc, SolverCfg cfg, int c, const float *__restrict__ qs,
                                                       uint32_t n, uint64_t seed, uint64_t stream_off,
                                                       float *__restrict__ value, int *__restrict__ count,
                                                       int *__restrict__ walks, SsScratch scr, DevCounters *ctr,
                                                       mlp::SeedProposal pr) {
    constexpr bool kRough = (kVar & 1) != 0, kTwo = (kVar & 2) != 0, kNM = (kVar & 4) != 0;
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
            float g0 = 0.f, g1 = 0.f;
            if (kTwo) {
                g0 = rng.next_f32();
                g1 = rng.next_f32();
                pos += 2u;
            }
            Vtx v;
            int it;
            bool ok = ss_walk<kRough, kTwo, kNM>(sc, cfg, caster, Q.x, L.p, sp, v, it, err, st, nullptr, no, g0, g1);
            st.walks++;
            st.newton += (unsigned)it;
            nw++;
            if (ok) {
                st.succ++;
                if (visible(sc, L.p, v.p, err, st)) {
                    f3 dir = normalize(v.p - Q.x);
                    f3 spec = contribution<kNM>(sc, Q.x, L, v, err, st);
                    // the caster's estimate is divided by the offset density (manifold_ss.cpp:199)
                    f3 val = kRough ? receiver_eval(sc, Q, dir, err) * spec * (1.f / p_off) : receiver_eval(sc, Q, dir, err) * spec;
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
template <bool kLearned, int G, int kVar, bool kTree = false>
__global__ void __launch_bounds__(128, SMS_SS_WALK_MIN_BLOCKS) ss_trials_kernel(DevScene sc, SolverCfg cfg, int c, const float *__restrict__ qs,
                                                        uint32_t n, uint64_t seed, uint64_t stream_off,
                                                        float *__restrict__ value, int *__restrict__ count,
                                                        int *__restrict__ walks, SsScratch scr, DevCounters *ctr,
                                                        mlp::SeedProposal pr) {
    static_assert(G == 8 || G == 16 || G == 32, "group size");
    constexpr bool kRough = (kVar & 1) != 0, kTwo = (kVar & 2) != 0, kNM = (kVar & 4) != 0;
    if (kTree) tree_smem_fill(sc);
    const unsigned full = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31;
    const unsigned gbase = lane & ~(unsigned)(G - 1), gl = lane - gbase;
    const unsigned gmask = (G == 32) ? full : (((1u << G) - 1u) << gbase);
    constexpr uint32_t kStride = (kLearned ? 3u : 2u) + (kTwo ? 2u : 0u);   // numbers per walk
    LaneStats st;
    uint32_t err = 0;
    const int cap = cfg.max_trials > 0 ? cfg.max_trials : kTrialHardLimit;
    const int caster = sc.casters_ss[c];
    const unsigned n_list = *(volatile unsigned *)&ctr->trial_count;
    // per-group state (replicated on the group's lanes)
    bool have = false, drained = false;
    const unsigned chunk = cfg.queue_chunk > 1 ? (unsigned)cfg.queue_chunk : 1u;
    unsigned cnext = 0, cend = 0;   // the group's claimed range of the queue
    uint32_t qi = 0, pos = 0;
    int t0 = 1;
    Query Q;
    Light L;
    Pcg32 base;
    f3 dir0 = splat(0.f);
    f3 no = mk(0.f, 0.f, 1.f);
    const DevShape &cshape = sc.shapes[caster];
    while (true) {
        // groups without a query take the next one, claiming `chunk` queue
        // entries per atomic
        const bool need = !have && !drained;
        const bool claim = need && cnext == cend;
        unsigned got = 0;
        if (claim && gl == 0) got = atomicAdd(&ctr->trial_head, chunk);
        got = __shfl_sync(full, got, gbase);
        if (claim) { cnext = got; cend = got + chunk; }
        const unsigned idx = cnext;
        if (need) {
            ++cnext;
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
            float g0 = 0.f, g1 = 0.f;
            if (kTwo) { g0 = rng.next_f32(); g1 = rng.next_f32(); }
            Vtx v;
            succ = ss_walk<kRough, kTwo, kNM, kTree>(sc, cfg, caster, Q.x, L.p, sp, v, it, err, st, nullptr, no, g0,
                                                     g1) &&
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

// ------------------------------------------------- per-variant launchers
template <int kVar>
cudaError_t ss_biased_launch(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                             uint64_t stream_off, float *value, int *count, int *walks, DevCounters *ctr,
                             int num_sms, int bps, PhaseTimer *tm, cudaStream_t s) {
    const int G = cfg.max_trials <= 16 ? 16 : 32;
    const uint32_t groups_per_block = 128 / G;
    uint32_t blocks_needed = (n + groups_per_block - 1) / groups_per_block;
    uint32_t blocks = std::min<uint32_t>(blocks_needed, (uint32_t)(num_sms * bps));
    phase_begin(tm, kPhaseSsBiased, s);
    auto biased = G == 16 ? ss_biased_kernel<16, kVar> : ss_biased_kernel<32, kVar>;
    biased<<<blocks, 128, 0, s>>>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr);
    phase_end(tm, s);
    return cudaGetLastError();
}

// First walks and Bernoulli trials of caster c (kLearnedOk: a learned
// proposal may seed it).
template <int kVar, bool kLearnedOk>
cudaError_t ss_caster_launch(const DevScene &sc, const SolverCfg &cfg, int c, const float *q, uint32_t n,
                             uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                             DevCounters *ctr, const SsScratch &scr, int num_sms, int bps, PhaseTimer *tm,
                             cudaStream_t s, const mlp::SeedProposal *prop, int trial_group, uint32_t treelet = 0) {
    const bool learned = kLearnedOk && prop && prop->shape == sc.casters_ss[c];
    // the trial kernel holds the top `treelet` node records in shared memory
    // (plain and rough casters)
    DevScene st = sc;
    st.n_tnodes = (kVar & 4) ? 0u : std::min<uint32_t>(treelet, sc.n_nodes);
    const size_t tsmem = (size_t)st.n_tnodes * 4 * sizeof(float4);
    const mlp::SeedProposal pr = learned ? *prop : mlp::SeedProposal{};
    phase_begin(tm, kPhaseSsFirst, s);
    cudaError_t e = cudaSuccess;
    if constexpr (kLearnedOk) {
        if (learned) {
            e = launch_ss_proposal(sc, cfg, q, n, seed, stream_off, pr, num_sms, s);
            if (e != cudaSuccess) return e;
            ss_first_kernel<true, kVar><<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, c, q, n, seed, stream_off, value,
                                                                        count, walks, scr, ctr, pr);
        }
    }
    if (!learned)
        ss_first_kernel<false, kVar><<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, c, q, n, seed, stream_off, value,
                                                                     count, walks, scr, ctr, pr);
    phase_end(tm, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    phase_begin(tm, kPhaseSsTrials, s);
    const int group = trial_group > 0 ? trial_group : (learned ? 8 : 32);
    if constexpr (kLearnedOk) {
        if (learned) {
            auto trials = group == 8 ? ss_trials_kernel<true, 8, kVar>
                          : group == 16 ? ss_trials_kernel<true, 16, kVar> : ss_trials_kernel<true, 32, kVar>;
            if constexpr ((kVar & 4) == 0) {   // the treelet serves the plain and rough casters
                if (st.n_tnodes)
                    trials = group == 8 ? ss_trials_kernel<true, 8, kVar, true>
                             : group == 16 ? ss_trials_kernel<true, 16, kVar, true>
                                           : ss_trials_kernel<true, 32, kVar, true>;
            }
            trials<<<num_sms * bps, 128, tsmem, s>>>(st, cfg, c, q, n, seed, stream_off, value, count, walks, scr, ctr,
                                                     pr);
        }
    }
    if (!learned) {
        auto trials = group == 8 ? ss_trials_kernel<false, 8, kVar>
                      : group == 16 ? ss_trials_kernel<false, 16, kVar> : ss_trials_kernel<false, 32, kVar>;
        if constexpr ((kVar & 4) == 0) {
            if (st.n_tnodes)
                trials = group == 8 ? ss_trials_kernel<false, 8, kVar, true>
                         : group == 16 ? ss_trials_kernel<false, 16, kVar, true>
                                       : ss_trials_kernel<false, 32, kVar, true>;
        }
        trials<<<num_sms * bps, 128, tsmem, s>>>(st, cfg, c, q, n, seed, stream_off, value, count, walks, scr, ctr,
                                                 pr);
    }
    phase_end(tm, s);
    return cudaGetLastError();
}

}  // namespace sms
