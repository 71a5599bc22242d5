// sms_ss.cu -- single-scatter SMS kernels for sm_103a.
//
//  ss_walk_kernel     one thread per walk: SpecularManifoldSingleScatter::
//                     sample_path with an explicit start point
//                     (src/librender/manifold_ss.cpp:203-279, 329-405).
//  ss_connect_kernel  persistent kernel: specular_manifold_sampling for a
//                     wavefront of shading points (manifold_ss.cpp:28-201).
//
// The connection kernel keeps one query per lane.  Each lane is a small state
// machine that issues exactly ONE ray per loop iteration (seed ray, Newton
// reprojection, light visibility or the area-light vertex ray), so the BVH
// traversal -- the expensive part -- runs converged across the warp whatever
// phase each lane is in.  When a lane's query is complete it takes the next one
// from a device work queue (one atomic per warp), so geometric Bernoulli-trial
// counts and uneven Newton iteration counts never idle a lane.
#include "sms_device.cuh"
#include "sms_kernels.h"

namespace sms {

// ------------------------------------------------------------ walk kernel
__global__ void ss_walk_kernel(DevScene sc, SolverCfg cfg, int caster, const float *__restrict__ q,
                               const float *__restrict__ w, uint32_t n, float *__restrict__ out,
                               DevCounters *ctr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    auto Q = [&](int k) { return __ldg(q + (size_t)k * n + i); };
    auto W = [&](int k) { return __ldg(w + (size_t)k * n + i); };
    f3 x = mk(Q(0), Q(1), Q(2));
    f3 lp = mk(W(0), W(1), W(2));
    f3 ps = mk(W(3), W(4), W(5));
    uint32_t err = 0;
    const DevShape &cs = sc.shapes[caster];
    f3 seed = sample_position(sc, cs, W(6), W(7));
    if (ps.x != 0.f || ps.y != 0.f || ps.z != 0.f) seed = ps;
    f3 d = normalize(seed - x);
    Hit h;
    trace<false>(sc, x, d, kRayEps, INFINITY, h, err);
    float res[11] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int it = 0;
    bool ok = false;
    if (h.shape >= 0) {
        // si_init.p
        Vtx v;
        vertex_from_hit(sc, x, d, h, v);
        res[5] = v.p.x; res[6] = v.p.y; res[7] = v.p.z;
        if (h.shape == caster) {
            float beta = 1.f;
            bool accepted = false, conv = false;
            while (it < cfg.max_iterations) {
                float c0, c1, dx0, dx1;
                bool sok = cfg.halfvector ? step_halfvector(x, v, lp, c0, c1, dx0, dx1)
                                          : step_anglediff(x, v, lp, c0, c1, dx0, dx1);
                if (!sok) break;
                if (sqrtf(c0 * c0 + c1 * c1) < cfg.solver_threshold) { conv = true; break; }
                f3 pp = v.p - (v.dp_du * dx0 + v.dp_dv * dx1) * (cfg.step_scale * beta);
                f3 dd = normalize(pp - x);
                Hit hh;
                trace<false>(sc, x, dd, kRayEps, INFINITY, hh, err);
                if (hh.shape < 0 || hh.shape != v.shape) {
                    beta = 0.5f * beta;
                    it += 1;
                    accepted = false;
                    continue;
                }
                beta = fminf(1.f, 2.f * beta);
                vertex_from_hit(sc, x, dd, hh, v);
                accepted = true;
                it++;
            }
            // si_current must be a valid hit on the walked shape: the last ray
            // was an accepted reprojection (newton_solver returns si_current).
            if (conv && accepted) {
                f3 wx = normalize(x - v.p), wy = normalize(lp - v.p);
                bool refraction = dot(v.gn, wx) * dot(v.gn, wy) < 0.f;
                ok = (v.eta == 1.f) ? !refraction : refraction;
            }
            if (ok) {
                res[2] = v.p.x; res[3] = v.p.y; res[4] = v.p.z;
                res[8] = v.n.x; res[9] = v.n.y; res[10] = v.n.z;
            }
        }
    }
    res[0] = ok ? 1.f : 0.f;
    res[1] = (float)it;
    #pragma unroll
    for (int k = 0; k < 11; ++k) out[(size_t)k * n + i] = res[k];
    if (err) atomicOr(&ctr->error, err);
}

// ------------------------------------------------------- connection kernel
enum Purpose : int { kNone = 0, kSeed = 1, kReproj = 2, kVis = 3, kEmit = 4 };

struct Lane {
    // query
    uint32_t q;
    f3 x, xn, albedo;
    float cos_i;
    // emitter interaction
    f3 lp, lw;
    int ekind, eidx;
    // random numbers
    Pcg32 rng;
    // caster loop / estimator
    int ci, caster;
    int stage;          // 0 first walk, 1 Bernoulli trial (unbiased); walk index m (biased)
    int iterations;     // Bernoulli iterations (unbiased)
    int count, walks;
    float inv_prob;
    f3 dir0, val, acc, cur;
    int n_sol;
    // walk
    Vtx v;
    float beta;
    int it;
    bool accepted;
    // pending ray
    f3 ro, rd;
    float rmin, rmax;
    int purpose;
};

struct LaneStats {
    unsigned long long succ, fail, calls, iters, imax, walks, newton, conns, rays, nodes, tris;
};

__device__ __forceinline__ void begin_walk(const DevScene &sc, Lane &L) {
    float sx = L.rng.next_f32(), sy = L.rng.next_f32();
    f3 seed = sample_position(sc, sc.shapes[L.caster], sx, sy);
    L.ro = L.x;
    L.rd = normalize(seed - L.x);
    L.rmin = kRayEps;
    L.rmax = INFINITY;
    L.purpose = kSeed;
}

__device__ __forceinline__ void finish_query(Lane &L, uint32_t n, float *__restrict__ value,
                                             int *__restrict__ count, int *__restrict__ walks) {
    value[L.q] = L.acc.x;
    value[(size_t)n + L.q] = L.acc.y;
    value[2 * (size_t)n + L.q] = L.acc.z;
    count[L.q] = L.count;
    walks[L.q] = L.walks;
    L.purpose = kNone;
}

// Start the estimator for caster L.ci, or finish the query.
__device__ __forceinline__ void begin_caster(const DevScene &sc, const SolverCfg &cfg, Lane &L, uint32_t n,
                                             float *value, int *count, int *walks) {
    // A biased estimator with max_trials <= 0 makes no walk (manifold_ss.cpp:146).
    if (cfg.biased && cfg.max_trials <= 0) L.ci = sc.n_casters_ss;
    if (L.ci >= sc.n_casters_ss) { finish_query(L, n, value, count, walks); return; }
    L.caster = sc.casters_ss[L.ci];
    L.stage = 0;
    L.cur = splat(0.f);
    L.n_sol = 0;
    if (!cfg.biased) L.count = 0;
    begin_walk(sc, L);
}

__device__ __forceinline__ void caster_done(const DevScene &sc, const SolverCfg &cfg, Lane &L, uint32_t n,
                                            float *value, int *count, int *walks) {
    L.acc = L.acc + L.cur;
    L.ci++;
    begin_caster(sc, cfg, L, n, value, count, walks);
}

// Diffuse receiver eval: albedo / pi * cos_o (both cosines positive).
__device__ __forceinline__ f3 diffuse_eval(const Lane &L, f3 dir) {
    float co = dot(dir, L.xn);
    if (L.cos_i <= 0.f || co <= 0.f) return splat(0.f);
    return (L.albedo * kInvPi) * co;
}

// Contribution of the solution in L.v once the emitter vertex is known
// (evaluate_path_contribution, manifold_ss.cpp:281-327).
__device__ __forceinline__ f3 contribution(const DevScene &sc, const Lane &L, bool have_y, f3 yp, f3 ydu,
                                           f3 ydv) {
    if (!have_y) return splat(0.f);
    Vtx vt = L.v;
    make_orthonormal(vt.dp_du, vt.dp_dv, vt.dn_du, vt.dn_dv);
    f3 lw = L.lw;
    f3 lp = L.lp;
    if (L.ekind == 0) {
        // point light re-sampled from the solution (manifold_ss.cpp:291-312)
        const DevEmitter &e = sc.emitters[L.eidx];
        lp = mk(e.px, e.py, e.pz);
        f3 d = lp - vt.p;
        float dist = length(d);
        float inv = 1.f / dist;
        float emitter_pdf = 1.f / (float)sc.n_emitters_ss;
        f3 spec = mk(e.r, e.g, e.b) * (inv * inv);
        lw = (spec * dist) * dist;
        lw = lw * (1.f / emitter_pdf);
    }
    float F = specular_reflectance(sc.shapes[vt.shape], vt.n, normalize(lp - vt.p));
    F *= geometric_term(L.x, vt, yp, ydu, ydv);
    return lw * F;
}

__device__ __forceinline__ void after_contribution(const DevScene &sc, const SolverCfg &cfg, Lane &L, f3 spec,
                                                   LaneStats &st, uint32_t n, float *value, int *count,
                                                   int *walks) {
    f3 dir = normalize(L.v.p - L.x);
    f3 bsdf = diffuse_eval(L, dir);
    if (!cfg.biased) {
        L.val = bsdf * spec;
        L.inv_prob = 1.f;
        L.iterations = 1;
        L.stage = 1;
        st.calls++;
        begin_walk(sc, L);
    } else {
        L.cur = L.cur + bsdf * spec;
        L.count++;
        L.stage++;
        if (L.stage >= cfg.max_trials) caster_done(sc, cfg, L, n, value, count, walks);
        else begin_walk(sc, L);
    }
}

// Emitter vertex for the contribution: point lights directly, area lights by
// one ray toward the sampled light point (manifold.h:264-302).
__device__ __forceinline__ void start_contribution(const DevScene &sc, const SolverCfg &cfg, Lane &L,
                                                   LaneStats &st, uint32_t n, float *value, int *count,
                                                   int *walks) {
    if (L.ekind == 1) {
        f3 d = normalize(L.lp - L.v.p);
        L.ro = L.v.p + d * kShadowEps;
        L.rd = d;
        L.rmin = kRayEps;
        L.rmax = INFINITY;
        L.purpose = kEmit;
        return;
    }
    const DevEmitter &e = sc.emitters[L.eidx];
    f3 ep = mk(e.px, e.py, e.pz);
    f3 d = normalize(L.v.p - ep);
    f3 du, dv;
    onb(d, du, dv);
    f3 spec = contribution(sc, L, true, ep, du, dv);
    after_contribution(sc, cfg, L, spec, st, n, value, count, walks);
}

__device__ __forceinline__ void after_visibility(const DevScene &sc, const SolverCfg &cfg, Lane &L, bool vis,
                                                 LaneStats &st, f3 *sol, uint32_t n, float *value,
                                                 int *count, int *walks, uint32_t &err) {
    if (!cfg.biased) {
        if (!vis) { caster_done(sc, cfg, L, n, value, count, walks); return; }
        start_contribution(sc, cfg, L, st, n, value, count, walks);
        return;
    }
    if (vis) {
        f3 dir = normalize(L.v.p - L.x);
        bool dup = false;
        for (int k = 0; k < L.n_sol; ++k)
            if (fabsf(dot(dir, sol[k]) - 1.f) < cfg.uniqueness_threshold) { dup = true; break; }
        if (!dup) {
            if (L.n_sol < kMaxSolutions) {
                sol[L.n_sol++] = dir;
                start_contribution(sc, cfg, L, st, n, value, count, walks);
                return;
            }
            err |= kErrSolutionOverflow;
        }
    }
    L.stage++;
    if (L.stage >= cfg.max_trials) caster_done(sc, cfg, L, n, value, count, walks);
    else begin_walk(sc, L);
}

// A walk ended (converged or failed): advance the estimator.
__device__ __forceinline__ void walk_done(const DevScene &sc, const SolverCfg &cfg, Lane &L, bool ok,
                                          LaneStats &st, f3 *sol, uint32_t n, float *value, int *count,
                                          int *walks, uint32_t &err) {
    L.walks++;
    st.walks++;
    st.newton += (unsigned long long)L.it;
    if (!cfg.biased && L.stage == 1) {
        // Bernoulli trial (manifold_ss.cpp:115-135)
        if (ok && fabsf(dot(L.dir0, normalize(L.v.p - L.x)) - 1.f) < cfg.uniqueness_threshold) {
            L.cur = L.val * L.inv_prob;
            L.count = L.iterations;
            st.iters += (unsigned long long)L.iterations;
            st.imax = max(st.imax, (unsigned long long)L.iterations);
            caster_done(sc, cfg, L, n, value, count, walks);
            return;
        }
        L.inv_prob += 1.f;
        L.iterations++;
        bool capped = cfg.max_trials > 0 && L.iterations > cfg.max_trials;
        bool limit = cfg.max_trials <= 0 && L.iterations > kTrialHardLimit;
        if (capped || limit) {
            if (limit) err |= kErrTrialLimit;
            L.inv_prob = 0.f;
            L.cur = L.val * 0.f;
            L.count = -1;
            st.iters += (unsigned long long)L.iterations;
            st.imax = max(st.imax, (unsigned long long)L.iterations);
            caster_done(sc, cfg, L, n, value, count, walks);
            return;
        }
        begin_walk(sc, L);
        return;
    }
    if (!ok) {
        st.fail++;
        if (!cfg.biased) { caster_done(sc, cfg, L, n, value, count, walks); return; }
        L.stage++;
        if (L.stage >= cfg.max_trials) caster_done(sc, cfg, L, n, value, count, walks);
        else begin_walk(sc, L);
        return;
    }
    st.succ++;
    if (!cfg.biased) L.dir0 = normalize(L.v.p - L.x);
    // visibility between the light and the solution (manifold_ss.cpp:88-102)
    f3 d = L.v.p - L.lp;
    float dist = length(d);
    d = d * (1.f / dist);
    L.ro = L.lp;
    L.rd = d;
    L.rmin = kRayEps * (1.f + fmaxf(fabsf(L.lp.x), fmaxf(fabsf(L.lp.y), fabsf(L.lp.z))));
    L.rmax = dist * (1.f - kRayEps);
    L.purpose = kVis;
    (void)sol; (void)err;
}

// One Newton iteration on the current vertex: converge, fail, or propose a
// reprojection ray (manifold_ss.cpp:344-384).
__device__ __forceinline__ void newton_advance(const DevScene &sc, const SolverCfg &cfg, Lane &L,
                                               LaneStats &st, f3 *sol, uint32_t n, float *value,
                                               int *count, int *walks, uint32_t &err) {
    bool fail = L.it >= cfg.max_iterations;
    float c0 = 0.f, c1 = 0.f, dx0 = 0.f, dx1 = 0.f;
    if (!fail) {
        bool ok = cfg.halfvector ? step_halfvector(L.x, L.v, L.lp, c0, c1, dx0, dx1)
                                 : step_anglediff(L.x, L.v, L.lp, c0, c1, dx0, dx1);
        fail = !ok;
    }
    if (fail) { walk_done(sc, cfg, L, false, st, sol, n, value, count, walks, err); return; }
    if (sqrtf(c0 * c0 + c1 * c1) < cfg.solver_threshold) {
        bool ok = L.accepted;
        if (ok) {
            f3 wx = normalize(L.x - L.v.p), wy = normalize(L.lp - L.v.p);
            bool refraction = dot(L.v.gn, wx) * dot(L.v.gn, wy) < 0.f;
            ok = (L.v.eta == 1.f) ? !refraction : refraction;
        }
        walk_done(sc, cfg, L, ok, st, sol, n, value, count, walks, err);
        return;
    }
    f3 pp = L.v.p - (L.v.dp_du * dx0 + L.v.dp_dv * dx1) * (cfg.step_scale * L.beta);
    L.ro = L.x;
    L.rd = normalize(pp - L.x);
    L.rmin = kRayEps;
    L.rmax = INFINITY;
    L.purpose = kReproj;
}

__device__ __forceinline__ void begin_query(const DevScene &sc, const SolverCfg &cfg, Lane &L, uint32_t qi,
                                            const float *__restrict__ qs, uint32_t n, uint64_t seed,
                                            uint64_t stream_off, LaneStats &st, float *value, int *count,
                                            int *walks) {
    L.q = qi;
    auto Q = [&](int k) { return __ldg(qs + (size_t)k * n + qi); };
    L.x = mk(Q(0), Q(1), Q(2));
    L.xn = mk(Q(3), Q(4), Q(5));
    L.albedo = mk(Q(12), Q(13), Q(14));
    L.cos_i = Q(15);
    L.rng.seed(seed, (uint64_t)qi + stream_off);
    L.acc = splat(0.f);
    L.count = 0;
    L.walks = 0;
    L.ci = 0;
    // sample_emitter_interaction (manifold.h:204-260)
    int ne = sc.n_emitters_ss;
    if (ne == 0 || sc.n_casters_ss == 0) { finish_query(L, n, value, count, walks); return; }
    float es = L.rng.next_f32();
    float emitter_pdf = 1.f / (float)ne;
    uint32_t idx = min((uint32_t)(es * (float)ne), (uint32_t)ne - 1);
    L.eidx = sc.emitters_ss[idx];
    const DevEmitter &e = sc.emitters[L.eidx];
    L.ekind = e.kind;
    float sx = L.rng.next_f32(), sy = L.rng.next_f32();
    f3 spec;
    if (e.kind == 1) {
        const DevShape &ls = sc.shapes[e.shape];
        L.lp = sample_position(sc, ls, sx, sy);
        float pdf = 1.f / (4.f * kPi * ls.radius * ls.radius);
        spec = mk(e.r / pdf, e.g / pdf, e.b / pdf);
    } else {
        L.lp = mk(e.px, e.py, e.pz);
        f3 d = L.lp - L.x;
        float dist = length(d);
        float inv = 1.f / dist;
        spec = mk(e.r, e.g, e.b) * (inv * inv);
        spec = (spec * dist) * dist;
    }
    L.lw = spec * (1.f / emitter_pdf);
    st.conns++;
    begin_caster(sc, cfg, L, n, value, count, walks);
}

// Warp-aggregated counter update; every lane of the warp must call it.
__device__ __forceinline__ void flush_stats(LaneStats &st, DevCounters *ctr, uint32_t err) {
    unsigned long long v[10] = {st.succ, st.fail, st.calls, st.iters, st.walks, st.newton, st.conns,
                                st.rays, st.nodes, st.tris};
    unsigned long long *dst[10] = {&ctr->solver_succeeded, &ctr->solver_failed, &ctr->bernoulli_calls,
                                   &ctr->bernoulli_iters, &ctr->walks, &ctr->newton_iters, &ctr->connections,
                                   &ctr->rays, &ctr->bvh_nodes, &ctr->tri_tests};
    __syncwarp();
    const unsigned mask = 0xffffffffu;
    #pragma unroll
    for (int k = 0; k < 10; ++k) {
        unsigned long long s = v[k];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(mask, s, off);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst[k], s);
    }
    unsigned long long m = st.imax;
    for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(mask, m, off));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(&ctr->bernoulli_max, m);
    if (err) atomicOr(&ctr->error, err);
}

__global__ void __launch_bounds__(128) ss_connect_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ qs,
                                                         uint32_t n, uint64_t seed, uint64_t stream_off,
                                                         float *__restrict__ value, int *__restrict__ count,
                                                         int *__restrict__ walks, DevCounters *ctr) {
    Lane L;
    L.purpose = kNone;
    LaneStats st = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t err = 0;
    f3 sol[kMaxSolutions];
    bool exhausted = false;
    const unsigned lane = threadIdx.x & 31;
    while (true) {
        // ---- refill idle lanes from the work queue (one atomic per warp)
        bool need = L.purpose == kNone && !exhausted;
        unsigned act = __activemask();
        unsigned want = __ballot_sync(act, need);
        if (want) {
            unsigned leader = __ffs(want) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(&ctr->queue_head, (unsigned)__popc(want));
            base = __shfl_sync(act, base, leader);
            if (need) {
                unsigned qi = base + __popc(want & ((1u << lane) - 1u));
                if (qi >= n) exhausted = true;
                else begin_query(sc, cfg, L, qi, qs, n, seed, stream_off, st, value, count, walks);
            }
        }
        if (L.purpose == kNone) {
            if (exhausted) break;
            continue;
        }
        // ---- one ray per lane
        Hit h;
        bool any;
        if (L.purpose == kVis) {
            any = trace<true>(sc, L.ro, L.rd, L.rmin, L.rmax, h, err);
        } else {
            any = trace<false>(sc, L.ro, L.rd, L.rmin, L.rmax, h, err);
        }
        st.rays++;
        st.nodes += h.nodes;
        st.tris += h.tests;
        // ---- consume
        switch (L.purpose) {
        case kSeed:
            if (any && h.shape == L.caster) {
                vertex_from_hit(sc, L.ro, L.rd, h, L.v);
                L.it = 0;
                L.beta = 1.f;
                L.accepted = false;
                newton_advance(sc, cfg, L, st, sol, n, value, count, walks, err);
            } else {
                L.it = 0;
                walk_done(sc, cfg, L, false, st, sol, n, value, count, walks, err);
            }
            break;
        case kReproj:
            if (!any || h.shape != L.v.shape) {
                L.beta = 0.5f * L.beta;
                L.accepted = false;
            } else {
                L.beta = fminf(1.f, 2.f * L.beta);
                vertex_from_hit(sc, L.ro, L.rd, h, L.v);
                L.accepted = true;
            }
            L.it++;
            newton_advance(sc, cfg, L, st, sol, n, value, count, walks, err);
            break;
        case kVis:
            after_visibility(sc, cfg, L, !any, st, sol, n, value, count, walks, err);
            break;
        case kEmit: {
            f3 spec = splat(0.f);
            if (any) {
                Vtx vy;
                vertex_from_hit(sc, L.ro, L.rd, h, vy);
                make_orthonormal(vy.dp_du, vy.dp_dv, vy.dn_du, vy.dn_dv);
                spec = contribution(sc, L, true, vy.p, vy.dp_du, vy.dp_dv);
            }
            after_contribution(sc, cfg, L, spec, st, n, value, count, walks);
            break;
        }
        default:
            break;
        }
    }
    flush_stats(st, ctr, err);
}

// ---------------------------------------------------------------- launchers
cudaError_t launch_ss_walk(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q,
                           const float *w, uint32_t n, float *out, DevCounters *ctr, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 block(128), grid((n + 127) / 128);
    ss_walk_kernel<<<grid, block, 0, s>>>(sc, cfg, caster, q, w, n, out, ctr);
    return cudaGetLastError();
}

cudaError_t launch_ss_connect(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n,
                              uint64_t seed, uint64_t stream_off, float *value, int *count, int *walks,
                              DevCounters *ctr, int blocks, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(&ctr->queue_head, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    ss_connect_kernel<<<blocks, 128, 0, s>>>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr);
    return cudaGetLastError();
}

int ss_connect_max_blocks_per_sm() {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ss_connect_kernel, 128, 0);
    return b;
}

}  // namespace sms
