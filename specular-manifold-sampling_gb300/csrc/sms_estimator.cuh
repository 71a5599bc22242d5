// sms_estimator.cuh -- device helpers shared by the SMS estimators and the
// path tracer: counters, shading-point queries, emitter sampling, light
// visibility, emitter vertex, diffuse receiver, the single-scatter walk and
// its contribution.
#pragma once
#include "sms_device.cuh"
#include "sms_kernels.h"

namespace sms {

#define SMS_D __device__ __forceinline__

// ------------------------------------------------------------- statistics
struct LaneStats {
    unsigned long long succ = 0, fail = 0, calls = 0, iters = 0, imax = 0, walks = 0, newton = 0, conns = 0,
                       rays = 0, nodes = 0, tris = 0, spec = 0;
    SMS_D void ray(const Hit &h) {
        rays++;
        nodes += h.nodes;
        tris += h.tests;
    }
};

// Warp-aggregated counter update; all 32 lanes must call it.
SMS_D void flush_stats(const LaneStats &st, DevCounters *ctr, uint32_t err, int phase) {
    unsigned long long v[11] = {st.succ, st.fail, st.calls, st.iters, st.walks, st.newton, st.conns,
                                st.rays, st.nodes, st.tris, st.spec};
    unsigned long long *dst[11] = {&ctr->solver_succeeded, &ctr->solver_failed, &ctr->bernoulli_calls,
                                   &ctr->bernoulli_iters, &ctr->walks, &ctr->newton_iters, &ctr->connections,
                                   &ctr->rays, &ctr->bvh_nodes, &ctr->tri_tests, &ctr->speculative_walks};
    const unsigned full = 0xffffffffu;
    #pragma unroll
    for (int k = 0; k < 11; ++k) {
        unsigned long long s = v[k];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(full, s, off);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst[k], s);
    }
    unsigned long long pv[3] = {st.rays, st.nodes, st.tris};
    unsigned long long *pd[3] = {&ctr->phase_rays[phase], &ctr->phase_nodes[phase], &ctr->phase_tris[phase]};
    #pragma unroll
    for (int k = 0; k < 3; ++k) {
        unsigned long long s = pv[k];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(full, s, off);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(pd[k], s);
    }
    unsigned long long m = st.imax;
    for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(full, m, off));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(&ctr->bernoulli_max, m);
    unsigned e = err;
    for (int off = 16; off > 0; off >>= 1) e |= __shfl_xor_sync(full, e, off);
    if ((threadIdx.x & 31) == 0 && e) atomicOr(&ctr->error, e);
}

// ------------------------------------------------------------ query / light
struct Query {
    f3 x, n, albedo;
    float cos_i;
};

SMS_D Query load_query(const float *__restrict__ q, uint32_t n, uint32_t i) {
    auto Q = [&](int k) { return __ldg(q + (size_t)k * n + i); };
    Query r;
    r.x = mk(Q(0), Q(1), Q(2));
    r.n = mk(Q(3), Q(4), Q(5));
    r.albedo = mk(Q(12), Q(13), Q(14));
    r.cos_i = Q(15);
    return r;
}

struct Light {
    int eidx, kind;   // kind 0 point, 1 area sphere
    int n_list;       // size of the emitter list it was drawn from
    f3 p, w;          // ei.p, ei.weight
};

// sample_emitter_interaction (manifold.h:204-260) over an emitter list
// (caustic_emitters_single_scatter or _multi_scatter): 3 draws.
SMS_D bool sample_emitter(const DevScene &sc, const int *list, int ne, Pcg32 &rng, f3 x, Light &L) {
    if (ne == 0) return false;
    float es = rng.next_f32();
    float emitter_pdf = 1.f / (float)ne;
    uint32_t idx = min((uint32_t)(es * (float)ne), (uint32_t)ne - 1);
    L.eidx = list[idx];
    L.n_list = ne;
    const DevEmitter &e = sc.emitters[L.eidx];
    L.kind = e.kind;
    float sx = rng.next_f32(), sy = rng.next_f32();
    f3 spec;
    if (e.kind == 1) {
        const DevShape &ls = sc.shapes[e.shape];
        L.p = sample_position(sc, ls, sx, sy);
        float pdf = 1.f / (4.f * kPi * ls.radius * ls.radius);
        spec = mk(e.r / pdf, e.g / pdf, e.b / pdf);
    } else {
        L.p = mk(e.px, e.py, e.pz);
        f3 d = L.p - x;
        float dist = length(d);
        float inv = 1.f / dist;
        spec = mk(e.r, e.g, e.b) * (inv * inv);
        spec = (spec * dist) * dist;
    }
    L.w = spec * (1.f / emitter_pdf);
    return true;
}

SMS_D uint64_t query_stream(const SolverCfg &cfg, uint64_t stream_off, uint32_t qi) {
    return cfg.streams ? __ldg(reinterpret_cast<const unsigned long long *>(cfg.streams) + qi)
                       : stream_off + (uint64_t)qi;
}

// Offset normal of a rough caster (manifold_ss.cpp:60-70): an isotropic
// Beckmann microfacet normal drawn from the next 2 numbers of rng (the
// caster's first draws), with density p_off = D(m) cos(theta_m); (0, 0, 1)
// and 1 for a smooth caster, which draws nothing.
SMS_D f3 caster_offset(const DevShape &s, Pcg32 &rng, float &p_off) {
    p_off = 1.f;
    if (!(s.alpha > 0.f)) return mk(0.f, 0.f, 1.f);
    const float u0 = rng.next_f32(), u1 = rng.next_f32();
    return beckmann_sample(s.alpha, u0, u1, p_off);
}

// Random numbers a caster takes before its walks (the offset normal).
SMS_D uint32_t caster_draws(const DevShape &s) { return s.alpha > 0.f ? 2u : 0u; }

SMS_D Pcg32 query_rng(uint64_t seed, uint64_t stream, uint64_t position) {
    Pcg32 r;
    r.seed(seed, stream);
    if (position) r.advance(position);
    return r;
}

// Light-to-solution visibility (manifold_ss.cpp:88-102).
SMS_D bool visible(const DevScene &sc, f3 lp, f3 p, uint32_t &err, LaneStats &st) {
    f3 d = p - lp;
    float dist = length(d);
    d = d * (1.f / dist);
    float mint = kRayEps * (1.f + fmaxf(fabsf(lp.x), fmaxf(fabsf(lp.y), fabsf(lp.z))));
    Hit h;
    bool occ = trace(sc, lp, d, mint, dist * (1.f - kRayEps), true, h, err);
    st.ray(h);
    return !occ;
}

// Emitter endpoint of the generalized geometric term (manifold.h:264-302) and
// the emitter weight for a solution whose last specular vertex is at p.
// Point lights are re-sampled from p (manifold_ss.cpp:291-312, manifold_ms.cpp:
// 234-257); area lights cast one ray toward the light sample.
SMS_D bool emitter_endpoint(const DevScene &sc, const Light &L, f3 p, f3 &yp, f3 &ydu, f3 &ydv, f3 &lw, f3 &lp,
                            uint32_t &err, LaneStats &st) {
    lw = L.w;
    lp = L.p;
    if (L.kind == 1) {
        f3 d = normalize(lp - p);
        f3 o = p + d * kShadowEps;
        Hit h;
        trace(sc, o, d, kRayEps, INFINITY, false, h, err);
        st.ray(h);
        if (h.shape < 0) return false;
        Vtx vy;
        vertex_from_hit<false>(sc, o, d, h, vy);
        make_orthonormal(vy.dp_du, vy.dp_dv, vy.dn_du, vy.dn_dv);
        yp = vy.p; ydu = vy.dp_du; ydv = vy.dp_dv;
        return true;
    }
    const DevEmitter &e = sc.emitters[L.eidx];
    lp = mk(e.px, e.py, e.pz);
    f3 d = lp - p;
    float dist = length(d);
    float inv = 1.f / dist;
    float emitter_pdf = 1.f / (float)L.n_list;
    f3 spec = mk(e.r, e.g, e.b) * (inv * inv);
    lw = (spec * dist) * dist;
    lw = lw * (1.f / emitter_pdf);
    yp = lp;
    onb(normalize(p - lp), ydu, ydv);
    return true;
}

// Diffuse receiver (src/bsdfs/diffuse.cpp): albedo / pi * cos_o.
SMS_D f3 diffuse_eval(const Query &Q, f3 dir) {
    float co = dot(dir, Q.n);
    if (Q.cos_i <= 0.f || co <= 0.f) return splat(0.f);
    return (Q.albedo * kInvPi) * co;
}

// ------------------------------------------------------------ roughplastic
// roughplastic.cpp:185-353: a Beckmann-rough dielectric coating (eta) over a
// diffuse base.  The external transmittance t(cos) is the tabulated integral
// (lerp_gather, :301-310); the base's internal scattering divides its albedo
// by 1 - Fdr (or 1 - albedo Fdr, nonlinear).  The coating's normals are drawn
// with density D(m) cos(theta_m) like the other rough BSDFs here (the
// reference's sample_visible = false branch of pdf, :346-348).
SMS_D float rp_transmittance(const DevShape &s, float c) {
    float x = c * (float)(kRoughPlasticRes - 1);
    const int i = min((int)x, kRoughPlasticRes - 2);
    const float v0 = s.rp_t[i], v1 = s.rp_t[i + 1];
    return v0 + (v1 - v0) * (x - (float)i);
}

SMS_D f3 roughplastic_eval(const DevShape &s, f3 wi, f3 wo) {
    const float ci = wi.z, co = wo.z;
    if (!(ci > 0.f && co > 0.f)) return splat(0.f);
    const f3 h = normalize(wo + wi);
    const float F = fresnel_dielectric(dot(wi, h), s.eta);
    const float G = beckmann_G1(wi, h, s.alpha) * beckmann_G1(wo, h, s.alpha);
    const float spec = F * beckmann_D(h, s.alpha) * G / (4.f * ci);
    const float t_i = rp_transmittance(s, ci), t_o = rp_transmittance(s, co);
    f3 diff = mk(s.albedo[0], s.albedo[1], s.albedo[2]);
    if (s.rp_nonlinear)
        diff = mk(diff.x / (1.f - diff.x * s.rp_fdr), diff.y / (1.f - diff.y * s.rp_fdr),
                  diff.z / (1.f - diff.z * s.rp_fdr));
    else
        diff = diff * (1.f / (1.f - s.rp_fdr));
    return splat(spec) + diff * (kInvPi * (1.f / (s.eta * s.eta)) * co * t_i * t_o);
}

// BSDF value x |cos(theta_o)| of the BSDFs emitter sampling and receivers
// evaluate: diffuse (diffuse.cpp eval), rough (roughconductor.cpp,
// roughdielectric.cpp eval) and roughplastic; delta BSDFs give 0.
SMS_D f3 bsdf_eval(const DevShape &s, f3 wi, f3 wo) {
    if (s.bsdf_type == kBsdfRoughPlastic) return roughplastic_eval(s, wi, wo);
    if (s.bsdf_type == kBsdfDiffuse) {
        if (!(wi.z > 0.f && wo.z > 0.f)) return splat(0.f);
        return mk(s.albedo[0], s.albedo[1], s.albedo[2]) * (kInvPi * wo.z);
    }
    if (!(s.alpha > 0.f)) return splat(0.f);
    return splat(s.bsdf_type == kBsdfConductor ? roughconductor_eval(s.alpha, s.eta, s.k, wi, wo)
                                               : roughdielectric_eval(s.alpha, s.eta, wi, wo));
}

// The receiver's BSDF toward the first specular vertex (manifold_ss.cpp:109,
// 191; manifold_ms.cpp:113, 190).  A query whose row 12 is >= 0 is a diffuse
// receiver with that albedo (diffuse_eval, unchanged).  A negative row 12 is
// -(1 + shape id) of the receiver shape, whose BSDF is evaluated in the frame
// onb(n) with the incident direction (row 13, row 14, cos_i); the isotropic
// BSDFs here depend on the frame's normal only.  An id outside the scene
// contributes nothing and raises the invalid-query error bit.
SMS_D f3 receiver_eval(const DevScene &sc, const Query &Q, f3 dir, uint32_t &err) {
    if (Q.albedo.x >= 0.f) return diffuse_eval(Q, dir);
    const int id = (int)(-Q.albedo.x) - 1;
    if (!(id >= 0 && id < sc.n_shapes)) {
        err |= kErrBadQuery;
        return splat(0.f);
    }
    f3 s, t;
    onb(Q.n, s, t);
    return bsdf_eval(sc.shapes[id], mk(Q.albedo.y, Q.albedo.z, Q.cos_i), mk(dot(dir, s), dot(dir, t), dot(dir, Q.n)));
}

// ------------------------------------------------------------------- walk
// sample_path + newton_solver (manifold_ss.cpp:206-279, 331-405) from an
// explicit seed point.  Returns ok; v holds the solution vertex.
// kOffset: the caster is rough and `no` is its offset normal; without it the
// constraint uses the vertex normal and `no` is ignored (compiled away).
// newton_solver (manifold_ss.cpp:331-405) from the vertex v with offset normal
// no; coarse: the two-stage solver's smoothed frames (smoothing = 1).  it
// counts this solve's iterations; h is its ray-cast scratch.  On success v is
// the accepted solution and, with kTrack, (h_acc, d_acc) the hit that
// produced it; true = converged there and admissible
// (reflection vs refraction, :391-402).
template <bool kTrack, bool kNM, bool kTree = false>
SMS_D bool ss_newton(const DevScene &sc, const SolverCfg &cfg, f3 x, f3 lp, Vtx &v, Hit &h, Hit &h_acc, f3 &d_acc,
                     int &it, uint32_t &err, LaneStats &st, f3 no, bool coarse) {
    float beta = 1.f;
    bool accepted = false, conv = false;
    it = 0;
    while (it < cfg.max_iterations) {
        float c0, c1, dx0, dx1;
        bool sok = cfg.halfvector ? step_halfvector(x, v, lp, c0, c1, dx0, dx1, no)
                                  : step_anglediff(x, v, lp, c0, c1, dx0, dx1, no);
        if (!sok) break;
        if (sqrtf(c0 * c0 + c1 * c1) < cfg.solver_threshold) { conv = true; break; }
        f3 pp = v.p - (v.dp_du * dx0 + v.dp_dv * dx1) * (cfg.step_scale * beta);
        f3 dd = normalize(pp - x);
        trace<kTree>(sc, x, dd, kRayEps, INFINITY, false, h, err);
        st.ray(h);
        it++;
        if (h.shape < 0 || h.shape != v.shape) {
            beta = 0.5f * beta;
            accepted = false;
            continue;
        }
        beta = fminf(1.f, 2.f * beta);
        vertex_from_hit<kNM>(sc, x, dd, h, v, nullptr, coarse);
        if constexpr (kTrack) {
            h_acc = h;
            d_acc = dd;
        }
        accepted = true;
    }
    // newton_solver returns si_current: valid only after an accepted step.
    if (!(conv && accepted)) return false;
    f3 wx = normalize(x - v.p), wy = normalize(lp - v.p);
    bool refraction = dot(v.gn, wx) * dot(v.gn, wy) < 0.f;
    return (v.eta == 1.f) ? !refraction : refraction;
}

// sample_gaussian (manifold.h:326-345): a slope from N(mu, sigma) with sigma =
// (a, c; c, b), through the standard normal of warp.h:184-190.
SMS_D float2 sample_slope_gaussian(float mx, float my, float sa, float sb, float scv, float u0, float u1) {
    const float r = sqrtf(-2.f * logf(1.f - u0));
    float sp, cp;
    sincosf(2.f * kPi * u1, &sp, &cp);
    const float px = cp * r, py = sp * r;
    const float sx = sqrtf(sa), sy = sqrtf(sb);
    const float rho = scv / (sx * sy);
    const float a = sqrtf(1.f + rho), b = sqrtf(1.f - rho);
    const float d0 = 0.5f * a + 0.5f * b, d1 = 0.5f * a - 0.5f * b;
    return make_float2((d0 * px + d1 * py) * sx + mx, (d1 * px + d0 * py) * sy + my);
}

// sample_path + newton_solver (manifold_ss.cpp:206-279, 331-405) from an
// explicit seed point.  kOffset: the caster is rough and `no` is its offset
// normal (otherwise ignored and compiled away).  kTwoStage: the two-stage
// solver on a normal-mapped caster (:253-270): first a solve on the smoothed
// surface toward a slope drawn from the map's LEAN distribution (g0, g1 the
// two numbers), then the solve on the full normal map from its solution.
// Returns ok; v holds the solution vertex; it counts all iterations.
// kNM: the caster may be normal-mapped (its manifold vertices read the map).
template <bool kOffset = false, bool kTwoStage = false, bool kNM = false, bool kTree = false>
SMS_D bool ss_walk(const DevScene &sc, const SolverCfg &cfg, int caster, f3 x, f3 lp, f3 seed, Vtx &v, int &it,
                   uint32_t &err, LaneStats &st, f3 *p_init = nullptr, f3 no_in = f3{0.f, 0.f, 1.f}, float g0 = 0.f,
                   float g1 = 0.f) {
    const f3 no = kOffset ? no_in : f3{0.f, 0.f, 1.f};
    f3 d = normalize((cfg.mnee_init ? mnee_target(sc.shapes[caster], lp) : seed) - x);
    Hit h;
    trace<kTree>(sc, x, d, kRayEps, INFINITY, false, h, err);
    st.ray(h);
    it = 0;
    if (h.shape < 0) return false;
    vertex_from_hit<kNM>(sc, x, d, h, v, nullptr, kTwoStage);
    if (p_init) *p_init = v.p;
    if (h.shape != caster) return false;
    if constexpr (kTwoStage) {
        Hit h_acc = h;
        f3 d_acc = d;
        float mx, my, sa, sb, scv;
        nm_top_lean(sc, mx, my, sa, sb, scv);
        const float2 sl = sample_slope_gaussian(0.5f * (mx - no.x / no.z), 0.5f * (my - no.y / no.z), sa, sb, scv,
                                                g0, g1);
        const f3 ln = normalize(mk(-sl.x, -sl.y, 1.f));
        int it1;
        const bool ok1 = ss_newton<true, kNM, kTree>(sc, cfg, x, lp, v, h, h_acc, d_acc, it1, err, st, ln, true);
        it = it1;
        if (!ok1) return false;
        vertex_from_hit<kNM>(sc, x, d_acc, h_acc, v, nullptr, false);   // ManifoldVertex(si_smooth, 0)
    }
    int it2;
    const bool ok = ss_newton<false, kNM, kTree>(sc, cfg, x, lp, v, h, h, d, it2, err, st, no, false);
    it += it2;
    return ok;
}

// evaluate_path_contribution (manifold_ss.cpp:281-327) for a flat receiver;
// kNM: the caster may carry the normal map.
template <bool kNM = false>
SMS_D f3 contribution(const DevScene &sc, f3 x, const Light &L, const Vtx &sol, uint32_t &err, LaneStats &st) {
    Vtx vt = sol;
    make_orthonormal(vt.dp_du, vt.dp_dv, vt.dn_du, vt.dn_dv);
    f3 yp, ydu, ydv, lw, lp;
    if (!emitter_endpoint(sc, L, vt.p, yp, ydu, ydv, lw, lp, err, st)) return splat(0.f);
    const DevShape &sh = sc.shapes[vt.shape];
    const bool nm = kNM && vt.shape == sc.nmap_shape && sh.nmap_frames;
    float F = sh.alpha > 0.f ? specular_reflectance_rough(sh, vt.n, vt.dp_du, normalize(x - vt.p), normalize(lp - vt.p),
                                                          vt.n0, nm)
                             : specular_reflectance(sh, vt.n, normalize(lp - vt.p));
    F *= geometric_term(x, vt, yp, ydu, ydv);
    return lw * F;
}

}  // namespace sms
