// sms_glints.cu -- glint SMS kernels (normal-mapped specular surfaces), sm_103a.
//
// Reference: SpecularManifoldGlints (src/librender/manifold_glints.cpp):
//   specular_manifold_sampling :28-223 (the SMS strategy, :45-176),
//   sample_glint :225-265, evaluate_glint_contribution :267-294,
//   newton_solver :296-343, compute_step :345-373,
//   specular_reflectance :375-409, geometric_term :411-554;
//   inside_parallelogram (include/mitsuba/render/manifold_glints.h:162-194);
// and the slope lookups of the normal-map BSDF (src/bsdfs/normalmap.cpp:218-336,
// include/mitsuba/render/normalmap.h:62-193).  SpecularManifoldGlintsVectorized
// (manifold_glints_vectorized.cpp) is the same biased estimator run 16 walks at
// a time on the CPU; here a lane group of 32 is the packet.
//
// The slope map is stored as FP16 (sx, sy) pairs, 4 bytes per texel, and one
// Newton iteration reads the 2x2 texel neighbourhood (16 bytes) for both the
// slope and its analytic bilinear derivative.
//
// Each query returns the SMS-strategy estimate sms_weight x ei.weight; the
// multiple-importance weight against BSDF sampling (LEAN pdf) and the sensor
// importance are applied by the integrator, which owns the camera and the BSDF
// sampling strategy.
#include <algorithm>

#include <cuda_fp16.h>

#include "sms_device.cuh"
#include "sms_estimator.cuh"
#include "sms_kernels.h"

namespace sms {

constexpr unsigned kFullG = 0xffffffffu;

struct f2 { float x, y; };

struct GQuery {
    f3 p, n, dp_du, dp_dv, sensor;
    f2 uv, duv_dx, duv_dy;
};

SMS_D GQuery load_gquery(const float *__restrict__ q, uint32_t n, uint32_t i) {
    auto Q = [&](int k) { return __ldg(q + (size_t)k * n + i); };
    GQuery r;
    r.p = mk(Q(0), Q(1), Q(2));
    r.n = mk(Q(3), Q(4), Q(5));
    r.dp_du = mk(Q(6), Q(7), Q(8));
    r.dp_dv = mk(Q(9), Q(10), Q(11));
    r.uv = {Q(12), Q(13)};
    r.duv_dx = {Q(14), Q(15)};
    r.duv_dy = {Q(16), Q(17)};
    r.sensor = mk(Q(18), Q(19), Q(20));
    return r;
}

SMS_D float2 texel(const DevScene &sc, uint32_t idx) {
    uint32_t bits = __ldg(sc.nmap + idx);
    __half2 h = *reinterpret_cast<__half2 *>(&bits);
    return __half22float2(h);
}

// Slope and its uv derivative at uv: the bilinear lookup of eval_normal /
// eval_normal_derivatives at level 0 after the tiling wrap.
SMS_D void nm_slope(const DevScene &sc, f2 uv_in, f2 &s, f2 &du, f2 &dv) {
    float u = uv_in.x * sc.nmap_tiles, v = uv_in.y * sc.nmap_tiles;
    u -= floorf(u);
    v -= floorf(v);
    const uint32_t R = sc.nmap_res;
    float res = (float)R;
    float duv = 1.f / res;
    float px = fminf(fmaxf((u - 0.5f * duv) * res, 0.f), res - 1.f);
    float py = fminf(fmaxf((v - 0.5f * duv) * res, 0.f), res - 1.f);
    uint32_t x0 = (uint32_t)floorf(px), y0 = (uint32_t)floorf(py);
    uint32_t x1 = min(x0 + 1, R - 1), y1 = min(y0 + 1, R - 1);
    x0 = min(x0, R - 1);
    y0 = min(y0, R - 1);
    float wx = px - (float)x0, wy = py - (float)y0;
    float2 t00 = texel(sc, y0 * R + x0), t10 = texel(sc, y0 * R + x1), t01 = texel(sc, y1 * R + x0),
           t11 = texel(sc, y1 * R + x1);
    float w0x = 1.f - wx, w0y = 1.f - wy;
    s.x = w0y * (w0x * t00.x + wx * t10.x) + wy * (w0x * t01.x + wx * t11.x);
    s.y = w0y * (w0x * t00.y + wx * t10.y) + wy * (w0x * t01.y + wx * t11.y);
    float tmpx = t01.x + t10.x - t11.x, tmpy = t01.y + t10.y - t11.y;
    du.x = (t10.x + t00.x * (wy - 1.f) - tmpx * wy) * res * sc.nmap_tiles;
    du.y = (t10.y + t00.y * (wy - 1.f) - tmpy * wy) * res * sc.nmap_tiles;
    dv.x = (t01.x + t00.x * (wx - 1.f) - tmpx * wx) * res * sc.nmap_tiles;
    dv.y = (t01.y + t00.y * (wx - 1.f) - tmpy * wx) * res * sc.nmap_tiles;
}

SMS_D bool inside_triangle(f2 p, f2 a, f2 b, f2 c) {
    f2 v0 = {c.x - a.x, c.y - a.y}, v1 = {b.x - a.x, b.y - a.y}, v2 = {p.x - a.x, p.y - a.y};
    float d00 = v0.x * v0.x + v0.y * v0.y, d01 = v0.x * v1.x + v0.y * v1.y, d02 = v0.x * v2.x + v0.y * v2.y,
          d11 = v1.x * v1.x + v1.y * v1.y, d12 = v1.x * v2.x + v1.y * v2.y;
    float inv = 1.f / (d00 * d11 - d01 * d01);
    float u = (d11 * d02 - d01 * d12) * inv, v = (d00 * d12 - d01 * d02) * inv;
    return u >= 0.f && v >= 0.f && u + v < 1.f;
}

SMS_D void base_frame(const GQuery &q, f3 &s, f3 &t) {
    s = normalize(q.dp_du - q.n * dot(q.n, q.dp_du));
    t = cross(q.n, s);
}

// Visible-normal sampling of an isotropic Beckmann distribution seen from wi
// (include/mitsuba/render/microfacet.h:287-314, sample_visible_11 :357-394,
// smith_g1 :331-355, Frame3f::sincos_phi frame.h:107-118): the offset normal
// of a rough glinty surface (manifold_glints.cpp:56-64); pdf = D G1 |wi.m| /
// cos_theta(wi).
SMS_D f3 beckmann_sample_visible(float alpha, f3 wi, float u0, float u1, float &pdf) {
    const f3 wp = normalize(mk(alpha * wi.x, alpha * wi.y, wi.z));
    const float st2 = wp.x * wp.x + wp.y * wp.y;
    float sin_phi = 0.f, cos_phi = 1.f;
    if (!(fabsf(st2) <= 4.f * 1.1920929e-7f)) {
        const float inv = 1.f / sqrtf(st2);
        cos_phi = fminf(1.f, fmaxf(-1.f, wp.x * inv));
        sin_phi = fminf(1.f, fmaxf(-1.f, wp.y * inv));
    }
    const float cos_i = wp.z;
    const float tan_i = sqrtf(fmaxf(1.f - cos_i * cos_i, 0.f)) / cos_i;
    const float cot_i = 1.f / tan_i;
    const float maxval = erff(cot_i);
    const float sx = fmaxf(fminf(u0, 1.f - 1e-6f), 1e-6f), sy = fmaxf(fminf(u1, 1.f - 1e-6f), 1e-6f);
    const float kInvSqrtPi = 0.56418958354775628695f;
    float x = maxval - (maxval + 1.f) * erff(sqrtf(-logf(sx)));
    const float target = sx * (1.f + maxval + kInvSqrtPi * tan_i * expf(-(cot_i * cot_i)));
    #pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        const float slope = erfinvf(x);
        const float value = 1.f + x + kInvSqrtPi * tan_i * expf(-(slope * slope)) - target;
        const float deriv = 1.f - slope * tan_i;
        x = x - value / deriv;
    }
    const float slx = erfinvf(x), sly = erfinvf(2.f * sy - 1.f);
    const float rx = (cos_phi * slx - sin_phi * sly) * alpha, ry = (sin_phi * slx + cos_phi * sly) * alpha;
    const f3 m = normalize(mk(-rx, -ry, 1.f));
    pdf = beckmann_D(m, alpha) * beckmann_G1(wi, m, alpha) * fabsf(dot(wi, m)) / wi.z;
    return m;
}

// Offset normal of the query's glinty surface, from the 2 numbers after the
// emitter sample: (0, 0, 1) and density 1 when the surface is smooth.
SMS_D f3 glint_offset(const DevScene &sc, const GQuery &q, Pcg32 rng_at_3, float &p_off) {
    p_off = 1.f;
    const DevShape &gs = sc.shapes[sc.glinty_shape];
    if (!(gs.alpha > 0.f)) return mk(0.f, 0.f, 1.f);
    const float u0 = rng_at_3.next_f32(), u1 = rng_at_3.next_f32();
    const f3 bs = normalize(q.dp_du - q.n * dot(q.n, q.dp_du)), bt = cross(q.n, bs);
    const f3 wiw = normalize(q.sensor - q.p);
    return beckmann_sample_visible(gs.alpha, mk(dot(wiw, bs), dot(wiw, bt), dot(wiw, q.n)), u0, u1, p_off);
}

// Random numbers the glint estimator takes after the emitter sample before its
// walks: the offset normal's 2 on a rough glinty surface.
SMS_D uint32_t glint_offset_numbers(const DevScene &sc) { return sc.shapes[sc.glinty_shape].alpha > 0.f ? 2u : 0u; }

// sample_glint (:225-265) from an explicit footprint sample fp; Newton in uv
// with footprint containment (:296-343).  Returns ok; uv = final position.
// no: the offset normal (local frame), added to the target slope (:243-246).
SMS_D bool glint_walk(const DevScene &sc, const SolverCfg &cfg, const GQuery &q, f3 lp, f2 fp, f2 &uv, f2 &uv_init,
                      int &it, f3 no = f3{0.f, 0.f, 1.f}) {
    it = 0;
    f3 s, t;
    base_frame(q, s, t);
    f3 wiw = normalize(q.sensor - q.p), wow = normalize(lp - q.p);
    f3 wi = mk(dot(wiw, s), dot(wiw, t), dot(wiw, q.n)), wo = mk(dot(wow, s), dot(wow, t), dot(wow, q.n));
    uv = {0.f, 0.f};
    uv_init = uv;
    if (wi.z <= 0.f || wo.z <= 0.f) return false;
    f3 h = normalize(wi + wo);
    f2 target = {-h.x / h.z + (-no.x / no.z), -h.y / h.z + (-no.y / no.z)};
    f2 duv = {(fp.x - 0.5f) * q.duv_dx.x + (fp.y - 0.5f) * q.duv_dy.x,
              (fp.x - 0.5f) * q.duv_dx.y + (fp.y - 0.5f) * q.duv_dy.y};
    uv_init = {q.uv.x + duv.x, q.uv.y + duv.y};
    uv = uv_init;
    auto corner = [&](float a, float b) {
        return f2{q.uv.x + a * q.duv_dx.x + b * q.duv_dy.x, q.uv.y + a * q.duv_dx.y + b * q.duv_dy.y};
    };
    f2 fa = corner(0.5f, 0.5f), fb = corner(0.5f, -0.5f), fc = corner(-0.5f, -0.5f), fd = corner(-0.5f, 0.5f);
    float beta = 1.f;
    while (it < cfg.max_iterations) {
        f2 sl, du, dv;
        nm_slope(sc, uv, sl, du, dv);
        float c0 = sl.x - target.x, c1 = sl.y - target.y;
        M2 J{du.x, dv.x, du.y, dv.y};
        float dj = det2(J);
        if (fabsf(dj) < 1e-6f) return false;
        if (sqrtf(c0 * c0 + c1 * c1) < cfg.solver_threshold) return true;
        float id = 1.f / dj;
        float sx = (J.d * id) * c0 + (-J.b * id) * c1;
        float sy = (-J.c * id) * c0 + (J.a * id) * c1;
        f2 prop = {uv.x - cfg.step_scale * beta * sx, uv.y - cfg.step_scale * beta * sy};
        it++;
        if (!(inside_triangle(prop, fa, fb, fc) || inside_triangle(prop, fa, fc, fd))) {
            beta = 0.5f * beta;
            continue;
        }
        beta = fminf(1.f, 2.f * beta);
        uv = prop;
    }
    return false;
}

// evaluate_glint_contribution (:267-294): Fresnel at the normal-mapped normal x
// the glint geometric term (:411-554, clamped to 1e-5).
SMS_D float glint_contribution(const DevScene &sc, const GQuery &q, const Light &L, f2 uv, uint32_t &err,
                               LaneStats &st) {
    f3 yp, ydu, ydv, lw, lp;
    if (L.kind == 1) {
        if (!emitter_endpoint(sc, L, q.p, yp, ydu, ydv, lw, lp, err, st)) return 0.f;
    } else {
        // point light: emitter_interaction_to_vertex without re-sampling
        yp = L.p;
        lp = L.p;
        onb(normalize(q.p - L.p), ydu, ydv);
    }
    f3 s, t;
    base_frame(q, s, t);
    f2 sl, du, dv;
    nm_slope(sc, uv, sl, du, dv);
    f3 wn = s * -sl.x + t * -sl.y + q.n;
    float inv_len = 1.f / length(wn);
    wn = wn * inv_len;
    f3 dnu = (s * -du.x + t * -du.y) * inv_len, dnv = (s * -dv.x + t * -dv.y) * inv_len;
    dnu = dnu - wn * dot(dnu, wn);
    dnv = dnv - wn * dot(dnv, wn);
    Vtx v;
    v.p = q.p; v.dp_du = q.dp_du; v.dp_dv = q.dp_dv; v.n = wn; v.gn = q.n; v.dn_du = dnu; v.dn_dv = dnv;
    v.eta = 1.f;
    v.shape = sc.glinty_shape;
    if (dot(v.n, v.gn) < 0.f) v.gn = -v.gn;
    float cos_theta = dot(wn, normalize(lp - q.p));
    const DevShape &shp = sc.shapes[sc.glinty_shape];
    float F;
    if (shp.alpha > 0.f) {
        // glossy (:383-393): NormalmapBSDF::eval, the nested rough BSDF in the
        // normal-mapped frame at uv (normalmap.cpp:172-181), x 4 |wo . h| in
        // the base frame
        const f3 wiw = normalize(q.sensor - q.p), wow = normalize(lp - q.p);
        const f3 fs = normalize(q.dp_du - wn * dot(wn, q.dp_du)), ft = cross(wn, fs);
        const f3 wip = mk(dot(wiw, fs), dot(wiw, ft), dot(wiw, wn)), wop = mk(dot(wow, fs), dot(wow, ft), dot(wow, wn));
        if (!(dot(wow, q.n) * wop.z > 0.f)) {
            F = 0.f;
        } else {
            const float f = shp.bsdf_type == kBsdfConductor ? roughconductor_eval(shp.alpha, shp.eta, shp.k, wip, wop)
                                                            : roughdielectric_eval(shp.alpha, shp.eta, wip, wop);
            const f3 wil = mk(dot(wiw, s), dot(wiw, t), dot(wiw, q.n)), wol = mk(dot(wow, s), dot(wow, t), dot(wow, q.n));
            const f3 hl = normalize(wil + wol);
            F = f * 4.f * fabsf(dot(wol, hl));
        }
    } else if (shp.bsdf_type == kBsdfConductor && shp.k != 0.f) F = fresnel_conductor(fabsf(cos_theta), shp.eta, shp.k);
    else if (shp.bsdf_type == kBsdfDielectric || shp.bsdf_type == kBsdfConductor)
        F = fresnel_dielectric(fabsf(cos_theta), shp.eta);
    else F = fresnel_conductor(fabsf(cos_theta), 0.f, 1.f);
    Vtx vo = v;
    make_orthonormal(vo.dp_du, vo.dp_dv, vo.dn_du, vo.dn_dv);
    // geometric term with eta = 1: the single-scatter form, then min(1e-5, G)
    // (manifold_glints.cpp:549-552; dx1/dx2 itself is not clamped here)
    f3 x = q.sensor;
    f3 wi = x - vo.p;
    float ili = length(wi);
    if (ili < 1e-3f) return 0.f;
    ili = 1.f / ili; wi = wi * ili;
    f3 wo = yp - vo.p;
    float ilo = length(wo);
    if (ilo < 1e-3f) return 0.f;
    ilo = 1.f / ilo; wo = wo * ilo;
    f3 h = wi + wo;
    float ilh = 1.f / length(h);
    h = h * ilh;
    ilo *= ilh;
    ili *= ilh;
    float dpdu_n = dot(vo.dp_du, vo.n), dpdv_n = dot(vo.dp_dv, vo.n);
    f3 ss = vo.dp_du - vo.n * dpdu_n, tt = vo.dp_dv - vo.n * dpdv_n;
    f3 dh_du = -vo.dp_du * (ili + ilo) + wi * (dot(wi, vo.dp_du) * ili) + wo * (dot(wo, vo.dp_du) * ilo);
    f3 dh_dv = -vo.dp_dv * (ili + ilo) + wi * (dot(wi, vo.dp_dv) * ili) + wo * (dot(wo, vo.dp_dv) * ilo);
    dh_du = dh_du - h * dot(dh_du, h);
    dh_dv = dh_dv - h * dot(dh_dv, h);
    float hn = dot(h, vo.n), hdu = dot(h, vo.dn_du), hdv = dot(h, vo.dn_dv);
    M2 A{dot(dh_du, ss) - dot(vo.dp_du, vo.dn_du) * hn - dpdu_n * hdu,
         dot(dh_dv, ss) - dot(vo.dp_du, vo.dn_dv) * hn - dpdu_n * hdv,
         dot(dh_du, tt) - dot(vo.dp_dv, vo.dn_du) * hn - dpdv_n * hdu,
         dot(dh_dv, tt) - dot(vo.dp_dv, vo.dn_dv) * hn - dpdv_n * hdv};
    dh_du = (ydu - wo * dot(wo, ydu)) * ilo;
    dh_dv = (ydv - wo * dot(wo, ydv)) * ilo;
    dh_du = dh_du - h * dot(dh_du, h);
    dh_dv = dh_dv - h * dot(dh_dv, h);
    M2 B{dot(dh_du, ss), dot(dh_dv, ss), dot(dh_du, tt), dot(dh_dv, tt)};
    float dA = det2(A);
    if (fabsf(dA) < 1e-6f) return 0.f;
    float id = 1.f / dA;
    M2 Ai{A.d * id, -A.b * id, -A.c * id, A.a * id};
    M2 P{Ai.a * B.a + Ai.b * B.c, Ai.a * B.b + Ai.b * B.d, Ai.c * B.a + Ai.d * B.c, Ai.c * B.b + Ai.d * B.d};
    float dx1_dx2 = fabsf(det2(P));
    f3 dd = x - vo.p;
    float inv_r2 = 1.f / dot(dd, dd);
    dd = dd * sqrtf(inv_r2);
    float G = fabsf(dot(dd, vo.gn)) * inv_r2 * dx1_dx2;
    G = fminf(1e-5f, G);
    return F * G;
}

// Emitter sample over all emitters plus the shadow test of :45-56.
SMS_D bool glint_light(const DevScene &sc, Pcg32 &rng, const GQuery &q, Light &L, bool &visible, uint32_t &err,
                       LaneStats &st) {
    visible = false;
    if (!sample_emitter(sc, sc.emitters_all, sc.n_emitters_all, rng, q.p, L)) return false;
    f3 d = L.p - q.p;
    float dist = length(d);
    d = d * (1.f / dist);
    float mint = kRayEps * (1.f + fmaxf(fabsf(q.p.x), fmaxf(fabsf(q.p.y), fabsf(q.p.z))));
    Hit h;
    visible = !trace(sc, q.p, d, mint, dist * (1.f - kRayEps), true, h, err);
    st.ray(h);
    return true;
}

// -------------------------------------------------------------- walk kernel
__global__ void __launch_bounds__(128) glint_walk_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ q,
                                                         const float *__restrict__ w, uint32_t n,
                                                         float *__restrict__ out, DevCounters *ctr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    LaneStats st;
    uint32_t err = 0;
    if (i < n) {
        GQuery Q = load_gquery(q, n, i);
        auto W = [&](int k) { return __ldg(w + (size_t)k * n + i); };
        f2 uv, uv0;
        int it = 0;
        bool ok = glint_walk(sc, cfg, Q, mk(W(0), W(1), W(2)), f2{W(3), W(4)}, uv, uv0, it);
        float res[kGlintWalkOutFields] = {ok ? 1.f : 0.f, (float)it, uv.x, uv.y, uv0.x, uv0.y};
        #pragma unroll
        for (int k = 0; k < kGlintWalkOutFields; ++k) out[(size_t)k * n + i] = res[k];
    }
    flush_stats(st, ctr, err, kPhaseGlintWalk);
}

// ------------------------------------------------------- biased estimator
// G lanes per query, walk m at stream position 3 + 2m; deduplication in uv in
// walk order (:117-138), contributions only for first occurrences.
template <int G>
__global__ void __launch_bounds__(128, 8) glint_biased_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ qs,
                                                           uint32_t n, uint64_t seed, uint64_t stream_off,
                                                           float *__restrict__ value, int *__restrict__ count,
                                                           int *__restrict__ walks, DevCounters *ctr) {
    constexpr int kGroupsPerBlock = 128 / G;
    __shared__ f2 rec[kGroupsPerBlock][kMaxSolutions];
    const unsigned lane = threadIdx.x & 31;
    const int gl = (int)(threadIdx.x % G);
    const int gib = (int)(threadIdx.x / G);
    const int gbase = (int)(lane & ~(unsigned)(G - 1));
    const unsigned gmask = (G == 32) ? kFullG : (((1u << G) - 1u) << gbase);
    LaneStats st;
    uint32_t err = 0;
    const int M = cfg.max_trials > 0 ? cfg.max_trials : 0;
    const uint32_t groups_total = gridDim.x * kGroupsPerBlock;
    const uint32_t rounds = (n + groups_total - 1) / groups_total;
    for (uint32_t r = 0; r < rounds; ++r) {
        uint32_t qi = (r * gridDim.x + blockIdx.x) * kGroupsPerBlock + gib;
        bool live = qi < n;
        GQuery Q{};
        Light L{};
        bool have_light = false, vis = false;
        if (live) {
            Q = load_gquery(qs, n, qi);
            Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
            // the shadow ray is the same for every lane of the group: one lane casts it
            Pcg32 r2 = rng;
            have_light = sample_emitter(sc, sc.emitters_all, sc.n_emitters_all, r2, Q.p, L);
            if (have_light && gl == 0) {
                Pcg32 r3 = rng;
                glint_light(sc, r3, Q, L, vis, err, st);
            }
        }
        vis = __shfl_sync(kFullG, vis, gbase);
        bool counted = live && have_light && sc.glinty_shape >= 0 && sc.nmap_res > 0;
        bool work = counted && vis;
        if (counted && gl == 0) st.conns++;
        int nrec = 0;
        float acc = 0.f;
        // offset normal of a rough glinty surface (:56-64), the same on every lane
        float p_off = 1.f;
        f3 no = mk(0.f, 0.f, 1.f);
        const uint32_t n_off = glint_offset_numbers(sc);
        if (work && n_off) no = glint_offset(sc, Q, query_rng(seed, query_stream(cfg, stream_off, qi), 3u), p_off);
        for (int m0 = 0; m0 < M; m0 += G) {
            int m = m0 + gl;
            bool ok = false;
            f2 uv = {0.f, 0.f};
            if (work && m < M) {
                Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), 3u + n_off + 2u * (uint64_t)m);
                float fx = rng.next_f32(), fy = rng.next_f32();
                f2 uv0;
                int it;
                ok = glint_walk(sc, cfg, Q, L.p, f2{fx, fy}, uv, uv0, it, no);
                st.walks++;
                st.newton += (unsigned)it;
                if (ok) st.succ++; else st.fail++;
            }
            bool keep = false;
            for (int k = 0; k < G; ++k) {
                const int src = gbase + k;
                bool ck = __shfl_sync(kFullG, ok, src);
                f2 uk = {__shfl_sync(kFullG, uv.x, src), __shfl_sync(kFullG, uv.y, src)};
                bool dup = false;
                if (ck)
                    for (int j = gl; j < nrec; j += G) {
                        float dx = uk.x - rec[gib][j].x, dy = uk.y - rec[gib][j].y;
                        if (sqrtf(dx * dx + dy * dy) < cfg.uniqueness_threshold) dup = true;
                    }
                unsigned anydup = __ballot_sync(kFullG, dup) & gmask;
                __syncwarp();
                if (ck && !anydup) {
                    if (nrec < kMaxSolutions) {
                        if (gl == 0) rec[gib][nrec] = uk;
                        nrec++;
                        if (gl == k) keep = true;
                    } else {
                        err |= kErrSolutionOverflow;
                    }
                }
                __syncwarp();
            }
            float c = keep ? glint_contribution(sc, Q, L, uv, err, st) : 0.f;
            for (int k = 0; k < G; ++k) {
                const int src = gbase + k;
                bool kk = __shfl_sync(kFullG, keep, src);
                float ck = __shfl_sync(kFullG, c, src);
                if (kk) acc += ck;
            }
        }
        if (live && gl == 0) {
            f3 v = L.w * (acc / p_off);   // sms_weight /= p_offset (:141)
            if (!work) v = splat(0.f);
            value[qi] = v.x;
            value[(size_t)n + qi] = v.y;
            value[2 * (size_t)n + qi] = v.z;
            count[qi] = nrec;
            walks[qi] = work ? M : 0;
        }
    }
    flush_stats(st, ctr, err, kPhaseGlints);
}

// ------------------------------------------------------ unbiased estimator
__global__ void __launch_bounds__(128) glint_first_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ qs,
                                                          uint32_t n, uint64_t seed, uint64_t stream_off,
                                                          float *__restrict__ value, int *__restrict__ count,
                                                          int *__restrict__ walks, SsScratch scr, DevCounters *ctr) {
    uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    LaneStats st;
    uint32_t err = 0;
    bool enqueue = false;
    if (qi < n) {
        GQuery Q = load_gquery(qs, n, qi);
        Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
        Light L;
        bool vis = false;
        bool have = glint_light(sc, rng, Q, L, vis, err, st) && sc.glinty_shape >= 0 && sc.nmap_res > 0;
        int nw = 0;
        if (have) st.conns++;
        const uint32_t n_off = have ? glint_offset_numbers(sc) : 0u;
        if (have && vis) {
            float p_off;
            const f3 no = glint_offset(sc, Q, rng, p_off);
            rng.advance(n_off);
            float fx = rng.next_f32(), fy = rng.next_f32();
            f2 uv, uv0;
            int it;
            bool ok = glint_walk(sc, cfg, Q, L.p, f2{fx, fy}, uv, uv0, it, no);
            st.walks++;
            st.newton += (unsigned)it;
            nw = 1;
            if (ok) {
                st.succ++;
                scr.dir0[qi] = uv.x;
                scr.dir0[(size_t)n + qi] = uv.y;
                scr.val[qi] = glint_contribution(sc, Q, L, uv, err, st);
                enqueue = true;
            } else {
                st.fail++;
            }
        }
        scr.pos[qi] = 5u + n_off;
        value[qi] = 0.f;
        value[(size_t)n + qi] = 0.f;
        value[2 * (size_t)n + qi] = 0.f;
        count[qi] = 0;
        walks[qi] = nw;
    }
    unsigned want = __ballot_sync(kFullG, enqueue);
    if (want) {
        unsigned lane = threadIdx.x & 31, leader = __ffs(want) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&ctr->trial_count, (unsigned)__popc(want));
        base = __shfl_sync(kFullG, base, leader);
        if (enqueue) scr.list[base + __popc(want & ((1u << lane) - 1u))] = qi;
    }
    flush_stats(st, ctr, err, kPhaseGlints);
}

// Bernoulli trials 32 at a time (:76-105): success when the trial converges
// within uniqueness_threshold (in uv) of the first glint.
__global__ void __launch_bounds__(128) glint_trials_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ qs,
                                                           uint32_t n, uint64_t seed, uint64_t stream_off,
                                                           float *__restrict__ value, int *__restrict__ count,
                                                           int *__restrict__ walks, SsScratch scr, DevCounters *ctr) {
    const unsigned lane = threadIdx.x & 31;
    LaneStats st;
    uint32_t err = 0;
    const int cap = cfg.max_trials > 0 ? cfg.max_trials : kTrialHardLimit;
    const unsigned n_list = *(volatile unsigned *)&ctr->trial_count;
    while (true) {
        unsigned idx = 0;
        if (lane == 0) idx = atomicAdd(&ctr->trial_head, 1u);
        idx = __shfl_sync(kFullG, idx, 0);
        if (idx >= n_list) break;
        uint32_t qi = scr.list[idx];
        GQuery Q = load_gquery(qs, n, qi);
        Pcg32 base = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
        Light L;
        sample_emitter(sc, sc.emitters_all, sc.n_emitters_all, base, Q.p, L);   // at position 3
        f2 uv0 = {scr.dir0[qi], scr.dir0[(size_t)n + qi]};
        float p_off;
        const f3 no = glint_offset(sc, Q, base, p_off);
        const uint32_t n_off = glint_offset_numbers(sc);
        int first = 0;
        for (int t0 = 1; t0 <= cap; t0 += 32) {
            int t = t0 + (int)lane;
            bool succ = false;
            int it = 0;
            if (t <= cap) {
                Pcg32 rng = base;
                rng.advance(2u + n_off + 2u * (uint64_t)(t - 1));
                float fx = rng.next_f32(), fy = rng.next_f32();
                f2 uv, uvi;
                bool ok = glint_walk(sc, cfg, Q, L.p, f2{fx, fy}, uv, uvi, it, no);
                float dx = uv.x - uv0.x, dy = uv.y - uv0.y;
                succ = ok && sqrtf(dx * dx + dy * dy) < cfg.uniqueness_threshold;
            }
            unsigned b = __ballot_sync(kFullG, succ);
            int f = b ? t0 + __ffs(b) - 1 : 0x7fffffff;
            if (t <= cap) {
                if (t <= f) { st.walks++; st.newton += (unsigned)it; }
                else st.spec++;
            }
            if (b) { first = f; break; }
        }
        if (lane == 0) {
            int iterations = first ? first : cap + 1;
            float inv_prob = first ? (float)first : 0.f;
            int trial_walks = first ? first : cap;
            if (!first && cfg.max_trials <= 0) err |= kErrTrialLimit;
            f3 v = L.w * ((scr.val[qi] * inv_prob) / p_off);   // sms_weight /= p_offset (:141)
            value[qi] = v.x;
            value[(size_t)n + qi] = v.y;
            value[2 * (size_t)n + qi] = v.z;
            count[qi] = first ? iterations : -1;
            walks[qi] += trial_walks;
            st.calls++;
            st.iters += (unsigned long long)iterations;
            st.imax = max(st.imax, (unsigned long long)iterations);
        }
    }
    flush_stats(st, ctr, err, kPhaseGlints);
}

// ---------------------------------------------------------------- launchers
// --------------------------------------------------------- LEAN pyramid
// Level 0 from the FP16 slope map (sx, sy, sx^2 + s0, sy^2 + s0, sx sy; s0 the
// base variance of normalmap.cpp:36-40), each coarser level the 2x2 average
// of the finer one (the box-filtered halving of normalmap.cpp:73-89).  Plain
// rounded multiplies and adds, so the pyramid matches a scalar build bit for
// bit.
__global__ void lean_level0_kernel(DevScene sc, float *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = sc.nmap_res * sc.nmap_res;
    if (i >= n) return;
    uint32_t bits = __ldg(sc.nmap + i);
    float2 t = __half22float2(*reinterpret_cast<__half2 *>(&bits));
    float *o = out + 5 * (size_t)i;
    const float s0 = 0.5f * 0.0001f * 0.0001f;
    o[0] = t.x;
    o[1] = t.y;
    o[2] = __fadd_rn(__fmul_rn(t.x, t.x), s0);
    o[3] = __fadd_rn(__fmul_rn(t.y, t.y), s0);
    o[4] = __fmul_rn(t.x, t.y);
}

__global__ void lean_downsample_kernel(const float *src, uint32_t res, float *dst) {
    const uint32_t r2 = res / 2;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r2 * r2) return;
    const uint32_t x = i % r2, y = i / r2;
    const size_t a0 = 5 * ((size_t)(2 * y) * res + 2 * x), a1 = a0 + 5;
    const size_t b0 = 5 * ((size_t)(2 * y + 1) * res + 2 * x), b1 = b0 + 5;
    #pragma unroll
    for (int c = 0; c < 5; ++c) {
        float a = __fadd_rn(src[a0 + c], src[a1 + c]), b = __fadd_rn(src[b0 + c], src[b1 + c]);
        dst[5 * (size_t)i + c] = __fmul_rn(0.25f, __fadd_rn(a, b));
    }
}

cudaError_t launch_lean_build(const DevScene &sc, float *out, const uint32_t *offsets, int levels, cudaStream_t s) {
    const uint32_t n0 = sc.nmap_res * sc.nmap_res;
    lean_level0_kernel<<<(n0 + 255) / 256, 256, 0, s>>>(sc, out + offsets[0]);
    cudaError_t e = cudaGetLastError();
    uint32_t res = sc.nmap_res;
    for (int l = 1; l < levels && e == cudaSuccess; ++l) {
        const uint32_t r2 = res / 2;
        lean_downsample_kernel<<<(r2 * r2 + 255) / 256, 256, 0, s>>>(out + offsets[l - 1], res, out + offsets[l]);
        e = cudaGetLastError();
        res = r2;
    }
    return e;
}

cudaError_t launch_glint_walk(const DevScene &sc, const SolverCfg &cfg, const float *q, const float *w, uint32_t n,
                              float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    phase_begin(tm, kPhaseGlintWalk, s);
    glint_walk_kernel<<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, q, w, n, out, ctr);
    phase_end(tm, s);
    return cudaGetLastError();
}

cudaError_t launch_glint_connect(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                                 uint64_t stream_off, float *value, int *count, int *walks, DevCounters *ctr,
                                 const SsScratch &scr, int num_sms, int blocks_per_sm, PhaseTimer *tm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int bps = blocks_per_sm > 0 ? blocks_per_sm : 16;
    phase_begin(tm, kPhaseGlints, s);
    if (cfg.biased) {
        const int G = cfg.max_trials <= 16 ? 16 : 32;
        const uint32_t gpb = 128 / G;
        uint32_t blocks = std::min<uint32_t>((n + gpb - 1) / gpb, (uint32_t)(num_sms * bps));
        if (G == 16) glint_biased_kernel<16><<<blocks, 128, 0, s>>>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr);
        else glint_biased_kernel<32><<<blocks, 128, 0, s>>>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr);
    } else {
        cudaError_t e = cudaMemsetAsync(&ctr->trial_count, 0, 2 * sizeof(unsigned), s);
        if (e != cudaSuccess) return e;
        glint_first_kernel<<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, q, n, seed, stream_off, value, count, walks, scr,
                                                           ctr);
        glint_trials_kernel<<<num_sms * bps, 128, 0, s>>>(sc, cfg, q, n, seed, stream_off, value, count, walks, scr,
                                                          ctr);
    }
    phase_end(tm, s);
    return cudaGetLastError();
}

}  // namespace sms
