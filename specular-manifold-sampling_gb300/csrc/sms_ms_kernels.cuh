// sms_ms_kernels.cuh -- multi-scatter SMS kernels (k-bounce specular chains) for
// sm_103a and their per-chain-length launchers, templated on the chain length
// K and on kNM (chain shapes may carry the normal map).  Each (K, kNM) pair is
// instantiated in its own translation unit (sms_ms_k1.cu .. sms_ms_k4.cu,
// sms_ms_nm_k1.cu .. sms_ms_nm_k4.cu) so they compile in parallel; sms_ms.cu
// dispatches.
//
// Reference: SpecularManifoldMultiScatter (src/librender/manifold_ms.cpp):
//   specular_manifold_sampling :27-201, sample_path :203-227,
//   evaluate_path_contribution :229-278, sample_seed_path :280-408,
//   newton_solver :410-498, compute_step_halfvector :500-629,
//   compute_step_anglediff :631-857, reproject :859-918,
//   specular_reflectance :920-1023, geometric_term :1025-1190,
//   invert_tridiagonal_step :1192-1232, invert_tridiagonal_geo :1234-1268.
//
// The chain length K is a template parameter (1..4), so a chain's vertices and
// its 2x2 Jacobian blocks live in registers and the block-tridiagonal (block
// Thomas) solve is fully unrolled.  Random numbers follow the single-scatter
// layout: 3 draws for the emitter, 2 per walk (the seed position).
//
// Seed-path template.  The reference keeps the shapes of the first complete
// seed path of an estimate (m_seed_path) and rejects later walks, and Newton
// reprojections, that hit other shapes.  With one walk per lane the template
// is the chain of the first lane, in walk order, whose seed path completed; a
// ballot finds it and a shuffle broadcasts its K shape ids.
#pragma once
#include <algorithm>

#include "sms_device.cuh"
#include "sms_estimator.cuh"
#include "sms_kernels.h"

namespace sms {

constexpr unsigned kFull = 0xffffffffu;

SMS_D M2 mmul(M2 a, M2 b) { return {a.a * b.a + a.b * b.c, a.a * b.b + a.b * b.d, a.c * b.a + a.d * b.c, a.c * b.b + a.d * b.d}; }
SMS_D M2 msub(M2 a, M2 b) { return {a.a - b.a, a.b - b.b, a.c - b.c, a.d - b.d}; }
SMS_D M2 mneg(M2 a) { return {-a.a, -a.b, -a.c, -a.d}; }
SMS_D void mvec(M2 a, float x, float y, float &ox, float &oy) { ox = a.a * x + a.b * y; oy = a.c * x + a.d * y; }
// inverse when det != 0 exactly (the reference's invert lambda, :1199-1206)
SMS_D bool minv(M2 a, M2 &r) {
    float dt = det2(a);
    if (fabsf(dt) == 0.f) return false;
    float id = 1.f / dt;
    r = {a.d * id, -a.b * id, -a.c * id, a.a * id};
    return true;
}
// block from d_sphcoords outputs (rows theta/phi, columns u/v)
SMS_D M2 sph_block(float dtu, float dpu, float dtv, float dpv) { return {dtu, dtv, dpu, dpv}; }

template <int K>
struct Chain {
    Vtx v[K];
};

SMS_D bool chain_shape(const DevScene &sc, int s) {
    uint32_t f = sc.shapes[s].flags;
    return (f & (kShapeFlagCasterMulti | kShapeFlagBouncer)) != 0;
}

// Offset normals of a rough chain (sample_seed_path :356-375): the walk of a
// first path draws them (draw: 2 numbers per vertex; a rough vertex samples a
// Beckmann offset from its pair, a smooth one keeps (0, 0, 1); out: the
// offsets and the product of their densities); later walks scatter about the
// template's offsets (offs).
template <int K>
struct ChainOffsets {
    const f3 *offs = nullptr;     // template offsets (K) or null
    const float *draw = nullptr;  // first path: 2 K numbers
    f3 *out = nullptr;            // first path: its offsets (K)
    float *pdf = nullptr;         // first path: product of the offset densities
};

// Trace a specular chain from x0 toward x1, reflecting or refracting at each
// hit (sample_seed_path :327-397, reproject :865-917).  tmpl (K shape ids) or
// null; check_flags restricts hits to caster_multi / bouncer shapes; straight
// keeps the direction at every hit (the MNEE seed path, :378-397).  kRough:
// scattering about the offset normals of co (:380-382, :894-897).
template <int K, bool kNM = false, bool kRough = false>
SMS_D bool trace_chain(const DevScene &sc, f3 x0, f3 x1, const int *tmpl, bool check_flags, Chain<K> &c,
                       int *shapes, uint32_t &err, LaneStats &st, bool straight = false,
                       ChainOffsets<K> co = ChainOffsets<K>()) {
    f3 wo = normalize(x1 - x0);
    f3 o = x0;
    float mint = kRayEps;
    if (kRough && co.draw) *co.pdf = 1.f;
    #pragma unroll
    for (int b = 0; b < K; ++b) {
        Hit h;
        trace(sc, o, wo, mint, INFINITY, false, h, err);
        st.ray(h);
        if (h.shape < 0) return false;
        if (check_flags && !chain_shape(sc, h.shape)) return false;
        if (tmpl && h.shape != tmpl[b]) return false;
        vertex_from_hit<kNM>(sc, o, wo, h, c.v[b]);
        if (shapes) shapes[b] = h.shape;
        f3 m = c.v[b].n;
        if constexpr (kRough) {
            if (co.draw || co.offs) {
                f3 on = mk(0.f, 0.f, 1.f);
                if (co.draw) {
                    const DevShape &hs = sc.shapes[h.shape];
                    if (hs.alpha > 0.f) {
                        float p;
                        on = beckmann_sample(hs.alpha, co.draw[2 * b], co.draw[2 * b + 1], p);
                        *co.pdf *= p;
                    }
                    co.out[b] = on;
                } else {
                    on = co.offs[b];
                }
                f3 fs, ft, fsdu, fsdv, ftdu, ftdv;
                frame_and_derivative(c.v[b], fs, ft, fsdu, fsdv, ftdu, ftdv);
                m = fs * on.x + ft * on.y + c.v[b].n * on.z;
            }
        }
        f3 wi = -wo;
        if (straight) {
            // no scattering: the chain continues along the straight line
        } else if (c.v[b].eta == 1.f) {
            wo = m * (2.f * dot(wi, m)) - wi;
        } else if (!refract(wi, m, c.v[b].eta, wo)) {
            return false;
        }
        o = c.v[b].p;
        mint = (1.f + fmaxf(fabsf(o.x), fmaxf(fabsf(o.y), fabsf(o.z)))) * kRayEps;
    }
    return true;
}

// The seed path of a walk (sample_seed_path :280-408): toward the sampled
// point x1, or with cfg.mnee_init along the straight line toward the MNEE
// target without scattering.
template <int K, bool kNM = false, bool kRough = false>
SMS_D bool seed_chain(const DevScene &sc, const SolverCfg &cfg, int caster, f3 x0, f3 x1, f3 lp, const int *tmpl,
                      Chain<K> &c, int *shapes, uint32_t &err, LaneStats &st,
                      ChainOffsets<K> co = ChainOffsets<K>()) {
    if (cfg.mnee_init)
        return trace_chain<K, kNM, kRough>(sc, x0, mnee_target(sc.shapes[caster], lp), tmpl, true, c, shapes, err,
                                           st, true, co);
    return trace_chain<K, kNM, kRough>(sc, x0, x1, tmpl, true, c, shapes, err, st, false, co);
}

// Angle-difference constraint of vertex i and its blocks w.r.t. the previous,
// current and next vertex (:631-857); `no` is the vertex's offset normal in
// its shading frame (:707-717; (0, 0, 1) keeps the vertex normal).
SMS_D bool vertex_anglediff(f3 xp, const Vtx &vc, f3 xn, const Vtx *vp, const Vtx *vn, float &c0, float &c1,
                            M2 &prev, M2 &cur, M2 &next, f3 no = f3{0.f, 0.f, 1.f}) {
    prev = {0.f, 0.f, 0.f, 0.f};
    cur = prev;
    next = prev;
    c0 = c1 = 0.f;
    f3 wo = xn - vc.p;
    float ilo = length(wo);
    if (ilo < 1e-3f) return false;
    ilo = 1.f / ilo; wo = wo * ilo;
    f3 dwo_du = (vc.dp_du - wo * dot(wo, vc.dp_du)) * -ilo;
    f3 dwo_dv = (vc.dp_dv - wo * dot(wo, vc.dp_dv)) * -ilo;
    f3 wi = xp - vc.p;
    float ili = length(wi);
    if (ili < 1e-3f) return false;
    ili = 1.f / ili; wi = wi * ili;
    f3 dwi_du = (vc.dp_du - wi * dot(wi, vc.dp_du)) * -ili;
    f3 dwi_dv = (vc.dp_dv - wi * dot(wi, vc.dp_dv)) * -ili;
    const bool refl = vc.eta == 1.f;
    const f3 z = splat(0.f);
    f3 nn = vc.n, nn_du = vc.dn_du, nn_dv = vc.dn_dv;
    if (no.x != 0.f || no.y != 0.f) {
        f3 fs, ft, fsdu, fsdv, ftdu, ftdv;
        frame_and_derivative(vc, fs, ft, fsdu, fsdv, ftdu, ftdv);
        nn = fs * no.x + ft * no.y + vc.n * no.z;
        nn_du = fsdu * no.x + ftdu * no.y + vc.dn_du * no.z;
        nn_dv = fsdv * no.x + ftdv * no.y + vc.dn_dv * no.z;
    }
    auto xform = [&](f3 w, f3 &out) {
        if (refl) { out = nn * (2.f * dot(w, nn)) - w; return true; }
        return refract(w, nn, vc.eta, out);
    };
    auto dxform = [&](f3 w, f3 du, f3 dv, f3 ndu, f3 ndv, f3 &ou, f3 &ov) {
        if (refl) d_reflect(w, du, dv, nn, ndu, ndv, ou, ov);
        else d_refract(w, du, dv, nn, ndu, ndv, vc.eta, ou, ov);
    };
    float a0, a1, a2, a3, b0, b1, b2, b3;
    f3 t;
    if (xform(wi, t)) {
        float to, po, tt, pt;
        sphcoords(wo, to, po);
        sphcoords(t, tt, pt);
        float dt = to - tt, dp = po - pt;
        if (dp < -kPi) dp += 2.f * kPi; else if (dp > kPi) dp -= 2.f * kPi;
        c0 = dt; c1 = dp;
        if (vp) {
            f3 du = (vp->dp_du - wi * dot(wi, vp->dp_du)) * ili, dv = (vp->dp_dv - wi * dot(wi, vp->dp_dv)) * ili;
            f3 ou, ov;
            dxform(wi, du, dv, z, z, ou, ov);
            d_sphcoords(t, ou, ov, b0, b1, b2, b3);
            prev = sph_block(-b0, -b1, -b2, -b3);
        }
        f3 ou, ov;
        dxform(wi, dwi_du, dwi_dv, nn_du, nn_dv, ou, ov);
        d_sphcoords(wo, dwo_du, dwo_dv, a0, a1, a2, a3);
        d_sphcoords(t, ou, ov, b0, b1, b2, b3);
        cur = sph_block(a0 - b0, a1 - b1, a2 - b2, a3 - b3);
        if (vn) {
            f3 du = (vn->dp_du - wo * dot(wo, vn->dp_du)) * ilo, dv = (vn->dp_dv - wo * dot(wo, vn->dp_dv)) * ilo;
            d_sphcoords(wo, du, dv, a0, a1, a2, a3);
            next = sph_block(a0, a1, a2, a3);
        }
        return true;
    }
    if (xform(wo, t)) {
        float ti, pi, tt, pt;
        sphcoords(wi, ti, pi);
        sphcoords(t, tt, pt);
        float dt = ti - tt, dp = pi - pt;
        if (dp < -kPi) dp += 2.f * kPi; else if (dp > kPi) dp -= 2.f * kPi;
        c0 = dt; c1 = dp;
        if (vp) {
            f3 du = (vp->dp_du - wi * dot(wi, vp->dp_du)) * ili, dv = (vp->dp_dv - wi * dot(wi, vp->dp_dv)) * ili;
            d_sphcoords(wi, du, dv, a0, a1, a2, a3);
            prev = sph_block(a0, a1, a2, a3);
        }
        f3 ou, ov;
        dxform(wo, dwo_du, dwo_dv, nn_du, nn_dv, ou, ov);
        d_sphcoords(wi, dwi_du, dwi_dv, a0, a1, a2, a3);
        d_sphcoords(t, ou, ov, b0, b1, b2, b3);
        cur = sph_block(a0 - b0, a1 - b1, a2 - b2, a3 - b3);
        if (vn) {
            f3 du = (vn->dp_du - wo * dot(wo, vn->dp_du)) * ilo, dv = (vn->dp_dv - wo * dot(wo, vn->dp_dv)) * ilo;
            dxform(wo, du, dv, z, z, ou, ov);
            d_sphcoords(t, ou, ov, b0, b1, b2, b3);
            next = sph_block(-b0, -b1, -b2, -b3);
        }
        return true;
    }
    return false;
}

// Half-vector constraint of vertex i and its blocks (:500-629); C = H - N with
// N the offset normal's (x, y) (:618-621).
SMS_D bool vertex_halfvector(f3 xp, const Vtx &vc, f3 xn, const Vtx *vp, const Vtx *vn, float &c0, float &c1,
                             M2 &prev, M2 &cur, M2 &next, f3 no = f3{0.f, 0.f, 1.f}) {
    prev = {0.f, 0.f, 0.f, 0.f};
    cur = prev;
    next = prev;
    f3 wo = xn - vc.p;
    float ilo = length(wo);
    if (ilo < 1e-3f) return false;
    ilo = 1.f / ilo; wo = wo * ilo;
    f3 wi = xp - vc.p;
    float ili = length(wi);
    if (ili < 1e-3f) return false;
    ili = 1.f / ili; wi = wi * ili;
    float eta = vc.eta;
    if (dot(wi, vc.gn) < 0.f) eta = 1.f / eta;
    f3 h = wi + wo * eta;
    if (eta != 1.f) h = h * -1.f;
    float ilh = 1.f / length(h);
    h = h * ilh;
    ilo *= eta * ilh;
    ili *= ilh;
    f3 s, t, dsdu, dsdv, dtdu, dtdv;
    frame_and_derivative(vc, s, t, dsdu, dsdv, dtdu, dtdv);
    f3 du, dv;
    if (vp) {
        du = (vp->dp_du - wi * dot(wi, vp->dp_du)) * ili;
        dv = (vp->dp_dv - wi * dot(wi, vp->dp_dv)) * ili;
        du = du - h * dot(du, h); dv = dv - h * dot(dv, h);
        if (eta != 1.f) { du = du * -1.f; dv = dv * -1.f; }
        prev = {dot(s, du), dot(s, dv), dot(t, du), dot(t, dv)};
    }
    du = -vc.dp_du * (ili + ilo) + wi * (dot(wi, vc.dp_du) * ili) + wo * (dot(wo, vc.dp_du) * ilo);
    dv = -vc.dp_dv * (ili + ilo) + wi * (dot(wi, vc.dp_dv) * ili) + wo * (dot(wo, vc.dp_dv) * ilo);
    du = du - h * dot(du, h); dv = dv - h * dot(dv, h);
    if (eta != 1.f) { du = du * -1.f; dv = dv * -1.f; }
    cur = {dot(dsdu, h) + dot(s, du), dot(dsdv, h) + dot(s, dv), dot(dtdu, h) + dot(t, du), dot(dtdv, h) + dot(t, dv)};
    if (vn) {
        du = (vn->dp_du - wo * dot(wo, vn->dp_du)) * ilo;
        dv = (vn->dp_dv - wo * dot(wo, vn->dp_dv)) * ilo;
        du = du - h * dot(du, h); dv = dv - h * dot(dv, h);
        if (eta != 1.f) { du = du * -1.f; dv = dv * -1.f; }
        next = {dot(s, du), dot(s, dv), dot(t, du), dot(t, dv)};
    }
    c0 = dot(s, h) - no.x;
    c1 = dot(t, h) - no.y;
    return true;
}

// Constraints, blocks and the block-Thomas Newton step (:1192-1232).  Returns
// false when a constraint or the solve fails; conv = all |C_i| <= threshold;
// dx0 = step of the first vertex (the only one reprojection uses).
template <int K, bool kRough = false>
SMS_D bool chain_step(const SolverCfg &cfg, f3 x0, f3 lp, const Chain<K> &c, bool &conv, float &dx0u, float &dx0v,
                      const f3 *offs = nullptr) {
    float C0[K], C1[K];
    M2 P[K], Cu[K], N[K];
    #pragma unroll
    for (int i = 0; i < K; ++i) {
        f3 xp = i == 0 ? x0 : c.v[i - 1].p;
        f3 xn = i == K - 1 ? lp : c.v[i + 1].p;
        const Vtx *vp = i > 0 ? &c.v[i - 1] : nullptr;
        const Vtx *vn = i < K - 1 ? &c.v[i + 1] : nullptr;
        const f3 no = kRough && offs ? offs[i] : f3{0.f, 0.f, 1.f};
        bool ok = cfg.halfvector ? vertex_halfvector(xp, c.v[i], xn, vp, vn, C0[i], C1[i], P[i], Cu[i], N[i], no)
                                 : vertex_anglediff(xp, c.v[i], xn, vp, vn, C0[i], C1[i], P[i], Cu[i], N[i], no);
        if (!ok) return false;
    }
    M2 tmp[K], il[K];
    float dxu[K], dxv[K];
    tmp[0] = P[0];
    if (!minv(Cu[0], il[0])) return false;
    #pragma unroll
    for (int i = 1; i < K; ++i) {
        tmp[i] = mmul(P[i], il[i - 1]);
        if (!minv(msub(Cu[i], mmul(tmp[i], N[i - 1])), il[i])) return false;
    }
    dxu[0] = C0[0]; dxv[0] = C1[0];
    #pragma unroll
    for (int i = 1; i < K; ++i) {
        float tu, tv;
        mvec(tmp[i], dxu[i - 1], dxv[i - 1], tu, tv);
        dxu[i] = C0[i] - tu; dxv[i] = C1[i] - tv;
    }
    {
        float u, v;
        mvec(il[K - 1], dxu[K - 1], dxv[K - 1], u, v);
        dxu[K - 1] = u; dxv[K - 1] = v;
    }
    #pragma unroll
    for (int i = K - 2; i >= 0; --i) {
        float nu, nv, u, v;
        mvec(N[i], dxu[i + 1], dxv[i + 1], nu, nv);
        mvec(il[i], dxu[i] - nu, dxv[i] - nv, u, v);
        dxu[i] = u; dxv[i] = v;
    }
    conv = true;
    #pragma unroll
    for (int i = 0; i < K; ++i)
        if (sqrtf(C0[i] * C0[i] + C1[i] * C1[i]) > cfg.solver_threshold) conv = false;
    dx0u = dxu[0];
    dx0v = dxv[0];
    return true;
}

// newton_solver (:410-498).  c holds the seed path on entry and the solution
// on success; tmpl = the estimate's template shapes.
template <int K, bool kNM = false, bool kRough = false>
SMS_D bool chain_newton(const DevScene &sc, const SolverCfg &cfg, f3 x0, f3 lp, const int *tmpl, Chain<K> &c,
                        int &it, uint32_t &err, LaneStats &st, const f3 *offs = nullptr) {
    ChainOffsets<K> co;
    co.offs = offs;
    it = 0;
    float beta = 1.f;
    bool need = true, conv = false, ok = true;
    float du = 0.f, dv = 0.f;
    while (it < cfg.max_iterations) {
        if (need) ok = chain_step<K, kRough>(cfg, x0, lp, c, conv, du, dv, offs);
        if (!ok) break;
        if (conv) break;
        f3 p0 = c.v[0].p - (c.v[0].dp_du * du + c.v[0].dp_dv * dv) * (cfg.step_scale * beta);
        Chain<K> prop;
        if (trace_chain<K, kNM, kRough>(sc, x0, p0, tmpl, false, prop, nullptr, err, st, false, co)) {
            beta = fminf(1.f, 2.f * beta);
            c = prop;
            need = true;
        } else {
            beta = 0.5f * beta;
            need = false;
        }
        it++;
    }
    if (!(ok && conv)) return false;
    #pragma unroll
    for (int i = 0; i < K; ++i) {
        f3 xp = i == 0 ? x0 : c.v[i - 1].p, xn = i == K - 1 ? lp : c.v[i + 1].p;
        f3 wi = normalize(xp - c.v[i].p), wo = normalize(xn - c.v[i].p);
        bool refraction = dot(c.v[i].gn, wi) * dot(c.v[i].gn, wo) < 0.f;
        if ((c.v[i].eta == 1.f) ? refraction : !refraction) return false;
    }
    return true;
}

// specular_reflectance (:920-1023): Fresnel along the re-traced chain, then
// the light visibility test.  At a rough vertex the reference computes the
// glossy BSDF value in the half-vector domain (:963-985) but multiplies only
// the delta branch's factor into the throughput (:1007): a rough vertex
// contributes 1, restated as is.
template <int K, bool kNM = false, bool kRough = false>
SMS_D float chain_reflectance(const DevScene &sc, f3 x0, f3 lp, const Chain<K> &c, uint32_t &err, LaneStats &st) {
    f3 o = x0, d = normalize(c.v[0].p - x0);
    float val = 1.f;
    f3 last = x0;
    #pragma unroll
    for (int k = 0; k < K; ++k) {
        Hit h;
        trace(sc, o, d, kRayEps, INFINITY, false, h, err);
        st.ray(h);
        if (h.shape < 0) return 0.f;
        Vtx hv;
        vertex_from_hit<kNM>(sc, o, d, h, hv);
        f3 wo = k + 1 < K ? normalize(c.v[k + 1].p - hv.p) : normalize(lp - hv.p);
        if (!kRough || !(sc.shapes[h.shape].alpha > 0.f)) val *= specular_reflectance(sc.shapes[h.shape], hv.n, wo);
        o = hv.p;
        d = wo;
        last = hv.p;
    }
    f3 dl = lp - last;
    float mint = kRayEps * (1.f + fmaxf(fabsf(last.x), fmaxf(fabsf(last.y), fabsf(last.z))));
    Hit h;
    bool occ = trace(sc, last, normalize(dl), mint, length(dl) * (1.f - kRayEps), true, h, err);
    st.ray(h);
    return occ ? 0.f : val;
}

// Generalized geometric term (:1025-1190) for a positional endpoint, with
// invert_tridiagonal_geo (:1234-1268).  c: orthonormalized chain.
template <int K>
SMS_D float chain_geometric(f3 x, const Chain<K> &c, f3 yp, f3 ydu, f3 ydv) {
    M2 P[K], Cu[K], N[K];
    #pragma unroll
    for (int i = 0; i < K; ++i) {
        const Vtx &v = c.v[i];
        f3 xn = i + 1 < K ? c.v[i + 1].p : yp;
        f3 ndu = i + 1 < K ? c.v[i + 1].dp_du : ydu, ndv = i + 1 < K ? c.v[i + 1].dp_dv : ydv;
        f3 wo = xn - v.p;
        float ilo = length(wo);
        if (ilo < 1e-3f) return 0.f;
        ilo = 1.f / ilo; wo = wo * ilo;
        f3 xp = i == 0 ? x : c.v[i - 1].p;
        f3 wi = xp - v.p;
        float ili = length(wi);
        if (ili < 1e-3f) return 0.f;
        ili = 1.f / ili; wi = wi * ili;
        float eta = v.eta;
        if (dot(wi, v.gn) < 0.f) eta = 1.f / eta;
        f3 h = wi + wo * eta;
        if (eta != 1.f) h = h * -1.f;
        float ilh = 1.f / length(h);
        h = h * ilh;
        ilo *= eta * ilh;
        ili *= ilh;
        float dpdu_n = dot(v.dp_du, v.n), dpdv_n = dot(v.dp_dv, v.n);
        f3 s = v.dp_du - v.n * dpdu_n, t = v.dp_dv - v.n * dpdv_n;
        f3 du, dv;
        P[i] = {0.f, 0.f, 0.f, 0.f};
        if (i > 0) {
            du = (c.v[i - 1].dp_du - wi * dot(wi, c.v[i - 1].dp_du)) * ili;
            dv = (c.v[i - 1].dp_dv - wi * dot(wi, c.v[i - 1].dp_dv)) * ili;
            du = du - h * dot(du, h); dv = dv - h * dot(dv, h);
            if (eta != 1.f) { du = du * -1.f; dv = dv * -1.f; }
            P[i] = {dot(s, du), dot(s, dv), dot(t, du), dot(t, dv)};
        }
        du = -v.dp_du * (ili + ilo) + wi * (dot(wi, v.dp_du) * ili) + wo * (dot(wo, v.dp_du) * ilo);
        dv = -v.dp_dv * (ili + ilo) + wi * (dot(wi, v.dp_dv) * ili) + wo * (dot(wo, v.dp_dv) * ilo);
        du = du - h * dot(du, h); dv = dv - h * dot(dv, h);
        if (eta != 1.f) { du = du * -1.f; dv = dv * -1.f; }
        float hn = dot(h, v.n), hdu = dot(h, v.dn_du), hdv = dot(h, v.dn_dv);
        Cu[i] = {dot(du, s) - dot(v.dp_du, v.dn_du) * hn - dpdu_n * hdu,
                 dot(dv, s) - dot(v.dp_du, v.dn_dv) * hn - dpdu_n * hdv,
                 dot(du, t) - dot(v.dp_dv, v.dn_du) * hn - dpdv_n * hdu,
                 dot(dv, t) - dot(v.dp_dv, v.dn_dv) * hn - dpdv_n * hdv};
        du = (ndu - wo * dot(wo, ndu)) * ilo;
        dv = (ndv - wo * dot(wo, ndv)) * ilo;
        du = du - h * dot(du, h); dv = dv - h * dot(dv, h);
        if (eta != 1.f) { du = du * -1.f; dv = dv * -1.f; }
        N[i] = {dot(s, du), dot(s, dv), dot(t, du), dot(t, dv)};
    }
    // block system of n = K + 1 vertices; blocks exist for the K chain vertices
    M2 Li, tmp[K], il[K];
    if (!minv(Cu[0], Li)) return 0.f;
    #pragma unroll
    for (int i = 0; i + 1 < K; ++i) {
        tmp[i] = mmul(Li, N[i]);
        if (!minv(msub(Cu[i + 1], mmul(P[i + 1], tmp[i])), Li)) return 0.f;
    }
    il[K - 1] = mmul(mneg(Li), N[K - 1]);
    #pragma unroll
    for (int i = K - 2; i >= 0; --i) il[i] = mmul(mneg(tmp[i]), il[i + 1]);
    float dx1_dxend = fabsf(det2(mneg(il[0])));
    f3 d = x - c.v[0].p;
    float inv_r2 = 1.f / dot(d, d);
    d = d * sqrtf(inv_r2);
    return fabsf(dot(d, c.v[0].gn)) * inv_r2 * dx1_dxend;
}

// evaluate_path_contribution (:229-278).
template <int K, bool kNM = false, bool kRough = false>
SMS_D f3 chain_contribution(const DevScene &sc, f3 x, const Light &L, const Chain<K> &sol, uint32_t &err,
                            LaneStats &st) {
    f3 yp, ydu, ydv, lw, lp;
    if (!emitter_endpoint(sc, L, sol.v[K - 1].p, yp, ydu, ydv, lw, lp, err, st)) return splat(0.f);
    Chain<K> c = sol;
    #pragma unroll
    for (int i = 0; i < K; ++i) make_orthonormal(c.v[i].dp_du, c.v[i].dp_dv, c.v[i].dn_du, c.v[i].dn_dv);
    float F = chain_reflectance<K, kNM, kRough>(sc, x, lp, c, err, st);
    F *= chain_geometric<K>(x, c, yp, ydu, ydv);
    return lw * F;
}

// -------------------------------------------------------------- walk kernel
template <int K, bool kNM>
__global__ void __launch_bounds__(128) ms_walk_kernel(DevScene sc, SolverCfg cfg, int caster, const float *__restrict__ q,
                                                      const float *__restrict__ w, uint32_t n, float *__restrict__ out,
                                                      DevCounters *ctr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    LaneStats st;
    uint32_t err = 0;
    if (i < n) {
        auto Q = [&](int k) { return __ldg(q + (size_t)k * n + i); };
        auto W = [&](int k) { return __ldg(w + (size_t)k * n + i); };
        f3 x = mk(Q(0), Q(1), Q(2));
        f3 lp = mk(W(0), W(1), W(2));
        f3 ps = mk(W(3), W(4), W(5));
        f3 x1 = sample_position(sc, sc.shapes[caster], W(6), W(7));
        if (ps.x != 0.f || ps.y != 0.f || ps.z != 0.f) x1 = ps;
        Chain<K> c;
        int shapes[K];
        int it = 0;
        bool seed_ok = seed_chain<K, kNM>(sc, cfg, caster, x, x1, lp, nullptr, c, shapes, err, st);
        bool ok = seed_ok && chain_newton<K, kNM>(sc, cfg, x, lp, shapes, c, it, err, st);
        float res[kMsWalkOutFields] = {ok ? 1.f : 0.f, (float)it, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, seed_ok ? 1.f : 0.f};
        if (ok) {
            res[2] = c.v[0].p.x; res[3] = c.v[0].p.y; res[4] = c.v[0].p.z;
            res[5] = c.v[K - 1].p.x; res[6] = c.v[K - 1].p.y; res[7] = c.v[K - 1].p.z;
        }
        #pragma unroll
        for (int k = 0; k < kMsWalkOutFields; ++k) out[(size_t)k * n + i] = res[k];
    }
    flush_stats(st, ctr, err, kPhaseMsWalk);
}

// ------------------------------------------------ unbiased-MNEE test
// The test of path_sms_ms.cpp:323-360 for the wavefront paths with want[i]
// (their BSDF-sampled ray reached a caustic emitter through a complete
// specular chain): the MNEE walk from the receiver point -- the straight seed
// chain toward the light point (or the first specular shape's box centre),
// its own shapes as the template, then Newton -- and, where it does not end on
// the chain the path recorded (every vertex within 1e-5), the path's emitter
// contribution is added to its radiance.  rec (16 rows of `stride`): receiver
// point (3), first specular shape (int bits), recorded vertices (3 K);
// stage rows 0-2 the light point, 3-5 the contribution; L: 3 rows.
template <int K, bool kNM>
__global__ void __launch_bounds__(128) ms_mnee_check_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ rec,
                                                            const float *__restrict__ stage,
                                                            const int *__restrict__ want, float *__restrict__ L,
                                                            uint32_t n, uint32_t stride, DevCounters *ctr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    LaneStats st;
    uint32_t err = 0;
    if (i < n && want[i]) {
        auto R = [&](int k) { return rec[(size_t)k * stride + i]; };
        auto S = [&](int k) { return stage[(size_t)k * stride + i]; };
        const f3 x0 = mk(R(0), R(1), R(2)), lp = mk(S(0), S(1), S(2));
        const int caster = __float_as_int(R(3));
        Chain<K> c;
        int shapes[K];
        int it = 0;
        bool ok = seed_chain<K, kNM>(sc, cfg, caster, x0, lp, lp, nullptr, c, shapes, err, st) &&
                  chain_newton<K, kNM>(sc, cfg, x0, lp, shapes, c, it, err, st);
        #pragma unroll
        for (int k = 0; k < K; ++k)
            if (ok && !(length(c.v[k].p - mk(R(4 + 3 * k), R(5 + 3 * k), R(6 + 3 * k))) < 1e-5f)) ok = false;
        if (!ok) {
            #pragma unroll
            for (int k = 0; k < 3; ++k) L[(size_t)k * stride + i] += S(3 + k);
        }
    }
    flush_stats(st, ctr, err, kPhaseMs);
}

// Random numbers per walk: the seed position's 2; with rough chain shapes
// (kRough) a fixed run of 2 + 2 K: the seed position, then 2 per chain vertex
// for its offset normal, used only by a first path at a rough vertex (the
// reference draws those only when it uses them; the fixed run keeps walks
// independent, as lanes running side by side need, with the same expectation).
template <int K, bool kRough>
constexpr uint32_t ms_walk_numbers() { return kRough ? 2u + 2u * (uint32_t)K : 2u; }

// Offset normals of an estimate's template in the unbiased estimator's scratch:
// rows 3 b + j (vertex b, component j) and row 3 kMaxBounces (the product of
// their densities) of the float block after the kMaxBounces template-shape rows.
SMS_D float *ms_offset_rows(int *tmpl, uint32_t n) { return reinterpret_cast<float *>(tmpl + (size_t)kMaxBounces * n); }

// -------------------------------------------------------- biased estimator
// G lanes per query, one walk per lane; walk m of caster c at stream position
// 3 + r (c M + m), r the walk's numbers.  Unlike the single-scatter estimator,
// solutions are deduplicated before the contribution, which itself tests
// visibility (:147-195).  kRough: the first complete seed path (the template)
// also fixes the offset normals; walks after it in its chunk retrace their
// seed paths about them (:160, :372-375).
template <int K, int G, bool kNM, bool kRough = false>
#ifndef SMS_MS_BIASED_MIN_BLOCKS
#define SMS_MS_BIASED_MIN_BLOCKS 8
#endif
__global__ void __launch_bounds__(128, SMS_MS_BIASED_MIN_BLOCKS) ms_biased_kernel(DevScene sc, SolverCfg cfg, const float *__restrict__ qs,
                                                        uint32_t n, uint64_t seed, uint64_t stream_off,
                                                        float *__restrict__ value, int *__restrict__ count,
                                                        int *__restrict__ walks, DevCounters *ctr) {
    constexpr int kGroupsPerBlock = 128 / G;
    __shared__ f3 rec[kGroupsPerBlock][kMaxSolutions];
    const unsigned lane = threadIdx.x & 31;
    const int gl = (int)(threadIdx.x % G);
    const int gib = (int)(threadIdx.x / G);
    const int gbase = (int)(lane & ~(unsigned)(G - 1));
    const unsigned gmask = (G == 32) ? kFull : (((1u << G) - 1u) << gbase);
    LaneStats st;
    uint32_t err = 0;
    const int M = cfg.max_trials > 0 ? cfg.max_trials : 0;
    constexpr uint32_t kRun = ms_walk_numbers<K, kRough>();
    const uint32_t groups_total = gridDim.x * kGroupsPerBlock;
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
            have_light = sample_emitter(sc, sc.emitters_ms, sc.n_emitters_ms, rng, Q.x, L);
        }
        bool work = live && have_light && sc.n_casters_ms > 0;
        if (work && gl == 0) st.conns++;
        f3 acc = splat(0.f);
        int n_unique = 0;
        for (int ci = 0; ci < sc.n_casters_ms; ++ci) {
            int caster = sc.casters_ms[ci];
            bool have_tmpl = false;
            int tmpl[K];
            #pragma unroll
            for (int b = 0; b < K; ++b) tmpl[b] = -1;
            int nrec = 0;
            f3 cur = splat(0.f);
            f3 toff[K];           // the template's offset normals (kRough)
            float tpdf = 1.f;
            #pragma unroll
            for (int b = 0; b < K; ++b) toff[b] = mk(0.f, 0.f, 1.f);
            for (int m0 = 0; m0 < M; m0 += G) {
                int m = m0 + gl;
                bool act = work && m < M;
                Chain<K> c;
                int shapes[K];
                #pragma unroll
                for (int b = 0; b < K; ++b) shapes[b] = -1;
                bool seed_ok = false;
                f3 x1 = splat(0.f);
                f3 own[K];
                float own_pdf = 1.f;
                #pragma unroll
                for (int b = 0; b < K; ++b) own[b] = mk(0.f, 0.f, 1.f);
                if (act) {
                    Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), 3u + kRun * ((uint64_t)ci * M + m));
                    float sx = rng.next_f32(), sy = rng.next_f32();
                    x1 = sample_position(sc, sc.shapes[caster], sx, sy);
                    if constexpr (kRough) {
                        float dr[2 * K];
                        #pragma unroll
                        for (int j = 0; j < 2 * K; ++j) dr[j] = rng.next_f32();
                        ChainOffsets<K> co;
                        if (have_tmpl) {
                            co.offs = toff;
                        } else {
                            co.draw = dr; co.out = own; co.pdf = &own_pdf;
                        }
                        seed_ok = seed_chain<K, kNM, true>(sc, cfg, caster, Q.x, x1, L.p, nullptr, c, shapes, err, st,
                                                           co);
                    } else {
                        seed_ok = seed_chain<K, kNM>(sc, cfg, caster, Q.x, x1, L.p, nullptr, c, shapes, err, st);
                    }
                }
                // the first completed seed path of the estimate is the template
                unsigned sb = __ballot_sync(kFull, seed_ok) & gmask;
                const int first_lane = sb ? (__ffs(sb) - 1) : -1;   // absolute lane id
                int tshape[K];
                #pragma unroll
                for (int b = 0; b < K; ++b)
                    tshape[b] = __shfl_sync(kFull, shapes[b], first_lane >= 0 ? first_lane : (int)lane);
                // the first completed lane's offsets, broadcast by the whole warp
                // (the two groups of a 16-lane split may differ in what follows)
                f3 foff[K];
                float fpdf = 1.f;
                if constexpr (kRough) {
                    const int src = first_lane >= 0 ? first_lane : (int)lane;
                    #pragma unroll
                    for (int b = 0; b < K; ++b)
                        foff[b] = mk(__shfl_sync(kFull, own[b].x, src), __shfl_sync(kFull, own[b].y, src),
                                     __shfl_sync(kFull, own[b].z, src));
                    fpdf = __shfl_sync(kFull, own_pdf, src);
                }
                bool is_template_walk = false;
                if (!have_tmpl && first_lane >= 0) {
                    #pragma unroll
                    for (int b = 0; b < K; ++b) tmpl[b] = tshape[b];
                    have_tmpl = true;
                    is_template_walk = (int)lane == first_lane;
                    if constexpr (kRough) {
                        #pragma unroll
                        for (int b = 0; b < K; ++b) toff[b] = foff[b];
                        tpdf = fpdf;
                        // walks after the template walk are not first paths:
                        // their seed paths scatter about the template's offsets
                        if (act && (int)lane > first_lane) {
                            ChainOffsets<K> co;
                            co.offs = toff;
                            seed_ok = seed_chain<K, kNM, true>(sc, cfg, caster, Q.x, x1, L.p, nullptr, c, shapes, err,
                                                               st, co);
                        }
                    }
                }
                bool ok = false;
                int it = 0;
                if (seed_ok) {
                    bool match = true;
                    if (!is_template_walk) {
                        #pragma unroll
                        for (int b = 0; b < K; ++b) match = match && shapes[b] == tmpl[b];
                    }
                    ok = match && chain_newton<K, kNM, kRough>(sc, cfg, Q.x, L.p, tmpl, c, it, err, st,
                                                               kRough ? toff : nullptr);
                }
                if (act) {
                    st.walks++;
                    st.newton += (unsigned)it;
                    if (ok) st.succ++; else st.fail++;
                }
                f3 dir = ok ? normalize(c.v[0].p - Q.x) : splat(0.f);
                // walk-ordered deduplication (no visibility test first, :162-184)
                bool keep = false;
                for (int k = 0; k < G; ++k) {
                    const int src = gbase + k;
                    bool ck = __shfl_sync(kFull, ok, src);
                    f3 dk = mk(__shfl_sync(kFull, dir.x, src), __shfl_sync(kFull, dir.y, src),
                               __shfl_sync(kFull, dir.z, src));
                    bool dup = false;
                    if (ck)
                        for (int j = gl; j < nrec; j += G)
                            if (fabsf(dot(dk, rec[gib][j]) - 1.f) < cfg.uniqueness_threshold) dup = true;
                    unsigned anydup = __ballot_sync(kFull, dup) & gmask;
                    __syncwarp();
                    if (ck && !anydup) {
                        if (nrec < kMaxSolutions) {
                            if (gl == 0) rec[gib][nrec] = dk;
                            nrec++;
                            if (gl == k) keep = true;
                        } else {
                            err |= kErrSolutionOverflow;
                        }
                    }
                    __syncwarp();
                }
                f3 contrib = splat(0.f);
                if (keep)
                    contrib = receiver_eval(sc, Q, dir, err) * chain_contribution<K, kNM, kRough>(sc, Q.x, L, c, err, st);
                // sum in walk order
                for (int k = 0; k < G; ++k) {
                    const int src = gbase + k;
                    bool kk = __shfl_sync(kFull, keep, src);
                    f3 vk = mk(__shfl_sync(kFull, contrib.x, src), __shfl_sync(kFull, contrib.y, src),
                               __shfl_sync(kFull, contrib.z, src));
                    if (kk) cur = cur + vk;
                }
            }
            // result += value / m_offset_normals_pdf (:198)
            if (kRough) cur = mk(cur.x / tpdf, cur.y / tpdf, cur.z / tpdf);
            acc = acc + cur;
            n_unique += nrec;
        }
        if (live && gl == 0) {
            value[qi] = acc.x;
            value[(size_t)n + qi] = acc.y;
            value[2 * (size_t)n + qi] = acc.z;
            count[qi] = n_unique;
            walks[qi] = work ? M * sc.n_casters_ms : 0;
        }
    }
    flush_stats(st, ctr, err, kPhaseMs);
}

// ------------------------------------------------------ unbiased estimator
// Part 1: one lane per query runs the first walk (its seed path is the
// template) and the contribution; every success is queued for trials
// (:95-110; the contribution tests visibility itself).  kRough: the first walk
// draws the offset normals the trials keep.
template <int K, bool kNM, bool kRough = false>
__global__ void __launch_bounds__(128) ms_first_kernel(DevScene sc, SolverCfg cfg, int ci, const float *__restrict__ qs,
                                                       uint32_t n, uint64_t seed, uint64_t stream_off,
                                                       float *__restrict__ value, int *__restrict__ count,
                                                       int *__restrict__ walks, SsScratch scr, int *__restrict__ tmpl_out,
                                                       DevCounters *ctr) {
    uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    LaneStats st;
    uint32_t err = 0;
    bool enqueue = false;
    if (qi < n) {
        Query Q = load_query(qs, n, qi);
        Pcg32 rng = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
        Light L;
        bool have_light = sample_emitter(sc, sc.emitters_ms, sc.n_emitters_ms, rng, Q.x, L);
        uint32_t pos = 3u;
        f3 acc = splat(0.f);
        int nw = 0;
        if (ci == 0) {
            if (have_light) st.conns++;
        } else {
            pos = scr.pos[qi];
            acc = mk(value[qi], value[(size_t)n + qi], value[2 * (size_t)n + qi]);
            nw = walks[qi];
        }
        if (have_light) {
            int caster = sc.casters_ms[ci];
            rng.advance(pos - 3u);
            float sx = rng.next_f32(), sy = rng.next_f32();
            pos += ms_walk_numbers<K, kRough>();
            f3 x1 = sample_position(sc, sc.shapes[caster], sx, sy);
            Chain<K> c;
            int shapes[K];
            int it = 0;
            f3 own[K];
            float own_pdf = 1.f;
            ChainOffsets<K> co;
            float dr[2 * K];
            if constexpr (kRough) {
                #pragma unroll
                for (int j = 0; j < 2 * K; ++j) dr[j] = rng.next_f32();
                co.draw = dr; co.out = own; co.pdf = &own_pdf;
            }
            bool ok = seed_chain<K, kNM, kRough>(sc, cfg, caster, Q.x, x1, L.p, nullptr, c, shapes, err, st, co) &&
                      chain_newton<K, kNM, kRough>(sc, cfg, Q.x, L.p, shapes, c, it, err, st, kRough ? own : nullptr);
            st.walks++;
            st.newton += (unsigned)it;
            nw++;
            if (ok) {
                st.succ++;
                f3 dir = normalize(c.v[0].p - Q.x);
                f3 spec = chain_contribution<K, kNM, kRough>(sc, Q.x, L, c, err, st);
                f3 val = receiver_eval(sc, Q, dir, err) * spec;
                scr.dir0[qi] = dir.x; scr.dir0[(size_t)n + qi] = dir.y; scr.dir0[2 * (size_t)n + qi] = dir.z;
                scr.val[qi] = val.x; scr.val[(size_t)n + qi] = val.y; scr.val[2 * (size_t)n + qi] = val.z;
                #pragma unroll
                for (int b = 0; b < K; ++b) tmpl_out[(size_t)b * n + qi] = shapes[b];
                if constexpr (kRough) {
                    float *orow = ms_offset_rows(tmpl_out, n);
                    #pragma unroll
                    for (int b = 0; b < K; ++b) {
                        orow[(size_t)(3 * b) * n + qi] = own[b].x;
                        orow[(size_t)(3 * b + 1) * n + qi] = own[b].y;
                        orow[(size_t)(3 * b + 2) * n + qi] = own[b].z;
                    }
                    orow[(size_t)(3 * kMaxBounces) * n + qi] = own_pdf;
                }
                enqueue = true;
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
    unsigned want = __ballot_sync(kFull, enqueue);
    if (want) {
        unsigned lane = threadIdx.x & 31, leader = __ffs(want) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&ctr->trial_count, (unsigned)__popc(want));
        base = __shfl_sync(kFull, base, leader);
        if (enqueue) scr.list[base + __popc(want & ((1u << lane) - 1u))] = qi;
    }
    flush_stats(st, ctr, err, kPhaseMs);
}

// Part 2: Bernoulli trials, 32 per warp step (:111-135); trial walks must
// reproduce the template's shapes (and, kRough, scatter about its offsets).
template <int K, bool kNM, bool kRough = false>
__global__ void __launch_bounds__(128) ms_trials_kernel(DevScene sc, SolverCfg cfg, int ci, const float *__restrict__ qs,
                                                        uint32_t n, uint64_t seed, uint64_t stream_off,
                                                        float *__restrict__ value, int *__restrict__ count,
                                                        int *__restrict__ walks, SsScratch scr,
                                                        const int *__restrict__ tmpl_in, DevCounters *ctr) {
    const unsigned lane = threadIdx.x & 31;
    LaneStats st;
    uint32_t err = 0;
    const int cap = cfg.max_trials > 0 ? cfg.max_trials : kTrialHardLimit;
    const int caster = sc.casters_ms[ci];
    const unsigned n_list = *(volatile unsigned *)&ctr->trial_count;
    while (true) {
        unsigned idx = 0;
        if (lane == 0) idx = atomicAdd(&ctr->trial_head, 1u);
        idx = __shfl_sync(kFull, idx, 0);
        if (idx >= n_list) break;
        uint32_t qi = scr.list[idx];
        Query Q = load_query(qs, n, qi);
        Pcg32 base = query_rng(seed, query_stream(cfg, stream_off, qi), 0);
        Light L;
        sample_emitter(sc, sc.emitters_ms, sc.n_emitters_ms, base, Q.x, L);
        uint32_t pos = scr.pos[qi];
        f3 dir0 = mk(scr.dir0[qi], scr.dir0[(size_t)n + qi], scr.dir0[2 * (size_t)n + qi]);
        int tmpl[K];
        #pragma unroll
        for (int b = 0; b < K; ++b) tmpl[b] = tmpl_in[(size_t)b * n + qi];
        f3 toff[K];
        float tpdf = 1.f;
        #pragma unroll
        for (int b = 0; b < K; ++b) toff[b] = mk(0.f, 0.f, 1.f);
        if constexpr (kRough) {
            const float *orow = ms_offset_rows(const_cast<int *>(tmpl_in), n);
            #pragma unroll
            for (int b = 0; b < K; ++b)
                toff[b] = mk(orow[(size_t)(3 * b) * n + qi], orow[(size_t)(3 * b + 1) * n + qi],
                             orow[(size_t)(3 * b + 2) * n + qi]);
            tpdf = orow[(size_t)(3 * kMaxBounces) * n + qi];
        }
        constexpr uint32_t kRun = ms_walk_numbers<K, kRough>();
        int first = 0;
        for (int t0 = 1; t0 <= cap; t0 += 32) {
            int t = t0 + (int)lane;
            bool succ = false;
            int it = 0;
            if (t <= cap) {
                Pcg32 rng = base;
                rng.advance((uint64_t)(pos - 3u) + kRun * (uint64_t)(t - 1));
                float sx = rng.next_f32(), sy = rng.next_f32();
                f3 x1 = sample_position(sc, sc.shapes[caster], sx, sy);
                Chain<K> c;
                ChainOffsets<K> co;
                co.offs = toff;
                bool ok = seed_chain<K, kNM, kRough>(sc, cfg, caster, Q.x, x1, L.p, tmpl, c, nullptr, err, st, co) &&
                          chain_newton<K, kNM, kRough>(sc, cfg, Q.x, L.p, tmpl, c, it, err, st,
                                                       kRough ? toff : nullptr);
                succ = ok && fabsf(dot(dir0, normalize(c.v[0].p - Q.x)) - 1.f) < cfg.uniqueness_threshold;
            }
            unsigned b = __ballot_sync(kFull, succ);
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
            f3 val = mk(scr.val[qi], scr.val[(size_t)n + qi], scr.val[2 * (size_t)n + qi]);
            f3 cur = val * inv_prob;
            // result += value / m_offset_normals_pdf (:198)
            if (kRough) cur = mk(cur.x / tpdf, cur.y / tpdf, cur.z / tpdf);
            value[qi] += cur.x;
            value[(size_t)n + qi] += cur.y;
            value[2 * (size_t)n + qi] += cur.z;
            count[qi] = first ? iterations : -1;
            walks[qi] += trial_walks;
            scr.pos[qi] = pos + kRun * (uint32_t)trial_walks;
            st.calls++;
            st.iters += (unsigned long long)iterations;
            st.imax = max(st.imax, (unsigned long long)iterations);
        }
    }
    flush_stats(st, ctr, err, kPhaseMs);
}

// ---------------------------------------------------------------- launchers
template <int K, bool kNM>
cudaError_t ms_mnee_check_k(const DevScene &sc, const SolverCfg &cfg, const float *rec, const float *stage,
                            const int *want, float *L, uint32_t n, uint32_t stride, DevCounters *ctr,
                            cudaStream_t s) {
    ms_mnee_check_kernel<K, kNM><<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, rec, stage, want, L, n, stride, ctr);
    return cudaGetLastError();
}

template <int K, bool kNM>
cudaError_t ms_walk_k(const DevScene &sc, const SolverCfg &cfg, int caster, const float *q, const float *w,
                      uint32_t n, float *out, DevCounters *ctr, PhaseTimer *tm, cudaStream_t s) {
    phase_begin(tm, kPhaseMsWalk, s);
    ms_walk_kernel<K, kNM><<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, caster, q, w, n, out, ctr);
    phase_end(tm, s);
    return cudaGetLastError();
}

template <int K, bool kNM, bool kRough = false>
cudaError_t ms_connect_k(const DevScene &sc, const SolverCfg &cfg, const float *q, uint32_t n, uint64_t seed,
                         uint64_t stream_off, float *value, int *count, int *walks, DevCounters *ctr,
                         const SsScratch &scr, int *tmpl, int num_sms, int bps, PhaseTimer *tm, cudaStream_t s) {
    if (cfg.biased) {
        const int G = cfg.max_trials <= 16 ? 16 : 32;
        const uint32_t gpb = 128 / G;
        uint32_t blocks = std::min<uint32_t>((n + gpb - 1) / gpb, (uint32_t)(num_sms * bps));
        phase_begin(tm, kPhaseMs, s);
        auto kernel = G == 16 ? ms_biased_kernel<K, 16, kNM, kRough> : ms_biased_kernel<K, 32, kNM, kRough>;
        kernel<<<blocks, 128, 0, s>>>(sc, cfg, q, n, seed, stream_off, value, count, walks, ctr);
        phase_end(tm, s);
        return cudaGetLastError();
    }
    for (int c = 0; c < sc.n_casters_ms; ++c) {
        cudaError_t e = cudaMemsetAsync(&ctr->trial_count, 0, 2 * sizeof(unsigned), s);
        if (e != cudaSuccess) return e;
        phase_begin(tm, kPhaseMs, s);
        auto first = ms_first_kernel<K, kNM, kRough>;
        auto trials = ms_trials_kernel<K, kNM, kRough>;
        first<<<(n + 127) / 128, 128, 0, s>>>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, scr, tmpl, ctr);
        trials<<<num_sms * bps, 128, 0, s>>>(sc, cfg, c, q, n, seed, stream_off, value, count, walks, scr, tmpl,
                                              ctr);
        phase_end(tm, s);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace sms
