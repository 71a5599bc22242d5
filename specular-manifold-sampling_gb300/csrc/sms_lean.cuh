// sms_lean.cuh -- LEAN mapping and the normal-mapped conductor for the glints
// integrator (device side).
//
// References: the LEAN mip pyramid of src/librender/normalmap.cpp:36-89 and
// its lookups (include/mitsuba/render/normalmap.h:62-104, 199-233), the
// footprint level of NormalmapBSDF::mipmap_level (src/bsdfs/normalmap.cpp:
// 374-388), the LEAN/LEADR distribution of include/mitsuba/render/lean.h
// (after Dupuy's reference implementation), SpecularManifoldGlints::lean_pdf
// (src/librender/manifold_glints.cpp:557-579), NormalmapBSDF::frame / sample
// with a smooth conductor inside (normalmap.cpp:116-139, 236-257).
#pragma once
#include <cuda_fp16.h>

#include "sms_device.cuh"

namespace sms {

// Base variance of the slopes at level 0: 0.5 * alpha^2, alpha = 1e-4
// (normalmap.cpp:36-40).
constexpr float kLeanBaseSigma2 = 0.5f * 0.0001f * 0.0001f;

// Footprint level (a footprint finer than one texel takes level 0).
SMS_D int lean_level(const DevScene &sc, float dxu, float dxv, float dyu, float dyv) {
    const float t = sc.nmap_tiles;
    float w = 2.f * fmaxf(fmaxf(fabsf(t * dxu), fabsf(t * dxv)), fmaxf(fabsf(t * dyu), fabsf(t * dyv)));
    float lv = ceilf((float)(sc.lean_levels - 1) + log2f(fmaxf(w, 1e-8f)));
    if (!(lv > 0.f)) return 0;
    return (int)fminf(lv, (float)(sc.lean_levels - 1));
}

// Bilinear LEAN lookup: mean slope and covariance (a, c; c, b) on level l.
SMS_D void lean_lookup(const DevScene &sc, float u_in, float v_in, int l, float &mx, float &my, float &sa,
                       float &sb, float &scv) {
    const uint32_t res = sc.nmap_res >> l;
    float u = u_in * sc.nmap_tiles, v = v_in * sc.nmap_tiles;
    u -= floorf(u);
    v -= floorf(v);
    float fr = (float)res, duv = 1.f / fr;
    float px = fminf(fmaxf((u - 0.5f * duv) * fr, 0.f), fr - 1.f);
    float py = fminf(fmaxf((v - 0.5f * duv) * fr, 0.f), fr - 1.f);
    uint32_t x0 = (uint32_t)floorf(px), y0 = (uint32_t)floorf(py);
    uint32_t x1 = min(x0 + 1, res - 1), y1 = min(y0 + 1, res - 1);
    x0 = min(x0, res - 1);
    y0 = min(y0, res - 1);
    float wx = px - (float)x0, wy = py - (float)y0;
    const float *d = sc.lean + sc.lean_off[l];
    float vv[5];
    #pragma unroll
    for (int c = 0; c < 5; ++c) {
        float v00 = __ldg(d + 5 * ((size_t)y0 * res + x0) + c), v10 = __ldg(d + 5 * ((size_t)y0 * res + x1) + c);
        float v01 = __ldg(d + 5 * ((size_t)y1 * res + x0) + c), v11 = __ldg(d + 5 * ((size_t)y1 * res + x1) + c);
        float a = (1.f - wx) * v00 + wx * v10, b = (1.f - wx) * v01 + wx * v11;
        vv[c] = (1.f - wy) * a + wy * b;
    }
    mx = vv[0];
    my = vv[1];
    sa = fmaxf(0.f, vv[2] - vv[0] * vv[0]);
    sb = fmaxf(0.f, vv[3] - vv[1] * vv[1]);
    scv = fmaxf(0.f, vv[4] - vv[0] * vv[1]);
}

struct LeanP {
    f3 n;
    float ax, ay, rho, srho, tx, ty;
};

SMS_D LeanP lean_params(float mx, float my, float sa, float sb, float scv, float alpha) {
    float lax = sqrtf(2.f * sa), lay = sqrtf(2.f * sb);
    float rho = 2.f * scv / (lax * lay);
    float e3 = 0.5f * lax * lax + mx * mx + 0.5f * alpha * alpha;
    float e4 = 0.5f * lay * lay + my * my + 0.5f * alpha * alpha;
    float e5 = 0.5f * rho * lax * lay + mx * my;
    LeanP p;
    p.tx = mx;
    p.ty = my;
    p.ax = sqrtf(2.f * fmaxf(0.f, e3 - mx * mx));
    p.ay = sqrtf(2.f * fmaxf(0.f, e4 - my * my));
    p.rho = 2.f * (e5 - mx * my) / (p.ax * p.ay);
    p.srho = sqrtf(1.f - p.rho * p.rho);
    p.n = normalize(mk(-p.tx, -p.ty, 1.f));
    return p;
}

SMS_D float lean_sigma_std(float ct) {
    if (ct == 1.f) return 1.f;
    float st = sqrtf(1.f - ct * ct), nu = ct / st;
    float tmp = expf(-nu * nu) * 0.56418958354775628695f;   // 1 / sqrt(pi)
    return 0.5f * (ct * (1.f + erff(nu)) + st * tmp);
}

SMS_D float lean_sigma(f3 k, const LeanP &p) {
    float a = k.x * p.ax + k.y * p.ay * p.rho, b = k.y * p.ay * p.srho, c = k.z - k.x * p.tx - k.y * p.ty;
    float nrm = sqrtf(a * a + b * b + c * c);
    return nrm * lean_sigma_std(c / nrm);
}

SMS_D float lean_g1(f3 k, const LeanP &p) { return dot(k, p.n) > 0.f ? k.z / lean_sigma(k, p) : 0.f; }

SMS_D float lean_ndf(f3 h, const LeanP &p) {
    if (!(h.z > 5.9604644775390625e-08f)) return 0.f;
    float t1 = h.z * h.z, t2 = t1 * t1;
    float sx = -h.x / h.z - p.tx, sy = -h.y / h.z - p.ty;
    float nrm = p.ax * p.ay * p.srho;
    float x = sx / p.ax, y = (p.ax * sy - p.rho * p.ay * sx) / (p.ax * p.ay * p.srho);
    return kInvPi * expf(-(x * x + y * y)) / nrm / t2;
}

// LEAN density of reflecting wi into wo over the footprint at uv.
SMS_D float glint_lean_pdf(const DevScene &sc, float u, float v, float dxu, float dxv, float dyu, float dyv, f3 wi,
                           f3 wo) {
    if (wi.z < 0.f || wo.z < 0.f) return 0.f;
    float mx, my, sa, sb, scv;
    lean_lookup(sc, u, v, lean_level(sc, dxu, dxv, dyu, dyv), mx, my, sa, sb, scv);
    LeanP p = lean_params(mx, my, sa, sb, scv, 0.f);
    f3 h = normalize(wo + wi);
    float G = lean_g1(wo, p) * lean_g1(wi, p);
    if (!(G > 0.f)) return 0.f;
    float dp = dot(wi, h);
    float vndf = dp > 0.f ? dp * lean_ndf(h, p) / lean_sigma(wi, p) : 0.f;
    return vndf / (4.f * dot(wi, h));
}

// ------------------------------------------------------- LEAN fallback BSDF
// NormalmapBSDF with lean_fallback (src/bsdfs/normalmap.cpp:46-55, 80-112,
// 142-170, 187-203): where the interaction has no uv partials -- every path
// vertex after the camera's first hit -- the normal-mapped surface reflects
// like the glossy LEAN/LEADR distribution of the map's top pyramid level (the
// whole map's mean slope and covariance), widened by the base roughness
// lean_fallback_alpha, times the Fresnel factor of (eta, k).  The visible-
// slope sampling is LEAN::sample_vndf (include/mitsuba/render/lean.h): the
// standard distribution's visible slopes by a Newton/bisection inversion of
// their CDF in the erf domain (qf2) and an erfinv (qf1), then the Cholesky
// map to the surface's slope distribution.

constexpr float kInvSqrtPi = 0.56418958354775628695f;

SMS_D float lean_qf2(float u, float ct, float st) {
    const float cot = ct / st, tan_t = st / ct;
    float a = -1.f, c = erff(cot);
    u = fmaxf(u, 1e-6f);
    // initial guess, then at most 9 Newton steps kept inside [a, c]
    const float fit = 1.f + ct * (-0.876f + ct * (0.4265f - 0.0594f * ct));
    float b = c - (1.f + c) * powf(1.f - u, fit);
    const float norm_cdf = 1.f / (1.f + c + kInvSqrtPi * tan_t * expf(-cot * cot));
    int it = 0;
    while (++it < 10) {
        if (!(b >= a && b <= c)) b = 0.5f * (a + c);
        const float ie = erfinvf(b);
        const float value = norm_cdf * (1.f + b + kInvSqrtPi * tan_t * expf(-ie * ie)) - u;
        const float deriv = norm_cdf * (1.f - ie * tan_t);
        if (fabsf(value) < 1e-5f) break;
        if (value > 0.f) c = b;
        else a = b;
        b -= value / deriv;
    }
    return erfinvf(fmaxf(-0.9999f, b));
}

// A visible slope of the standard distribution for direction wi (z up).
SMS_D float2 lean_sample_vp22_std(f3 wi, float u0, float u1) {
    const float ct = wi.z;
    const float st = ct < 1.f ? sqrtf(1.f - ct * ct) : 0.f;
    const float tx = lean_qf2(u0, ct, st);
    const float ty = erfinvf(2.f * u1 - 1.f);
    if (st == 0.f) return make_float2(tx, ty);
    const float nrm = 1.f / sqrtf(wi.x * wi.x + wi.y * wi.y);
    const float cp = wi.x * nrm, sp = wi.y * nrm;
    return make_float2(cp * tx - sp * ty, sp * tx + cp * ty);
}

// A visible microfacet normal of the LEAN distribution p for wi.
SMS_D f3 lean_sample_vndf(f3 wi, float u0, float u1, const LeanP &p) {
    const float a = wi.x * p.ax + wi.y * p.ay * p.rho, b = wi.y * p.ay * p.srho;
    const float c = wi.z - wi.x * p.tx - wi.y * p.ty;
    const f3 ws = normalize(mk(a, b, c));
    if (!(ws.z > 0.f)) return mk(0.f, 0.f, 1.f);
    const float2 t = lean_sample_vp22_std(ws, u0, u1);
    const float txh = p.ax * t.x + p.tx;
    const float chol = p.rho * t.x + p.srho * t.y;
    const float tyh = p.ay * chol + p.ty;
    return normalize(mk(-txh, -tyh, 1.f));
}

SMS_D float lean_vndf(f3 h, f3 wi, const LeanP &p) {
    const float dp = dot(wi, h);
    return dp > 0.f ? dp * lean_ndf(h, p) / lean_sigma(wi, p) : 0.f;
}

// LEAN::gaf as the reference computes it: the product of the two G1 (its
// height-correlated form is unreachable code there).
SMS_D float lean_gaf(f3 a, f3 b, const LeanP &p) {
    const float g = lean_g1(a, p) * lean_g1(b, p);
    return g > 0.f ? g : 0.f;
}

// The fallback's distribution: the top pyramid level and the base roughness.
SMS_D LeanP lean_fb_params(const DevScene &sc) {
    float mx, my, sa, sb, scv;
    lean_lookup(sc, 0.f, 0.f, sc.lean_levels - 1, mx, my, sa, sb, scv);
    return lean_params(mx, my, sa, sb, scv, sc.lf_alpha);
}

SMS_D float lean_fb_fresnel(const DevScene &sc, float c) {
    return sc.lf_k == 0.f ? fresnel_dielectric(c, sc.lf_eta) : fresnel_conductor(c, sc.lf_eta, sc.lf_k);
}

// NormalmapBSDF::sample, lean_fallback branch (normalmap.cpp:80-112), local
// shading frame: reflected direction, weight F G / G1 and the density.
SMS_D bool lean_fb_sample(const DevScene &sc, f3 wi, float u0, float u1, f3 &wo, float &weight, float &pdf) {
    if (!(wi.z > 0.f)) return false;
    const LeanP p = lean_fb_params(sc);
    const f3 m = lean_sample_vndf(wi, u0, u1, p);
    const float dm = dot(wi, m);
    wo = m * (2.f * dm) - wi;
    const float G = lean_gaf(wo, wi, p);   // LEAN::gaf(m, wo, wi): G1 ignores m
    if (!(G > 0.f && wo.z > 0.f)) return false;
    const float F = lean_fb_fresnel(sc, dm);
    pdf = lean_vndf(m, wi, p) / (4.f * dm);
    weight = F * G / lean_g1(wi, p);
    return true;
}

// NormalmapBSDF::eval, lean_fallback branch (normalmap.cpp:142-170).
SMS_D float lean_fb_eval(const DevScene &sc, f3 wi, f3 wo) {
    if (!(wi.z > 0.f && wo.z > 0.f)) return 0.f;
    const LeanP p = lean_fb_params(sc);
    const f3 h = normalize(wo + wi);
    return lean_fb_fresnel(sc, dot(wi, h)) * lean_ndf(h, p) * lean_gaf(wi, wo, p) / (4.f * wi.z);
}

// NormalmapBSDF::pdf, lean_fallback branch (normalmap.cpp:187-203): the
// reference returns the density wherever G > 0, whatever the cosines.
SMS_D float lean_fb_pdf(const DevScene &sc, f3 wi, f3 wo) {
    const LeanP p = lean_fb_params(sc);
    const f3 h = normalize(wo + wi);
    return lean_gaf(wo, wi, p) > 0.f ? lean_vndf(h, wi, p) / (4.f * dot(wi, h)) : 0.f;
}

// Normal-mapped smooth conductor: reflection about the bilinear slope normal
// of level 0 at uv; world-space directions; weight = Fresnel.
SMS_D bool nm_conductor_sample(const DevScene &sc, const DevShape &s, f3 n, f3 dp_du, float u, float v, f3 wi_w,
                               f3 &wo_w, float &weight) {
    f3 bs = normalize(dp_du - n * dot(n, dp_du)), bt = cross(n, bs);
    float2 sl = nm_slope0(sc, u, v);
    f3 pn = normalize(bs * -sl.x + bt * -sl.y + n);
    float ci = dot(wi_w, pn);
    if (!(ci > 0.f)) return false;
    wo_w = pn * (2.f * ci) - wi_w;
    if (!(dot(wo_w, n) * dot(wo_w, pn) > 0.f)) return false;
    weight = fresnel_conductor(ci, s.eta, s.k);
    return true;
}

}  // namespace sms
