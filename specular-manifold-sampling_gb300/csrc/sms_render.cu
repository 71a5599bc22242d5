// sms_render.cu -- wavefront path tracer around the SMS solvers (sm_103a).
//
// The reference's integrators (src/integrators/path.cpp, path_sms_ss.cpp,
// path_sms_ms.cpp) trace one camera path per host thread and call the SMS
// solver inline at every caustic receiver.  Here a wavefront of up to 2^20
// paths advances one bounce per launch:
//
//   pt_camera_kernel   camera ray, first intersection, directly seen emitters
//   pt_bounce_kernel   one bounce of every live path: Russian roulette, the SMS
//                      query of a receiver vertex (staged, not solved), emitter
//                      sampling with MIS, BSDF sampling, the next intersection
//                      and the emitter it hits (filtered like the reference,
//                      with the unbiased-MNEE check walk of path_sms_ss)
//   pt_scan_kernel     ordered prefix sum of the per-block query counts
//   pt_gather_kernel   appends the staged queries of this bounce to the
//                      wavefront's pending SMS batch, in path order, each
//                      with its random-number stream (path, bounce)
//   pt_pack_kernel     the pending batch as one SoA query array
//   (SMS estimator)    the context's single- or multi-scatter connection
//                      kernels on the whole pending batch: the queries of all
//                      bounces of a wavefront are solved by one call, so the
//                      trial kernel's tail is paid once, not once per bounce
//   pt_sms_add_kernel  adds throughput x SMS estimate to each path's radiance,
//                      one launch per bounce in bounce order
//   pt_resolve_kernel  sums the samples of each pixel in sample order
//
// One host read per bounce (query and live-path counts) drives the loop.
// Every sum runs in a fixed order, so images are bit-reproducible, and since
// all random numbers are keyed by path and bounce they do not depend on the
// wavefront size.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sms_gb300.h"
#include "sms_device.cuh"
#include "sms_estimator.cuh"
#include "sms_kernels.h"
#include "sms_lean.cuh"

namespace sms {
namespace {

constexpr int kPtBlock = 256;
constexpr uint32_t kPtDefaultPaths = 1u << 20;
constexpr int kPtHardDepth = 4096;        // bounce limit of an unbounded path
constexpr int kQueryRowsMax = 21;        // glint queries; single / multi scatter use 16
constexpr int kStageRows = 24;            // query rows, then 3 throughput rows at 21..23

// path flags; bits 3-4 and 5-7 hold the multi-bounce filter's path record
// (path_filtered_ms.cpp:219-301): its state and chain bounce count
constexpr int kAlive = 1, kPrevReceiver = 2, kSpecularCamera = 4;
constexpr int kRecShift = 3, kRecBounceShift = 5;
constexpr int kRecDefault = 0, kRecReceiver = 1, kRecCaster = 2, kRecEmitter = 3;
// path_filtered_teaser's path record (path_filtered_teaser.cpp:36-43,
// 334-410): its state in bits 8-10, its chain bounce count in bits 5-7
constexpr int kTfShift = 8;
constexpr int kTfDefault = 0, kTfReceiver = 1, kTfSingleCaster = 2, kTfSingleEmitter = 3, kTfMultiCaster = 4,
              kTfMultiEmitter = 5;
// rows of the MNEE record: receiver point (3), first specular shape (int
// bits), specular vertices (3 per bounce)
constexpr int kMneeRows = 4 + 3 * kMaxBounces;

struct PtCam {
    float m[12];          // rows 0..2 of camera-to-world
    float tx, ty;         // tan of the half field of view along x and y
    float near_clip, far_clip;
    int width, height;
};

struct PtParams {
    int integrator;       // SMS_INTEGRATOR_*
    int max_depth, rr_depth;
    int disable_reflected_emitters, biased_mnee;
    int bounces;          // SMS chain length (path_sms_ms)
    int mnee_check;       // path_sms_ss with mnee_init and !biased_mnee
    int mnee_ms;          // path_sms_ms with mnee_init and !biased_mnee
    uint64_t seed;
    SolverCfg solver;     // for the MNEE check walk
    float diff_scale;     // ray-differential scale (glints)
    int bsdf_strategy_only, sms_strategy_only;
    // path_sms_teaser: the pass being rendered (0 single-scatter caustics and
    // the paths SMS does not handle, 1 multi-scatter caustics, 2 glints) and
    // its switches
    int teaser_pass;
    int caustics_enabled, glints_enabled, non_sms_paths;
};

struct PtState {
    uint64_t *rng_state, *rng_inc;
    float *o, *d, *thr, *L, *prev_p;      // 3 x cap
    float *eta, *hit_t, *hit_u, *hit_v;   // cap
    float *cam_s;                         // 2 x cap: the camera sample position
    int *hit_shape, *flags;               // cap
    uint32_t *hit_prim;                   // cap
    float *stage;                         // kStageRows x cap
    int *want;                            // cap
    // path_sms_ms unbiased MNEE (MNEEHelper, path_sms_ms.cpp:54-142): per
    // path the receiver point, the first specular shape and the specular
    // vertices since (kMneeRows x cap; null when off), and the paths whose
    // emitter hit awaits the MNEE test of this bounce
    float *mnee;
    int *mnee_want;
    uint32_t *block_q, *block_a;          // per block
    uint32_t *totals;                     // [0] queries, [1] live paths
    // pending SMS batch (qcap entries, appended bounce by bounce)
    int qrows;                            // query rows: 16, or 21 for glints
    float *qraw;                          // qrows x qcap, stride qcap
    float *qw;                            // 3 x qcap: path throughput
    uint32_t *qmap;                       // qcap: query -> path
    uint64_t *qstream;                    // qcap: random-number stream
    float *q;                             // qrows x nq packed (stride nq)
    float *value;                         // 3 x nq
    int *count, *walks;                   // nq
    uint32_t cap, qcap;
};

SMS_D f3 ld3s(const float *a, uint32_t cap, uint32_t i) { return mk(a[i], a[cap + i], a[2 * (size_t)cap + i]); }
SMS_D void st3s(float *a, uint32_t cap, uint32_t i, f3 v) {
    a[i] = v.x; a[cap + i] = v.y; a[2 * (size_t)cap + i] = v.z;
}
SMS_D float hmax3(f3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
SMS_D float max_abs(f3 v) { return fmaxf(fabsf(v.x), fmaxf(fabsf(v.y), fabsf(v.z))); }

// Power heuristic (path.cpp:227-231).
SMS_D float mis_weight(float a, float b) {
    a *= a;
    b *= b;
    return a > 0.f ? a / (a + b) : 0.f;
}

// Surface data of a closest hit: position, geometric and shading normals,
// position partials (sphere.cpp:322-373, mesh.cpp:618-687).
SMS_D void surface_at(const DevScene &sc, f3 o, f3 d, float t, int shape, uint32_t prim, float u, float v,
                      SurfPt &si) {
    const DevShape &s = sc.shapes[shape];
    if (s.kind == kShapeSphere) {
        sphere_surface(s, o, d, t, si);
    } else {
        MeshTri m;
        load_tri(sc, s, prim, m);
        mesh_surface(m, s.has_normals, u, v, si);
    }
}

// Shading frame: normal n, tangent from dp_du (the reference's surface
// interaction frame, kdtree.h:2334-2366), Duff et al. basis when dp_du is
// degenerate or parallel to n.
SMS_D void shading_frame(const SurfPt &si, f3 &s, f3 &t) {
    f3 n = si.shn;
    f3 a = si.dp_du - n * dot(n, si.dp_du);
    float l2 = dot(a, a);
    if (l2 > 1e-20f) {
        s = a * (1.f / sqrtf(l2));
        t = cross(n, s);
    } else {
        onb(n, s, t);
    }
}

// Emitted radiance of an area emitter seen along direction d from its front
// side (area.cpp: eval, cos_theta(wi) > 0).  Only spheres carry emitters.
SMS_D f3 emitted(const DevScene &sc, const DevShape &s, f3 p, f3 d) {
    if (s.emitter < 0) return splat(0.f);
    f3 n = normalize(p - mk(s.cx, s.cy, s.cz));
    if (s.flip) n = -n;
    if (!(dot(n, -d) > 0.f)) return splat(0.f);
    const DevEmitter &e = sc.emitters[s.emitter];
    return mk(e.r, e.g, e.b);
}

// Sphere::pdf_direction (sphere.cpp) x the emitter pick (scene.cpp:206-220):
// density of emitter sampling from x for the emitter point p (normal n).
SMS_D float emitter_pdf(const DevScene &sc, const DevShape &s, f3 x, f3 p, f3 d, float dist) {
    f3 n = normalize(p - mk(s.cx, s.cy, s.cz));
    if (s.flip) n = -n;
    if (!(dot(d, n) < 0.f)) return 0.f;
    f3 c = mk(s.cx, s.cy, s.cz);
    float sin_a = s.radius / length(c - x);
    float cos_a = safe_sqrt(1.f - sin_a * sin_a);
    float pdf;
    if (sin_a < 1.f - 5.9604644775390625e-08f)
        pdf = (0.5f * kInvPi) / (1.f - cos_a);
    else
        pdf = (1.f / (4.f * kPi * s.radius * s.radius)) * dist * dist / fabsf(dot(d, n));
    return sc.n_emitters_all > 1 ? pdf * (1.f / (float)sc.n_emitters_all) : pdf;
}

struct DirSample {
    f3 d, spec;
    float dist, pdf;
    bool delta;
};

// Scene::sample_emitter_direction over an emitter list (scene.cpp:156-196;
// all emitters, or a caustic list as path_filtered_teaser.cpp:331-378 picks
// them): point.cpp sample_direction; area.cpp + Sphere::sample_direction
// (cone sampling from outside, uniform sphere from inside).  Visibility is
// tested by the caller.
SMS_D bool sample_emitter_direction_from(const DevScene &sc, const int *list, int ne, f3 x, float ux, float uy,
                                         DirSample &ds) {
    if (ne == 0) return false;
    int idx = 0;
    if (ne > 1) {
        const float epdf = 1.f / (float)ne;
        idx = (int)min((uint32_t)(ux * (float)ne), (uint32_t)ne - 1);
        ux = (ux - (float)idx * epdf) * (float)ne;
    }
    const DevEmitter &e = sc.emitters[list[idx]];
    if (e.kind == 0) {
        f3 d = mk(e.px, e.py, e.pz) - x;
        ds.dist = length(d);
        float inv = 1.f / ds.dist;
        ds.d = d * inv;
        ds.pdf = 1.f;
        ds.delta = true;
        ds.spec = mk(e.r, e.g, e.b) * (inv * inv);
    } else {
        const DevShape &s = sc.shapes[e.shape];
        f3 c = mk(s.cx, s.cy, s.cz);
        f3 dc = c - x;
        float dc2 = dot(dc, dc);
        float r_adj = s.radius * (s.flip ? (1.f + kRayEps) : (1.f - kRayEps));
        f3 p, n;
        if (dc2 > r_adj * r_adj) {
            float inv_dc = 1.f / sqrtf(dc2);
            float sin_max = s.radius * inv_dc, sin2_max = sin_max * sin_max, inv_sin_max = 1.f / sin_max;
            float cos_max = safe_sqrt(1.f - sin2_max);
            // small cones: first-order expansion of 1 - cos^2 (1.5 degrees)
            float a = (cos_max - 1.f) * ux + 1.f;
            float sin2 = sin2_max > 0.00068523f ? 1.f - a * a : sin2_max * ux;
            float cos_t = safe_sqrt(1.f - sin2);
            // point on the visible cap (Akalin, "Sampling the visible sphere")
            float cos_al = sin2 * inv_sin_max + cos_t * safe_sqrt(1.f - sin2 * inv_sin_max * inv_sin_max);
            float sin_al = safe_sqrt(1.f - cos_al * cos_al);
            float sp, cp;
            sincosf(uy * (2.f * kPi), &sp, &cp);
            f3 fz = dc * -inv_dc, fs, ft;
            onb(fz, fs, ft);
            f3 dl = fs * (cp * sin_al) + ft * (sp * sin_al) + fz * cos_al;
            p = dl * s.radius + c;
            n = dl;
            f3 dv = p - x;
            ds.dist = length(dv);
            ds.d = dv * (1.f / ds.dist);
            ds.pdf = ds.dist == 0.f ? 0.f : (0.5f * kInvPi) / (1.f - cos_max);
        } else {
            float z = 1.f - 2.f * uy;
            float r = safe_sqrt(1.f - z * z);
            float sp, cp;
            sincosf(2.f * kPi * ux, &sp, &cp);
            f3 dl = mk(r * cp, r * sp, z);
            p = dl * s.radius + c;
            n = dl;
            f3 dv = p - x;
            float dist2 = dot(dv, dv);
            ds.dist = sqrtf(dist2);
            ds.d = dv * (1.f / ds.dist);
            ds.pdf = (1.f / (4.f * kPi * s.radius * s.radius)) * dist2 / fabsf(dot(ds.d, n));
        }
        if (s.flip) n = -n;
        ds.delta = false;
        if (!(dot(ds.d, n) < 0.f && ds.pdf != 0.f)) return false;
        ds.spec = mk(e.r, e.g, e.b) * (1.f / ds.pdf);
    }
    if (ne > 1) {
        ds.pdf *= 1.f / (float)ne;
        ds.spec = ds.spec * (float)ne;
    }
    return ds.pdf != 0.f;
}

SMS_D bool sample_emitter_direction(const DevScene &sc, f3 x, float ux, float uy, DirSample &ds) {
    return sample_emitter_direction_from(sc, sc.emitters_all, sc.n_emitters_all, x, ux, uy, ds);
}

// Fresnel equations for a dielectric (fresnel.h:34-80): reflectance, signed
// cosine of the transmitted direction and the two relative indices.
SMS_D float fresnel_full(float cos_i, float eta, float &cos_t, float &eta_it, float &eta_ti) {
    bool outside = cos_i >= 0.f;
    float rcp_eta = 1.f / eta;
    eta_it = outside ? eta : rcp_eta;
    eta_ti = outside ? rcp_eta : eta;
    float ct2 = 1.f - (1.f - cos_i * cos_i) * (eta_ti * eta_ti);
    float ci = fabsf(cos_i), ct = safe_sqrt(ct2);
    float a_s = (ci - eta_it * ct) / (ci + eta_it * ct);
    float a_p = (ct - eta_it * ci) / (ct + eta_it * ci);
    float r = 0.5f * (a_s * a_s + a_p * a_p);
    if (eta == 1.f) r = 0.f;
    else if (ci == 0.f) r = 1.f;
    cos_t = cos_i >= 0.f ? -ct : ct;
    return r;
}

// Concentric square-to-disk map (Shirley and Chiu 1997, in the branch-free
// form of warp.h:54-90) lifted to the cosine-weighted hemisphere.
SMS_D f3 cosine_hemisphere(float u1, float u2) {
    float x = 2.f * u1 - 1.f, y = 2.f * u2 - 1.f;
    float r, phi;
    if (x == 0.f && y == 0.f) {
        r = 0.f; phi = 0.f;
    } else if (fabsf(x) < fabsf(y)) {
        r = y; phi = 0.5f * kPi - (x / y) * (0.25f * kPi);
    } else {
        r = x; phi = (y / x) * (0.25f * kPi);
    }
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float px = r * cp, py = r * sp;
    return mk(px, py, safe_sqrt(1.f - px * px - py * py));
}

struct BsdfSample {
    f3 wo, weight;
    float pdf, eta;
    bool delta;
    bool transmit;   // BSDFFlags::Transmission of the sampled lobe
};

// Density of rough_sample below for the pair (wi, wo): microfacet normal m of
// the pair, D(m) cos(theta_m) times the Jacobian of the reflection or
// refraction (the densities of roughconductor.cpp / roughdielectric.cpp pdf
// with normals drawn from D cos instead of the visible normals).
SMS_D float rough_pdf(const DevShape &s, f3 wi, f3 wo) {
    const float ci = wi.z, co = wo.z;
    if (s.bsdf_type == kBsdfConductor) {
        if (!(ci > 0.f && co > 0.f)) return 0.f;
        f3 h = normalize(wo + wi);
        return beckmann_D(h, s.alpha) * h.z / (4.f * dot(wo, h));
    }
    if (ci == 0.f) return 0.f;
    const bool reflect = ci * co > 0.f;
    const float eta = ci > 0.f ? s.eta : 1.f / s.eta;
    f3 m = normalize(wi + wo * (reflect ? 1.f : eta));
    if (m.z < 0.f) m = -m;
    if (dot(wi, m) * ci <= 0.f || dot(wo, m) * co <= 0.f) return 0.f;
    const float F = fresnel_dielectric(dot(wi, m), s.eta);
    const float pm = beckmann_D(m, s.alpha) * m.z;
    if (reflect) return F * pm / (4.f * fabsf(dot(wo, m)));
    const float den = dot(wi, m) + eta * dot(wo, m);
    return (1.f - F) * pm * eta * eta * fabsf(dot(wo, m)) / (den * den);
}

// ------------------------------------------------------------ roughplastic
// roughplastic_eval, its transmittance table and bsdf_eval are shared with the
// estimators' receiver evaluation (sms_estimator.cuh).
// the probability of sampling the coating's specular lobe at cos theta_i
SMS_D float rp_prob_specular(const DevShape &s, float ci) {
    const float t_i = rp_transmittance(s, ci);
    const float ps = (1.f - t_i) * s.rp_ws, pd = t_i * (1.f - s.rp_ws);
    return ps / (ps + pd);
}

SMS_D float roughplastic_pdf(const DevShape &s, f3 wi, f3 wo) {
    const float ci = wi.z, co = wo.z;
    if (!(ci > 0.f && co > 0.f)) return 0.f;
    const float ps = rp_prob_specular(s, ci);
    const f3 h = normalize(wo + wi);
    return beckmann_D(h, s.alpha) * h.z / (4.f * dot(wo, h)) * ps + (1.f - ps) * kInvPi * co;
}

SMS_D float bsdf_pdf(const DevShape &s, f3 wi, f3 wo) {
    if (s.bsdf_type == kBsdfRoughPlastic) return roughplastic_pdf(s, wi, wo);
    if (s.bsdf_type == kBsdfDiffuse) return (wi.z > 0.f && wo.z > 0.f) ? kInvPi * wo.z : 0.f;
    return s.alpha > 0.f ? rough_pdf(s, wi, wo) : 0.f;
}

// Rough conductor / dielectric sampling: microfacet normal m with density
// D(m) cos(theta_m) (microfacet.h, sample_visible = false), then reflection
// about m, or for a dielectric reflection / refraction chosen by the Fresnel
// reflectance at m (roughdielectric.cpp sample); weight = value / density.
SMS_D bool rough_sample(const DevShape &s, f3 wi, float u1, float u2, float u3, BsdfSample &bs) {
    const float ci = wi.z;
    float pm;
    const f3 m = beckmann_sample(s.alpha, u2, u3, pm);
    bs.delta = false;
    bs.eta = 1.f;
    if (s.bsdf_type == kBsdfConductor) {
        if (!(ci > 0.f)) return false;
        bs.wo = m * (2.f * dot(wi, m)) - wi;
        if (!(bs.wo.z > 0.f)) return false;
    } else {
        float cos_t, eta_it, eta_ti;
        const float F = fresnel_full(dot(wi, m), s.eta, cos_t, eta_it, eta_ti);
        if (u1 <= F) {
            bs.wo = m * (2.f * dot(wi, m)) - wi;
            if (!(bs.wo.z * ci > 0.f)) return false;
        } else {
            bs.wo = m * (dot(wi, m) * eta_ti + cos_t) - wi * eta_ti;
            if (!(bs.wo.z * ci < 0.f)) return false;
            bs.eta = eta_it;
        }
    }
    bs.pdf = rough_pdf(s, wi, bs.wo);
    if (!(bs.pdf > 0.f)) return false;
    bs.weight = bsdf_eval(s, wi, bs.wo) * (1.f / bs.pdf);
    return true;
}

// BSDF::sample of diffuse.cpp, dielectric.cpp, conductor.cpp (smooth) and the
// rough variants above, radiance transport, local frame.  Returns false for a
// zero weight.
SMS_D bool bsdf_sample(const DevShape &s, f3 wi, float u1, float u2, float u3, BsdfSample &bs) {
    const float ci = wi.z;
    if (s.bsdf_type == kBsdfRoughPlastic) {
        // roughplastic.cpp:185-241: the coating's lobe or the base's cosine lobe
        if (!(ci > 0.f)) return false;
        if (u1 < rp_prob_specular(s, ci)) {
            float pm;
            const f3 m = beckmann_sample(s.alpha, u2, u3, pm);
            bs.wo = m * (2.f * dot(wi, m)) - wi;
        } else {
            bs.wo = cosine_hemisphere(u2, u3);
        }
        bs.delta = false;
        bs.eta = 1.f;
        bs.pdf = roughplastic_pdf(s, wi, bs.wo);
        if (!(bs.pdf > 0.f)) return false;
        bs.weight = roughplastic_eval(s, wi, bs.wo) * (1.f / bs.pdf);
        return true;
    }
    if (s.bsdf_type != kBsdfDiffuse && s.alpha > 0.f) return rough_sample(s, wi, u1, u2, u3, bs);
    if (s.bsdf_type == kBsdfDiffuse) {
        if (!(ci > 0.f)) return false;
        bs.wo = cosine_hemisphere(u2, u3);
        bs.pdf = kInvPi * bs.wo.z;
        bs.eta = 1.f;
        bs.delta = false;
        bs.weight = mk(s.albedo[0], s.albedo[1], s.albedo[2]);
        return bs.pdf > 0.f;
    }
    if (s.bsdf_type == kBsdfDielectric) {
        float cos_t, eta_it, eta_ti;
        float r = fresnel_full(ci, s.eta, cos_t, eta_it, eta_ti);
        bs.delta = true;
        if (u1 <= r) {
            bs.wo = mk(-wi.x, -wi.y, wi.z);
            bs.pdf = r;
            bs.eta = 1.f;
            bs.weight = splat(1.f);
        } else {
            bs.wo = mk(-eta_ti * wi.x, -eta_ti * wi.y, cos_t);
            bs.pdf = 1.f - r;
            bs.eta = eta_it;
            bs.weight = splat(eta_ti * eta_ti);
        }
        return true;
    }
    // conductor
    if (!(ci > 0.f)) return false;
    bs.wo = mk(-wi.x, -wi.y, wi.z);
    bs.pdf = 1.f;
    bs.eta = 1.f;
    bs.delta = true;
    bs.weight = splat(fresnel_conductor(ci, s.eta, s.k));
    return true;
}

// NormalmapBSDF::sample (normalmap.cpp:118-135) around any smooth nested BSDF:
// sampled in the frame of the level-0 slope normal at uv, the direction taken
// back to the shading frame (fs, ft, n) and kept when it lies on the same side
// of both frames' normals.
SMS_D bool nm_bsdf_sample(const DevScene &sc, const DevShape &s, f3 fs, f3 ft, f3 n, f3 dp_du, float u, float v,
                          f3 wi_w, float u1, float u2, float u3, BsdfSample &bs) {
    const f3 bs0 = normalize(dp_du - n * dot(n, dp_du)), bt0 = cross(n, bs0);
    const float2 sl = nm_slope0(sc, u, v);
    const f3 pn = normalize(bs0 * -sl.x + bt0 * -sl.y + n);
    const f3 ps = normalize(dp_du - pn * dot(pn, dp_du)), pt = cross(pn, ps);
    const f3 wi = mk(dot(wi_w, ps), dot(wi_w, pt), dot(wi_w, pn));
    if (!bsdf_sample(s, wi, u1, u2, u3, bs)) return false;
    bs.transmit = bs.wo.z * wi.z < 0.f;
    const f3 wo_w = ps * bs.wo.x + pt * bs.wo.y + pn * bs.wo.z;
    const f3 wo = mk(dot(wo_w, fs), dot(wo_w, ft), dot(wo_w, n));
    if (!(bs.wo.z * wo.z > 0.f)) return false;
    bs.wo = wo;
    return true;
}

// Caustic single-scatter flag of emitter e (used by the MNEE check).
SMS_D bool emitter_is_caustic_ss(const DevScene &sc, int e) {
    for (int k = 0; k < sc.n_emitters_ss; ++k)
        if (sc.emitters_ss[k] == e) return true;
    return false;
}

SMS_D bool emitter_is_caustic_ms(const DevScene &sc, int e) {
    for (int k = 0; k < sc.n_emitters_ms; ++k)
        if (sc.emitters_ms[k] == e) return true;
    return false;
}

SMS_D Pcg32 load_rng(const PtState &S, uint32_t i) {
    Pcg32 r;
    r.state = S.rng_state[i];
    r.inc = S.rng_inc[i];
    return r;
}
SMS_D void store_rng(const PtState &S, uint32_t i, const Pcg32 &r) {
    S.rng_state[i] = r.state;
    S.rng_inc[i] = r.inc;
}

// ------------------------------------------------------------------ camera
// Perspective sensor (perspective.cpp sample_ray) through a box-filtered pixel
// sample; first intersection and directly visible emitters.
__global__ void __launch_bounds__(kPtBlock) pt_camera_kernel(DevScene sc, PtCam cam, PtState S, uint64_t base,
                                                             uint32_t n, uint64_t seed, int add_emitted) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t g = base + i;
    const uint64_t wh = (uint64_t)cam.width * (uint64_t)cam.height;
    const uint32_t pix = (uint32_t)(g % wh);
    const uint32_t px = pix % (uint32_t)cam.width, py = pix / (uint32_t)cam.width;
    Pcg32 rng;
    rng.seed(seed, g);
    float ux = rng.next_f32(), uy = rng.next_f32();
    (void)rng.next_f32();   // wavelength sample (integrator.cpp render_sample)
    float sx = ((float)px + ux) / (float)cam.width, sy = ((float)py + uy) / (float)cam.height;
    f3 dc = normalize(mk(cam.tx * (1.f - 2.f * sx), cam.ty * (1.f - 2.f * sy), 1.f));
    float inv_z = 1.f / dc.z;
    f3 d = normalize(mk(cam.m[0] * dc.x + cam.m[1] * dc.y + cam.m[2] * dc.z,
                        cam.m[4] * dc.x + cam.m[5] * dc.y + cam.m[6] * dc.z,
                        cam.m[8] * dc.x + cam.m[9] * dc.y + cam.m[10] * dc.z));
    f3 o = mk(cam.m[3], cam.m[7], cam.m[11]);
    Hit h;
    uint32_t err = 0;
    trace(sc, o, d, cam.near_clip * inv_z, cam.far_clip * inv_z, false, h, err);
    f3 L = splat(0.f);
    if (h.shape >= 0) {
        const DevShape &s = sc.shapes[h.shape];
        if (s.emitter >= 0 && add_emitted) L = emitted(sc, s, o + d * h.t, d);
    }
    st3s(S.o, S.cap, i, o);
    st3s(S.d, S.cap, i, d);
    st3s(S.thr, S.cap, i, splat(1.f));
    st3s(S.L, S.cap, i, L);
    S.eta[i] = 1.f;
    S.hit_t[i] = h.t; S.hit_u[i] = h.u; S.hit_v[i] = h.v;
    S.hit_shape[i] = h.shape; S.hit_prim[i] = h.prim;
    // path record of the multi-bounce filter after the camera ray
    // (state_transition(si, si, ...) of path_filtered_ms.cpp:79)
    const int rec = (h.shape >= 0 && (sc.shapes[h.shape].flags & kShapeFlagReceiver)) ? kRecReceiver : kRecDefault;
    if (S.mnee && rec == kRecReceiver) st3s(S.mnee, S.cap, i, o + d * h.t);
    const int tf = rec == kRecReceiver ? kTfReceiver : kTfDefault;
    S.flags[i] = (h.shape >= 0 ? kAlive : 0) | kSpecularCamera | (rec << kRecShift) | (tf << kTfShift);
    S.cam_s[i] = sx;
    S.cam_s[(size_t)S.cap + i] = sy;
    store_rng(S, i, rng);
}

// World-space direction through the image-plane sample (sx, sy).
SMS_D f3 cam_dir(const PtCam &cam, float sx, float sy) {
    f3 dc = normalize(mk(cam.tx * (1.f - 2.f * sx), cam.ty * (1.f - 2.f * sy), 1.f));
    return normalize(mk(cam.m[0] * dc.x + cam.m[1] * dc.y + cam.m[2] * dc.z,
                        cam.m[4] * dc.x + cam.m[5] * dc.y + cam.m[6] * dc.z,
                        cam.m[8] * dc.x + cam.m[9] * dc.y + cam.m[10] * dc.z));
}

// PerspectiveCamera::importance (perspective.cpp:224-276) x film size for the
// world-space direction d from the camera (camera-to-world taken as rigid).
SMS_D float cam_importance(const PtCam &cam, f3 d) {
    f3 dl = mk(cam.m[0] * d.x + cam.m[4] * d.y + cam.m[8] * d.z, cam.m[1] * d.x + cam.m[5] * d.y + cam.m[9] * d.z,
               cam.m[2] * d.x + cam.m[6] * d.y + cam.m[10] * d.z);
    if (!(dl.z > 0.f)) return 0.f;
    float ic = 1.f / dl.z;
    float px = dl.x * ic, py = dl.y * ic;
    if (!(px >= -cam.tx && px <= cam.tx && py >= -cam.ty && py <= cam.ty)) return 0.f;
    return (1.f / (4.f * cam.tx * cam.ty)) * ic * ic * ic * (float)cam.width * (float)cam.height;
}

// ------------------------------------------------------------------ bounce
template <bool kMneeCheck>
__global__ void __launch_bounds__(kPtBlock) pt_bounce_kernel(DevScene sc, PtParams P, PtState S, int depth,
                                                             uint32_t n, DevCounters *ctr, PtCam cam) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    int want = 0, alive_out = 0;
    uint32_t err = 0;
    if (i < n && S.mnee_want) S.mnee_want[i] = 0;
    if (i < n && (S.flags[i] & kAlive)) {
        int flags = S.flags[i];
        Pcg32 rng = load_rng(S, i);
        f3 o = ld3s(S.o, S.cap, i), d = ld3s(S.d, S.cap, i);
        f3 thr = ld3s(S.thr, S.cap, i), L = ld3s(S.L, S.cap, i);
        float eta = S.eta[i];
        const int shape = S.hit_shape[i];
        SurfPt si;
        surface_at(sc, o, d, S.hit_t[i], shape, S.hit_prim[i], S.hit_u[i], S.hit_v[i], si);
        const DevShape &s = sc.shapes[shape];
        bool alive = true;
        // Russian roulette (path.cpp:139-144; path_sms_ss.cpp:102-107)
        if (depth > P.rr_depth) {
            float q = fminf(hmax3(thr) * eta * eta, 0.95f);
            float u = rng.next_f32();
            if (P.integrator == SMS_INTEGRATOR_PATH ? !(u < q) : (u > q)) alive = false;
            thr = thr * (1.f / q);
        }
        if ((uint32_t)depth >= (uint32_t)P.max_depth) alive = false;
        if (alive) {
            f3 fs, ft;
            shading_frame(si, fs, ft);
            // a twosided BSDF seen from the back (cos_theta(wi) <= 0) works in
            // the local frame with its normal reflected (twosided.cpp)
            const f3 n_sh = (s.twosided && !(dot(-d, si.shn) > 0.f)) ? -si.shn : si.shn;
            const f3 wiw = -d;
            const f3 wi = mk(dot(wiw, fs), dot(wiw, ft), dot(wiw, n_sh));
            const bool receiver = (s.flags & kShapeFlagReceiver) != 0;
            const bool teaser = P.integrator == SMS_INTEGRATOR_PATH_SMS_TEASER;
            // the teaser's passes trace the same paths (every draw below is
            // made in each pass); only pass 0 adds the non-SMS contributions
            const bool add_paths = !teaser || P.teaser_pass == 0;
            bool on_caster = false;
            if (teaser)
                on_caster = (s.flags & (kShapeFlagCasterSingle | kShapeFlagCasterMulti | kShapeFlagBouncer)) != 0;
            else if (P.integrator == SMS_INTEGRATOR_PATH_SMS_SS) on_caster = (s.flags & kShapeFlagCasterSingle) != 0;
            else if (P.integrator == SMS_INTEGRATOR_PATH_SMS_MS || P.integrator == SMS_INTEGRATOR_PATH_FILTERED_MS)
                on_caster = (s.flags & (kShapeFlagCasterMulti | kShapeFlagBouncer)) != 0;
            else if (P.integrator == SMS_INTEGRATOR_PATH_FILTERED_SS)
                on_caster = (s.flags & (kShapeFlagCasterSingle | kShapeFlagCasterMulti)) != 0;
            const bool filtered_teaser = P.integrator == SMS_INTEGRATOR_PATH_FILTERED_TEASER;
            if (filtered_teaser)
                on_caster = (s.flags & (kShapeFlagCasterSingle | kShapeFlagCasterMulti | kShapeFlagBouncer)) != 0;
            int tf = (flags >> kTfShift) & 7;
            const bool filtered_ss = P.integrator == SMS_INTEGRATOR_PATH_FILTERED_SS;
            const bool filtered_ms = P.integrator == SMS_INTEGRATOR_PATH_FILTERED_MS;
            const bool filtered = filtered_ss || filtered_ms;
            const bool glint_case = depth == 1 && !P.disable_reflected_emitters;
            int rec = (flags >> kRecShift) & 3, rec_b = (flags >> kRecBounceShift) & 7;
            // the connection the SMS estimators would have made from here
            // (path_filtered_ss.cpp:109-110; light_connection_valid,
            // path_filtered_ms.cpp:240-242)
            const bool valid_conn = filtered_ss ? on_caster && ((flags & kPrevReceiver) || glint_case)
                                                : filtered_ms && rec == kRecCaster && rec_b == P.bounces;
            const bool diffuse = s.bsdf_type == kBsdfDiffuse;
            // the normal-mapped shape (glinty, or a caster / bouncer) carries the
            // normalmap BSDF around its smooth conductor or dielectric
            const bool nmapped = shape == sc.glinty_shape && sc.nmap_res > 0;
            // with the LEAN fallback the normalmap BSDF is also glossy; it
            // takes the fallback where the interaction has no uv partials,
            // i.e. after the camera's first hit (normalmap.cpp:80, 142, 187)
            const bool lean_fb = nmapped && sc.lean_fb;
            const bool lean_now = lean_fb && depth > 1;
            const bool smooth =
                (!nmapped && (diffuse || s.alpha > 0.f || s.bsdf_type == kBsdfRoughPlastic)) || lean_fb;   // BSDFFlags::Smooth
            const bool on_glinty = (P.integrator == SMS_INTEGRATOR_PATH_SMS_GLINTS || (teaser && P.glints_enabled)) &&
                                   depth == 1 && nmapped && (s.flags & kShapeFlagGlinty);
            const bool glint_pass = !teaser || P.teaser_pass == 2;
            const f3 albedo = mk(s.albedo[0], s.albedo[1], s.albedo[2]);
            if (on_glinty) {
                // ray differentials of the camera ray (perspective.cpp:198-220),
                // scaled (integrator.cpp:164-165), then compute_partials
                // (interaction.h:216-248)
                const float sx = S.cam_s[i], sy = S.cam_s[(size_t)S.cap + i];
                const f3 rdx = d + (cam_dir(cam, sx + 1.f / (float)cam.width, sy) - d) * P.diff_scale;
                const f3 rdy = d + (cam_dir(cam, sx, sy + 1.f / (float)cam.height) - d) * P.diff_scale;
                const float dn = dot(si.n, si.p);
                const f3 dp_dx = o + rdx * ((dn - dot(si.n, o)) / dot(si.n, rdx)) - si.p;
                const f3 dp_dy = o + rdy * ((dn - dot(si.n, o)) / dot(si.n, rdy)) - si.p;
                const float a00 = dot(si.dp_du, si.dp_du), a01 = dot(si.dp_du, si.dp_dv);
                const float a11 = dot(si.dp_dv, si.dp_dv);
                float inv_det = 1.f / (a00 * a11 - a01 * a01);
                if (!isfinite(inv_det)) inv_det = 0.f;
                const float b0x = dot(si.dp_du, dp_dx), b1x = dot(si.dp_dv, dp_dx);
                const float b0y = dot(si.dp_du, dp_dy), b1y = dot(si.dp_dv, dp_dy);
                const float dxu = (a11 * b0x - a01 * b1x) * inv_det, dxv = (a00 * b1x - a01 * b0x) * inv_det;
                const float dyu = (a11 * b0y - a01 * b1y) * inv_det, dyv = (a00 * b1y - a01 * b0y) * inv_det;
                // SMS strategy: stage the glint query (solved after this launch)
                const float row[kStageRows] = {si.p.x, si.p.y, si.p.z, n_sh.x, n_sh.y, n_sh.z,
                                               si.dp_du.x, si.dp_du.y, si.dp_du.z, si.dp_dv.x, si.dp_dv.y, si.dp_dv.z,
                                               si.u, si.v, dxu, dxv, dyu, dyv, o.x, o.y, o.z, thr.x, thr.y, thr.z};
                if (glint_pass) {
                    #pragma unroll
                    for (int k = 0; k < kStageRows; ++k) S.stage[(size_t)k * S.cap + i] = row[k];
                    want = 1;
                }
                // BSDF strategy inside the footprint (manifold_glints.cpp:178-220)
                const float fpx = rng.next_f32(), fpy = rng.next_f32();
                (void)rng.next_f32(); (void)rng.next_f32(); (void)rng.next_f32();
                const float uo = si.u + (fpx - 0.5f) * dxu + (fpy - 0.5f) * dyu;
                const float vo = si.v + (fpx - 0.5f) * dxv + (fpy - 0.5f) * dyv;
                f3 bwo;
                float bw;
                if (nm_conductor_sample(sc, s, n_sh, si.dp_du, uo, vo, wiw, bwo, bw)) {
                    Hit hb;
                    trace(sc, si.p, bwo, kRayEps * (1.f + max_abs(si.p)), INFINITY, false, hb, err);
                    if (hb.shape >= 0 && sc.shapes[hb.shape].emitter >= 0) {
                        const DevShape &es = sc.shapes[hb.shape];
                        const f3 ep = si.p + bwo * hb.t;
                        const f3 Le = emitted(sc, es, ep, bwo);
                        const f3 bwo_l = mk(dot(bwo, fs), dot(bwo, ft), dot(bwo, n_sh));
                        const float p_bsdf = glint_lean_pdf(sc, uo, vo, dxu, dxv, dyu, dyv, wi, bwo_l) + 1.f;
                        const float p_sms = emitter_pdf(sc, es, si.p, ep, bwo, hb.t);
                        const float mis = P.sms_strategy_only ? 0.f : mis_weight(p_bsdf, p_sms);
                        if (glint_pass) L = L + thr * Le * (mis * bw);
                    }
                }
            }
            // ---- SMS query of a receiver vertex (solved after this launch); the
            // teaser's caustics (path_sms_teaser.cpp:152-162): single scatter
            // if depth + 1 < max_depth (pass 0), multi scatter if depth +
            // bounces < max_depth (pass 1)
            // any receiver whose BSDF has a non-delta lobe takes SMS queries
            // (path_sms_ss.cpp:120-124 calls the solver at every receiver;
            // a delta BSDF's eval toward the chain is zero)
            const bool sms_receiver = receiver && smooth && !nmapped;
            const bool teaser_caustic =
                teaser && P.caustics_enabled && sms_receiver &&
                ((P.teaser_pass == 0 && (P.max_depth < 0 || depth + 1 < P.max_depth)) ||
                 (P.teaser_pass == 1 && (P.max_depth < 0 || depth + P.bounces < P.max_depth)));
            if (teaser_caustic ||
                (!teaser && P.integrator != SMS_INTEGRATOR_PATH && !filtered && !filtered_teaser && receiver &&
                 !on_caster && sms_receiver &&
                 (P.max_depth < 0 || depth + P.bounces < P.max_depth))) {
                // a diffuse receiver passes its albedo; any other names its
                // shape and the incident direction in the frame onb(n_sh)
                f3 rx = albedo;
                if (!diffuse) {
                    f3 os, ot;
                    onb(n_sh, os, ot);
                    rx = mk(-1.f - (float)shape, dot(wiw, os), dot(wiw, ot));
                }
                const float row[SMS_QUERY_FIELDS] = {si.p.x, si.p.y, si.p.z, n_sh.x, n_sh.y, n_sh.z,
                                                     si.dp_du.x, si.dp_du.y, si.dp_du.z,
                                                     si.dp_dv.x, si.dp_dv.y, si.dp_dv.z,
                                                     rx.x, rx.y, rx.z, wi.z};
                #pragma unroll
                for (int k = 0; k < SMS_QUERY_FIELDS; ++k) S.stage[(size_t)k * S.cap + i] = row[k];
                S.stage[(size_t)21 * S.cap + i] = thr.x;
                S.stage[(size_t)22 * S.cap + i] = thr.y;
                S.stage[(size_t)23 * S.cap + i] = thr.z;
                want = 1;
            }
            // ---- emitter sampling
            bool nee = smooth && !on_caster && !on_glinty;
            if (P.integrator == SMS_INTEGRATOR_PATH_SMS_SS)
                nee = nee || (depth == 1 && !P.disable_reflected_emitters);
            if (teaser) nee = smooth && !on_caster && P.non_sms_paths;   // path_sms_teaser.cpp:185
            if (filtered) nee = smooth && (!on_caster || valid_conn);
            if (filtered_teaser) nee = smooth;   // path_filtered_teaser.cpp:108
            if (nee) {
                float ux = rng.next_f32(), uy = rng.next_f32();
                DirSample ds;
                bool got;
                if (filtered_teaser && on_caster) {
                    // sample_filtered_emitter_direction (:331-378): only the
                    // caustic emitters that end the caster's chain here
                    const bool single_em = tf == kTfSingleCaster && rec_b == 1;
                    const bool multi_em = tf == kTfMultiCaster && rec_b == P.bounces;
                    got = (single_em || multi_em) &&
                          sample_emitter_direction_from(sc, single_em ? sc.emitters_ss : sc.emitters_ms,
                                                        single_em ? sc.n_emitters_ss : sc.n_emitters_ms, si.p, ux,
                                                        uy, ds);
                } else {
                    got = sample_emitter_direction(sc, si.p, ux, uy, ds);
                }
                if (got) {
                    Hit hs;
                    float mint = kRayEps * (1.f + max_abs(si.p));
                    bool occ = trace(sc, si.p, ds.d, mint, ds.dist * (1.f - kShadowEps), true, hs, err);
                    if (!occ && smooth) {
                        const f3 wo = mk(dot(ds.d, fs), dot(ds.d, ft), dot(ds.d, n_sh));
                        // the normalmap BSDF with uv partials evaluates its
                        // smooth nested BSDF: nothing
                        const f3 bv = lean_now  ? splat(lean_fb_eval(sc, wi, wo))
                                      : nmapped ? splat(0.f)
                                                : bsdf_eval(s, wi, wo);
                        if (bv.x != 0.f || bv.y != 0.f || bv.z != 0.f) {
                            const float bp = lean_now ? lean_fb_pdf(sc, wi, wo) : bsdf_pdf(s, wi, wo);
                            float w = ds.delta ? 1.f : mis_weight(ds.pdf, bp);
                            // a filtered caustic connection must scatter the way
                            // SMS solves it: reflection on conductors, refraction
                            // on dielectrics (path_filtered_ss.cpp:127-142)
                            if (valid_conn && (filtered_ms || depth > 1)) {
                                const bool refraction = wo.z * wi.z < 0.f;
                                if (s.spec_eta == 1.f ? refraction : !refraction) w = 0.f;
                            }
                            // path_filtered_teaser.cpp:131-150: on a caster only
                            // the scattering SMS solves, elsewhere only with
                            // the non-SMS paths
                            if (filtered_teaser) {
                                const bool refraction = wo.z * wi.z < 0.f;
                                if (on_caster ? (s.spec_eta == 1.f ? refraction : !refraction) : !P.non_sms_paths)
                                    w = 0.f;
                            }
                            if (add_paths) L = L + thr * bv * ds.spec * w;
                        }
                    }
                }
            }
            // ---- BSDF sampling
            float u1 = rng.next_f32(), u2 = rng.next_f32(), u3 = rng.next_f32();
            BsdfSample bs;
            bool ok;
            if (lean_now) {
                // the LEAN fallback (normalmap.cpp:80-112): glossy reflection
                f3 lwo;
                float lw, lpdf;
                ok = lean_fb_sample(sc, wi, u2, u3, lwo, lw, lpdf);
                if (ok) {
                    bs.wo = lwo;
                    bs.weight = splat(lw);
                    bs.pdf = lpdf;
                    bs.eta = 1.f;
                    bs.delta = false;
                    bs.transmit = false;
                }
            } else if (nmapped) {
                // the normal-mapped BSDF at the hit's own uv
                ok = nm_bsdf_sample(sc, s, fs, ft, n_sh, si.dp_du, si.u, si.v, wiw, u1, u2, u3, bs);
            } else {
                ok = bsdf_sample(s, wi, u1, u2, u3, bs);
                bs.transmit = bs.wo.z * wi.z < 0.f;
            }
            if (ok) {
                thr = thr * bs.weight;
                eta *= bs.eta;
                if (!bs.delta) flags &= ~kSpecularCamera;
            }
            if (!ok || (thr.x == 0.f && thr.y == 0.f && thr.z == 0.f)) {
                alive = false;
            } else {
                f3 d2 = fs * bs.wo.x + ft * bs.wo.y + n_sh * bs.wo.z;
                Hit h2;
                trace(sc, si.p, d2, kRayEps * (1.f + max_abs(si.p)), INFINITY, false, h2, err);
                if (filtered_ms) {
                    // PathRecord::state_transition (path_filtered_ms.cpp:244-300)
                    const bool nv = h2.shape >= 0;
                    const uint32_t nf = nv ? sc.shapes[h2.shape].flags : 0u;
                    if (nv && (nf & kShapeFlagReceiver)) {
                        rec = kRecReceiver; rec_b = 0;
                    } else if (rec == kRecReceiver) {
                        if (nv && (nf & kShapeFlagCasterMulti)) { rec = kRecCaster; rec_b = 1; }
                        else { rec = kRecDefault; rec_b = 0; }
                    } else if (rec == kRecCaster) {
                        if (rec_b < P.bounces && nv && (nf & (kShapeFlagCasterMulti | kShapeFlagBouncer))) {
                            // the chain continues only with the scattering SMS solves
                            if (s.spec_eta == 1.f ? bs.transmit : !bs.transmit) { rec = kRecDefault; rec_b = 0; }
                            else rec_b++;
                        } else if (rec_b == P.bounces && nv && sc.shapes[h2.shape].emitter >= 0 &&
                                   emitter_is_caustic_ms(sc, sc.shapes[h2.shape].emitter)) {
                            rec = kRecEmitter;
                        } else {
                            rec = kRecDefault; rec_b = 0;
                        }
                    } else {
                        rec = kRecDefault; rec_b = 0;
                    }
                    flags = (flags & ~(0x1F << kRecShift)) | (rec << kRecShift) | (rec_b << kRecBounceShift);
                }
                if (filtered_teaser) {
                    // PathRecord::state_transition (path_filtered_teaser.cpp:334-410)
                    const bool nv = h2.shape >= 0;
                    const uint32_t nf = nv ? sc.shapes[h2.shape].flags : 0u;
                    const int em = nv ? sc.shapes[h2.shape].emitter : -1;
                    // the scattering SMS solves: reflection off a conductor,
                    // refraction through a dielectric
                    const bool wrong = s.spec_eta == 1.f ? bs.transmit : !bs.transmit;
                    if (nv && (nf & kShapeFlagReceiver)) {
                        tf = kTfReceiver; rec_b = 0;
                    } else if (tf == kTfReceiver) {
                        if (nv && (nf & kShapeFlagCasterSingle)) { tf = kTfSingleCaster; rec_b = 1; }
                        else if (nv && (nf & kShapeFlagCasterMulti)) { tf = kTfMultiCaster; rec_b = 1; }
                        else { tf = kTfDefault; rec_b = 0; }
                    } else if (tf == kTfSingleCaster) {
                        if (!wrong && rec_b == 1 && em >= 0 && emitter_is_caustic_ss(sc, em)) tf = kTfSingleEmitter;
                        else { tf = kTfDefault; rec_b = 0; }
                    } else if (tf == kTfMultiCaster) {
                        if (wrong) { tf = kTfDefault; rec_b = 0; }
                        else if (rec_b < P.bounces && nv && (nf & (kShapeFlagCasterMulti | kShapeFlagBouncer))) rec_b++;
                        else if (rec_b == P.bounces && em >= 0 && emitter_is_caustic_ms(sc, em)) tf = kTfMultiEmitter;
                        else { tf = kTfDefault; rec_b = 0; }
                    } else {
                        tf = kTfDefault; rec_b = 0;
                    }
                    flags = (flags & ~((7 << kTfShift) | (7 << kRecBounceShift))) | (tf << kTfShift) |
                            (rec_b << kRecBounceShift);
                }
                if (P.mnee_ms) {
                    // MNEEHelper::state_transition (path_sms_ms.cpp:84-140): like
                    // the filter's record, without its scattering-type test, and
                    // keeping the receiver point and the specular vertices
                    const bool nv = h2.shape >= 0;
                    const uint32_t nf = nv ? sc.shapes[h2.shape].flags : 0u;
                    const f3 p2 = si.p + d2 * h2.t;
                    if (nv && (nf & kShapeFlagReceiver)) {
                        rec = kRecReceiver; rec_b = 0;
                        st3s(S.mnee, S.cap, i, p2);
                    } else if (rec == kRecReceiver) {
                        if (nv && (nf & kShapeFlagCasterMulti)) {
                            rec = kRecCaster; rec_b = 1;
                            S.mnee[(size_t)3 * S.cap + i] = __int_as_float(h2.shape);
                            st3s(S.mnee + (size_t)4 * S.cap, S.cap, i, p2);
                        } else {
                            rec = kRecDefault; rec_b = 0;
                        }
                    } else if (rec == kRecCaster) {
                        if (rec_b < P.bounces && nv && (nf & (kShapeFlagCasterMulti | kShapeFlagBouncer))) {
                            st3s(S.mnee + (size_t)(4 + 3 * rec_b) * S.cap, S.cap, i, p2);
                            rec_b++;
                        } else if (rec_b == P.bounces && nv && sc.shapes[h2.shape].emitter >= 0 &&
                                   emitter_is_caustic_ms(sc, sc.shapes[h2.shape].emitter)) {
                            rec = kRecEmitter;
                        } else {
                            rec = kRecDefault; rec_b = 0;
                        }
                    } else {
                        rec = kRecDefault; rec_b = 0;
                    }
                    flags = (flags & ~(0x1F << kRecShift)) | (rec << kRecShift) | (rec_b << kRecBounceShift);
                }
                if (h2.shape >= 0 && sc.shapes[h2.shape].emitter >= 0) {
                    const DevShape &es = sc.shapes[h2.shape];
                    const f3 ep = si.p + d2 * h2.t;
                    const f3 Le = emitted(sc, es, ep, d2);
                    bool allow = true;
                    if (P.integrator == SMS_INTEGRATOR_PATH_SMS_SS)
                        allow = !on_caster || (depth == 1 && !P.disable_reflected_emitters);
                    else if (P.integrator == SMS_INTEGRATOR_PATH_SMS_MS)
                        allow = !on_caster || (flags & kSpecularCamera);
                    else if (P.integrator == SMS_INTEGRATOR_PATH_SMS_GLINTS)
                        allow = !on_glinty;
                    else if (teaser)   // path_sms_teaser.cpp:276
                        allow = !on_caster && P.non_sms_paths && !on_glinty;
                    else if (filtered_ss)   // path_filtered_ss.cpp:166-172
                        allow = !on_caster || ((flags & kPrevReceiver) && (s.spec_eta == 1.f ? !bs.transmit : bs.transmit)) ||
                                glint_case;
                    else if (filtered_ms)   // light_hit_valid, path_filtered_ms.cpp:191
                        allow = !on_caster || (rec == kRecEmitter && rec_b == P.bounces) || (flags & kSpecularCamera);
                    else if (filtered_teaser)   // filtered_emitter_hit_valid (:380-393), :186-195
                        allow = on_caster ? (((tf == kTfSingleEmitter && rec_b == 1) ||
                                              (tf == kTfMultiEmitter && rec_b == P.bounces)) &&
                                             emitter_is_caustic_ms(sc, es.emitter))
                                          : P.non_sms_paths != 0;
                    if (allow) {
                        float epdf = bs.delta ? 0.f : emitter_pdf(sc, es, si.p, ep, d2, h2.t);
                        if (add_paths) L = L + thr * Le * mis_weight(bs.pdf, epdf);
                    } else if (P.mnee_ms && rec == kRecEmitter && rec_b == P.bounces) {
                        // path_sms_ms.cpp:323-360: the MNEE test runs after this
                        // launch (ms_mnee_check_kernel); stage the light point and
                        // the contribution it adds when MNEE misses this chain
                        const f3 c = thr * Le;
                        const float row[6] = {ep.x, ep.y, ep.z, c.x, c.y, c.z};
                        #pragma unroll
                        for (int k = 0; k < 6; ++k) S.stage[(size_t)k * S.cap + i] = row[k];
                        S.mnee_want[i] = 1;
                    } else if (kMneeCheck && (flags & kPrevReceiver) &&
                               (sc.emitters[es.emitter].kind == 1) && emitter_is_caustic_ss(sc, es.emitter)) {
                        // path_sms_ss.cpp:207-241: add the path unless the MNEE
                        // walk from the previous vertex finds this very solution
                        const f3 xp = ld3s(S.prev_p, S.cap, i);
                        Vtx v;
                        int it;
                        LaneStats st;
                        bool found = ss_walk<false, false, true>(sc, P.solver, shape, xp, ep, si.p, v, it, err, st);
                        if (found) {
                            f3 dpt = normalize(si.p - xp), dmn = normalize(v.p - xp);
                            found = fabsf(dot(dpt, dmn) - 1.f) < P.solver.uniqueness_threshold;
                        }
                        if (!found) L = L + thr * Le;
                    }
                }
                st3s(S.prev_p, S.cap, i, si.p);
                flags = receiver ? (flags | kPrevReceiver) : (flags & ~kPrevReceiver);
                st3s(S.o, S.cap, i, si.p);
                st3s(S.d, S.cap, i, d2);
                S.hit_t[i] = h2.t; S.hit_u[i] = h2.u; S.hit_v[i] = h2.v;
                S.hit_shape[i] = h2.shape; S.hit_prim[i] = h2.prim;
                alive = h2.shape >= 0;
            }
        }
        st3s(S.thr, S.cap, i, thr);
        st3s(S.L, S.cap, i, L);
        S.eta[i] = eta;
        S.flags[i] = alive ? (flags | kAlive) : (flags & ~kAlive);
        store_rng(S, i, rng);
        alive_out = alive;
    }
    if (i < n) S.want[i] = want;
    const int bq = __syncthreads_count(want);
    const int ba = __syncthreads_count(alive_out);
    if (threadIdx.x == 0) {
        S.block_q[blockIdx.x] = (uint32_t)bq;
        S.block_a[blockIdx.x] = (uint32_t)ba;
    }
    if (err) atomicOr(&ctr->error, err);
}

// ------------------------------------------------------------ compaction
// Exclusive prefix sum of the per-block query counts (one block, in order)
// and the totals of queries and live paths.
__global__ void __launch_bounds__(1024) pt_scan_kernel(PtState S, uint32_t n_blocks) {
    __shared__ uint32_t warp_sum[32];
    __shared__ uint32_t carry;
    __shared__ uint32_t alive_sum;
    if (threadIdx.x == 0) { carry = 0; alive_sum = 0; }
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t alive_local = 0;
    for (uint32_t b0 = 0; b0 < n_blocks; b0 += 1024) {
        const uint32_t b = b0 + threadIdx.x;
        const uint32_t v = b < n_blocks ? S.block_q[b] : 0u;
        alive_local += b < n_blocks ? S.block_a[b] : 0u;
        uint32_t x = v;
        #pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if ((int)lane >= off) x += y;
        }
        if (lane == 31) warp_sum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = warp_sum[lane];
            #pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
                if ((int)lane >= off) w += y;
            }
            warp_sum[lane] = w;   // inclusive
        }
        __syncthreads();
        const uint32_t before = carry + (wid ? warp_sum[wid - 1] : 0u) + x - v;
        if (b < n_blocks) S.block_q[b] = before;   // now the block's offset
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_sum[31];
        __syncthreads();
    }
    atomicAdd(&alive_sum, alive_local);
    __syncthreads();
    if (threadIdx.x == 0) {
        S.totals[0] = carry;
        S.totals[1] = alive_sum;
    }
}

// Staged queries of this bounce -> entries base + r of the pending batch
// (r = rank in path order); their stream is path + bounce * 2^48.
__global__ void __launch_bounds__(kPtBlock) pt_gather_kernel(PtState S, uint32_t n, uint32_t base, uint64_t g0,
                                                             int depth) {
    __shared__ uint32_t warp_cnt[kPtBlock / 32];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = i < n ? S.want[i] : 0;
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, w);
    if (lane == 0) warp_cnt[wid] = __popc(m);
    __syncthreads();
    if (!w) return;
    uint32_t r = S.block_q[blockIdx.x] + __popc(m & ((1u << lane) - 1u));
    for (unsigned k = 0; k < wid; ++k) r += warp_cnt[k];
    const uint32_t e = base + r;
    for (int k = 0; k < S.qrows; ++k) S.qraw[(size_t)k * S.qcap + e] = S.stage[(size_t)k * S.cap + i];
    #pragma unroll
    for (int k = 0; k < 3; ++k) S.qw[(size_t)k * S.qcap + e] = S.stage[(size_t)(21 + k) * S.cap + i];
    S.qmap[e] = i;
    S.qstream[e] = g0 + i + ((uint64_t)depth << 48);
}

// Pending batch (stride qcap) -> packed SoA queries (stride nq).
__global__ void __launch_bounds__(kPtBlock) pt_pack_kernel(PtState S, uint32_t nq) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nq) return;
    for (int f = 0; f < S.qrows; ++f) S.q[(size_t)f * nq + k] = S.qraw[(size_t)f * S.qcap + k];
}

// Glint estimates of entries [b, b + cnt) -> path radiance: the SMS strategy
// of manifold_glints.cpp:150-176 with its MIS weight against the BSDF
// strategy (emitter-sampling density vs LEAN density + 1) and the sensor
// importance.  The emitter sample is redrawn from the query's stream (its
// first 3 numbers, as the estimator drew it).
__global__ void __launch_bounds__(kPtBlock) pt_glint_add_kernel(DevScene sc, PtCam cam, PtState S, uint32_t nq,
                                                                uint32_t b, uint32_t cnt, uint64_t sseed,
                                                                int bsdf_strategy_only) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= cnt) return;
    const uint32_t k = b + r;
    const f3 v = mk(S.value[k], S.value[(size_t)nq + k], S.value[2 * (size_t)nq + k]);
    if (v.x == 0.f && v.y == 0.f && v.z == 0.f) return;
    auto Q = [&](int f) { return S.q[(size_t)f * nq + k]; };
    const f3 p = mk(Q(0), Q(1), Q(2)), n = mk(Q(3), Q(4), Q(5)), dpdu = mk(Q(6), Q(7), Q(8));
    const float u = Q(12), vv = Q(13), dxu = Q(14), dxv = Q(15), dyu = Q(16), dyv = Q(17);
    const f3 sensor = mk(Q(18), Q(19), Q(20));
    Pcg32 rng = query_rng(sseed, S.qstream[k], 0);
    Light Lt;
    if (!sample_emitter(sc, sc.emitters_all, sc.n_emitters_all, rng, p, Lt)) return;
    f3 ed = Lt.p - p;
    const float edist = length(ed);
    ed = ed * (1.f / edist);
    float p_sms = 1.f;
    if (Lt.kind == 1) p_sms = emitter_pdf(sc, sc.shapes[sc.emitters[Lt.eidx].shape], p, Lt.p, ed, edist);
    const f3 fs = normalize(dpdu - n * dot(n, dpdu)), ft = cross(n, fs);
    const f3 wiw = normalize(sensor - p);
    const f3 wi = mk(dot(wiw, fs), dot(wiw, ft), dot(wiw, n)), wo = mk(dot(ed, fs), dot(ed, ft), dot(ed, n));
    const float p_bsdf = glint_lean_pdf(sc, u, vv, dxu, dxv, dyu, dyv, wi, wo) + 1.f;
    const float mis = bsdf_strategy_only ? 0.f : mis_weight(p_sms, p_bsdf);
    const float We = cam_importance(cam, normalize(p - sensor));
    const uint32_t i = S.qmap[k];
    const f3 w = mk(S.qw[k], S.qw[(size_t)S.qcap + k], S.qw[2 * (size_t)S.qcap + k]);
    st3s(S.L, S.cap, i, ld3s(S.L, S.cap, i) + w * v * (mis * We));
}

// Entries [b, b + cnt) of the solved batch (one bounce: each path at most
// once) -> path radiance.
__global__ void __launch_bounds__(kPtBlock) pt_sms_add_kernel(PtState S, uint32_t nq, uint32_t b, uint32_t cnt) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= cnt) return;
    const uint32_t k = b + r;
    const uint32_t i = S.qmap[k];
    f3 w = mk(S.qw[k], S.qw[(size_t)S.qcap + k], S.qw[2 * (size_t)S.qcap + k]);
    f3 v = mk(S.value[k], S.value[(size_t)nq + k], S.value[2 * (size_t)nq + k]);
    st3s(S.L, S.cap, i, ld3s(S.L, S.cap, i) + w * v);
}

// image[pix0 + j] += sum over the chunk's samples k of L[k * n_pix + j].
__global__ void __launch_bounds__(kPtBlock) pt_resolve_kernel(PtState S, float *image, uint32_t pix0,
                                                              uint32_t n_pix, uint32_t n_samples) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_pix) return;
    f3 acc = splat(0.f);
    for (uint32_t k = 0; k < n_samples; ++k) acc = acc + ld3s(S.L, S.cap, k * n_pix + j);
    float *px = image + 3 * (size_t)(pix0 + j);
    px[0] += acc.x; px[1] += acc.y; px[2] += acc.z;
}

__global__ void pt_scale_kernel(float *image, size_t n, float s) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) image[i] *= s;
}

// The Gaussian reconstruction filter as the reference film applies it: the
// filter tabulated at kFilterRes + 1 points (rfilter.cpp:9-20), n weights per
// axis around each sample (imageblock.cpp:111-135).
constexpr int kFilterRes = 31;
struct PtFilter {
    float table[kFilterRes + 1];
    float radius, scale;
    int n;       // weights per axis of one sample
    int reach;   // source pixels a destination pixel gathers from, each side
};

// Weight of a sample at pixel coordinate pos (the sample position minus 0.5)
// on pixel x of one axis; false when x is not among its n pixels.
SMS_D bool filter_weight(const PtFilter &F, float pos, int x, float &w) {
    const int lo = (int)ceilf(pos - F.radius), hi = (int)floorf(pos + F.radius);
    const int i = x - lo;
    if (i < 0 || i >= F.n || x > hi) return false;
    const float p = ((float)lo - pos) + (float)i;
    w = F.table[min((int)fabsf(p * F.scale), kFilterRes)];
    return true;
}

// ImageBlock::put of one chunk's samples (imageblock.cpp:111-160) as a
// gather: each destination pixel of rows [y0, y0 + rows) sums w L and w over
// the chunk's samples that splat onto it, source pixel by source pixel in
// sample order, so the image is reproducible; chunks add in order.  The
// weight sum is kept only when `weights` (the teaser's later passes trace
// the same samples).
__global__ void __launch_bounds__(kPtBlock) pt_splat_kernel(PtState S, PtFilter F, float *image, float *wsum,
                                                            uint32_t width, uint32_t height, uint32_t pix0,
                                                            uint32_t n_pix, uint32_t n_samples, uint32_t y0,
                                                            uint32_t rows, int weights) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= rows * width) return;
    const int x = (int)(j % width), y = (int)(y0 + j / width);
    f3 acc = splat(0.f);
    float wacc = 0.f;
    for (int dy = -F.reach; dy <= F.reach; ++dy) {
        const int sy = y + dy;
        if (sy < 0 || sy >= (int)height) continue;
        for (int dx = -F.reach; dx <= F.reach; ++dx) {
            const int sx = x + dx;
            if (sx < 0 || sx >= (int)width) continue;
            const uint32_t src = (uint32_t)sy * width + (uint32_t)sx;
            if (src < pix0 || src >= pix0 + n_pix) continue;
            for (uint32_t k = 0; k < n_samples; ++k) {
                const uint32_t i = k * n_pix + (src - pix0);
                const float px = S.cam_s[i] * (float)width - 0.5f;
                const float py = S.cam_s[(size_t)S.cap + i] * (float)height - 0.5f;
                float wx, wy;
                if (!filter_weight(F, px, x, wx) || !filter_weight(F, py, y, wy)) continue;
                const float w = wy * wx;
                acc = acc + ld3s(S.L, S.cap, i) * w;
                wacc += w;
            }
        }
    }
    const size_t d = (size_t)y * width + (size_t)x;
    float *px = image + 3 * d;
    px[0] += acc.x; px[1] += acc.y; px[2] += acc.z;
    if (weights) wsum[d] += wacc;
}

// The film's weighted mean: pixels without weight stay 0.
__global__ void pt_normalize_kernel(float *image, const float *wsum, size_t n_pix) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pix) return;
    const float w = wsum[i];
    const float s = w != 0.f ? 1.f / w : 0.f;
    image[3 * i] *= s; image[3 * i + 1] *= s; image[3 * i + 2] *= s;
}

sms_status rfail(sms_status st, const std::string &msg) {
    return (sms_status)set_last_error_impl((int)st, msg.c_str());
}

#define PT_TRY(call)                                                                         \
    do {                                                                                     \
        cudaError_t _e = (call);                                                             \
        if (_e != cudaSuccess) {                                                             \
            st = rfail(SMS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));    \
            goto done;                                                                       \
        }                                                                                    \
    } while (0)

}  // namespace

}  // namespace sms

using namespace sms;

extern "C" void sms_render_options_default(sms_render_options *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->integrator = SMS_INTEGRATOR_PATH_SMS_SS;
    o->max_depth = -1;
    o->rr_depth = 5;
    o->spp = 1;
    o->caustics_enabled = o->glints_enabled = o->non_sms_paths_enabled = 1;
    sms_config_default(&o->glints);
    o->rfilter = SMS_RFILTER_BOX;
    o->rfilter_stddev = 0.5f;
}

extern "C" uint64_t sms_render_sms_seed(uint64_t seed) {
    // SplitMix64 (Steele, Lea and Flood 2014) of seed + golden gamma
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static bool camera_params(const sms_camera *c, PtCam &out, std::string &why) {
    if (c->width <= 0 || c->height <= 0) { why = "film size must be positive"; return false; }
    if (!(c->fov > 0.f && c->fov < 180.f)) { why = "fov must lie in (0, 180) degrees"; return false; }
    const double aspect = (double)c->width / (double)c->height;
    const double t = std::tan(0.5 * (double)c->fov * M_PI / 180.0);
    double tx;
    switch (c->fov_axis) {
        case SMS_FOV_X: tx = t; break;
        case SMS_FOV_Y: tx = t * aspect; break;
        case SMS_FOV_DIAGONAL: tx = t / std::sqrt(1.0 + 1.0 / (aspect * aspect)); break;
        case SMS_FOV_SMALLER: tx = aspect >= 1.0 ? t * aspect : t; break;
        case SMS_FOV_LARGER: tx = aspect >= 1.0 ? t : t * aspect; break;
        default: why = "unknown fov_axis"; return false;
    }
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 4; ++k) out.m[4 * r + k] = c->to_world[4 * r + k];
    out.tx = (float)tx;
    out.ty = (float)(tx / aspect);
    out.near_clip = c->near_clip > 0.f ? c->near_clip : 1e-2f;
    out.far_clip = c->far_clip > out.near_clip ? c->far_clip : 1e4f;
    out.width = c->width;
    out.height = c->height;
    return true;
}

extern "C" sms_status sms_render_device(sms_ctx *c, const sms_camera *cam, const sms_render_options *opt,
                                        float *image) {
    if (!c || !cam || !opt || !image) return rfail(SMS_ERR_INVALID_ARG, "sms_render_device: null argument");
    CtxView v;
    if (!ctx_view(c, v)) return rfail(SMS_ERR_INVALID_ARG, "sms_render_device: bad context");
    PtCam pc;
    std::string why;
    if (!camera_params(cam, pc, why)) return rfail(SMS_ERR_INVALID_ARG, "sms_render: " + why);
    if (opt->spp <= 0) return rfail(SMS_ERR_INVALID_ARG, "sms_render: spp must be positive");
    const uint32_t spp_pass = opt->samples_per_pass == 0 ? (uint32_t)opt->spp
                                                         : std::min<uint32_t>(opt->samples_per_pass, (uint32_t)opt->spp);
    if ((uint32_t)opt->spp % spp_pass != 0)
        return rfail(SMS_ERR_INVALID_ARG, "sms_render: spp must be a multiple of samples_per_pass");
    if (opt->integrator < SMS_INTEGRATOR_PATH || opt->integrator > SMS_INTEGRATOR_PATH_FILTERED_TEASER)
        return rfail(SMS_ERR_INVALID_ARG, "sms_render: unknown integrator");
    const bool teaser = opt->integrator == SMS_INTEGRATOR_PATH_SMS_TEASER;
    // the teaser's glints need a glinty shape with a slope map
    const bool teaser_glints = teaser && opt->glints_enabled && v.scene->glinty_shape >= 0 && v.scene->nmap_res > 0;
    bool glints = opt->integrator == SMS_INTEGRATOR_PATH_SMS_GLINTS;
    if (glints || teaser_glints || v.scene->lean_fb) {
        // the footprint MIS and the LEAN fallback BSDF read the LEAN pyramid
        if (sms_status est = ctx_ensure_lean(c)) return est;
    }
    if (teaser && opt->timeout > 0.f)
        return rfail(SMS_ERR_UNSUPPORTED, "path_sms_teaser: a timeout is not supported (the image is rendered in "
                                          "three passes over the same paths)");
    if (teaser && opt->caustics_enabled && (v.bounces < 1 || v.bounces > kMaxBounces))
        return rfail(SMS_ERR_UNSUPPORTED, "path_sms_teaser: caustics_bounces must be between 1 and 4");
    if (opt->integrator == SMS_INTEGRATOR_PATH_SMS_SS && v.solver.mnee_init && !opt->biased_mnee &&
        v.solver.twostage)
        return rfail(SMS_ERR_UNSUPPORTED, "path_sms_ss: unbiased MNEE with the twostage solver is not supported");
    if (v.nm_rough)
        return rfail(SMS_ERR_UNSUPPORTED, "sms_render: a rough (alpha > 0) normal-mapped shape is not supported");
    if (opt->rr_depth <= 0) return rfail(SMS_ERR_INVALID_ARG, "sms_render: rr_depth must be positive");
    if (opt->max_depth < -1) return rfail(SMS_ERR_INVALID_ARG, "sms_render: max_depth must be -1 or >= 0");
    if (opt->integrator == SMS_INTEGRATOR_PATH_FILTERED_MS && (v.bounces < 1 || v.bounces > kMaxBounces))
        return rfail(SMS_ERR_UNSUPPORTED, "path_filtered_ms: bounces must be between 1 and 4");
    if (opt->integrator == SMS_INTEGRATOR_PATH_FILTERED_TEASER && (v.bounces < 1 || v.bounces > kMaxBounces))
        return rfail(SMS_ERR_UNSUPPORTED, "path_filtered_teaser: multi_caustic_bounces must be between 1 and 4");
    const bool gauss = opt->rfilter == SMS_RFILTER_GAUSSIAN;
    if (opt->rfilter != SMS_RFILTER_BOX && !gauss) return rfail(SMS_ERR_INVALID_ARG, "sms_render: unknown rfilter");
    PtFilter F{};
    if (gauss) {
        if (!(opt->rfilter_stddev > 0.f && opt->rfilter_stddev <= 2.f))
            return rfail(SMS_ERR_INVALID_ARG, "sms_render: rfilter_stddev must lie in (0, 2]");
        // gaussian.cpp: radius 4 stddev, max(0, exp(alpha x^2) - exp(alpha r^2))
        const float sd = opt->rfilter_stddev, r = 4.f * sd, alpha = -1.f / (2.f * sd * sd);
        const float bias = std::exp(alpha * r * r);
        for (int i = 0; i < kFilterRes; ++i) {
            const float x = (r * (float)i) / (float)kFilterRes;
            F.table[i] = std::max(0.f, std::exp(alpha * (x * x)) - bias);
        }
        F.table[kFilterRes] = 0.f;
        F.radius = r;
        F.scale = (float)kFilterRes / r;
        F.n = (int)std::ceil((r - 2.f * kRayEps) * 2.f);
        F.reach = (int)std::ceil(r + 0.5f);
    }
    PtParams P{};
    P.integrator = opt->integrator;
    P.max_depth = opt->max_depth;
    P.rr_depth = opt->rr_depth;
    P.disable_reflected_emitters = opt->disable_reflected_emitters;
    P.biased_mnee = opt->biased_mnee;
    P.bounces = (opt->integrator == SMS_INTEGRATOR_PATH_SMS_MS || opt->integrator == SMS_INTEGRATOR_PATH_FILTERED_MS ||
                 opt->integrator == SMS_INTEGRATOR_PATH_FILTERED_TEASER || teaser)
                    ? v.bounces : 1;
    P.mnee_check = opt->integrator == SMS_INTEGRATOR_PATH_SMS_SS && v.solver.mnee_init && !opt->biased_mnee;
    P.mnee_ms = opt->integrator == SMS_INTEGRATOR_PATH_SMS_MS && v.solver.mnee_init && !opt->biased_mnee;
    P.seed = opt->seed;
    P.solver = v.solver;
    P.diff_scale = std::max(1.f / std::sqrt((float)opt->spp), opt->glint_diff_scale_factor_clamp);
    P.bsdf_strategy_only = teaser ? 0 : v.bsdf_strategy_only;
    P.sms_strategy_only = teaser ? 0 : v.sms_strategy_only;
    P.caustics_enabled = opt->caustics_enabled;
    P.glints_enabled = teaser_glints ? 1 : 0;
    P.non_sms_paths = opt->non_sms_paths_enabled;
    // the teaser's passes; -1: any other integrator (one pass)
    std::vector<int> passes;
    if (teaser) {
        if (opt->caustics_enabled || opt->non_sms_paths_enabled) passes.push_back(0);
        if (opt->caustics_enabled) passes.push_back(1);
        if (teaser_glints) passes.push_back(2);
        if (passes.empty()) passes.push_back(0);
    } else {
        passes.push_back(-1);
    }
    sms_config glint_cfg = opt->glints;
    glint_cfg.biased = 1;   // path_sms_teaser.cpp:347-350

    const uint64_t wh = (uint64_t)cam->width * (uint64_t)cam->height;
    const uint64_t total = wh * (uint64_t)opt->spp;
    const uint64_t pass = wh * (uint64_t)spp_pass;   // paths per pass
    std::chrono::steady_clock::time_point t_start;
    if (total >= (1ull << 48)) return rfail(SMS_ERR_INVALID_ARG, "sms_render: more than 2^48 samples");
    uint32_t cap = opt->max_paths ? opt->max_paths : kPtDefaultPaths;
    if (wh <= cap) cap = (uint32_t)(std::min<uint64_t>(cap / wh, (uint64_t)opt->spp) * wh);
    cap = std::max<uint32_t>(cap, 1u);
    const uint32_t qcap = 2u * cap;
    const uint32_t n_blocks_cap = (cap + kPtBlock - 1) / kPtBlock;

    // one device block for the whole path state and the pending SMS batch
    size_t bytes = 0;
    auto take = [&](size_t b) { size_t o = bytes; bytes += (b + 255) & ~(size_t)255; return o; };
    const size_t o_rs = take(8 * (size_t)cap), o_ri = take(8 * (size_t)cap), o_o = take(12 * (size_t)cap),
                 o_d = take(12 * (size_t)cap), o_thr = take(12 * (size_t)cap), o_L = take(12 * (size_t)cap),
                 o_pp = take(12 * (size_t)cap), o_eta = take(4 * (size_t)cap), o_ht = take(4 * (size_t)cap),
                 o_hu = take(4 * (size_t)cap), o_hv = take(4 * (size_t)cap), o_hs = take(4 * (size_t)cap),
                 o_fl = take(4 * (size_t)cap), o_hp = take(4 * (size_t)cap), o_cs = take(8 * (size_t)cap),
                 o_st = take(4 * (size_t)kStageRows * cap), o_w = take(4 * (size_t)cap),
                 o_bq = take(4 * (size_t)n_blocks_cap), o_ba = take(4 * (size_t)n_blocks_cap), o_tot = take(16),
                 o_qr = take(4 * (size_t)kQueryRowsMax * qcap), o_qw = take(12 * (size_t)qcap),
                 o_qm = take(4 * (size_t)qcap), o_qs = take(8 * (size_t)qcap),
                 o_q = take(4 * (size_t)kQueryRowsMax * qcap), o_val = take(12 * (size_t)qcap),
                 o_cnt = take(4 * (size_t)qcap), o_wk = take(4 * (size_t)qcap),
                 o_mn = take(P.mnee_ms ? 4 * (size_t)kMneeRows * cap : 0),
                 o_mw = take(P.mnee_ms ? 4 * (size_t)cap : 0), o_ws = take(gauss ? 4 * (size_t)wh : 0);
    char *blk = nullptr;
    float *wsum = nullptr;   // the Gaussian filter's weight per pixel
    uint32_t *host_tot = nullptr;
    sms_status st = SMS_OK;
    cudaStream_t s = v.stream;
    PtState S{};
    uint64_t g0 = 0;
    const size_t img_n = 3 * (size_t)wh;
    uint64_t sseed = sms_render_sms_seed(P.seed);
    std::vector<uint32_t> seg_base, seg_cnt;   // pending batch: one segment per bounce
    uint32_t pending = 0;
    // Solves the pending batch and adds it to the paths' radiance.
    auto flush = [&]() -> sms_status {
        if (pending == 0) { seg_base.clear(); seg_cnt.clear(); return SMS_OK; }
        pt_pack_kernel<<<(pending + kPtBlock - 1) / kPtBlock, kPtBlock, 0, s>>>(S, pending);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return rfail(SMS_ERR_CUDA, std::string("pt_pack_kernel: ") + cudaGetErrorString(e));
        sms_result r{S.value, S.count, S.walks};
        sms_status fs;
        if (glints && teaser) {
            // the teaser's glints run with their own config
            sms_config caustics_cfg;
            if (!ctx_swap_config(c, &glint_cfg, &caustics_cfg))
                return rfail(SMS_ERR_INVALID_ARG, "path_sms_teaser: invalid glints config");
            fs = ctx_glint_connect(c, S.q, pending, sseed, 0, S.qstream, &r);
            ctx_swap_config(c, &caustics_cfg, nullptr);
        } else {
            fs = glints ? ctx_glint_connect(c, S.q, pending, sseed, 0, S.qstream, &r)
                 : (P.integrator == SMS_INTEGRATOR_PATH_SMS_MS || P.teaser_pass == 1)
                     ? ctx_ms_connect(c, S.q, pending, sseed, 0, S.qstream, &r)
                     : ctx_ss_connect(c, S.q, pending, sseed, 0, S.qstream, &r);
        }
        if (fs) return fs;
        for (size_t k = 0; k < seg_base.size(); ++k) {
            const uint32_t g = (seg_cnt[k] + kPtBlock - 1) / kPtBlock;
            if (glints)
                pt_glint_add_kernel<<<g, kPtBlock, 0, s>>>(*v.scene, pc, S, pending, seg_base[k], seg_cnt[k], sseed,
                                                            P.bsdf_strategy_only);
            else
                pt_sms_add_kernel<<<g, kPtBlock, 0, s>>>(S, pending, seg_base[k], seg_cnt[k]);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return rfail(SMS_ERR_CUDA, std::string("pt_sms_add_kernel: ") + cudaGetErrorString(e));
        pending = 0;
        seg_base.clear();
        seg_cnt.clear();
        return SMS_OK;
    };
    PT_TRY(cudaSetDevice(v.device));
    PT_TRY(cudaMalloc(&blk, bytes));
    PT_TRY(cudaMallocHost(&host_tot, 2 * sizeof(uint32_t)));
    S.rng_state = reinterpret_cast<uint64_t *>(blk + o_rs);
    S.rng_inc = reinterpret_cast<uint64_t *>(blk + o_ri);
    S.o = reinterpret_cast<float *>(blk + o_o);
    S.d = reinterpret_cast<float *>(blk + o_d);
    S.thr = reinterpret_cast<float *>(blk + o_thr);
    S.L = reinterpret_cast<float *>(blk + o_L);
    S.prev_p = reinterpret_cast<float *>(blk + o_pp);
    S.eta = reinterpret_cast<float *>(blk + o_eta);
    S.hit_t = reinterpret_cast<float *>(blk + o_ht);
    S.hit_u = reinterpret_cast<float *>(blk + o_hu);
    S.hit_v = reinterpret_cast<float *>(blk + o_hv);
    S.hit_shape = reinterpret_cast<int *>(blk + o_hs);
    S.flags = reinterpret_cast<int *>(blk + o_fl);
    S.hit_prim = reinterpret_cast<uint32_t *>(blk + o_hp);
    S.cam_s = reinterpret_cast<float *>(blk + o_cs);
    S.stage = reinterpret_cast<float *>(blk + o_st);
    S.want = reinterpret_cast<int *>(blk + o_w);
    S.block_q = reinterpret_cast<uint32_t *>(blk + o_bq);
    S.block_a = reinterpret_cast<uint32_t *>(blk + o_ba);
    S.totals = reinterpret_cast<uint32_t *>(blk + o_tot);
    S.qraw = reinterpret_cast<float *>(blk + o_qr);
    S.qw = reinterpret_cast<float *>(blk + o_qw);
    S.qmap = reinterpret_cast<uint32_t *>(blk + o_qm);
    S.qstream = reinterpret_cast<uint64_t *>(blk + o_qs);
    S.q = reinterpret_cast<float *>(blk + o_q);
    S.value = reinterpret_cast<float *>(blk + o_val);
    S.count = reinterpret_cast<int *>(blk + o_cnt);
    S.walks = reinterpret_cast<int *>(blk + o_wk);
    S.mnee = P.mnee_ms ? reinterpret_cast<float *>(blk + o_mn) : nullptr;
    S.mnee_want = P.mnee_ms ? reinterpret_cast<int *>(blk + o_mw) : nullptr;
    S.cap = cap;
    S.qcap = qcap;
    wsum = gauss ? reinterpret_cast<float *>(blk + o_ws) : nullptr;
    PT_TRY(cudaMemsetAsync(image, 0, img_n * sizeof(float), s));
    if (gauss) PT_TRY(cudaMemsetAsync(wsum, 0, (size_t)wh * sizeof(float), s));
    ctx_set_render_spp(c, 0);
    for (const int tp : passes) {
    if (teaser) {
        P.teaser_pass = tp;
        glints = tp == 2;
        sseed = sms_render_sms_seed(P.seed + (uint64_t)tp);
        g0 = 0;
    }
    S.qrows = glints ? kQueryRowsMax : SMS_QUERY_FIELDS;
    t_start = std::chrono::steady_clock::now();
    while (g0 < total) {
        // timeout: stop at a pass boundary once the time is up
        if (opt->timeout > 0.f && g0 > 0 && g0 % pass == 0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() > opt->timeout)
            break;
        uint32_t n;
        if (wh <= cap) n = (uint32_t)std::min<uint64_t>(cap, total - g0);
        else n = (uint32_t)std::min<uint64_t>(cap, wh - g0 % wh);
        n = (uint32_t)std::min<uint64_t>(n, pass - g0 % pass);
        const uint32_t nb = (n + kPtBlock - 1) / kPtBlock;
        pt_camera_kernel<<<nb, kPtBlock, 0, s>>>(*v.scene, pc, S, g0, n, P.seed, teaser ? (tp == 0 ? 1 : 0) : 1);
        PT_TRY(cudaGetLastError());
        uint32_t alive_bound = n;   // paths that can stage a query at the next bounce
        for (int depth = 1;; ++depth) {
            if (depth > kPtHardDepth) {
                st = rfail(SMS_ERR_DEVICE_LIMIT, "sms_render: a path exceeded 4096 bounces (raise rr pressure or "
                                                 "bound max_depth)");
                goto done;
            }
            if (pending + alive_bound > qcap) {
                st = flush();
                if (st) goto done;
            }
            if (P.mnee_check)
                pt_bounce_kernel<true><<<nb, kPtBlock, 0, s>>>(*v.scene, P, S, depth, n, v.counters, pc);
            else
                pt_bounce_kernel<false><<<nb, kPtBlock, 0, s>>>(*v.scene, P, S, depth, n, v.counters, pc);
            PT_TRY(cudaGetLastError());
            if (P.mnee_ms) {
                PT_TRY(launch_ms_mnee_check(*v.scene, P.solver, P.bounces, S.mnee, S.stage, S.mnee_want, S.L, n,
                                            S.cap, v.counters, s));
            }
            pt_scan_kernel<<<1, 1024, 0, s>>>(S, nb);
            PT_TRY(cudaGetLastError());
            pt_gather_kernel<<<nb, kPtBlock, 0, s>>>(S, n, pending, g0, depth);
            PT_TRY(cudaGetLastError());
            PT_TRY(cudaMemcpyAsync(host_tot, S.totals, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            PT_TRY(cudaStreamSynchronize(s));
            const uint32_t nq = host_tot[0], n_alive = host_tot[1];
            if (nq) {
                seg_base.push_back(pending);
                seg_cnt.push_back(nq);
                pending += nq;
            }
            alive_bound = n_alive;
            if (n_alive == 0) break;
        }
        st = flush();
        if (st) goto done;
        {
            const uint32_t n_pix = (uint32_t)std::min<uint64_t>(n, wh);
            const uint32_t pix0 = (uint32_t)(g0 % wh);
            if (gauss) {
                // destination rows: the chunk's rows and `reach` rows either side
                const uint32_t W = (uint32_t)cam->width, H = (uint32_t)cam->height;
                const int r0 = (int)(pix0 / W) - F.reach, r1 = (int)((pix0 + n_pix - 1) / W) + F.reach;
                const uint32_t y0 = (uint32_t)std::max(r0, 0), y1 = (uint32_t)std::min(r1, (int)H - 1);
                const uint32_t rows = y1 - y0 + 1;
                const int weights = !teaser || tp == passes.front();
                pt_splat_kernel<<<(rows * W + kPtBlock - 1) / kPtBlock, kPtBlock, 0, s>>>(
                    S, F, image, wsum, W, H, pix0, n_pix, n / n_pix, y0, rows, weights);
            } else {
                pt_resolve_kernel<<<(n_pix + kPtBlock - 1) / kPtBlock, kPtBlock, 0, s>>>(S, image, pix0, n_pix,
                                                                                         n / n_pix);
            }
            PT_TRY(cudaGetLastError());
        }
        g0 += n;
    }
    }   // passes
    {
        const uint32_t spp_done = (uint32_t)(g0 / wh);
        if (gauss)
            pt_normalize_kernel<<<(unsigned)((wh + 255) / 256), 256, 0, s>>>(image, wsum, (size_t)wh);
        else
            pt_scale_kernel<<<(unsigned)((img_n + 255) / 256), 256, 0, s>>>(image, img_n, 1.f / (float)spp_done);
        PT_TRY(cudaGetLastError());
        ctx_set_render_spp(c, spp_done);
    }
    st = ctx_check_device_error(c);
done:
    if (blk) {
        cudaStreamSynchronize(s);
        cudaFree(blk);
    }
    if (host_tot) cudaFreeHost(host_tot);
    return st;
}

extern "C" sms_status sms_render(sms_ctx *c, const sms_camera *cam, const sms_render_options *opt, float *image) {
    if (!c || !cam || !opt || !image) return rfail(SMS_ERR_INVALID_ARG, "sms_render: null argument");
    if (cam->width <= 0 || cam->height <= 0) return rfail(SMS_ERR_INVALID_ARG, "sms_render: bad film size");
    CtxView v;
    if (!ctx_view(c, v)) return rfail(SMS_ERR_INVALID_ARG, "sms_render: bad context");
    const size_t bytes = 3 * (size_t)cam->width * (size_t)cam->height * sizeof(float);
    float *dimg = nullptr;
    cudaError_t e = cudaSetDevice(v.device);
    if (e == cudaSuccess) e = cudaMalloc(&dimg, bytes);
    if (e != cudaSuccess) return rfail(SMS_ERR_CUDA, std::string("sms_render: ") + cudaGetErrorString(e));
    sms_status st = sms_render_device(c, cam, opt, dimg);
    if (st == SMS_OK) {
        e = cudaMemcpyAsync(image, dimg, bytes, cudaMemcpyDeviceToHost, v.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
        if (e != cudaSuccess) st = rfail(SMS_ERR_CUDA, std::string("sms_render: ") + cudaGetErrorString(e));
    }
    cudaFree(dimg);
    return st;
}
