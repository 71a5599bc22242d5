// sms_host.cpp -- host side of the GB300 SMS library: scene builder, BVH
// builder, device contexts and the extern "C" entry points of sms_gb300.h.
//
// The reference builds a SAH kd-tree over the scene (include/mitsuba/render/
// kdtree.h) and answers one ray at a time per host thread.  Here the host
// builds a binned-SAH BVH2 whose nodes carry both children's boxes (one 64-byte
// record per node), uploads it once per context, and every query batch runs as
// one persistent kernel on the context's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sms_gb300.h"
#include "sms_device.cuh"
#include "sms_kernels.h"
#include "sms_bvh.h"

using namespace sms;

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

static sms_status fail(sms_status st, const std::string &msg) {
    g_last_error = msg;
    return st;
}

static sms_status cuda_fail(cudaError_t e, const char *what) {
    return fail(SMS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CUDA_TRY(call)                                        \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);   \
    } while (0)

extern "C" const char *sms_last_error(void) { return g_last_error.c_str(); }

// ------------------------------------------------------------------ config
extern "C" void sms_config_default(sms_config *c) {
    if (!c) return;
    c->biased = 0;
    c->twostage = 0;
    c->halfvector_constraints = 0;
    c->mnee_init = 0;
    c->step_scale = 1.f;
    c->max_iterations = 20;
    c->solver_threshold = 1e-5f;
    c->uniqueness_threshold = 1e-4f;
    c->max_trials = -1;
    c->bounces = 1;
    c->bsdf_strategy_only = 0;
    c->sms_strategy_only = 0;
    c->glints_vectorized = 0;
}

static bool attr(const std::string &tag, const char *name, std::string &out) {
    std::string key = std::string(name) + "=\"";
    size_t p = tag.find(key);
    if (p == std::string::npos) return false;
    p += key.size();
    size_t e = tag.find('"', p);
    if (e == std::string::npos) return false;
    out = tag.substr(p, e - p);
    return true;
}

static bool parse_bool(const std::string &v, bool &ok) {
    ok = true;
    if (v == "true" || v == "1") return true;
    if (v == "false" || v == "0") return false;
    ok = false;
    return false;
}

// Reads the parameters the reference integrators read (path_sms_ss.cpp:47-61,
// path_sms_ms.cpp:149-161, path_sms_glints.cpp:42-54).  Unknown names are
// ignored, as Properties lookups ignore them.
extern "C" sms_status sms_config_parse_xml(const char *xml, sms_config *cfg, char *type_out,
                                           size_t type_cap) {
    if (!xml || !cfg) return fail(SMS_ERR_INVALID_ARG, "sms_config_parse_xml: null argument");
    std::string s(xml);
    size_t ip = s.find("<integrator");
    if (ip == std::string::npos) return fail(SMS_ERR_PARSE, "no <integrator> element");
    size_t ie = s.find('>', ip);
    if (ie == std::string::npos) return fail(SMS_ERR_PARSE, "unterminated <integrator> tag");
    std::string itag = s.substr(ip, ie - ip + 1);
    std::string type;
    if (!attr(itag, "type", type)) return fail(SMS_ERR_PARSE, "<integrator> without type");
    sms_config c;
    sms_config_default(&c);
    if (type == "path_sms_ms" || type == "path_filtered_ms") c.bounces = 2;   // path_sms_ms.cpp:152, path_filtered_ms.cpp:58
    // path_sms_teaser: the context config is its caustics_* block (bounces
    // default 2, path_sms_teaser.cpp:60-70); glints_* and the switches are
    // render options
    const bool teaser = type == "path_sms_teaser";
    if (teaser) c.bounces = 2;
    // path_filtered_teaser: multi_caustic_bounces (default 2,
    // path_filtered_teaser.cpp:46) is the chain length of its filter
    const bool filtered_teaser = type == "path_filtered_teaser";
    if (filtered_teaser) c.bounces = 2;
    size_t end = s.find("</integrator>", ie);
    if (end == std::string::npos) end = s.size();
    size_t pos = ie + 1;
    while (true) {
        size_t t = s.find('<', pos);
        if (t == std::string::npos || t >= end) break;
        size_t te = s.find('>', t);
        if (te == std::string::npos) return fail(SMS_ERR_PARSE, "unterminated tag");
        std::string tag = s.substr(t, te - t + 1);
        pos = te + 1;
        std::string kind;
        if (tag.compare(0, 8, "<boolean") == 0) kind = "boolean";
        else if (tag.compare(0, 8, "<integer") == 0) kind = "integer";
        else if (tag.compare(0, 6, "<float") == 0) kind = "float";
        else continue;
        std::string name, value;
        if (!attr(tag, "name", name) || !attr(tag, "value", value))
            return fail(SMS_ERR_PARSE, "parameter without name/value: " + tag);
        if (teaser) {
            if (name.compare(0, 9, "caustics_") != 0) continue;
            name = name.substr(9);
        }
        char *ep = nullptr;
        if (kind == "boolean") {
            bool ok;
            bool b = parse_bool(value, ok);
            if (!ok) return fail(SMS_ERR_PARSE, "bad boolean value for " + name + ": " + value);
            int iv = b ? 1 : 0;
            if (name == "biased") c.biased = iv;
            else if (name == "twostage") c.twostage = iv;
            else if (name == "halfvector_constraints") c.halfvector_constraints = iv;
            else if (name == "mnee_init") c.mnee_init = iv;
            else if (name == "bsdf_strategy_only") c.bsdf_strategy_only = iv;
            else if (name == "sms_strategy_only") c.sms_strategy_only = iv;
            else if (name == "glints_vectorized") c.glints_vectorized = iv;
        } else if (kind == "integer") {
            long v = std::strtol(value.c_str(), &ep, 10);
            if (ep == value.c_str() || *ep) return fail(SMS_ERR_PARSE, "bad integer for " + name);
            if (name == "max_iterations") c.max_iterations = (int32_t)v;
            else if (name == "max_trials") c.max_trials = (int32_t)v;
            else if (name == "bounces") c.bounces = (int32_t)v;
            else if (filtered_teaser && name == "multi_caustic_bounces") c.bounces = (int32_t)v;
        } else {
            float v = std::strtof(value.c_str(), &ep);
            if (ep == value.c_str() || *ep) return fail(SMS_ERR_PARSE, "bad float for " + name);
            if (name == "step_scale") c.step_scale = v;
            else if (name == "solver_threshold") c.solver_threshold = v;
            else if (name == "uniqueness_threshold") c.uniqueness_threshold = v;
        }
    }
    *cfg = c;
    if (type_out && type_cap) {
        std::snprintf(type_out, type_cap, "%s", type.c_str());
    }
    return SMS_OK;
}

// ------------------------------------------------------------------- scene
struct HostShape {
    int kind = kShapeSphere;
    float center[3] = {0, 0, 0};
    float radius = 1.f;
    int flip = 0;
    std::vector<float> P, N, UV;
    std::vector<uint32_t> F;
    sms_bsdf bsdf{};
    uint32_t flags = 0;
    int emitter = -1;
};

struct HostEmitter {
    int kind = 0;
    float p[3] = {0, 0, 0};
    float rgb[3] = {0, 0, 0};
    int shape = -1;
    uint32_t flags = 0;
};

struct sms_scene {
    std::vector<HostShape> shapes;
    std::vector<HostEmitter> emitters;
    // glint normal map (slope based, level 0)
    int nmap_shape = -1;
    uint32_t nmap_res = 0;
    float nmap_tiles = 1.f;
    std::vector<uint16_t> nmap;   // res * res * 2 FP16 (sx, sy)
    // the normal map's LEAN fallback BSDF (normalmap.cpp:46-55), off by default
    bool lean_fb = false;
    float lf_alpha = 1e-4f, lf_eta = 0.f, lf_k = 1.f;
};

extern "C" sms_status sms_scene_create(sms_scene **out) {
    if (!out) return fail(SMS_ERR_INVALID_ARG, "sms_scene_create: null out");
    *out = new sms_scene();
    return SMS_OK;
}

extern "C" void sms_scene_destroy(sms_scene *s) { delete s; }

// roughplastic.cpp:355-399 (parameters_changed): the coating's external
// transmittance T at the 64 cosines mu_i = max(1e-6, i / 63) and the base's
// internal diffuse reflectance 2 mean_i(mu_i R_int(mu_i)).  T and R are the
// integrals of microfacet.h:454-550 (eval_transmittance / eval_reflectance)
// over the Beckmann visible normals of wi; here by Gauss-Legendre quadrature
// in the normal's polar angle on [0, atan(6 alpha)] (where the density lives)
// and the midpoint rule in its azimuth, in double precision.
namespace {
double rp_g1(const double v[3], const double m[3], double alpha) {   // microfacet.h smith_g1 (Beckmann)
    if ((v[0] * m[0] + v[1] * m[1] + v[2] * m[2]) * v[2] <= 0.0) return 0.0;
    const double xy = alpha * alpha * (v[0] * v[0] + v[1] * v[1]);
    if (xy == 0.0) return 1.0;
    const double a = 1.0 / std::sqrt(xy / (v[2] * v[2])), a2 = a * a;
    return a >= 1.6 ? 1.0 : (3.535 * a + 2.181 * a2) / (1.0 + 2.276 * a + 2.577 * a2);
}
// dielectric Fresnel (fresnel.h:34-80): reflectance, cos of the transmitted
// direction, eta_ti
double rp_fresnel(double ci, double eta, double &ct, double &eta_ti) {
    const double eta_it = ci >= 0.0 ? eta : 1.0 / eta;
    eta_ti = ci >= 0.0 ? 1.0 / eta : eta;
    const double ct2 = 1.0 - (1.0 - ci * ci) * eta_ti * eta_ti;
    const double aci = std::fabs(ci), act = std::sqrt(std::max(0.0, ct2));
    const double as = (aci - eta_it * act) / (aci + eta_it * act), ap = (act - eta_it * aci) / (act + eta_it * aci);
    ct = ci >= 0.0 ? -act : act;
    if (ct2 <= 0.0) return 1.0;
    return aci == 0.0 ? 1.0 : 0.5 * (as * as + ap * ap);
}
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-15) break;
        }
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}
// the visible-normal integral of g over m for direction wi (wi.z > 0)
template <typename G>
double rp_visible_integral(const double wi[3], double alpha, const std::vector<double> &gx,
                           const std::vector<double> &gw, int n_phi, G g) {
    const double tmax = std::atan(6.0 * alpha);
    double sum = 0.0;
    for (size_t i = 0; i < gx.size(); ++i) {
        const double th = 0.5 * tmax * (gx[i] + 1.0), wth = 0.5 * tmax * gw[i];
        const double st = std::sin(th), ct = std::cos(th), t = st / ct;
        const double D = std::exp(-(t * t) / (alpha * alpha)) / (M_PI * alpha * alpha * ct * ct * ct * ct);
        for (int j = 0; j < n_phi; ++j) {
            const double ph = 2.0 * M_PI * (j + 0.5) / n_phi;
            const double m[3] = {st * std::cos(ph), st * std::sin(ph), ct};
            const double dm = wi[0] * m[0] + wi[1] * m[1] + wi[2] * m[2];
            if (dm <= 0.0) continue;
            const double dvis = rp_g1(wi, m, alpha) * dm * D / wi[2];
            sum += dvis * g(m, dm) * st * wth * (2.0 * M_PI / n_phi);
        }
    }
    return sum;
}
}  // namespace

static void roughplastic_tables(double eta, double alpha, float table[kRoughPlasticRes], float &fdr) {
    std::vector<double> gx, gw;
    gauss_legendre(128, gx, gw);
    const int n_phi = 128;
    double rsum = 0.0;
    for (int i = 0; i < kRoughPlasticRes; ++i) {
        const double mu = std::max(1e-6, (double)i / (kRoughPlasticRes - 1));
        const double wi[3] = {std::sqrt(1.0 - mu * mu), 0.0, mu};
        // external transmittance: refraction into the coating, G1 of the refracted direction
        const double T = rp_visible_integral(wi, alpha, gx, gw, n_phi, [&](const double m[3], double dm) {
            double ct, eta_ti;
            const double F = rp_fresnel(dm, eta, ct, eta_ti);
            const double k = dm * eta_ti + ct;
            const double wt[3] = {m[0] * k - wi[0] * eta_ti, m[1] * k - wi[1] * eta_ti, m[2] * k - wi[2] * eta_ti};
            return wt[2] * wi[2] >= 0.0 ? 0.0 : rp_g1(wt, m, alpha) * (1.0 - F);
        });
        // internal reflectance (eta inverted), G1 of the reflected direction
        const double R = rp_visible_integral(wi, alpha, gx, gw, n_phi, [&](const double m[3], double dm) {
            double ct, eta_ti;
            const double F = rp_fresnel(dm, 1.0 / eta, ct, eta_ti);
            const double wo[3] = {2.0 * dm * m[0] - wi[0], 2.0 * dm * m[1] - wi[1], 2.0 * dm * m[2] - wi[2]};
            return wo[2] <= 0.0 ? 0.0 : rp_g1(wo, m, alpha) * F;
        });
        table[i] = (float)T;
        rsum += R * mu;
    }
    fdr = (float)(rsum / kRoughPlasticRes * 2.0);
}

static sms_status check_bsdf(const sms_bsdf *b) {
    if (!b) return fail(SMS_ERR_INVALID_ARG, "null bsdf");
    if (b->type < SMS_BSDF_DIFFUSE || b->type > SMS_BSDF_ROUGHPLASTIC)
        return fail(SMS_ERR_INVALID_ARG, "unknown bsdf type");
    if (b->type == SMS_BSDF_ROUGHPLASTIC && !(b->eta > 0.f && b->eta != 1.f && b->alpha > 0.f))
        return fail(SMS_ERR_INVALID_ARG, "roughplastic needs eta > 0, eta != 1 and alpha > 0");
    if (b->type == SMS_BSDF_DIELECTRIC && !(b->eta > 0.f))
        return fail(SMS_ERR_INVALID_ARG, "dielectric eta must be positive");
    if (!(b->alpha >= 0.f) || !std::isfinite(b->alpha))
        return fail(SMS_ERR_INVALID_ARG, "bsdf roughness alpha must be finite and >= 0");
    // twosided.cpp: only BSDFs without transmission may be nested
    if (b->twosided && b->type == SMS_BSDF_DIELECTRIC)
        return fail(SMS_ERR_UNSUPPORTED, "a twosided bsdf cannot wrap a dielectric (transmission)");
    return SMS_OK;
}


extern "C" sms_status sms_scene_add_sphere(sms_scene *s, const float center[3], float radius, int32_t flip,
                                           const sms_bsdf *bsdf, uint32_t flags, int32_t *id) {
    if (!s || !center) return fail(SMS_ERR_INVALID_ARG, "sms_scene_add_sphere: null argument");
    if (sms_status st = check_bsdf(bsdf)) return st;
    if (!(radius != 0.f) || !std::isfinite(radius)) return fail(SMS_ERR_INVALID_ARG, "sphere radius must be nonzero");
    HostShape h;
    h.kind = kShapeSphere;
    std::memcpy(h.center, center, sizeof(h.center));
    // sphere.cpp:128-131: a negative radius flips the normals
    h.radius = std::fabs(radius);
    h.flip = (flip != 0) != (radius < 0.f);
    h.bsdf = *bsdf;
    h.flags = flags;
    s->shapes.push_back(h);
    if (id) *id = (int32_t)s->shapes.size() - 1;
    return SMS_OK;
}

extern "C" sms_status sms_scene_add_mesh(sms_scene *s, const float *P, const float *N, const float *UV,
                                         uint32_t nv, const uint32_t *F, uint32_t nf, const sms_bsdf *bsdf,
                                         uint32_t flags, int32_t *id) {
    if (!s || !P || !F) return fail(SMS_ERR_INVALID_ARG, "sms_scene_add_mesh: null argument");
    if (nv == 0 || nf == 0) return fail(SMS_ERR_INVALID_ARG, "sms_scene_add_mesh: empty mesh");
    if (sms_status st = check_bsdf(bsdf)) return st;
    for (size_t i = 0; i < 3 * (size_t)nf; ++i)
        if (F[i] >= nv) return fail(SMS_ERR_INVALID_ARG, "sms_scene_add_mesh: face index out of range");
    HostShape h;
    h.kind = kShapeMesh;
    h.P.assign(P, P + 3 * (size_t)nv);
    if (N) h.N.assign(N, N + 3 * (size_t)nv);
    if (UV) h.UV.assign(UV, UV + 2 * (size_t)nv);
    h.F.assign(F, F + 3 * (size_t)nf);
    h.bsdf = *bsdf;
    h.flags = flags;
    s->shapes.push_back(std::move(h));
    if (id) *id = (int32_t)s->shapes.size() - 1;
    return SMS_OK;
}

extern "C" sms_status sms_scene_add_point_emitter(sms_scene *s, const float p[3], const float I[3],
                                                  uint32_t flags) {
    if (!s || !p || !I) return fail(SMS_ERR_INVALID_ARG, "sms_scene_add_point_emitter: null argument");
    HostEmitter e;
    e.kind = 0;
    std::memcpy(e.p, p, sizeof(e.p));
    std::memcpy(e.rgb, I, sizeof(e.rgb));
    e.flags = flags;
    s->emitters.push_back(e);
    return SMS_OK;
}

extern "C" sms_status sms_scene_add_area_emitter(sms_scene *s, int32_t shape, const float L[3],
                                                 uint32_t flags) {
    if (!s || !L) return fail(SMS_ERR_INVALID_ARG, "sms_scene_add_area_emitter: null argument");
    if (shape < 0 || shape >= (int32_t)s->shapes.size())
        return fail(SMS_ERR_INVALID_ARG, "sms_scene_add_area_emitter: unknown shape id");
    if (s->shapes[shape].kind != kShapeSphere)
        return fail(SMS_ERR_UNSUPPORTED, "area emitters are supported on spheres only");
    if (s->shapes[shape].emitter >= 0)
        return fail(SMS_ERR_INVALID_ARG, "an area emitter can only be attached to a single shape");
    HostEmitter e;
    e.kind = 1;
    e.shape = shape;
    std::memcpy(e.rgb, L, sizeof(e.rgb));
    e.flags = flags;
    s->emitters.push_back(e);
    s->shapes[shape].emitter = (int)s->emitters.size() - 1;
    return SMS_OK;
}

extern "C" sms_status sms_scene_set_normalmap(sms_scene *s, int32_t shape, const uint16_t *slopes, uint32_t res,
                                              float tiles) {
    if (!s || !slopes) return fail(SMS_ERR_INVALID_ARG, "sms_scene_set_normalmap: null argument");
    if (shape < 0 || shape >= (int32_t)s->shapes.size())
        return fail(SMS_ERR_INVALID_ARG, "sms_scene_set_normalmap: unknown shape id");
    if (res == 0 || res > 65536) return fail(SMS_ERR_INVALID_ARG, "sms_scene_set_normalmap: bad resolution");
    if (!(tiles > 0.f)) return fail(SMS_ERR_INVALID_ARG, "sms_scene_set_normalmap: tiles must be positive");
    s->nmap_shape = shape;
    s->nmap_res = res;
    s->nmap_tiles = tiles;
    s->nmap.assign(slopes, slopes + 2 * (size_t)res * res);
    // a shape that is no caster / bouncer becomes glinty; a caster or bouncer
    // keeps its role and its manifold vertices take the normal-mapped frame
    const uint32_t chain = SMS_SHAPE_CAUSTIC_CASTER_SINGLE | SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER;
    if (!(s->shapes[shape].flags & chain)) s->shapes[shape].flags |= SMS_SHAPE_GLINTY;
    return SMS_OK;
}

extern "C" sms_status sms_scene_set_lean_fallback(sms_scene *s, float alpha, float eta, float k) {
    if (!s) return fail(SMS_ERR_INVALID_ARG, "sms_scene_set_lean_fallback: null scene");
    if (s->nmap_res == 0)
        return fail(SMS_ERR_INVALID_ARG, "sms_scene_set_lean_fallback: the scene has no normal map");
    if (!(alpha >= 0.f && alpha < 1e3f) || !(eta >= 0.f && eta < 1e3f) || !(k >= 0.f && k < 1e3f))
        return fail(SMS_ERR_INVALID_ARG, "sms_scene_set_lean_fallback: alpha, eta and k must be finite and >= 0");
    if (eta == 0.f && k == 0.f)
        return fail(SMS_ERR_INVALID_ARG, "sms_scene_set_lean_fallback: eta and k cannot both be 0");
    s->lean_fb = true;
    s->lf_alpha = alpha;
    s->lf_eta = eta;
    s->lf_k = k;
    return SMS_OK;
}

// ----------------------------------------------------------- phase timing
namespace sms {
struct PhaseTimer {
    bool enabled = false;
    struct Rec { int phase; cudaEvent_t a, b; };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    int open_phase = -1;
    cudaEvent_t open_ev = nullptr;
    double ms[kPhases] = {0};
    unsigned long long launches[kPhases] = {0};
    cudaEvent_t get() {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void collect() {
        for (Rec &r : pending) {
            float t = 0.f;
            if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
                ms[r.phase] += t;
                launches[r.phase]++;
            }
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        pending.clear();
    }
    ~PhaseTimer() {
        collect();
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
    }
};

void phase_begin(PhaseTimer *tm, int phase, cudaStream_t s) {
    if (!tm || !tm->enabled) return;
    tm->open_phase = phase;
    tm->open_ev = tm->get();
    cudaEventRecord(tm->open_ev, s);
}

void phase_end(PhaseTimer *tm, cudaStream_t s) {
    if (!tm || !tm->enabled || tm->open_phase < 0) return;
    cudaEvent_t b = tm->get();
    cudaEventRecord(b, s);
    tm->pending.push_back({tm->open_phase, tm->open_ev, b});
    tm->open_phase = -1;
}
}  // namespace sms

// ---------------------------------------------------------------- context
struct sms_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    sms_config cfg{};
    DevScene dsc{};
    DevCounters *ctr = nullptr;
    std::vector<void *> allocs;
    int num_sms = 0;
    int blocks_per_sm = 0;
    int threads = 128;
    int trial_group = 0;          // lanes per query of the Bernoulli-trial kernel (0: auto)
    uint32_t treelet = 0;         // node records the trial kernel stages in shared memory
    int queue_chunk = 1;          // queries a trial-kernel lane group claims per atomic
    // device staging for the host-pointer entry points
    void *io = nullptr;
    size_t io_bytes = 0;
    // per-query scratch of the unbiased estimators
    void *scratch = nullptr;
    uint32_t scratch_n = 0;
    int *ms_tmpl = nullptr;       // multi-scatter templates, (4 kMaxBounces + 1) x n words
    uint32_t ms_tmpl_n = 0;
    PhaseTimer timer;
    std::vector<int> casters_ss;
    // learned seed proposal: uv frame of every shape, the bound proposal and
    // its per-query mixture scratch (kGmmParams x gmm_n floats)
    std::vector<mlp::SeedFrame> frames;
    sms_proposal *prop = nullptr;                 // bound to the SS estimator
    std::vector<sms_proposal *> proposals;        // every live proposal made on this context
    float defensive = 0.1f;
    float *gmm = nullptr;
    uint32_t gmm_n = 0;
    // offset normals of rough shapes are built for the single-scatter
    // estimator only: rough multi-scatter chain shapes / glinty shapes
    bool ms_rough = false, glint_rough = false;
    bool ms_nm = false;   // a multi-scatter chain shape carries the normal map
    uint32_t render_spp = 0;   // samples per pixel of the last render
    bool nm_rough = false;   // the normal-mapped shape is rough
    float *lean = nullptr;   // LEAN pyramid of the slope map (glints integrator), built on first use
};

template <typename T>
static sms_status upload(sms_ctx *c, const std::vector<T> &v, const T **out) {
    *out = nullptr;
    if (v.empty()) return SMS_OK;
    void *p = nullptr;
    CUDA_TRY(cudaMalloc(&p, v.size() * sizeof(T)));
    c->allocs.push_back(p);
    CUDA_TRY(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    *out = reinterpret_cast<const T *>(p);
    return SMS_OK;
}

static SolverCfg solver_cfg(const sms_config &c) {
    SolverCfg s;
    s.biased = c.biased;
    s.halfvector = c.halfvector_constraints;
    s.max_iterations = c.max_iterations;
    s.max_trials = c.max_trials;
    s.solver_threshold = c.solver_threshold;
    s.uniqueness_threshold = c.uniqueness_threshold;
    s.step_scale = c.step_scale;
    s.mnee_init = c.mnee_init;
    s.twostage = c.twostage;
    s.streams = nullptr;
    s.queue_chunk = 1;
    return s;
}

static sms_status validate_cfg(const sms_config *c) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null config");
    if (c->max_iterations < 0) return fail(SMS_ERR_INVALID_ARG, "max_iterations must be >= 0");
    return SMS_OK;
}

extern "C" void sms_ctx_destroy(sms_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->timer.collect();
    for (void *p : c->allocs) cudaFree(p);
    if (c->io) cudaFree(c->io);
    if (c->scratch) cudaFree(c->scratch);
    if (c->lean) cudaFree(c->lean);
    if (c->ms_tmpl) cudaFree(c->ms_tmpl);
    if (c->gmm) cudaFree(c->gmm);
    for (sms_proposal *p : c->proposals) proposal_detach(p);
    if (c->ctr) cudaFree(c->ctr);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

// uv frame of the learned proposal for one shape (sms_proposal_create):
// spheres (theta / pi, phi / 2 pi); meshes their bounding box over the two
// widest axes, the third axis at mid-height.
static mlp::SeedFrame seed_frame(const HostShape &h) {
    mlp::SeedFrame f;
    std::memset(&f, 0, sizeof(f));
    if (h.kind == kShapeSphere) {
        f.kind = 1;
        for (int k = 0; k < 3; ++k) f.org[k] = h.center[k];
        f.ax_u[0] = h.radius;
        return f;
    }
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i + 2 < h.P.size(); i += 3)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], h.P[i + k]);
            hi[k] = std::max(hi[k], h.P[i + k]);
        }
    int ax[3] = {0, 1, 2};
    std::sort(ax, ax + 3, [&](int a, int b) { return hi[a] - lo[a] > hi[b] - lo[b] || (hi[a] - lo[a] == hi[b] - lo[b] && a < b); });
    f.kind = 0;
    for (int k = 0; k < 3; ++k) f.org[k] = lo[k];
    f.org[ax[2]] = 0.5f * (lo[ax[2]] + hi[ax[2]]);
    f.ax_u[ax[0]] = hi[ax[0]] - lo[ax[0]];
    f.ax_v[ax[1]] = hi[ax[1]] - lo[ax[1]];
    return f;
}

static sms_status ctx_build(sms_ctx *c, const sms_scene *s) {
    // shapes, meshes and area CDFs
    std::vector<DevShape> shapes;
    std::vector<float> P, N, UV, cdf, pmf;
    std::vector<uint32_t> F;
    std::vector<uint32_t> tri_shape, tri_face;
    DevScene &d = c->dsc;
    std::memset(&d, 0, sizeof(d));
    for (size_t i = 0; i < s->shapes.size(); ++i) {
        const HostShape &h = s->shapes[i];
        DevShape ds;
        std::memset(&ds, 0, sizeof(ds));
        ds.kind = h.kind;
        ds.flags = h.flags;
        ds.bsdf_type = h.bsdf.type;
        ds.eta = h.bsdf.eta;
        ds.k = h.bsdf.k;
        ds.albedo[0] = h.bsdf.albedo[0]; ds.albedo[1] = h.bsdf.albedo[1]; ds.albedo[2] = h.bsdf.albedo[2];
        ds.alpha = h.bsdf.type == SMS_BSDF_DIFFUSE ? 0.f : h.bsdf.alpha;
        ds.twosided = h.bsdf.twosided ? 1 : 0;
        if (h.bsdf.type == SMS_BSDF_ROUGHPLASTIC) {
            if (h.flags & (SMS_SHAPE_CAUSTIC_CASTER_SINGLE | SMS_SHAPE_CAUSTIC_CASTER_MULTI |
                           SMS_SHAPE_CAUSTIC_BOUNCER | SMS_SHAPE_GLINTY))
                return fail(SMS_ERR_UNSUPPORTED, "a roughplastic shape cannot be a caustic caster, bouncer or glinty");
            roughplastic_tables(h.bsdf.eta, h.bsdf.alpha, ds.rp_t, ds.rp_fdr);
            // specular sampling weight: s_mean / (d_mean + s_mean), s_mean = 1
            const float d_mean = (h.bsdf.albedo[0] + h.bsdf.albedo[1] + h.bsdf.albedo[2]) / 3.f;
            ds.rp_ws = 1.f / (d_mean + 1.f);
            ds.rp_nonlinear = h.bsdf.nonlinear ? 1 : 0;
        }
        ds.nmap_frames = ((int)i == s->nmap_shape && s->nmap_res > 0 &&
                          (h.flags & (SMS_SHAPE_CAUSTIC_CASTER_SINGLE | SMS_SHAPE_CAUSTIC_CASTER_MULTI |
                                      SMS_SHAPE_CAUSTIC_BOUNCER))) ? 1 : 0;
        if (ds.alpha > 0.f && (h.flags & (SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER)))
            c->ms_rough = true;
        if (ds.alpha > 0.f && (h.flags & SMS_SHAPE_GLINTY)) c->glint_rough = true;
        if (ds.nmap_frames && (h.flags & (SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER)))
            c->ms_nm = true;
        if ((int)i == s->nmap_shape && s->nmap_res > 0 && ds.alpha > 0.f) c->nm_rough = true;
        // manifold.h:94-96: real ior -> eta, complex or non-specular -> 1
        bool real_ior = h.bsdf.type == SMS_BSDF_DIELECTRIC ||
                        (h.bsdf.type == SMS_BSDF_CONDUCTOR && h.bsdf.k == 0.f);
        ds.spec_eta = real_ior ? h.bsdf.eta : 1.f;
        ds.emitter = h.emitter;
        // MNEE initialisation target (manifold_ss.cpp:229-241): the bounding-box
        // centre for a complex-ior (reflecting) BSDF, else the light sample
        ds.reflective = real_ior ? 0 : 1;
        if (h.kind == kShapeSphere) {
            ds.bcx = h.center[0]; ds.bcy = h.center[1]; ds.bcz = h.center[2];
        } else {
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (size_t k = 0; k + 2 < h.P.size(); k += 3)
                for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], h.P[k + a]); hi[a] = std::max(hi[a], h.P[k + a]); }
            ds.bcx = 0.5f * (lo[0] + hi[0]); ds.bcy = 0.5f * (lo[1] + hi[1]); ds.bcz = 0.5f * (lo[2] + hi[2]);
        }
        c->frames.push_back(seed_frame(h));
        if (h.kind == kShapeSphere) {
            ds.cx = h.center[0]; ds.cy = h.center[1]; ds.cz = h.center[2];
            ds.radius = h.radius;
            ds.flip = h.flip;
            if (d.n_spheres >= kMaxSpheres) return fail(SMS_ERR_UNSUPPORTED, "too many spheres");
            d.sphere_shape[d.n_spheres] = (int)i;
            d.sphere[d.n_spheres] = make_float4(h.center[0], h.center[1], h.center[2], h.radius);
            d.n_spheres++;
        } else {
            uint32_t nv = (uint32_t)(h.P.size() / 3), nf = (uint32_t)(h.F.size() / 3);
            ds.v_off = (uint32_t)(P.size() / 3);
            ds.f_off = (uint32_t)(F.size() / 3);
            ds.n_faces = nf;
            ds.has_normals = !h.N.empty();
            ds.has_uvs = !h.UV.empty();
            P.insert(P.end(), h.P.begin(), h.P.end());
            if (ds.has_normals) N.insert(N.end(), h.N.begin(), h.N.end());
            else N.resize(N.size() + 3 * (size_t)nv, 0.f);
            if (ds.has_uvs) UV.insert(UV.end(), h.UV.begin(), h.UV.end());
            else UV.resize(UV.size() + 2 * (size_t)nv, 0.f);
            F.insert(F.end(), h.F.begin(), h.F.end());
            // mesh.cpp:505-528 + distr_1d.h:60-88: double accumulation, float storage
            ds.cdf_off = (uint32_t)cdf.size();
            double sum = 0.0;
            bool first = true;
            for (uint32_t f = 0; f < nf; ++f) {
                const float *p0 = &h.P[3 * h.F[3 * f]], *p1 = &h.P[3 * h.F[3 * f + 1]],
                            *p2 = &h.P[3 * h.F[3 * f + 2]];
                float e0[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                float e1[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                float cx = e0[1] * e1[2] - e0[2] * e1[1], cy = e0[2] * e1[0] - e0[0] * e1[2],
                      cz = e0[0] * e1[1] - e0[1] * e1[0];
                float a = 0.5f * std::sqrt(cx * cx + cy * cy + cz * cz);
                pmf.push_back(a);
                sum += (double)a;
                cdf.push_back((float)sum);
                if (a > 0.f) {
                    if (first) { ds.valid_lo = f; first = false; }
                    ds.valid_hi = f;
                }
                tri_shape.push_back((uint32_t)i);
                tri_face.push_back(f);
            }
            if (first) return fail(SMS_ERR_INVALID_ARG, "mesh has no face with positive area");
            ds.area_sum = (float)sum;
            ds.area_norm = (float)(1.0 / sum);
        }
        if (h.flags & SMS_SHAPE_CAUSTIC_CASTER_SINGLE) {
            if (d.n_casters_ss >= kMaxCasters) return fail(SMS_ERR_UNSUPPORTED, "too many casters");
            if (ds.alpha > 0.f) d.casters_ss_rough |= 1u << d.n_casters_ss;
            if (ds.nmap_frames) d.casters_ss_nm |= 1u << d.n_casters_ss;
            d.casters_ss[d.n_casters_ss++] = (int)i;
        }
        if (h.flags & SMS_SHAPE_CAUSTIC_CASTER_MULTI) {
            if (d.n_casters_ms >= kMaxCasters) return fail(SMS_ERR_UNSUPPORTED, "too many casters");
            d.casters_ms[d.n_casters_ms++] = (int)i;
        }
        shapes.push_back(ds);
    }
    std::vector<DevEmitter> em;
    d.glinty_shape = s->nmap_shape;
    d.nmap_shape = s->nmap_res > 0 ? s->nmap_shape : -1;
    d.ms_nm = c->ms_nm ? 1 : 0;
    d.ms_rough = c->ms_rough ? 1 : 0;
    d.nmap_res = s->nmap_res;
    d.nmap_tiles = s->nmap_tiles;
    d.lean_fb = s->lean_fb && s->nmap_res > 0 ? 1 : 0;
    d.lf_alpha = s->lf_alpha;
    d.lf_eta = s->lf_eta;
    d.lf_k = s->lf_k;
    for (size_t i = 0; i < s->emitters.size(); ++i) {
        if (d.n_emitters_all >= kMaxEmitters) return fail(SMS_ERR_UNSUPPORTED, "too many emitters");
        d.emitters_all[d.n_emitters_all++] = (int)i;
        const HostEmitter &h = s->emitters[i];
        DevEmitter e;
        std::memset(&e, 0, sizeof(e));
        e.kind = h.kind;
        e.px = h.p[0]; e.py = h.p[1]; e.pz = h.p[2];
        e.r = h.rgb[0]; e.g = h.rgb[1]; e.b = h.rgb[2];
        e.shape = h.shape;
        em.push_back(e);
        if (h.flags & SMS_EMITTER_CAUSTIC_SINGLE) {
            if (d.n_emitters_ss >= kMaxEmitters) return fail(SMS_ERR_UNSUPPORTED, "too many emitters");
            d.emitters_ss[d.n_emitters_ss++] = (int)i;
        }
        if (h.flags & SMS_EMITTER_CAUSTIC_MULTI) {
            if (d.n_emitters_ms >= kMaxEmitters) return fail(SMS_ERR_UNSUPPORTED, "too many emitters");
            d.emitters_ms[d.n_emitters_ms++] = (int)i;
        }
    }
    // BVH over all mesh triangles
    std::vector<BvhInputTri> in;
    in.reserve(tri_shape.size());
    for (size_t k = 0; k < tri_shape.size(); ++k) {
        const HostShape &h = s->shapes[tri_shape[k]];
        uint32_t f = tri_face[k];
        BvhInputTri t;
        for (int j = 0; j < 3; ++j) {
            t.p0[j] = h.P[3 * h.F[3 * f] + j];
            t.p1[j] = h.P[3 * h.F[3 * f + 1] + j];
            t.p2[j] = h.P[3 * h.F[3 * f + 2] + j];
        }
        t.shape = (int)tri_shape[k];
        t.face = (int)f;
        in.push_back(t);
    }
    BvhResult bvh;
    std::string berr;
    if (!in.empty() && (!build_bvh(in, bvh, berr) || !validate_bvh(bvh, berr)))
        return fail(SMS_ERR_INVALID_ARG, "BVH build: " + berr);
    const std::vector<float4> &nodes = bvh.nodes, &tris = bvh.tris;
    if (sms_status st = upload(c, nodes, &d.nodes)) return st;
    if (sms_status st = upload(c, tris, &d.tris)) return st;
    d.n_nodes = (uint32_t)(nodes.size() / 4);
    d.n_tris = (uint32_t)(tris.size() / 3);
    if (sms_status st = upload(c, shapes, &d.shapes)) return st;
    d.n_shapes = (int)shapes.size();
    if (sms_status st = upload(c, P, &d.mesh_P)) return st;
    if (sms_status st = upload(c, N, &d.mesh_N)) return st;
    if (sms_status st = upload(c, UV, &d.mesh_UV)) return st;
    if (sms_status st = upload(c, F, &d.mesh_F)) return st;
    if (sms_status st = upload(c, cdf, &d.cdf)) return st;
    if (sms_status st = upload(c, pmf, &d.pmf)) return st;
    if (sms_status st = upload(c, em, &d.emitters)) return st;
    {
        const uint16_t *nm = nullptr;
        if (sms_status st = upload(c, s->nmap, &nm)) return st;
        d.nmap = reinterpret_cast<const uint32_t *>(nm);
    }
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return SMS_OK;
}

extern "C" sms_status sms_ctx_create(const sms_scene *s, const sms_config *cfg, int32_t device, sms_ctx **out) {
    if (!s || !out) return fail(SMS_ERR_INVALID_ARG, "sms_ctx_create: null argument");
    *out = nullptr;
    if (sms_status st = validate_cfg(cfg)) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(SMS_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(SMS_ERR_INVALID_ARG, "device id out of range");
    sms_ctx *c = new sms_ctx();
    c->device = device;
    c->cfg = *cfg;
    sms_status st = SMS_OK;
    do {
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) { st = cuda_fail(e, "cudaSetDevice"); break; }
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { st = cuda_fail(e, "cudaStreamCreate"); break; }
        e = cudaMalloc(&c->ctr, sizeof(DevCounters));
        if (e != cudaSuccess) { st = cuda_fail(e, "cudaMalloc(counters)"); break; }
        e = cudaMemsetAsync(c->ctr, 0, sizeof(DevCounters), c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "cudaMemset(counters)"); break; }
        cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
        st = ctx_build(c, s);
    } while (0);
    if (st != SMS_OK) { sms_ctx_destroy(c); return st; }
    *out = c;
    return SMS_OK;
}

extern "C" sms_status sms_ctx_set_config(sms_ctx *c, const sms_config *cfg) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null context");
    if (sms_status st = validate_cfg(cfg)) return st;
    c->cfg = *cfg;
    return SMS_OK;
}

extern "C" void *sms_ctx_stream(sms_ctx *c) { return c ? (void *)c->stream : nullptr; }

extern "C" sms_status sms_ctx_set_trial_group(sms_ctx *c, int32_t group) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null context");
    if (group != 0 && group != 8 && group != 16 && group != 32)
        return fail(SMS_ERR_INVALID_ARG, "trial group must be 0 (auto), 8, 16 or 32");
    c->trial_group = group;
    return SMS_OK;
}

extern "C" sms_status sms_ctx_set_treelet(sms_ctx *c, int32_t nodes) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null context");
    if (nodes < 0 || nodes > kMaxTreeletNodes)
        return fail(SMS_ERR_INVALID_ARG, "treelet size must be in [0, 384] node records");
    c->treelet = (uint32_t)nodes;
    return SMS_OK;
}

extern "C" sms_status sms_ctx_set_queue_chunk(sms_ctx *c, int32_t chunk) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null context");
    if (chunk < 1 || chunk > 64) return fail(SMS_ERR_INVALID_ARG, "queue chunk must be in [1, 64]");
    c->queue_chunk = chunk;
    return SMS_OK;
}

extern "C" sms_status sms_ctx_set_launch(sms_ctx *c, int32_t bps, int32_t tpb) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null context");
    if (bps < 0 || tpb < 0) return fail(SMS_ERR_INVALID_ARG, "negative launch parameter");
    if (tpb != 0 && tpb != 128) return fail(SMS_ERR_UNSUPPORTED, "threads per block must be 128");
    if (bps > 64) return fail(SMS_ERR_INVALID_ARG, "blocks per SM too large");
    c->blocks_per_sm = bps;
    return SMS_OK;
}

sms_status ctx_check_device_error(sms_ctx *c);
static sms_status check_device_error(sms_ctx *c) { return ctx_check_device_error(c); }
sms_status ctx_check_device_error(sms_ctx *c) {
    unsigned err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, &c->ctr->error, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (err) {
        CUDA_TRY(cudaMemsetAsync(&c->ctr->error, 0, sizeof(unsigned), c->stream));
        std::string m = "device limit hit:";
        if (err & kErrStackOverflow) m += " BVH traversal stack overflow;";
        if (err & kErrTrialLimit) m += " Bernoulli trials exceeded the hard limit;";
        if (err & kErrSolutionOverflow) m += " more unique solutions than the per-query capacity;";
        if (err & kErrBadQuery) m += " a query names a receiver shape outside the scene;";
        return fail(SMS_ERR_DEVICE_LIMIT, m);
    }
    return SMS_OK;
}

extern "C" sms_status sms_stats_read(sms_ctx *c, sms_stats *out) {
    if (!c || !out) return fail(SMS_ERR_INVALID_ARG, "null argument");
    DevCounters h;
    CUDA_TRY(cudaSetDevice(c->device));
    CUDA_TRY(cudaMemcpyAsync(&h, c->ctr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    out->solver_succeeded = h.solver_succeeded;
    out->solver_failed = h.solver_failed;
    out->bernoulli_trial_calls = h.bernoulli_calls;
    out->bernoulli_trial_iterations = h.bernoulli_iters;
    out->bernoulli_trial_iterations_max = h.bernoulli_max;
    out->walks = h.walks;
    out->newton_iterations = h.newton_iters;
    out->connections = h.connections;
    out->rays = h.rays;
    out->bvh_nodes = h.bvh_nodes;
    out->tri_tests = h.tri_tests;
    out->speculative_walks = h.speculative_walks;
    return SMS_OK;
}

extern "C" sms_status sms_stats_reset(sms_ctx *c) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null context");
    CUDA_TRY(cudaSetDevice(c->device));
    CUDA_TRY(cudaMemsetAsync(c->ctr, 0, sizeof(DevCounters), c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->timer.collect();
    for (int k = 0; k < kPhases; ++k) { c->timer.ms[k] = 0.0; c->timer.launches[k] = 0; }
    return SMS_OK;
}

extern "C" sms_status sms_ctx_set_profiling(sms_ctx *c, int32_t enable) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null context");
    c->timer.enabled = enable != 0;
    return SMS_OK;
}

extern "C" sms_status sms_profile_read(sms_ctx *c, sms_profile *out) {
    if (!c || !out) return fail(SMS_ERR_INVALID_ARG, "null argument");
    static_assert(SMS_PHASES == kPhases, "phase count");
    DevCounters h;
    CUDA_TRY(cudaSetDevice(c->device));
    CUDA_TRY(cudaMemcpyAsync(&h, c->ctr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->timer.collect();
    for (int k = 0; k < kPhases; ++k) {
        out->ms[k] = c->timer.ms[k];
        out->launches[k] = c->timer.launches[k];
        out->rays[k] = h.phase_rays[k];
        out->bvh_nodes[k] = h.phase_nodes[k];
        out->tri_tests[k] = h.phase_tris[k];
    }
    return SMS_OK;
}

static sms_status ensure_scratch(sms_ctx *c, uint32_t n, SsScratch &scr) {
    if (c->scratch_n < n) {
        if (c->scratch) {
            CUDA_TRY(cudaStreamSynchronize(c->stream));
            cudaFree(c->scratch);
            c->scratch = nullptr;
            c->scratch_n = 0;
        }
        CUDA_TRY(cudaMalloc(&c->scratch, ss_scratch_bytes(n)));
        c->scratch_n = n;
    }
    char *b = reinterpret_cast<char *>(c->scratch);
    size_t cap = c->scratch_n;
    scr.pos = reinterpret_cast<uint32_t *>(b);
    scr.dir0 = reinterpret_cast<float *>(b + 4 * cap);
    scr.val = reinterpret_cast<float *>(b + 16 * cap);
    scr.list = reinterpret_cast<uint32_t *>(b + 28 * cap);
    return SMS_OK;
}

// Normal-mapped single-scatter casters: the two-stage solver
// (manifold_ss.cpp:253-270) draws its first slope from the map's LEAN
// distribution, so it needs the pyramid, and every caster must carry the map
// (on a caster without one the reference's lean() is zero and the sampled
// slope is NaN: no walk converges).  A learned proposal seeds plain casters only.
static sms_status check_ss_normalmap(sms_ctx *c) {
    const uint32_t all = c->dsc.n_casters_ss >= 32 ? ~0u : ((1u << c->dsc.n_casters_ss) - 1u);
    if (c->cfg.twostage) {
        if (c->dsc.n_casters_ss > 0 && (c->dsc.casters_ss_nm & all) != all)
            return fail(SMS_ERR_UNSUPPORTED, "the twostage solver needs every single-scatter caster normal-mapped");
        if (c->dsc.n_casters_ss > 0)
            if (sms_status st = ctx_build_lean(c)) return st;
    }
    mlp::SeedProposal pr{};
    if (c->prop && proposal_seed_desc(c->prop, pr))
        for (int k = 0; k < c->dsc.n_casters_ss; ++k)
            if (c->dsc.casters_ss[k] == pr.shape && ((c->dsc.casters_ss_nm >> k) & 1u))
                return fail(SMS_ERR_UNSUPPORTED, "a learned proposal cannot seed a normal-mapped caster");
    return SMS_OK;
}

// Configuration checks of a single-scatter connection call, shared by the
// device entry point and the allocation-free one so both accept and refuse the
// same configurations.  With may_allocate false a missing LEAN pyramid is
// reported instead of built (building it allocates).
sms_status ctx_ss_check(sms_ctx *c, bool may_allocate) {
    if (c->cfg.biased && c->cfg.max_trials > (1 << 24))
        return fail(SMS_ERR_INVALID_ARG, "max_trials too large for the biased estimator");
    if (c->prop && c->cfg.biased)
        return fail(SMS_ERR_UNSUPPORTED, "a learned proposal seeds the unbiased estimator only");
    if (!may_allocate && c->cfg.twostage && c->dsc.n_casters_ss > 0 && !c->lean) {
        const uint32_t all = c->dsc.n_casters_ss >= 32 ? ~0u : ((1u << c->dsc.n_casters_ss) - 1u);
        if ((c->dsc.casters_ss_nm & all) != all)
            return fail(SMS_ERR_UNSUPPORTED, "the twostage solver needs every single-scatter caster normal-mapped");
        return fail(SMS_ERR_UNSUPPORTED, "the twostage solver needs the LEAN pyramid, which the first "
                                         "sms_ss_connect_batch_device call builds");
    }
    return check_ss_normalmap(c);
}

// Single-scatter connection of n device-resident queries; streams (may be
// null) as SolverCfg::streams.
sms_status ctx_ss_connect(sms_ctx *c, const float *q, uint32_t n, uint64_t seed, uint64_t stream_off,
                          const uint64_t *streams, sms_result *out) {
    if (!c || !out || (n && (!q || !out->value || !out->count || !out->walks)))
        return fail(SMS_ERR_INVALID_ARG, "sms_ss_connect_batch_device: null argument");
    if (n == 0) return SMS_OK;
    if (sms_status st = ctx_ss_check(c, true)) return st;
    CUDA_TRY(cudaSetDevice(c->device));
    SsScratch scr{};
    if (!c->cfg.biased)
        if (sms_status st = ensure_scratch(c, n, scr)) return st;
    mlp::SeedProposal pr{};
    if (c->prop) {
        if (c->gmm_n < n) {
            if (c->gmm) {
                CUDA_TRY(cudaStreamSynchronize(c->stream));
                cudaFree(c->gmm);
                c->gmm = nullptr;
                c->gmm_n = 0;
            }
            CUDA_TRY(cudaMalloc(&c->gmm, (size_t)mlp::kGmmParams * n * sizeof(float)));
            c->gmm_n = n;
        }
        if (!proposal_seed_desc(c->prop, pr)) return fail(SMS_ERR_INVALID_ARG, "proposal is not usable");
        pr.defensive = c->defensive;
        pr.gmm = c->gmm;
    }
    SolverCfg sc = solver_cfg(c->cfg);
    sc.streams = streams;
    sc.queue_chunk = c->queue_chunk;
    CUDA_TRY(launch_ss_connect(c->dsc, sc, q, n, seed, stream_off, out->value, out->count, out->walks, c->ctr, scr,
                               c->num_sms, c->blocks_per_sm, &c->timer, c->stream, c->prop ? &pr : nullptr,
                               c->trial_group, c->treelet));
    return SMS_OK;
}

extern "C" sms_status sms_ss_connect_batch_device(sms_ctx *c, const float *q, uint32_t n, uint64_t seed,
                                                  uint64_t stream_off, sms_result *out) {
    return ctx_ss_connect(c, q, n, seed, stream_off, nullptr, out);
}

extern "C" sms_status sms_ctx_set_proposal(sms_ctx *c, sms_proposal *p, float defensive) {
    if (!c) return fail(SMS_ERR_INVALID_ARG, "null context");
    if (!p) {
        c->prop = nullptr;
        return SMS_OK;
    }
    if (proposal_ctx(p) != c) return fail(SMS_ERR_INVALID_ARG, "proposal belongs to another context");
    if (!(defensive > 0.f && defensive <= 1.f))
        return fail(SMS_ERR_INVALID_ARG, "defensive share must lie in (0, 1]");
    c->prop = p;
    c->defensive = defensive;
    return SMS_OK;
}

// Context side of a proposal's lifetime (sms_proposal.cu).
void ctx_register_proposal(sms_ctx *c, sms_proposal *p) {
    if (c) c->proposals.push_back(p);
}
void ctx_forget_proposal(sms_ctx *c, sms_proposal *p) {
    if (!c) return;
    if (c->prop == p) c->prop = nullptr;
    c->proposals.erase(std::remove(c->proposals.begin(), c->proposals.end(), p), c->proposals.end());
}

// Device staging buffer of the host-pointer entry points, grown on demand and
// kept for the context's lifetime.
static sms_status ensure_io(sms_ctx *c, size_t bytes) {
    if (c->io_bytes >= bytes) return SMS_OK;
    if (c->io) {
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        cudaFree(c->io);
        c->io = nullptr;
        c->io_bytes = 0;
    }
    CUDA_TRY(cudaMalloc(&c->io, bytes));
    c->io_bytes = bytes;
    return SMS_OK;
}

extern "C" sms_status sms_ss_connect_batch(sms_ctx *c, const float *q, uint32_t n, uint64_t seed,
                                           uint64_t stream_off, sms_result *out) {
    if (!c || !out || (n && (!q || !out->value || !out->count || !out->walks)))
        return fail(SMS_ERR_INVALID_ARG, "sms_ss_connect_batch: null argument");
    if (n == 0) return SMS_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    size_t qb = (size_t)SMS_QUERY_FIELDS * n * sizeof(float);
    size_t vb = 3 * (size_t)n * sizeof(float), ib = (size_t)n * sizeof(int32_t);
    if (sms_status st = ensure_io(c, qb + vb + 2 * ib)) return st;
    char *dbuf = reinterpret_cast<char *>(c->io);
    float *dq = reinterpret_cast<float *>(dbuf);
    float *dv = reinterpret_cast<float *>(dbuf + qb);
    int32_t *dc = reinterpret_cast<int32_t *>(dbuf + qb + vb);
    int32_t *dw = reinterpret_cast<int32_t *>(dbuf + qb + vb + ib);
    sms_status st = SMS_OK;
    do {
        cudaError_t e = cudaMemcpyAsync(dq, q, qb, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy queries"); break; }
        sms_result r{dv, dc, dw};
        st = sms_ss_connect_batch_device(c, dq, n, seed, stream_off, &r);
        if (st) break;
        e = cudaMemcpyAsync(out->value, dv, vb, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->count, dc, ib, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->walks, dw, ib, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy results"); break; }
    } while (0);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(e, "sms_ss_connect_batch");
    return check_device_error(c);
}

extern "C" sms_status sms_ss_walk_batch(sms_ctx *c, int32_t caster, const float *q, const float *w, uint32_t n,
                                        float *out) {
    if (!c || (n && (!q || !w || !out))) return fail(SMS_ERR_INVALID_ARG, "sms_ss_walk_batch: null argument");
    if (caster < 0 || caster >= c->dsc.n_shapes) return fail(SMS_ERR_INVALID_ARG, "unknown caster shape id");
    if (n == 0) return SMS_OK;
    if (c->cfg.twostage) {
        bool nm = false;
        for (int k = 0; k < c->dsc.n_casters_ss; ++k)
            nm |= c->dsc.casters_ss[k] == caster && ((c->dsc.casters_ss_nm >> k) & 1u);
        if (!nm) return fail(SMS_ERR_UNSUPPORTED, "the twostage solver needs a normal-mapped single-scatter caster");
        if (sms_status st = ctx_build_lean(c)) return st;
    }
    CUDA_TRY(cudaSetDevice(c->device));
    const int wrows = c->cfg.twostage ? SMS_SS_WALK_IN_FIELDS_TWOSTAGE : SMS_WALK_IN_FIELDS;
    size_t qb = (size_t)SMS_QUERY_FIELDS * n * sizeof(float), wb = (size_t)wrows * n * sizeof(float),
           ob = (size_t)SMS_WALK_OUT_FIELDS * n * sizeof(float);
    if (sms_status st = ensure_io(c, qb + wb + ob)) return st;
    char *dbuf = reinterpret_cast<char *>(c->io);
    sms_status st = SMS_OK;
    do {
        cudaError_t e = cudaMemcpyAsync(dbuf, q, qb, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dbuf + qb, w, wb, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy walk inputs"); break; }
        e = launch_ss_walk(c->dsc, solver_cfg(c->cfg), caster, reinterpret_cast<float *>(dbuf),
                           reinterpret_cast<float *>(dbuf + qb), n, reinterpret_cast<float *>(dbuf + qb + wb),
                           c->ctr, &c->timer, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "launch ss_walk"); break; }
        e = cudaMemcpyAsync(out, dbuf + qb + wb, ob, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy walk outputs"); break; }
    } while (0);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(e, "sms_ss_walk_batch");
    return check_device_error(c);
}

// ------------------------------------------------- accessors for other TUs
bool ctx_swap_config(sms_ctx *c, const sms_config *in, sms_config *old) {
    if (!c || !in || validate_cfg(in) != SMS_OK) return false;
    if (old) *old = c->cfg;
    c->cfg = *in;
    return true;
}

bool ctx_view(sms_ctx *c, CtxView &out) {
    if (!c) return false;
    out.device = c->device;
    out.stream = c->stream;
    out.scene = &c->dsc;
    out.solver = solver_cfg(c->cfg);
    out.counters = c->ctr;
    out.num_sms = c->num_sms;
    out.blocks_per_sm = c->blocks_per_sm;
    out.timer = &c->timer;
    out.frames = c->frames.data();
    out.n_shapes = (int)c->frames.size();
    out.proposal_bound = c->prop != nullptr;
    out.trial_group = c->trial_group;
    out.bounces = c->cfg.bounces;
    out.bsdf_strategy_only = c->cfg.bsdf_strategy_only;
    out.nm_rough = c->nm_rough;
    out.sms_strategy_only = c->cfg.sms_strategy_only;
    return true;
}

int set_last_error_impl(int st, const char *msg) {
    g_last_error = msg ? msg : "";
    return st;
}

// -------------------------------------------------------------- multi scatter
static sms_status check_ms_cfg(sms_ctx *c) {
    if (c->cfg.bounces < 1 || c->cfg.bounces > kMaxBounces)
        return fail(SMS_ERR_UNSUPPORTED, "bounces must be between 1 and 4");
    if (c->ms_rough && c->ms_nm)
        return fail(SMS_ERR_UNSUPPORTED, "rough (alpha > 0) normal-mapped multi-scatter chain shapes are not supported");
    return SMS_OK;
}

sms_status ctx_ms_connect(sms_ctx *c, const float *q, uint32_t n, uint64_t seed, uint64_t stream_off,
                          const uint64_t *streams, sms_result *out) {
    if (!c || !out || (n && (!q || !out->value || !out->count || !out->walks)))
        return fail(SMS_ERR_INVALID_ARG, "sms_ms_connect_batch_device: null argument");
    if (sms_status st = check_ms_cfg(c)) return st;
    if (n == 0) return SMS_OK;
    if (c->cfg.biased && c->cfg.max_trials > (1 << 24))
        return fail(SMS_ERR_INVALID_ARG, "max_trials too large for the biased estimator");
    CUDA_TRY(cudaSetDevice(c->device));
    SsScratch scr{};
    if (!c->cfg.biased) {
        if (sms_status st = ensure_scratch(c, n, scr)) return st;
        if (c->ms_tmpl_n < n) {
            if (c->ms_tmpl) {
                CUDA_TRY(cudaStreamSynchronize(c->stream));
                cudaFree(c->ms_tmpl);
                c->ms_tmpl = nullptr;
                c->ms_tmpl_n = 0;
            }
            // template shapes (kMaxBounces rows), then the template's offset
            // normals (3 kMaxBounces rows) and their density (1 row)
            CUDA_TRY(cudaMalloc(&c->ms_tmpl, (size_t)(4 * kMaxBounces + 1) * n * sizeof(int)));
            c->ms_tmpl_n = n;
        }
    }
    SolverCfg sc = solver_cfg(c->cfg);
    sc.streams = streams;
    CUDA_TRY(launch_ms_connect(c->dsc, sc, c->cfg.bounces, q, n, seed, stream_off, out->value, out->count,
                               out->walks, c->ctr, scr, c->ms_tmpl, c->num_sms, c->blocks_per_sm, &c->timer,
                               c->stream));
    return SMS_OK;
}

extern "C" sms_status sms_ms_connect_batch_device(sms_ctx *c, const float *q, uint32_t n, uint64_t seed,
                                                  uint64_t stream_off, sms_result *out) {
    return ctx_ms_connect(c, q, n, seed, stream_off, nullptr, out);
}

extern "C" sms_status sms_ms_connect_batch(sms_ctx *c, const float *q, uint32_t n, uint64_t seed,
                                           uint64_t stream_off, sms_result *out) {
    if (!c || !out || (n && (!q || !out->value || !out->count || !out->walks)))
        return fail(SMS_ERR_INVALID_ARG, "sms_ms_connect_batch: null argument");
    if (sms_status st = check_ms_cfg(c)) return st;
    if (n == 0) return SMS_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    size_t qb = (size_t)SMS_QUERY_FIELDS * n * sizeof(float);
    size_t vb = 3 * (size_t)n * sizeof(float), ib = (size_t)n * sizeof(int32_t);
    if (sms_status st = ensure_io(c, qb + vb + 2 * ib)) return st;
    char *dbuf = reinterpret_cast<char *>(c->io);
    float *dq = reinterpret_cast<float *>(dbuf);
    sms_result r{reinterpret_cast<float *>(dbuf + qb), reinterpret_cast<int32_t *>(dbuf + qb + vb),
                 reinterpret_cast<int32_t *>(dbuf + qb + vb + ib)};
    sms_status st = SMS_OK;
    do {
        cudaError_t e = cudaMemcpyAsync(dq, q, qb, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy queries"); break; }
        st = sms_ms_connect_batch_device(c, dq, n, seed, stream_off, &r);
        if (st) break;
        e = cudaMemcpyAsync(out->value, r.value, vb, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->count, r.count, ib, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->walks, r.walks, ib, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy results"); break; }
    } while (0);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(e, "sms_ms_connect_batch");
    return check_device_error(c);
}

extern "C" sms_status sms_ms_walk_batch(sms_ctx *c, int32_t caster, const float *q, const float *w, uint32_t n,
                                        float *out) {
    if (!c || (n && (!q || !w || !out))) return fail(SMS_ERR_INVALID_ARG, "sms_ms_walk_batch: null argument");
    if (caster < 0 || caster >= c->dsc.n_shapes) return fail(SMS_ERR_INVALID_ARG, "unknown caster shape id");
    if (sms_status st = check_ms_cfg(c)) return st;
    if (n == 0) return SMS_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    size_t qb = (size_t)SMS_QUERY_FIELDS * n * sizeof(float), wb = (size_t)SMS_WALK_IN_FIELDS * n * sizeof(float),
           ob = (size_t)SMS_MS_WALK_OUT_FIELDS * n * sizeof(float);
    if (sms_status st = ensure_io(c, qb + wb + ob)) return st;
    char *dbuf = reinterpret_cast<char *>(c->io);
    sms_status st = SMS_OK;
    do {
        cudaError_t e = cudaMemcpyAsync(dbuf, q, qb, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dbuf + qb, w, wb, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy walk inputs"); break; }
        e = launch_ms_walk(c->dsc, solver_cfg(c->cfg), c->cfg.bounces, caster, reinterpret_cast<float *>(dbuf),
                           reinterpret_cast<float *>(dbuf + qb), n, reinterpret_cast<float *>(dbuf + qb + wb), c->ctr,
                           &c->timer, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "launch ms_walk"); break; }
        e = cudaMemcpyAsync(out, dbuf + qb + wb, ob, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy walk outputs"); break; }
    } while (0);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(e, "sms_ms_walk_batch");
    return check_device_error(c);
}

// --------------------------------------------------------------------- glints
static sms_status check_glint_scene(sms_ctx *c) {
    if (c->dsc.glinty_shape < 0 || c->dsc.nmap_res == 0)
        return fail(SMS_ERR_INVALID_ARG, "the scene has no normal map (sms_scene_set_normalmap)");
    return SMS_OK;
}

sms_status ctx_glint_connect(sms_ctx *c, const float *q, uint32_t n, uint64_t seed, uint64_t stream_off,
                             const uint64_t *streams, sms_result *out) {
    if (!c || !out || (n && (!q || !out->value || !out->count || !out->walks)))
        return fail(SMS_ERR_INVALID_ARG, "sms_glint_connect_batch_device: null argument");
    if (sms_status st = check_glint_scene(c)) return st;
    if (n == 0) return SMS_OK;
    if (c->cfg.biased && c->cfg.max_trials > (1 << 24))
        return fail(SMS_ERR_INVALID_ARG, "max_trials too large for the biased estimator");
    CUDA_TRY(cudaSetDevice(c->device));
    SsScratch scr{};
    if (!c->cfg.biased)
        if (sms_status st = ensure_scratch(c, n, scr)) return st;
    SolverCfg sc = solver_cfg(c->cfg);
    sc.streams = streams;
    CUDA_TRY(launch_glint_connect(c->dsc, sc, q, n, seed, stream_off, out->value, out->count, out->walks, c->ctr,
                                  scr, c->num_sms, c->blocks_per_sm, &c->timer, c->stream));
    return SMS_OK;
}

extern "C" sms_status sms_glint_connect_batch_device(sms_ctx *c, const float *q, uint32_t n, uint64_t seed,
                                                     uint64_t stream_off, sms_result *out) {
    return ctx_glint_connect(c, q, n, seed, stream_off, nullptr, out);
}

void ctx_set_render_spp(sms_ctx *c, uint32_t spp) {
    if (c) c->render_spp = spp;
}

extern "C" uint32_t sms_render_spp_done(const sms_ctx *c) { return c ? c->render_spp : 0u; }

sms_status ctx_ensure_lean(sms_ctx *c) {
    if (sms_status st = check_glint_scene(c)) return st;
    return ctx_build_lean(c);
}

sms_status ctx_build_lean(sms_ctx *c) {
    if (c->lean) return SMS_OK;
    if (c->dsc.nmap_res == 0) return fail(SMS_ERR_INVALID_ARG, "the scene has no normal map (sms_scene_set_normalmap)");
    const uint32_t res = c->dsc.nmap_res;
    if (res & (res - 1)) return fail(SMS_ERR_UNSUPPORTED, "the LEAN pyramid needs a power-of-two slope map");
    int levels = 0;
    size_t total = 0;
    uint32_t offs[kMaxLeanLevels];
    for (uint32_t r = res; r >= 1 && levels < kMaxLeanLevels; r /= 2) {
        offs[levels++] = (uint32_t)total;
        total += 5 * (size_t)r * r;
        if (r == 1) break;
    }
    if (total > 0xffffffffull) return fail(SMS_ERR_UNSUPPORTED, "slope map too large for the LEAN pyramid");
    CUDA_TRY(cudaSetDevice(c->device));
    void *p = nullptr;
    CUDA_TRY(cudaMalloc(&p, total * sizeof(float)));
    c->lean = reinterpret_cast<float *>(p);
    CUDA_TRY(launch_lean_build(c->dsc, c->lean, offs, levels, c->stream));
    c->dsc.lean = c->lean;
    for (int l = 0; l < levels; ++l) c->dsc.lean_off[l] = offs[l];
    c->dsc.lean_levels = levels;
    return SMS_OK;
}

extern "C" sms_status sms_glint_connect_batch(sms_ctx *c, const float *q, uint32_t n, uint64_t seed,
                                              uint64_t stream_off, sms_result *out) {
    if (!c || !out || (n && (!q || !out->value || !out->count || !out->walks)))
        return fail(SMS_ERR_INVALID_ARG, "sms_glint_connect_batch: null argument");
    if (sms_status st = check_glint_scene(c)) return st;
    if (n == 0) return SMS_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    size_t qb = (size_t)SMS_GLINT_QUERY_FIELDS * n * sizeof(float);
    size_t vb = 3 * (size_t)n * sizeof(float), ib = (size_t)n * sizeof(int32_t);
    if (sms_status st = ensure_io(c, qb + vb + 2 * ib)) return st;
    char *dbuf = reinterpret_cast<char *>(c->io);
    float *dq = reinterpret_cast<float *>(dbuf);
    sms_result r{reinterpret_cast<float *>(dbuf + qb), reinterpret_cast<int32_t *>(dbuf + qb + vb),
                 reinterpret_cast<int32_t *>(dbuf + qb + vb + ib)};
    sms_status st = SMS_OK;
    do {
        cudaError_t e = cudaMemcpyAsync(dq, q, qb, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy queries"); break; }
        st = sms_glint_connect_batch_device(c, dq, n, seed, stream_off, &r);
        if (st) break;
        e = cudaMemcpyAsync(out->value, r.value, vb, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->count, r.count, ib, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->walks, r.walks, ib, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy results"); break; }
    } while (0);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(e, "sms_glint_connect_batch");
    return check_device_error(c);
}

extern "C" sms_status sms_glint_walk_batch(sms_ctx *c, const float *q, const float *w, uint32_t n, float *out) {
    if (!c || (n && (!q || !w || !out))) return fail(SMS_ERR_INVALID_ARG, "sms_glint_walk_batch: null argument");
    if (sms_status st = check_glint_scene(c)) return st;
    if (n == 0) return SMS_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    size_t qb = (size_t)SMS_GLINT_QUERY_FIELDS * n * sizeof(float),
           wb = (size_t)SMS_GLINT_WALK_IN_FIELDS * n * sizeof(float),
           ob = (size_t)SMS_GLINT_WALK_OUT_FIELDS * n * sizeof(float);
    if (sms_status st = ensure_io(c, qb + wb + ob)) return st;
    char *dbuf = reinterpret_cast<char *>(c->io);
    sms_status st = SMS_OK;
    do {
        cudaError_t e = cudaMemcpyAsync(dbuf, q, qb, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dbuf + qb, w, wb, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy walk inputs"); break; }
        e = launch_glint_walk(c->dsc, solver_cfg(c->cfg), reinterpret_cast<float *>(dbuf),
                              reinterpret_cast<float *>(dbuf + qb), n, reinterpret_cast<float *>(dbuf + qb + wb),
                              c->ctr, &c->timer, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "launch glint_walk"); break; }
        e = cudaMemcpyAsync(out, dbuf + qb + wb, ob, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) { st = cuda_fail(e, "copy walk outputs"); break; }
    } while (0);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (st) return st;
    if (e != cudaSuccess) return cuda_fail(e, "sms_glint_walk_batch");
    return check_device_error(c);
}
