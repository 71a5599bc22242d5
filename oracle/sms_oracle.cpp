/*
 * sms_oracle.cpp -- CPU oracle for the Specular Manifold Sampling hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a scalar, one-walk-per-thread
 * restatement of the reference's scalar_rgb SMS code.  It is the checker the
 * GPU library is compared against, and the CPU baseline bench.py times; the
 * library itself never links, loads or calls it.
 *
 * Parity status: the reference (Mitsuba 2 + SMS) cannot be built in this
 * environment (its enoki/tbb/pybind11 submodules are empty), so no output of the
 * reference itself pins this file.  It is pinned against (a) the known-answer
 * values of the reference's own dependency tests (Fresnel, warps) and (b)
 * analytic solutions of the specular constraint computed independently in FP64
 * (tests/golden/).  SMS-level outputs are otherwise "parity unpinned".
 *
 * All arithmetic is FP32 like scalar_rgb, except the sphere intersection, which
 * the reference does in FP64 (src/shapes/sphere.cpp:275-297).  Build with
 * -ffp-contract=off so x86-64 and aarch64 produce the same results.
 *
 * Every function cites the reference lines it restates (paths relative to the
 * reference project root).
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <type_traits>
#include <vector>

#include "../include/sms_gb300.h"

#if defined(ORC_OPCOUNT)
#include "op_count.h"
#endif

namespace orc {

/* The scalar type of every walk computation.  float is the oracle proper;
 * liboracle_f64.so builds the same source with double (the basin classifier:
 * a walk whose outcome is the same in FP32, FP32 with FMA contraction and FP64
 * is well conditioned), and liboracle_ops.so with the counting float of
 * op_count.h (algorithmic FLOPs; results identical to the float build). */
#if defined(ORC_OPCOUNT)
typedef orc_opcount::CFloat Float;
#define ORC_COUNT_FP64_OPS(n) (orc_opcount::counters().add += (n))
#define ORC_TRAVERSAL_SCOPE(is_tri) orc_opcount::TraversalScope orc_scope_(is_tri)
#define ORC_COUNT_RAY() (++orc_opcount::counters().rays)
#elif defined(ORC_DOUBLE)
typedef double Float;
#define ORC_COUNT_FP64_OPS(n) ((void)0)
#define ORC_TRAVERSAL_SCOPE(is_tri) ((void)0)
#define ORC_COUNT_RAY() ((void)0)
#else
typedef float Float;
#define ORC_COUNT_FP64_OPS(n) ((void)0)
#define ORC_TRAVERSAL_SCOPE(is_tri) ((void)0)
#define ORC_COUNT_RAY() ((void)0)
#endif

/* std::max / std::min for operands that may differ in type (a Float and a
 * float literal when Float is double); same selection rule as std::max/min. */
template <class A, class B>
static inline typename std::common_type<A, B>::type omax(A a, B b) {
    typedef typename std::common_type<A, B>::type T;
    return ((T)a < (T)b) ? (T)b : (T)a;
}
template <class A, class B>
static inline typename std::common_type<A, B>::type omin(A a, B b) {
    typedef typename std::common_type<A, B>::type T;
    return ((T)b < (T)a) ? (T)b : (T)a;
}

static const Float kInf = std::numeric_limits<float>::infinity();
static const Float kPi = 3.14159265358979323846f;
static const Float kInvPi = 0.31830988618379067154f;
/* include/mitsuba/core/math.h:37-38 */
static const Float kRayEps = (std::numeric_limits<float>::epsilon() / 2.f) * 1500.f;
static const Float kShadowEps = kRayEps * 10.f;

/* ------------------------------------------------------------ vector math */
struct V3 {
    Float x = 0.f, y = 0.f, z = 0.f;
    V3() {}
    V3(Float a) : x(a), y(a), z(a) {}
    V3(Float a, Float b, Float c) : x(a), y(b), z(c) {}
    Float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3 operator*(V3 a, Float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(Float s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 &operator+=(V3 &a, V3 b) { a = a + b; return a; }
static inline V3 &operator-=(V3 &a, V3 b) { a = a - b; return a; }
static inline V3 &operator*=(V3 &a, Float s) { a = a * s; return a; }
static inline Float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline Float norm(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 normalize(V3 a) { return a * (1.f / norm(a)); }
static inline Float hmax_abs(V3 a) {
    return omax(std::fabs(a.x), omax(std::fabs(a.y), std::fabs(a.z)));
}
static inline Float safe_sqrt(Float v) { return std::sqrt(omax(v, 0.f)); }
static inline Float safe_acos(Float v) { return std::acos(omin(1.f, omax(-1.f, v))); }
static inline Float safe_asin(Float v) { return std::asin(omin(1.f, omax(-1.f, v))); }

struct V2 { Float x = 0.f, y = 0.f; };

/* 2x2 matrix, row-major m[r][c] */
struct M2 {
    Float m[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
};
static inline Float det(const M2 &a) { return a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]; }
static inline M2 inverse(const M2 &a) {
    Float id = 1.f / det(a);
    M2 r;
    r.m[0][0] = a.m[1][1] * id;  r.m[0][1] = -a.m[0][1] * id;
    r.m[1][0] = -a.m[1][0] * id; r.m[1][1] = a.m[0][0] * id;
    return r;
}
static inline M2 mul(const M2 &a, const M2 &b) {
    M2 r;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j];
    return r;
}
static inline V2 mul(const M2 &a, V2 v) {
    return {a.m[0][0] * v.x + a.m[0][1] * v.y, a.m[1][0] * v.x + a.m[1][1] * v.y};
}

/* Orthonormal basis of Duff et al. 2017, as used by the reference's
 * coordinate_system (include/mitsuba/core/vector.h:116-135). */
static void coordinate_system(V3 n, V3 &s, V3 &t) {
    Float sign = std::copysign(1.f, n.z);
    Float a = -1.f / (sign + n.z);
    Float b = n.x * n.y * a;
    s = V3(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    t = V3(b, sign + n.y * n.y * a, -n.y);
}

/* ------------------------------------------------------------------ PCG32 */
/* O'Neill's PCG32 (XSH-RR 64/32), the generator behind the reference's
 * independent sampler (include/mitsuba/core/random.h:50-52).  Floats take the
 * high 23 bits as the mantissa of a number in [1, 2). */
struct PCG32 {
    uint64_t state = 0, inc = 1;
    void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next_u32();
        state += initstate;
        next_u32();
    }
    uint32_t next_u32() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((~rot + 1u) & 31u));
    }
    Float next_f32() {
        uint32_t bits = (next_u32() >> 9) | 0x3f800000u;
        float f;
        std::memcpy(&f, &bits, 4);
        return Float(f - 1.f);
    }
    V2 next_2d() { V2 r; r.x = next_f32(); r.y = next_f32(); return r; }
};

/* ------------------------------------------------------------------ scene */
/* roughplastic's precomputed coating terms (roughplastic.cpp:364-396):
 * external transmittance at 64 cosines, internal diffuse reflectance,
 * specular sampling weight */
constexpr int kRoughPlasticRes = 64;   /* MTS_ROUGH_TRANSMITTANCE_RES */
struct RoughPlastic {
    Float t[kRoughPlasticRes] = {};
    Float fdr = 0.f, ws = 0.f;
};

struct Shape {
    int kind = 0; /* 0 sphere, 1 mesh */
    V3 center; Float radius = 1.f; bool flip = false;
    std::vector<V3> P, N;
    std::vector<V2> UV;
    std::vector<uint32_t> F;
    std::vector<Float> pmf, cdf; /* area distribution over faces */
    Float area_sum = 0.f, area_norm = 0.f;
    uint32_t valid_lo = 0, valid_hi = 0;
    sms_bsdf bsdf{};
    RoughPlastic rp;  /* set for SMS_BSDF_ROUGHPLASTIC */
    uint32_t flags = 0;
    int emitter = -1;
    V3 bbox_center;   /* Shape::bbox().center(), for the MNEE initialisation */
};

struct Emitter {
    int kind = 0; /* 0 point, 1 area (sphere shape) */
    V3 p; V3 radiance; int shape = -1; uint32_t flags = 0;
};

struct BNode { Float lo[3], hi[3]; int left = -1, right = -1; uint32_t first = 0, count = 0; int axis = 0; };

/* Slope-based normal map, level 0 (channels sx, sy of the reference's LEAN
 * data, src/librender/normalmap.cpp:7-36), stored as FP16 by the library and
 * widened to FP32 here. */
struct NormalMap {
    uint32_t res = 0;
    Float tiles = 1.f;
    std::vector<Float> sx, sy;
    /* LEAN mip pyramid (src/librender/normalmap.cpp:36-89): per level, 5
     * floats per texel (sx, sy, sx^2 + s0, sy^2 + s0, sx sy); built on first use */
    std::vector<std::vector<Float>> lean;
};

/* The normal map's LEAN fallback BSDF (normalmap.cpp:46-55), off by default. */
struct LeanFallback {
    bool on = false;
    Float alpha = 1e-4f, eta = 0.f, k = 1.f;
};

struct Scene {
    std::vector<Shape> shapes;
    std::vector<Emitter> emitters;
    std::vector<int> emitters_all;
    NormalMap nmap;
    LeanFallback lean_fb;
    int glinty_shape = -1;
    /* triangle BVH over all mesh shapes: primitive = (shape, face) */
    std::vector<uint32_t> tri_shape, tri_face;
    std::vector<BNode> nodes;
    std::vector<int> casters_ss, casters_ms, bouncers, emitters_ss, emitters_ms;
    bool finalized = false;
};

/* Surface interaction: the subset of the reference's SurfaceInteraction3f the
 * SMS path reads (include/mitsuba/render/interaction.h). */
struct SI {
    Float t = kInf;
    V3 p, n, shn, dp_du, dp_dv;
    V2 uv;
    int shape = -1;
    uint32_t prim = 0;
    bool valid() const { return t != kInf; }
};

struct Ray {
    V3 o, d;
    Float mint = kRayEps, maxt = kInf;
};

/* ---- sphere: src/shapes/sphere.cpp:275-297 (FP64 quadratic), math.h:371 */
static bool solve_quadratic(double a, double b, double c, double &x0, double &x1) {
    bool linear = (a == 0.0);
    bool active = !linear || (b > 0.0);
    x0 = x1 = -c / b;
    double discrim = b * b - 4.0 * a * c;
    active = active && (linear || discrim >= 0.0);
    if (active && !linear) {
        double sq = std::sqrt(discrim);
        double temp = -0.5 * (b + std::copysign(sq, b));
        double x0p = temp / a, x1p = c / temp;
        x0 = omin(x0p, x1p);
        x1 = omax(x0p, x1p);
    }
    return active;
}

static bool sphere_intersect(const Shape &s, const Ray &r, Float &t_out) {
    ORC_COUNT_FP64_OPS(31);   /* the FP64 arithmetic below: 30 add/mul/div + 1 sqrt */
    double mint = (double)r.mint, maxt = (double)r.maxt;
    double ox = (double)r.o.x - (double)s.center.x, oy = (double)r.o.y - (double)s.center.y,
           oz = (double)r.o.z - (double)s.center.z;
    double dx = (double)r.d.x, dy = (double)r.d.y, dz = (double)r.d.z;
    double A = dx * dx + dy * dy + dz * dz;
    double B = 2.0 * (ox * dx + oy * dy + oz * dz);
    double C = ox * ox + oy * oy + oz * oz - (double)s.radius * (double)s.radius;
    double n0, f0;
    bool found = solve_quadratic(A, B, C, n0, f0);
    bool out_bounds = !(n0 <= maxt && f0 >= mint);
    bool in_bounds = n0 < mint && f0 > maxt;
    if (!(found && !out_bounds && !in_bounds)) return false;
    t_out = (Float)(n0 < mint ? f0 : n0);
    return true;
}

/* src/shapes/sphere.cpp:322-382 (uv, dp_du, dp_dv; no rotation in to_world) */
static void sphere_fill(const Shape &s, const Ray &r, SI &si) {
    V3 hit = r.o + r.d * si.t;
    V3 n = normalize(hit - s.center);
    si.p = n * s.radius + s.center;
    V3 local = (si.p - s.center) * (1.f / s.radius);
    Float rd2 = local.x * local.x + local.y * local.y;
    /* angle to +z, robust form: 2 asin(|v - (0,0,+-1)| / 2) */
    Float sz = std::copysign(1.f, local.z);
    Float tmp = 2.f * safe_asin(0.5f * norm(V3(local.x, local.y, local.z - sz)));
    Float theta = local.z >= 0.f ? tmp : kPi - tmp;
    Float phi = std::atan2(local.y, local.x);
    if (phi < 0.f) phi += 2.f * kPi;
    si.uv.x = phi * (0.5f / kPi);
    si.uv.y = theta * (1.f / kPi);
    V3 dpdu(-local.y, local.x, 0.f);
    Float rd = std::sqrt(rd2), inv_rd = 1.f / rd;
    Float cphi = local.x * inv_rd, sphi = local.y * inv_rd;
    V3 dpdv(local.z * cphi, local.z * sphi, -rd);
    if (rd == 0.f) dpdv = V3(1.f, 0.f, 0.f);
    si.dp_du = dpdu * (s.radius * 2.f * kPi);
    si.dp_dv = dpdv * (s.radius * kPi);
    if (s.flip) n = -n;
    si.n = n;
    si.shn = n;
}

/* ---- triangles: include/mitsuba/render/mesh.h:203-228 (Moller-Trumbore) */
static bool tri_intersect(const Shape &m, uint32_t f, const Ray &r, Float &u, Float &v, Float &t) {
    ORC_TRAVERSAL_SCOPE(true);
    V3 p0 = m.P[m.F[3 * f]], p1 = m.P[m.F[3 * f + 1]], p2 = m.P[m.F[3 * f + 2]];
    V3 e1 = p1 - p0, e2 = p2 - p0;
    V3 pvec = cross(r.d, e2);
    Float inv_det = 1.f / dot(e1, pvec);
    V3 tvec = r.o - p0;
    u = dot(tvec, pvec) * inv_det;
    bool active = u >= 0.f && u <= 1.f;
    V3 qvec = cross(tvec, e1);
    v = dot(r.d, qvec) * inv_det;
    active = active && v >= 0.f && u + v <= 1.f;
    t = dot(e2, qvec) * inv_det;
    active = active && t >= r.mint && t <= r.maxt;
    return active;
}

/* src/librender/mesh.cpp:618-687 */
static void mesh_fill(const Shape &m, Float b1, Float b2, SI &si) {
    uint32_t f = si.prim;
    uint32_t i0 = m.F[3 * f], i1 = m.F[3 * f + 1], i2 = m.F[3 * f + 2];
    Float b0 = 1.f - b1 - b2;
    V3 p0 = m.P[i0], p1 = m.P[i1], p2 = m.P[i2];
    V3 dp0 = p1 - p0, dp1 = p2 - p0;
    si.p = p0 * b0 + p1 * b1 + p2 * b2;
    V3 n = normalize(cross(dp0, dp1));
    si.n = n;
    V3 dpdu, dpdv;
    coordinate_system(n, dpdu, dpdv);
    V2 uv0, uv1, uv2;
    if (!m.UV.empty()) { uv0 = m.UV[i0]; uv1 = m.UV[i1]; uv2 = m.UV[i2]; }
    else { uv0 = {0.f, 0.f}; uv1 = {1.f, 0.f}; uv2 = {0.f, 1.f}; }
    /* use_default_uv_parameterization defaults to true (mesh.cpp:42) */
    V2 uv;
    uv.x = uv0.x * b0 + uv1.x * b1 + uv2.x * b2;
    uv.y = uv0.y * b0 + uv1.y * b1 + uv2.y * b2;
    V2 duv0{uv1.x - uv0.x, uv1.y - uv0.y}, duv1{uv2.x - uv0.x, uv2.y - uv0.y};
    Float dt = duv0.x * duv1.y - duv0.y * duv1.x;
    if (dt != 0.f) {
        Float inv = 1.f / dt;
        dpdu = (dp0 * duv1.y - dp1 * duv0.y) * inv;
        dpdv = (dp1 * duv0.x - dp0 * duv1.x) * inv;
    }
    si.uv = uv;
    if (!m.N.empty()) n = normalize(m.N[i0] * b0 + m.N[i1] * b1 + m.N[i2] * b2);
    si.shn = n;
    si.dp_du = dpdu;
    si.dp_dv = dpdv;
}

/* src/librender/mesh.cpp:693-765 (needs vertex normals; none -> flat, as the
 * reference's rectangle, src/shapes/rectangle.cpp:210-214) */
static void mesh_normal_derivative(const Shape &m, const SI &si, V3 &dndu, V3 &dndv) {
    if (m.N.empty()) { dndu = V3(0.f); dndv = V3(0.f); return; }
    uint32_t f = si.prim;
    uint32_t i0 = m.F[3 * f], i1 = m.F[3 * f + 1], i2 = m.F[3 * f + 2];
    V3 p0 = m.P[i0], p1 = m.P[i1], p2 = m.P[i2];
    V3 n0 = m.N[i0], n1 = m.N[i1], n2 = m.N[i2];
    V3 rel = si.p - p0, du = p1 - p0, dv = p2 - p0;
    Float b1 = dot(du, rel), b2 = dot(dv, rel), a11 = dot(du, du), a12 = dot(du, dv),
          a22 = dot(dv, dv);
    Float inv_det = 1.f / (a11 * a22 - a12 * a12);
    Float u = (a22 * b1 - a12 * b2) * inv_det, v = (a11 * b2 - a12 * b1) * inv_det,
          w = 1.f - u - v;
    V3 N = n1 * u + n2 * v + n0 * w;
    Float il = 1.f / std::sqrt(dot(N, N));
    N *= il;
    dndu = (n1 - n0) * il;
    dndv = (n2 - n0) * il;
    dndu = dndu - N * dot(N, dndu);
    dndv = dndv - N * dot(N, dndv);
    V2 uv0, uv1, uv2;
    if (!m.UV.empty()) { uv0 = m.UV[i0]; uv1 = m.UV[i1]; uv2 = m.UV[i2]; }
    else { uv0 = {0.f, 0.f}; uv1 = {1.f, 0.f}; uv2 = {0.f, 1.f}; }
    V2 duv1{uv1.x - uv0.x, uv1.y - uv0.y}, duv2{uv2.x - uv0.x, uv2.y - uv0.y};
    Float id = 1.f / (duv1.x * duv2.y - duv1.y * duv2.x);
    V3 a = (dndu * duv2.y - dndv * duv1.y) * id;
    V3 b = (dndv * duv1.x - dndu * duv2.x) * id;
    dndu = a;
    dndv = b;
}

/* ---- oracle BVH: binned SAH (16 bins per axis, leaves of at most 4
 * triangles), exact closest hit.  Any exact structure gives the reference
 * kd-tree's closest-hit result; the SAH split only makes the CPU baseline
 * traverse fewer nodes. */
static void bvh_bounds(const Scene &sc, uint32_t prim, Float lo[3], Float hi[3], Float c[3]) {
    const Shape &m = sc.shapes[sc.tri_shape[prim]];
    uint32_t f = sc.tri_face[prim];
    for (int k = 0; k < 3; ++k) { lo[k] = kInf; hi[k] = -kInf; }
    for (int j = 0; j < 3; ++j) {
        V3 p = m.P[m.F[3 * f + j]];
        for (int k = 0; k < 3; ++k) { lo[k] = omin(lo[k], p[k]); hi[k] = omax(hi[k], p[k]); }
    }
    for (int k = 0; k < 3; ++k) c[k] = 0.5f * (lo[k] + hi[k]);
}

/* Half surface area of a box given as lo/hi arrays (doubles: build only). */
static double bvh_half_area(const double lo[3], const double hi[3]) {
    double d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
    if (d0 < 0 || d1 < 0 || d2 < 0) return 0.0;
    return d0 * d1 + d1 * d2 + d2 * d0;
}

static int bvh_build_rec(Scene &sc, std::vector<uint32_t> &idx, std::vector<Float> &cen,
                         uint32_t first, uint32_t count, std::vector<BNode> &out) {
    const int kBins = 16;
    BNode node;
    for (int k = 0; k < 3; ++k) { node.lo[k] = kInf; node.hi[k] = -kInf; }
    Float clo[3] = {kInf, kInf, kInf}, chi[3] = {-kInf, -kInf, -kInf};
    for (uint32_t i = first; i < first + count; ++i) {
        Float lo[3], hi[3], c[3];
        bvh_bounds(sc, idx[i], lo, hi, c);
        for (int k = 0; k < 3; ++k) {
            node.lo[k] = omin(node.lo[k], lo[k]); node.hi[k] = omax(node.hi[k], hi[k]);
            clo[k] = omin(clo[k], c[k]); chi[k] = omax(chi[k], c[k]);
        }
    }
    /* pad so that Float rounding in the slab test never drops a triangle that
       the exact triangle test would accept */
    for (int k = 0; k < 3; ++k) {
        Float pad = 1e-6f * omax(1.f, omax(std::fabs(node.lo[k]), std::fabs(node.hi[k])));
        node.lo[k] -= pad; node.hi[k] += pad;
    }
    int id = (int)out.size();
    out.push_back(node);
    if (count <= 4) { out[id].first = first; out[id].count = count; return id; }
    /* binned SAH over the centroid bounds */
    int best_axis = -1, best_split = 0;
    double best_cost = std::numeric_limits<double>::infinity();
    for (int axis = 0; axis < 3; ++axis) {
        double ext = (double)chi[axis] - (double)clo[axis];
        if (!(ext > 0.0)) continue;
        uint32_t cnt[kBins] = {};
        double blo[kBins][3], bhi[kBins][3];
        for (int b = 0; b < kBins; ++b)
            for (int k = 0; k < 3; ++k) { blo[b][k] = 1e30; bhi[b][k] = -1e30; }
        for (uint32_t i = first; i < first + count; ++i) {
            int b = (int)(kBins * (((double)cen[3 * idx[i] + axis] - (double)clo[axis]) / ext));
            b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
            Float lo[3], hi[3], c[3];
            bvh_bounds(sc, idx[i], lo, hi, c);
            ++cnt[b];
            for (int k = 0; k < 3; ++k) {
                blo[b][k] = std::min(blo[b][k], (double)lo[k]);
                bhi[b][k] = std::max(bhi[b][k], (double)hi[k]);
            }
        }
        double rarea[kBins]; uint32_t rcnt[kBins];
        double acc_lo[3] = {1e30, 1e30, 1e30}, acc_hi[3] = {-1e30, -1e30, -1e30};
        uint32_t acc = 0;
        for (int b = kBins - 1; b > 0; --b) {
            for (int k = 0; k < 3; ++k) { acc_lo[k] = std::min(acc_lo[k], blo[b][k]); acc_hi[k] = std::max(acc_hi[k], bhi[b][k]); }
            acc += cnt[b];
            rarea[b] = bvh_half_area(acc_lo, acc_hi); rcnt[b] = acc;
        }
        double l_lo[3] = {1e30, 1e30, 1e30}, l_hi[3] = {-1e30, -1e30, -1e30};
        uint32_t lc = 0;
        for (int b = 0; b < kBins - 1; ++b) {
            for (int k = 0; k < 3; ++k) { l_lo[k] = std::min(l_lo[k], blo[b][k]); l_hi[k] = std::max(l_hi[k], bhi[b][k]); }
            lc += cnt[b];
            if (lc == 0 || rcnt[b + 1] == 0) continue;
            double cost = bvh_half_area(l_lo, l_hi) * lc + rarea[b + 1] * rcnt[b + 1];
            if (cost < best_cost) { best_cost = cost; best_axis = axis; best_split = b; }
        }
    }
    uint32_t mid;
    int axis = best_axis;
    if (axis >= 0) {
        double ext = (double)chi[axis] - (double)clo[axis];
        auto it = std::partition(idx.begin() + first, idx.begin() + first + count, [&](uint32_t a) {
            int b = (int)(kBins * (((double)cen[3 * a + axis] - (double)clo[axis]) / ext));
            b = b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
            return b <= best_split;
        });
        mid = (uint32_t)(it - idx.begin());
    } else {
        /* every centroid coincides: split the range in half */
        axis = 0;
        mid = first + count / 2;
    }
    if (mid == first || mid == first + count) mid = first + count / 2;
    int l = bvh_build_rec(sc, idx, cen, first, mid - first, out);
    int r = bvh_build_rec(sc, idx, cen, mid, first + count - mid, out);
    out[id].left = l; out[id].right = r; out[id].count = 0; out[id].axis = axis;
    return id;
}

static bool box_hit(const BNode &n, const Ray &r, Float tmax) {
    ORC_TRAVERSAL_SCOPE(false);
    Float t0 = r.mint, t1 = tmax;
    for (int k = 0; k < 3; ++k) {
        Float inv = 1.f / r.d[k];
        Float a = (n.lo[k] - r.o[k]) * inv, b = (n.hi[k] - r.o[k]) * inv;
        if (a > b) std::swap(a, b);
        /* NaN (0 * inf) leaves the interval unchanged */
        if (a > t0) t0 = a;
        if (b < t1) t1 = b;
        if (t0 > t1) return false;
    }
    return true;
}

/* Scene::ray_intersect (src/librender/scene.cpp:123-131, kdtree.h:2334-2366) */
static bool ray_is_nan(const Ray &r) {
    return std::isnan(r.o.x) || std::isnan(r.o.y) || std::isnan(r.o.z) || std::isnan(r.d.x) ||
           std::isnan(r.d.y) || std::isnan(r.d.z);
}

static SI ray_intersect(const Scene &sc, const Ray &ray) {
    ORC_COUNT_RAY();
    SI si;
    /* a NaN ray hits nothing (all intersection comparisons are false) */
    if (ray_is_nan(ray)) return si;
    Float best = ray.maxt;
    int best_shape = -1; uint32_t best_prim = 0; Float bu = 0.f, bv = 0.f;
    bool hit = false;
    for (size_t s = 0; s < sc.shapes.size(); ++s) {
        if (sc.shapes[s].kind != 0) continue;
        Float t;
        Ray r = ray; r.maxt = best;
        if (sphere_intersect(sc.shapes[s], r, t) && (!hit || t < best)) {
            best = t; best_shape = (int)s; hit = true;
        }
    }
    if (!sc.nodes.empty()) {
        int stack[128]; int sp = 0; stack[sp++] = 0;
        while (sp) {
            const BNode &n = sc.nodes[stack[--sp]];
            if (!box_hit(n, ray, best)) continue;
            if (n.count) {
                for (uint32_t i = n.first; i < n.first + n.count; ++i) {
                    const Shape &m = sc.shapes[sc.tri_shape[i]];
                    Float u, v, t;
                    Ray r = ray; r.maxt = best;
                    /* equal distances (a ray through a shared edge) go to the lower
                       (shape, face) index, so the hit does not depend on the tree */
                    if (tri_intersect(m, sc.tri_face[i], r, u, v, t) &&
                        (!hit || t < best ||
                         (t == best && best_shape >= 0 && sc.shapes[best_shape].kind != 0 &&
                          ((int)sc.tri_shape[i] < best_shape ||
                           ((int)sc.tri_shape[i] == best_shape && sc.tri_face[i] < best_prim))))) {
                        best = t; best_shape = (int)sc.tri_shape[i]; best_prim = sc.tri_face[i];
                        bu = u; bv = v; hit = true;
                    }
                }
            } else if (ray.d[n.axis] < 0.f) {   /* near child last, so it pops first */
                stack[sp++] = n.left; stack[sp++] = n.right;
            } else {
                stack[sp++] = n.right; stack[sp++] = n.left;
            }
        }
    }
    if (!hit) return si;
    si.t = best; si.shape = best_shape; si.prim = best_prim;
    const Shape &s = sc.shapes[best_shape];
    if (s.kind == 0) sphere_fill(s, ray, si);
    else mesh_fill(s, bu, bv, si);
    return si;
}

/* Scene::ray_test (src/librender/scene.cpp:144-152) */
static bool ray_test(const Scene &sc, const Ray &ray) {
    ORC_COUNT_RAY();
    if (ray_is_nan(ray)) return false;
    for (const Shape &s : sc.shapes) {
        Float t;
        if (s.kind == 0 && sphere_intersect(s, ray, t)) return true;
    }
    if (sc.nodes.empty()) return false;
    int stack[128]; int sp = 0; stack[sp++] = 0;
    while (sp) {
        const BNode &n = sc.nodes[stack[--sp]];
        if (!box_hit(n, ray, ray.maxt)) continue;
        if (n.count) {
            for (uint32_t i = n.first; i < n.first + n.count; ++i) {
                Float u, v, t;
                if (tri_intersect(sc.shapes[sc.tri_shape[i]], sc.tri_face[i], ray, u, v, t)) return true;
            }
        } else { stack[sp++] = n.left; stack[sp++] = n.right; }
    }
    return false;
}

/* ---- sampling: warp.h:153-156,262-267; mesh.cpp:541-586; distr_1d.h:144-201 */
static V3 square_to_uniform_sphere(V2 s) {
    Float z = 1.f - 2.f * s.y;
    Float r = safe_sqrt(1.f - z * z);
    Float ang = 2.f * kPi * s.x;
    return V3(r * std::cos(ang), r * std::sin(ang), z);
}

static V3 sample_position(const Shape &s, V2 sample, V3 *n_out = nullptr) {
    if (s.kind == 0) {
        V3 local = square_to_uniform_sphere(sample);
        if (n_out) *n_out = s.flip ? -local : local;
        return local * s.radius + s.center;
    }
    /* DiscreteDistribution::sample_reuse on sample.y */
    Float value = sample.y * s.area_sum;
    uint32_t lo = s.valid_lo, hi = s.valid_hi;
    /* first index in [lo, hi] whose cdf >= value (hi if none) */
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (s.cdf[mid] < value) lo = mid + 1; else hi = mid;
    }
    uint32_t f = lo;
    Float pmf = s.pmf[f] * s.area_norm;
    Float cdf_prev = f > 0 ? s.cdf[f - 1] * s.area_norm : Float(0.f);
    Float y = (sample.y - cdf_prev) / pmf;
    Float tq = safe_sqrt(1.f - sample.x);
    Float bx = 1.f - tq, by = tq * y;
    V3 p0 = s.P[s.F[3 * f]], p1 = s.P[s.F[3 * f + 1]], p2 = s.P[s.F[3 * f + 2]];
    V3 e0 = p1 - p0, e1 = p2 - p0;
    if (n_out) {
        if (!s.N.empty())
            *n_out = normalize(s.N[s.F[3 * f]] * (1.f - bx - by) + s.N[s.F[3 * f + 1]] * bx +
                               s.N[s.F[3 * f + 2]] * by);
        else
            *n_out = normalize(cross(e0, e1));
    }
    return p0 + e0 * bx + e1 * by;
}

/* ------------------------------------------------------- ManifoldVertex */
/* include/mitsuba/render/manifold.h:50-141 */
struct MVertex {
    V3 p, dp_du, dp_dv, n, gn, dn_du, dn_dv, s, t, ds_du, ds_dv, dt_du, dt_dv;
    Float eta = 1.f;
    V2 uv;
    int shape = -1;
    bool fixed_direction = false;
};

/* manifold.h:94-96: eta = real(ior) when imag(ior) == 0, else 1.  Conductors
 * with k = 0 therefore behave like dielectrics; non-specular BSDFs have
 * ior = (0, 1) (bsdf.cpp:58-60) -> 1. */
static Float bsdf_eta(const sms_bsdf &b) {
    if (b.type == SMS_BSDF_DIELECTRIC) return b.eta;
    if (b.type == SMS_BSDF_CONDUCTOR && b.k == 0.f) return b.eta;
    return 1.f;
}

/* MNEE initialisation target (manifold_ss.cpp:229-241, manifold_ms.cpp:305-316):
 * complex ior (imag != 0: conductors with k != 0, and the diffuse BSDF whose
 * ior() is (0, 1)) -> the shape's bounding-box centre, else the light point. */
static V3 mnee_target(const Shape &s, V3 lp) {
    const sms_bsdf &b = s.bsdf;
    bool real_ior = b.type == SMS_BSDF_DIELECTRIC || (b.type == SMS_BSDF_CONDUCTOR && b.k == 0.f);
    return real_ior ? lp : s.bbox_center;
}

static V2 nm_slope(const NormalMap &m, V2 uv);
static void nm_slope_derivative(const NormalMap &m, V2 uv, V2 &du, V2 &dv);

/* A caster / bouncer carrying the scene's normal map (the reference's
 * normalmap BSDF around its dielectric / conductor). */
static bool nm_frames(const Scene &sc, int shape) {
    const uint32_t chain = SMS_SHAPE_CAUSTIC_CASTER_SINGLE | SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER;
    return shape == sc.glinty_shape && sc.nmap.res > 0 && (sc.shapes[shape].flags & chain) != 0;
}

/* NormalmapBSDF::frame / frame_derivative (normalmap.cpp:236-290): the base
 * frame (n0, tangent from dp_du) and its derivative applied to the slope
 * normal (-s_x, -s_y, 1) at level 0 and its derivative; coarse = the
 * two-stage solver's smoothing 1: the top LEAN level (mean slope, no
 * derivative). */
static void nm_vertex_frame(const Scene &sc, const SI &si, V3 n0, V3 dn0_du, V3 dn0_dv, bool coarse, V3 &n,
                            V3 &dn_du, V3 &dn_dv) {
    V3 s0 = si.dp_du - n0 * dot(n0, si.dp_du);
    const Float inv_len = 1.f / norm(s0);
    s0 *= inv_len;
    const V3 t0 = cross(n0, s0);
    V3 ds_du = (-dn0_du * dot(n0, si.dp_du) - n0 * dot(dn0_du, si.dp_du)) * inv_len;
    V3 ds_dv = (-dn0_dv * dot(n0, si.dp_du) - n0 * dot(dn0_dv, si.dp_du)) * inv_len;
    ds_du -= s0 * dot(ds_du, s0);
    ds_dv -= s0 * dot(ds_dv, s0);
    const V3 dt_du = cross(dn0_du, s0) + cross(n0, ds_du), dt_dv = cross(dn0_dv, s0) + cross(n0, ds_dv);
    V3 nl, dl_du, dl_dv;
    if (coarse) {
        const std::vector<Float> &t = sc.nmap.lean.back();
        nl = V3(-t[0], -t[1], 1.f);
        dl_du = V3(0.f); dl_dv = V3(0.f);
    } else {
        V2 sl = nm_slope(sc.nmap, si.uv), du, dv;
        nm_slope_derivative(sc.nmap, si.uv, du, dv);
        nl = V3(-sl.x, -sl.y, 1.f);
        dl_du = V3(-du.x, -du.y, 0.f);
        dl_dv = V3(-dv.x, -dv.y, 0.f);
    }
    V3 wn = s0 * nl.x + t0 * nl.y + n0 * nl.z;
    const Float il = 1.f / norm(wn);
    wn *= il;
    V3 a = (s0 * dl_du.x + t0 * dl_du.y + n0 * dl_du.z + ds_du * nl.x + dt_du * nl.y + dn0_du * nl.z) * il;
    V3 b = (s0 * dl_dv.x + t0 * dl_dv.y + n0 * dl_dv.z + ds_dv * nl.x + dt_dv * nl.y + dn0_dv * nl.z) * il;
    n = wn;
    dn_du = a - wn * dot(a, wn);
    dn_dv = b - wn * dot(b, wn);
}

/* frame.h:197-240 (compute_shading_frame{,_derivative}); bsdf.cpp:17-31;
 * nm_coarse: the two-stage solver's smoothed frame on a normal-mapped shape */
static void vertex_from_si(const Scene &sc, const SI &si, MVertex &v, bool nm_coarse = false) {
    const Shape &sh = sc.shapes[si.shape];
    v.p = si.p; v.dp_du = si.dp_du; v.dp_dv = si.dp_dv; v.gn = si.n; v.uv = si.uv;
    v.shape = si.shape; v.fixed_direction = false;
    v.eta = bsdf_eta(sh.bsdf);
    V3 n = si.shn;
    V3 dndu, dndv;
    if (sh.kind == 0) {
        Float inv_r = (sh.flip ? -1.f : 1.f) / sh.radius;   /* sphere.cpp:376-382 */
        dndu = si.dp_du * inv_r; dndv = si.dp_dv * inv_r;
    } else {
        mesh_normal_derivative(sh, si, dndu, dndv);
    }
    if (nm_frames(sc, si.shape)) nm_vertex_frame(sc, si, si.shn, dndu, dndv, nm_coarse, n, dndu, dndv);
    V3 s = normalize(si.dp_du - n * dot(n, si.dp_du));
    v.n = n; v.s = s; v.t = cross(n, s);
    V3 s0 = si.dp_du - n * dot(n, si.dp_du);
    Float inv_len_s = 1.f / norm(s0);
    s0 *= inv_len_s;
    V3 dsdu = (-dndu * dot(n, si.dp_du) - n * dot(dndu, si.dp_du)) * inv_len_s;
    V3 dsdv = (-dndv * dot(n, si.dp_du) - n * dot(dndv, si.dp_du)) * inv_len_s;
    dsdu -= s0 * dot(dsdu, s0);
    dsdv -= s0 * dot(dsdv, s0);
    v.ds_du = dsdu; v.ds_dv = dsdv;
    v.dt_du = cross(dndu, s0) + cross(n, dsdu);
    v.dt_dv = cross(dndv, s0) + cross(n, dsdv);
    v.dn_du = dndu; v.dn_dv = dndv;
    if (dot(v.n, v.gn) < 0.f) v.gn = -v.gn;
}

/* manifold.h:115-126 */
static void make_orthonormal(MVertex &v) {
    Float inv = 1.f / norm(v.dp_du);
    v.dp_du *= inv; v.dn_du *= inv;
    Float dp = dot(v.dp_du, v.dp_dv);
    V3 a = v.dp_dv - v.dp_du * dp, b = v.dn_dv - v.dn_du * dp;
    inv = 1.f / norm(a);
    v.dp_dv = a * inv; v.dn_dv = b * inv;
}

/* ------------------------------------------------ emitter interaction */
struct EI {
    V3 p, n, d, weight;
    Float pdf = 0.f;
    int emitter = -1;
    bool is_point = false, is_area = false;
};

/* ---------------------------------------------- specular transforms */
/* manifold.h:348-418 */
static bool reflect(V3 w, V3 n, V3 &out) { out = n * (2.f * dot(w, n)) - w; return true; }
static void d_reflect(V3 w, V3 dwdu, V3 dwdv, V3 n, V3 dndu, V3 dndv, V3 &ou, V3 &ov) {
    Float dwn = dot(w, n), dun = dot(dwdu, n), dvn = dot(dwdv, n), wdu = dot(w, dndu),
          wdv = dot(w, dndv);
    ou = ((n * (dun + wdu)) + dndu * dwn) * 2.f - dwdu;
    ov = ((n * (dvn + wdv)) + dndv * dwn) * 2.f - dwdv;
}
static bool refract(V3 w, V3 n, Float eta_, V3 &out) {
    Float eta = 1.f / eta_;
    if (dot(w, n) < 0.f) { eta = 1.f / eta; n = -n; }
    Float dwn = dot(w, n);
    Float root = 1.f - eta * eta * (1.f - dwn * dwn);
    if (root < 0.f) { out = V3(0.f); return false; }
    out = -(w - n * dwn) * eta - n * std::sqrt(root);
    return true;
}
static void d_refract(V3 w, V3 dwdu, V3 dwdv, V3 n, V3 dndu, V3 dndv, Float eta_, V3 &ou, V3 &ov) {
    Float eta = 1.f / eta_;
    if (dot(w, n) < 0.f) { eta = 1.f / eta; n = -n; dndu = -dndu; dndv = -dndv; }
    Float dwn = dot(w, n), dun = dot(dwdu, n), dvn = dot(dwdv, n), wdu = dot(w, dndu),
          wdv = dot(w, dndv);
    Float root = std::sqrt(1.f - eta * eta * (1.f - dwn * dwn));
    V3 a_u = -(dwdu - (n * (dun + wdu) + dndu * dwn)) * eta;
    V3 b_u = -(dndu * root + n * (1.f / (2.f * root)) * (-eta * eta * (-2.f * dwn * (dun + wdu))));
    V3 a_v = -(dwdv - (n * (dvn + wdv) + dndv * dwn)) * eta;
    V3 b_v = -(dndv * root + n * (1.f / (2.f * root)) * (-eta * eta * (-2.f * dwn * (dvn + wdv))));
    ou = a_u + b_u;
    ov = a_v + b_v;
}
/* manifold.h:420-443 */
static void sphcoords(V3 w, Float &theta, Float &phi) {
    theta = safe_acos(w.z);
    phi = std::atan2(w.y, w.x);
    if (phi < 0.f) phi += 2.f * kPi;
}
static void d_sphcoords(V3 w, V3 dwdu, V3 dwdv, Float &dtu, Float &dpu, Float &dtv, Float &dpv) {
    Float d_acos = -1.f / safe_sqrt(1.f - w.z * w.z);
    dtu = d_acos * dwdu.z;
    dtv = d_acos * dwdv.z;
    Float yx = w.y / w.x;
    Float d_atan = 1.f / (1.f + yx * yx);
    Float inv = 1.f / (w.x * w.x);
    dpu = d_atan * (w.x * dwdu.y - w.y * dwdu.x) * inv;
    dpv = d_atan * (w.x * dwdv.y - w.y * dwdv.x) * inv;
    if (w.x == 0.f) { dpu = 0.f; dpv = 0.f; }
}

/* ------------------------------------------------------ constraints */
/* manifold_ss.cpp:494-636 */
static bool step_anglediff(V3 x, const MVertex &v1, const EI &ei, V2 &C, V2 &dX, M2 *J_out = nullptr,
                           V3 no = V3(0.f, 0.f, 1.f)) {
    V3 wi = x - v1.p;
    Float ili = norm(wi);
    if (ili < 1e-3f) return false;
    ili = 1.f / ili; wi *= ili;
    V3 dwi_du = (v1.dp_du - wi * dot(wi, v1.dp_du)) * -ili;
    V3 dwi_dv = (v1.dp_dv - wi * dot(wi, v1.dp_dv)) * -ili;
    V3 wo = ei.p - v1.p;
    Float ilo = norm(wo);
    if (ilo < 1e-3f) return false;
    ilo = 1.f / ilo; wo *= ilo;
    V3 dwo_du = (v1.dp_du - wo * dot(wo, v1.dp_du)) * -ilo;
    V3 dwo_dv = (v1.dp_dv - wo * dot(wo, v1.dp_dv)) * -ilo;
    /* offset normal (manifold_ss.cpp:560-569); (0,0,1) keeps the vertex's own */
    V3 n = v1.n, dndu = v1.dn_du, dndv = v1.dn_dv;
    if (no.x != 0.f || no.y != 0.f) {
        n = v1.s * no.x + v1.t * no.y + v1.n * no.z;
        dndu = v1.ds_du * no.x + v1.dt_du * no.y + v1.dn_du * no.z;
        dndv = v1.ds_dv * no.x + v1.dt_dv * no.y + v1.dn_dv * no.z;
    }
    bool success = false;
    M2 J;
    C = V2{0.f, 0.f};
    auto transform = [&](V3 w, V3 &out) {
        return v1.eta == 1.f ? reflect(w, n, out) : refract(w, n, v1.eta, out);
    };
    auto d_transform = [&](V3 w, V3 du, V3 dv, V3 &ou, V3 &ov) {
        if (v1.eta == 1.f) d_reflect(w, du, dv, n, dndu, dndv, ou, ov);
        else d_refract(w, du, dv, n, dndu, dndv, v1.eta, ou, ov);
    };
    V3 wio;
    if (transform(wi, wio)) {
        V3 dwio_du, dwio_dv;
        d_transform(wi, dwi_du, dwi_dv, dwio_du, dwio_dv);
        Float to, po, tio, pio;
        sphcoords(wo, to, po); sphcoords(wio, tio, pio);
        Float dt = to - tio, dp = po - pio;
        if (dp < -kPi) dp += 2.f * kPi; else if (dp > kPi) dp -= 2.f * kPi;
        C = V2{dt, dp};
        Float a0, a1, a2, a3, b0, b1, b2, b3;
        d_sphcoords(wo, dwo_du, dwo_dv, a0, a1, a2, a3);
        d_sphcoords(wio, dwio_du, dwio_dv, b0, b1, b2, b3);
        J.m[0][0] = a0 - b0; J.m[1][0] = a1 - b1; J.m[0][1] = a2 - b2; J.m[1][1] = a3 - b3;
        success = true;
    }
    V3 woi;
    if (transform(wo, woi) && !success) {
        V3 dwoi_du, dwoi_dv;
        d_transform(wo, dwo_du, dwo_dv, dwoi_du, dwoi_dv);
        Float ti, pi, toi, poi;
        sphcoords(wi, ti, pi); sphcoords(woi, toi, poi);
        Float dt = ti - toi, dp = pi - poi;
        if (dp < -kPi) dp += 2.f * kPi; else if (dp > kPi) dp -= 2.f * kPi;
        C = V2{dt, dp};
        Float a0, a1, a2, a3, b0, b1, b2, b3;
        d_sphcoords(wi, dwi_du, dwi_dv, a0, a1, a2, a3);
        d_sphcoords(woi, dwoi_du, dwoi_dv, b0, b1, b2, b3);
        J.m[0][0] = a0 - b0; J.m[1][0] = a1 - b1; J.m[0][1] = a2 - b2; J.m[1][1] = a3 - b3;
        success = true;
    }
    if (J_out) *J_out = J;
    Float d = det(J);
    if (std::fabs(d) < 1e-6f) return false;
    dX = mul(inverse(J), C);
    return success;
}

/* manifold_ss.cpp:407-492 */
static bool step_halfvector(V3 x, const MVertex &v1, const EI &ei, V2 &C, V2 &dX, M2 *J_out = nullptr,
                            V3 no = V3(0.f, 0.f, 1.f)) {
    V3 wo = ei.p - v1.p;
    Float ilo = norm(wo);
    if (ilo < 1e-3f) return false;
    ilo = 1.f / ilo; wo *= ilo;
    V3 wi = x - v1.p;
    Float ili = norm(wi);
    if (ili < 1e-3f) return false;
    ili = 1.f / ili; wi *= ili;
    Float eta = v1.eta;
    if (dot(wi, v1.gn) < 0.f) eta = 1.f / eta;
    V3 h = wi + wo * eta;
    if (eta != 1.f) h *= -1.f;
    Float ilh = 1.f / norm(h);
    h *= ilh;
    ilo *= eta * ilh;
    ili *= ilh;
    V3 dh_du = -v1.dp_du * (ili + ilo) + wi * (dot(wi, v1.dp_du) * ili) + wo * (dot(wo, v1.dp_du) * ilo);
    V3 dh_dv = -v1.dp_dv * (ili + ilo) + wi * (dot(wi, v1.dp_dv) * ili) + wo * (dot(wo, v1.dp_dv) * ilo);
    dh_du -= h * dot(dh_du, h);
    dh_dv -= h * dot(dh_dv, h);
    if (eta != 1.f) { dh_du *= -1.f; dh_dv *= -1.f; }
    M2 J;
    J.m[0][0] = dot(v1.ds_du, h) + dot(v1.s, dh_du);
    J.m[1][0] = dot(v1.dt_du, h) + dot(v1.t, dh_du);
    J.m[0][1] = dot(v1.ds_dv, h) + dot(v1.s, dh_dv);
    J.m[1][1] = dot(v1.dt_dv, h) + dot(v1.t, dh_dv);
    if (J_out) { *J_out = J; C = V2{dot(v1.s, h) - no.x, dot(v1.t, h) - no.y}; }
    Float d = det(J);
    if (std::fabs(d) < 1e-6f) return false;
    C = V2{dot(v1.s, h) - no.x, dot(v1.t, h) - no.y};   /* H - N (manifold_ss.cpp:485-488) */
    dX = mul(inverse(J), C);
    return true;
}

/* ------------------------------------------------------ Newton solver */
struct Cfg {
    sms_config c;
};

/* manifold_ss.cpp:329-405.  Returns (ok, si_current, iterations); coarse:
 * smoothing = 1 (the two-stage solver's first solve, manifold_ss.cpp:262). */
static bool newton_solver(const Scene &sc, const sms_config &cfg, V3 x, const MVertex &init,
                          const EI &ei, SI &si_out, int &iters_out, V3 no = V3(0.f, 0.f, 1.f),
                          bool coarse = false) {
    MVertex vtx = init;
    bool success = false;
    int it = 0;
    Float beta = 1.f;
    SI si_current;
    while (it < cfg.max_iterations) {
        V2 C, dX;
        bool ok = cfg.halfvector_constraints ? step_halfvector(x, vtx, ei, C, dX, nullptr, no)
                                             : step_anglediff(x, vtx, ei, C, dX, nullptr, no);
        if (!ok) break;
        if (std::sqrt(C.x * C.x + C.y * C.y) < cfg.solver_threshold) { success = true; break; }
        V3 p_prop = vtx.p - (vtx.dp_du * dX.x + vtx.dp_dv * dX.y) * (cfg.step_scale * beta);
        Ray r; r.o = x; r.d = normalize(p_prop - x);
        si_current = ray_intersect(sc, r);
        if (!si_current.valid() || vtx.shape != si_current.shape) {
            beta = 0.5f * beta;
            it += 1;
            continue;
        }
        beta = omin(1.f, 2.f * beta);
        vertex_from_si(sc, si_current, vtx, coarse);
        it++;
    }
    iters_out = it;
    si_out = si_current;
    if (!success) return false;
    V3 wx = normalize(x - vtx.p);
    V3 wy = normalize(ei.p - vtx.p);
    Float cx = dot(vtx.gn, wx), cy = dot(vtx.gn, wy);
    bool refraction = cx * cy < 0.f;
    bool reflection = !refraction;
    if ((vtx.eta == 1.f && !reflection) || (vtx.eta != 1.f && !refraction)) return false;
    return true;
}

/* ----------------------------------------------------------- query */
struct Query {
    V3 p, n, dp_du, dp_dv, albedo;
    Float cos_i = 1.f;
};

static Query load_query(const float *q, uint32_t n, uint32_t i) {
    Query r;
    auto f = [&](int k) { return q[(size_t)k * n + i]; };
    r.p = V3(f(0), f(1), f(2)); r.n = V3(f(3), f(4), f(5));
    r.dp_du = V3(f(6), f(7), f(8)); r.dp_dv = V3(f(9), f(10), f(11));
    r.albedo = V3(f(12), f(13), f(14)); r.cos_i = f(15);
    return r;
}

/* sample_gaussian (manifold.h:326-345) through square_to_std_normal
 * (warp.h:184-190): a slope from N(mu, sigma), sigma = (a, c; c, b). */
static V2 sample_slope_gaussian(V2 mu, Float a, Float b, Float c, V2 u) {
    const Float r = std::sqrt(-2.f * std::log(1.f - u.x)), ph = 2.f * kPi * u.y;
    const Float px = std::cos(ph) * r, py = std::sin(ph) * r;
    const Float sx = std::sqrt(a), sy = std::sqrt(b);
    const Float rho = c / (sx * sy);
    const Float ka = std::sqrt(1.f + rho), kb = std::sqrt(1.f - rho);
    const Float d0 = 0.5f * ka + 0.5f * kb, d1 = 0.5f * ka - 0.5f * kb;
    return V2{(d0 * px + d1 * py) * sx + mu.x, (d1 * px + d0 * py) * sy + mu.y};
}

/* manifold_ss.cpp:203-279; no = offset normal.  cfg.twostage (:253-270, a
 * normal-mapped caster): a first solve on the smoothed surface (the top LEAN
 * level's frame) toward a slope drawn from that level's Gaussian around the
 * mean of its mean slope and the offset slope (the two numbers g), then the
 * solve on the full map from its solution.  g is drawn for every walk (the
 * reference draws it after the first ray hit the caster), so that every walk
 * owns a fixed run of random numbers. */
static bool sample_path(const Scene &sc, const sms_config &cfg, int caster, const Query &q,
                        const EI &ei, V2 sample, V3 p_start, SI &si_final, SI &si_init,
                        int &iters, V3 no = V3(0.f, 0.f, 1.f), V2 g = V2{0.f, 0.f}) {
    const Shape &shape = sc.shapes[caster];
    V3 p = sample_position(shape, sample);
    if (p_start.x != 0.f || p_start.y != 0.f || p_start.z != 0.f) p = p_start;
    V3 d_tmp = normalize(p - q.p);
    if (cfg.mnee_init) d_tmp = normalize(mnee_target(shape, ei.p) - q.p);
    Ray r; r.o = q.p; r.d = d_tmp;
    si_init = ray_intersect(sc, r);
    iters = 0;
    if (!si_init.valid() || caster != si_init.shape) return false;
    MVertex v0;
    vertex_from_si(sc, si_init, v0, cfg.twostage != 0);
    int it1 = 0;
    if (cfg.twostage) {
        const std::vector<Float> &t = sc.nmap.lean.back();
        const Float a = omax(0.f, t[2] - t[0] * t[0]), b = omax(0.f, t[3] - t[1] * t[1]),
                    c = omax(0.f, t[4] - t[0] * t[1]);
        const V2 mu{0.5f * (t[0] - no.x / no.z), 0.5f * (t[1] - no.y / no.z)};
        const V2 sl = sample_slope_gaussian(mu, a, b, c, g);
        const V3 ln = normalize(V3(-sl.x, -sl.y, 1.f));
        SI si_smooth;
        const bool ok1 = newton_solver(sc, cfg, q.p, v0, ei, si_smooth, it1, ln, true);
        if (!ok1 || !si_smooth.valid()) { iters = it1; return false; }
        vertex_from_si(sc, si_smooth, v0, false);
    }
    bool ok = newton_solver(sc, cfg, q.p, v0, ei, si_final, iters, no);
    iters += it1;
    return ok && si_final.valid();
}

/* manifold.h:204-260 (em: the caustic emitter list of the estimator) */
static EI sample_emitter_interaction(const Scene &sc, const std::vector<int> &em, const Query &q, PCG32 &rng) {
    EI ei;
    if (em.empty()) return ei;
    Float es = rng.next_f32();
    Float emitter_pdf = 1.f / (Float)em.size();
    uint32_t idx = omin((uint32_t)(es * (Float)em.size()), (uint32_t)em.size() - 1);
    const Emitter &e = sc.emitters[em[idx]];
    ei.emitter = em[idx];
    V3 spec(0.f);
    if (e.kind == 1) {
        ei.is_area = true;
        const Shape &s = sc.shapes[e.shape];
        V3 n;
        V3 p = sample_position(s, rng.next_2d(), &n);
        Float area = 4.f * kPi * s.radius * s.radius;
        Float pdf = 1.f / area;
        /* area.cpp:71-79 with wi = (0,0,1): cos_theta > 0 -> radiance */
        spec = V3(e.radiance.x / pdf, e.radiance.y / pdf, e.radiance.z / pdf);
        ei.p = p; ei.n = n; ei.d = normalize(p - q.p); ei.pdf = pdf;
    } else {
        ei.is_point = true;
        (void)rng.next_2d(); /* point.cpp:74-100 consumes a 2D sample */
        V3 d = e.p - q.p;
        Float dist = norm(d);
        Float inv = 1.f / dist;
        d *= inv;
        V3 s = e.radiance * (inv * inv);
        ei.p = e.p; ei.d = d; ei.n = d; ei.pdf = 1.f;
        spec = (s * dist) * dist;
    }
    ei.pdf *= emitter_pdf;
    ei.weight = spec * (1.f / emitter_pdf);
    return ei;
}

/* fresnel.h:34-80 */
static Float fresnel(Float cos_i, Float eta, Float *cos_t_out = nullptr) {
    bool outside = cos_i >= 0.f;
    Float rcp_eta = 1.f / eta;
    Float eta_it = outside ? eta : rcp_eta, eta_ti = outside ? rcp_eta : eta;
    Float ct2 = 1.f - (1.f - cos_i * cos_i) * (eta_ti * eta_ti);
    Float ci = std::fabs(cos_i), ct = safe_sqrt(ct2);
    bool index_matched = eta == 1.f;
    bool special = index_matched || ci == 0.f;
    Float r_sc = index_matched ? 0.f : 1.f;
    Float a_s = (ci - eta_it * ct) / (ci + eta_it * ct);
    Float a_p = (ct - eta_it * ci) / (ct + eta_it * ci);
    Float r = 0.5f * (a_s * a_s + a_p * a_p);
    if (special) r = r_sc;
    if (cos_t_out) *cos_t_out = cos_i >= 0.f ? -ct : ct;
    return r;
}
/* fresnel.h:92-120 */
static Float fresnel_conductor(Float cos_i, Float er, Float ei_) {
    Float c2 = cos_i * cos_i, s2 = 1.f - c2, s4 = s2 * s2;
    Float t1 = er * er - ei_ * ei_ - s2;
    Float a2pb2 = safe_sqrt(t1 * t1 + 4.f * ei_ * ei_ * er * er);
    Float a = safe_sqrt(0.5f * (a2pb2 + t1));
    Float term1 = a2pb2 + c2, term2 = 2.f * cos_i * a;
    Float rs = (term1 - term2) / (term1 + term2);
    Float term3 = a2pb2 * c2 + s4, term4 = term2 * s2;
    Float rp = rs * (term3 - term4) / (term3 + term4);
    return 0.5f * (rs + rp);
}

/* manifold_ss.cpp:638-693 (smooth BSDFs) */
static Float specular_reflectance(const Scene &sc, const SI &si, V3 wo) {
    if (!si.valid()) return 0.f;
    const sms_bsdf &b = sc.shapes[si.shape].bsdf;
    V3 n = si.shn;
    Float cos_theta = dot(n, wo);
    if (b.type == SMS_BSDF_CONDUCTOR && b.k != 0.f)
        return fresnel_conductor(std::fabs(cos_theta), b.eta, b.k);
    if (b.type == SMS_BSDF_DIELECTRIC || b.type == SMS_BSDF_CONDUCTOR) {
        /* real ior: the "reflection" mask is false -> transmission branch */
        Float eta = b.eta;
        if (cos_theta < 0.f) eta = 1.f / eta;
        Float F = fresnel(cos_theta, eta);
        return (1.f - F) * eta * eta;
    }
    /* diffuse: ior (0,1) has a nonzero imaginary part -> conductor formula */
    return fresnel_conductor(std::fabs(cos_theta), 0.f, 1.f);
}

/* ---- isotropic Beckmann microfacets (include/mitsuba/render/microfacet.h):
 * D(m) with its underflow cut-off; Smith G1 by the rational approximation of
 * Walter et al. 2007 (eq. 27); sampling of m with density D(m) cos(theta_m). */
static Float beckmann_D(V3 m, Float alpha) {
    Float c2 = m.z * m.z;
    Float r = std::exp(-((m.x * m.x + m.y * m.y) / (alpha * alpha)) / c2) / (kPi * alpha * alpha * c2 * c2);
    return r * m.z > 1e-20f ? r : Float(0.f);
}
static Float beckmann_G1(V3 v, V3 m, Float alpha) {
    Float xy = alpha * alpha * (v.x * v.x + v.y * v.y);
    Float r = 1.f;
    if (xy != 0.f) {
        Float a = 1.f / std::sqrt(xy / (v.z * v.z)), a2 = a * a;
        r = a >= 1.6f ? Float(1.f) : (3.535f * a + 2.181f * a2) / (1.f + 2.276f * a + 2.577f * a2);
    }
    return dot(v, m) * v.z <= 0.f ? Float(0.f) : r;
}
static V3 beckmann_sample(Float alpha, Float u0, Float u1, Float &pdf) {
    Float ang = 2.f * kPi * u1;
    Float sp = std::sin(ang), cp = std::cos(ang);
    Float ct = 1.f / std::sqrt(1.f - alpha * alpha * std::log(1.f - u0));
    Float c2 = ct * ct;
    pdf = (1.f - u0) / (kPi * alpha * alpha * omax(c2 * ct, 1e-20f));
    Float st = std::sqrt(1.f - c2);
    return V3(cp * st, sp * st, ct);
}
/* roughconductor.cpp eval (value x cos_theta_o), local frame */
static Float roughconductor_eval(Float alpha, Float er, Float ek, V3 wi, V3 wo) {
    if (!(wi.z > 0.f && wo.z > 0.f)) return 0.f;
    V3 h = normalize(wo + wi);
    Float D = beckmann_D(h, alpha);
    if (D == 0.f) return 0.f;
    Float G = beckmann_G1(wi, h, alpha) * beckmann_G1(wo, h, alpha);
    return D * G / (4.f * wi.z) * fresnel_conductor(dot(wi, h), er, ek);
}
/* roughdielectric.cpp eval (value x |cos_theta_o|, radiance transport), local frame */
static Float roughdielectric_eval(Float alpha, Float eta_, V3 wi, V3 wo) {
    const Float ci = wi.z, co = wo.z;
    if (ci == 0.f) return 0.f;
    const bool reflect = ci * co > 0.f;
    const Float eta = ci > 0.f ? eta_ : 1.f / eta_, inv_eta = ci > 0.f ? 1.f / eta_ : eta_;
    V3 m = normalize(wi + wo * (reflect ? Float(1.f) : eta));
    if (m.z < 0.f) m = -m;
    Float D = beckmann_D(m, alpha);
    Float F = fresnel(dot(wi, m), eta_);
    Float G = beckmann_G1(wi, m, alpha) * beckmann_G1(wo, m, alpha);
    if (reflect) return F * D * G / (4.f * std::fabs(ci));
    Float den = dot(wi, m) + eta * dot(wo, m);
    return std::fabs((inv_eta * inv_eta) * (1.f - F) * D * G * eta * eta * dot(wi, m) * dot(wo, m) /
                     (ci * den * den));
}
/* manifold_ss.cpp:648-669: a rough BSDF's value in the half-vector domain;
 * wi toward the shading point, wo toward the light (world space). */
/* On a normal-mapped shape, NormalmapBSDF::eval (normalmap.cpp:172-181)
 * evaluates the nested BSDF in the perturbed frame and keeps wo only on the
 * same side of the perturbed and the unperturbed normal; the half-vector
 * factor flips eta by the side of wi in the unperturbed frame (si.wi). */
static Float specular_reflectance_rough(const Scene &sc, const SI &si, V3 wi_w, V3 wo_w) {
    const sms_bsdf &b = sc.shapes[si.shape].bsdf;
    const bool nm = nm_frames(sc, si.shape);
    V3 n = si.shn;
    if (nm) {
        MVertex v;
        vertex_from_si(sc, si, v);
        n = v.n;
    }
    V3 fs = normalize(si.dp_du - n * dot(n, si.dp_du));
    V3 ft = cross(n, fs);
    V3 wi(dot(wi_w, fs), dot(wi_w, ft), dot(wi_w, n));
    V3 wo(dot(wo_w, fs), dot(wo_w, ft), dot(wo_w, n));
    if (nm && !(dot(wo_w, si.shn) * wo.z > 0.f)) return 0.f;
    if (b.type == SMS_BSDF_CONDUCTOR && b.k != 0.f) {
        Float f = roughconductor_eval(b.alpha, b.eta, b.k, wi, wo);
        V3 h = normalize(wi + wo);
        return f * 4.f * std::fabs(dot(wo, h));
    }
    Float f = b.type == SMS_BSDF_CONDUCTOR ? roughconductor_eval(b.alpha, b.eta, b.k, wi, wo)
                                           : roughdielectric_eval(b.alpha, b.eta, wi, wo);
    Float eta = b.eta;
    if ((nm ? dot(wi_w, si.shn) : wi.z) < 0.f) eta = 1.f / eta;
    V3 h = -normalize(wi + wo * eta);
    Float a = dot(wi, h) + eta * dot(wo, h);
    return f * a * a / (eta * eta * std::fabs(dot(wo, h)));
}

static bool is_rough(const sms_bsdf &b) { return b.type != SMS_BSDF_DIFFUSE && b.alpha > 0.f; }

/* manifold_ss.cpp:695-857 */
static Float geometric_term(const MVertex &v0, const MVertex &v1, const MVertex &v2) {
    V3 wi = v0.p - v1.p;
    Float ili = norm(wi);
    if (ili < 1e-3f) return 0.f;
    ili = 1.f / ili; wi *= ili;
    V3 wo = v2.p - v1.p;
    Float ilo = norm(wo);
    if (ilo < 1e-3f) return 0.f;
    ilo = 1.f / ilo; wo *= ilo;
    Float eta = v1.eta;
    if (dot(wi, v1.gn) < 0.f) eta = 1.f / eta;
    V3 h = wi + wo * eta;
    if (eta != 1.f) h *= -1.f;
    Float ilh = 1.f / norm(h);
    h *= ilh;
    ilo *= eta * ilh;
    ili *= ilh;
    Float dpdu_n = dot(v1.dp_du, v1.n), dpdv_n = dot(v1.dp_dv, v1.n);
    V3 s = v1.dp_du - v1.n * dpdu_n, t = v1.dp_dv - v1.n * dpdv_n;
    V3 dh_du = -v1.dp_du * (ili + ilo) + wi * (dot(wi, v1.dp_du) * ili) + wo * (dot(wo, v1.dp_du) * ilo);
    V3 dh_dv = -v1.dp_dv * (ili + ilo) + wi * (dot(wi, v1.dp_dv) * ili) + wo * (dot(wo, v1.dp_dv) * ilo);
    dh_du -= h * dot(dh_du, h);
    dh_dv -= h * dot(dh_dv, h);
    if (eta != 1.f) { dh_du *= -1.f; dh_dv *= -1.f; }
    Float hn = dot(h, v1.n), hdu = dot(h, v1.dn_du), hdv = dot(h, v1.dn_dv);
    M2 d11;
    d11.m[0][0] = dot(dh_du, s) - dot(v1.dp_du, v1.dn_du) * hn - dpdu_n * hdu;
    d11.m[0][1] = dot(dh_dv, s) - dot(v1.dp_du, v1.dn_dv) * hn - dpdu_n * hdv;
    d11.m[1][0] = dot(dh_du, t) - dot(v1.dp_dv, v1.dn_du) * hn - dpdv_n * hdu;
    d11.m[1][1] = dot(dh_dv, t) - dot(v1.dp_dv, v1.dn_dv) * hn - dpdv_n * hdv;
    dh_du = (v2.dp_du - wo * dot(wo, v2.dp_du)) * ilo;
    dh_dv = (v2.dp_dv - wo * dot(wo, v2.dp_dv)) * ilo;
    dh_du -= h * dot(dh_du, h);
    dh_dv -= h * dot(dh_dv, h);
    if (eta != 1.f) { dh_du *= -1.f; dh_dv *= -1.f; }
    M2 d12;
    d12.m[0][0] = dot(dh_du, s); d12.m[0][1] = dot(dh_dv, s);
    d12.m[1][0] = dot(dh_du, t); d12.m[1][1] = dot(dh_dv, t);
    Float d = det(d11);
    if (std::fabs(d) < 1e-6f) return 0.f;
    Float dx1_dx2 = std::fabs(det(mul(inverse(d11), d12)));
    dx1_dx2 = omin(dx1_dx2, 1.f);
    V3 dd = v0.p - v1.p;
    Float inv_r2 = 1.f / dot(dd, dd);
    dd *= std::sqrt(inv_r2);
    Float dw0_dx1 = std::fabs(dot(dd, v1.gn)) * inv_r2;
    return dw0_dx1 * dx1_dx2;
}

/* manifold.h:264-302 */
static bool emitter_vertex(const Scene &sc, const EI &ei, V3 p, MVertex &vy) {
    if (ei.is_area) {
        V3 d = normalize(ei.p - p);
        Ray r; r.o = p + d * kShadowEps; r.d = d;
        SI si_y = ray_intersect(sc, r);
        if (!si_y.valid()) return false;
        vertex_from_si(sc, si_y, vy);
        make_orthonormal(vy);
        return true;
    }
    vy = MVertex();
    vy.p = ei.p;
    V3 d = normalize(p - ei.p);
    vy.n = vy.gn = d;
    coordinate_system(d, vy.dp_du, vy.dp_dv);
    return true;
}

/* manifold_ss.cpp:281-327 */
static V3 evaluate_path_contribution(const Scene &sc, const Query &q, const EI &ei_in,
                                     const SI &si_final) {
    MVertex vtx;
    vertex_from_si(sc, si_final, vtx);
    make_orthonormal(vtx);
    EI ei = ei_in;
    if (ei.is_point) {
        const Emitter &e = sc.emitters[ei.emitter];
        V3 d = e.p - si_final.p;
        Float dist = norm(d);
        Float inv = 1.f / dist;
        d *= inv;
        V3 spec = e.radiance * (inv * inv);
        ei.p = e.p; ei.d = d; ei.n = d;
        Float emitter_pdf = ei.pdf;
        ei.pdf = 1.f;
        ei.weight = (spec * dist) * dist;
        ei.pdf *= emitter_pdf;
        ei.weight = ei.weight * (1.f / emitter_pdf);
    }
    MVertex vy;
    if (!emitter_vertex(sc, ei, vtx.p, vy)) return V3(0.f);
    /* shading point vertex: flat receiver (dn = 0) */
    MVertex vx;
    vx.p = q.p; vx.dp_du = q.dp_du; vx.dp_dv = q.dp_dv; vx.gn = q.n; vx.n = q.n;
    vx.dn_du = V3(0.f); vx.dn_dv = V3(0.f);
    make_orthonormal(vx);
    /* path_throughput = 1 * F * G * weight (manifold_ss.cpp:322-326) */
    Float f = is_rough(sc.shapes[si_final.shape].bsdf)
                  ? specular_reflectance_rough(sc, si_final, normalize(q.p - si_final.p), normalize(ei.p - si_final.p))
                  : specular_reflectance(sc, si_final, normalize(ei.p - si_final.p));
    f *= geometric_term(vx, vtx, vy);
    return V3(f * ei.weight.x, f * ei.weight.y, f * ei.weight.z);
}

/* src/bsdfs/diffuse.cpp eval: albedo / pi * cos_theta_o (both cosines > 0) */
static V3 diffuse_eval(const Query &q, V3 dir) {
    Float co = dot(dir, q.n);
    if (q.cos_i <= 0.f || co <= 0.f) return V3(0.f);
    return (q.albedo * kInvPi) * co;
}

/* The receiver's BSDF toward the first specular vertex (manifold_ss.cpp:109,
 * 191; manifold_ms.cpp:113, 190): a query with albedo.x >= 0 is a diffuse
 * receiver; albedo.x = -(1 + shape id) names a receiver shape whose BSDF is
 * evaluated in the frame coordinate_system(n) with the incident direction
 * (albedo.y, albedo.z, cos_i). */
static V3 shape_bsdf_eval(const Shape &sh, V3 wi, V3 wo);
static V3 receiver_eval(const Scene &sc, const Query &q, V3 dir) {
    if (q.albedo.x >= 0.f) return diffuse_eval(q, dir);
    const int id = (int)(-q.albedo.x) - 1;
    if (id < 0 || id >= (int)sc.shapes.size()) return V3(0.f);
    V3 s, t;
    coordinate_system(q.n, s, t);
    return shape_bsdf_eval(sc.shapes[id], V3(q.albedo.y, q.albedo.z, q.cos_i), V3(dot(dir, s), dot(dir, t), dot(dir, q.n)));
}

static bool visible(const Scene &sc, const EI &ei, V3 p) {
    V3 d = p - ei.p;
    Float dist = norm(d);
    d *= 1.f / dist;
    Ray r; r.o = ei.p; r.d = d;
    r.mint = kRayEps * (1.f + hmax_abs(ei.p));
    r.maxt = dist * (1.f - kRayEps);
    return !ray_test(sc, r);
}

struct Stats {
    std::atomic<uint64_t> succeeded{0}, failed{0}, calls{0}, iters{0}, iters_max{0}, walks{0},
        newton{0}, connections{0};
};

static void update_max(std::atomic<uint64_t> &a, uint64_t v) {
    uint64_t cur = a.load();
    while (cur < v && !a.compare_exchange_weak(cur, v)) {}
}

/* manifold_ss.cpp:28-201 */
/* Learned seed proposal (no counterpart in the reference: it always seeds
 * uniformly, manifold_ss.cpp:223).  For the proposal's caster every walk
 * draws three numbers: u_sel, then the 2D sample.  u_sel < defensive keeps
 * the reference's uniform seeding with the 2D sample; otherwise component k
 * of the query's mixture (first k with u' < cdf[k], u' = (u_sel - defensive)
 * / (1 - defensive)) gives uv = mean_k + sigma_k * z with z from Box-Muller
 * (r = sqrt(-2 ln(1 - x)), angle 2 pi y), mapped to a seed point through the
 * caster's uv frame.  mix: 40 values of this query (cdf 8, means 16, sigmas
 * 16) with stride `stride`. */
struct Learned {
    int shape = -1;
    Float defensive = 1.f;
    int kind = 0;               /* 0 box frame, 1 sphere */
    V3 org, ax_u, ax_v;
    const float *mix = nullptr;
    size_t stride = 0;
};

static V3 learned_seed_point(const Learned &L, Float u, Float v) {
    if (L.kind == 1) {
        Float th = kPi * u, ph = 2.f * kPi * v;
        return L.org + V3(std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th)) * L.ax_u.x;
    }
    return L.org + L.ax_u * u + L.ax_v * v;
}

/* one walk's seed: returns p_start for sample_path (zero = uniform seeding
 * with `sample`) */
static V3 learned_seed(const Learned &L, PCG32 &rng, V2 &sample) {
    Float us = rng.next_f32();
    sample = rng.next_2d();
    if (us < L.defensive) return V3(0.f);
    Float u2 = (us - L.defensive) / (1.f - L.defensive);
    int k = 0;
    while (k < 7 && u2 >= L.mix[(size_t)k * L.stride]) ++k;
    Float r = std::sqrt(-2.f * std::log(1.f - sample.x));
    Float ang = 2.f * kPi * sample.y;
    Float u = L.mix[(size_t)(8 + 2 * k) * L.stride] + L.mix[(size_t)(24 + 2 * k) * L.stride] * (r * std::cos(ang));
    Float v = L.mix[(size_t)(9 + 2 * k) * L.stride] + L.mix[(size_t)(25 + 2 * k) * L.stride] * (r * std::sin(ang));
    return learned_seed_point(L, u, v);
}

static V3 ss_connect(const Scene &sc, const sms_config &cfg, const Query &q, PCG32 &rng,
                     int &count_out, int &walks_out, Stats &st, const Learned *learned = nullptr) {
    count_out = 0; walks_out = 0;
    EI ei = sample_emitter_interaction(sc, sc.emitters_ss, q, rng);
    V3 result(0.f);
    if (sc.casters_ss.empty() || ei.emitter < 0) return result;
    st.connections++;
    for (int caster : sc.casters_ss) {
        V3 value(0.f);
        SI si_final, si_init;
        int it = 0;
        /* offset normal of a rough caster (manifold_ss.cpp:60-70) */
        V3 no(0.f, 0.f, 1.f);
        Float p_offset = 1.f;
        if (is_rough(sc.shapes[caster].bsdf)) {
            V2 u = rng.next_2d();
            no = beckmann_sample(sc.shapes[caster].bsdf.alpha, u.x, u.y, p_offset);
        }
        if (!cfg.biased) {
            count_out = 0;
            const bool lrn = learned && learned->shape == caster;
            auto seed_of = [&](V2 &smp) -> V3 {
                if (lrn) return learned_seed(*learned, rng, smp);
                smp = rng.next_2d();
                return V3(0.f);
            };
            auto stage_of = [&]() { return cfg.twostage ? rng.next_2d() : V2{0.f, 0.f}; };
            V2 smp;
            V3 ps = seed_of(smp);
            V2 g = stage_of();
            bool ok = sample_path(sc, cfg, caster, q, ei, smp, ps, si_final, si_init, it, no, g);
            walks_out++; st.walks++; st.newton += it;
            if (!ok) { st.failed++; continue; }
            st.succeeded++;
            V3 direction = normalize(si_final.p - q.p);
            if (!visible(sc, ei, si_final.p)) continue;
            V3 spec = evaluate_path_contribution(sc, q, ei, si_final);
            V3 bsdf = receiver_eval(sc, q, direction);
            Float inv_prob = 1.f;
            int iterations = 1;
            st.calls++;
            while (true) {
                SI sf, si0;
                int it2 = 0;
                V2 smp2;
                V3 ps2 = seed_of(smp2);
                V2 g2 = stage_of();
                bool ok2 = sample_path(sc, cfg, caster, q, ei, smp2, ps2, sf, si0, it2, no, g2);
                walks_out++; st.walks++; st.newton += it2;
                if (ok2) {
                    V3 dt = normalize(sf.p - q.p);
                    if (std::fabs(dot(direction, dt) - 1.f) < cfg.uniqueness_threshold) break;
                }
                inv_prob += 1.f;
                iterations++;
                if (cfg.max_trials > 0 && iterations > cfg.max_trials) { inv_prob = 0.f; break; }
            }
            st.iters += (uint64_t)iterations;
            update_max(st.iters_max, (uint64_t)iterations);
            count_out = inv_prob == 0.f ? -1 : iterations;
            value = bsdf * spec * inv_prob;
        } else {
            std::vector<V3> solutions;
            for (int m = 0; m < cfg.max_trials; ++m) {
                const V2 smp = rng.next_2d();
                const V2 g = cfg.twostage ? rng.next_2d() : V2{0.f, 0.f};
                bool ok = sample_path(sc, cfg, caster, q, ei, smp, V3(0.f), si_final, si_init, it, no, g);
                walks_out++; st.walks++; st.newton += it;
                if (!ok) { st.failed++; continue; }
                st.succeeded++;
                V3 direction = normalize(si_final.p - q.p);
                if (!visible(sc, ei, si_final.p)) continue;
                bool dup = false;
                for (const V3 &s : solutions)
                    if (std::fabs(dot(direction, s) - 1.f) < cfg.uniqueness_threshold) { dup = true; break; }
                if (dup) continue;
                solutions.push_back(direction);
                V3 bsdf = receiver_eval(sc, q, direction);
                V3 spec = evaluate_path_contribution(sc, q, ei, si_final);
                value += bsdf * spec;
            }
            count_out += (int)solutions.size();
        }
        result += value * (1.f / p_offset);
    }
    return result;
}


/* ====================================================================
 * Multi-scatter SMS (src/librender/manifold_ms.cpp)
 * ==================================================================== */
struct MSBlock {
    V2 C, dx;
    M2 prev, cur, next, tmp, inv_lambda;
};

static M2 msub(const M2 &a, const M2 &b) {
    M2 r;
    for (int i = 0; i < 2; ++i) for (int j = 0; j < 2; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j];
    return r;
}
static M2 mneg(const M2 &a) {
    M2 r;
    for (int i = 0; i < 2; ++i) for (int j = 0; j < 2; ++j) r.m[i][j] = -a.m[i][j];
    return r;
}
static V2 vsub(V2 a, V2 b) { V2 r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }

/* manifold_ms.cpp:1192-1232 (block Thomas, Kaplanyan et al. 2014) */
static bool invert_tridiagonal_step(std::vector<MSBlock> &b) {
    auto inv = [](const M2 &A, M2 &Ai) {
        if (std::fabs(det(A)) == 0.f) return false;
        Ai = inverse(A);
        return true;
    };
    int n = (int)b.size();
    if (n == 0) return true;
    b[0].tmp = b[0].prev;
    if (!inv(b[0].cur, b[0].inv_lambda)) return false;
    for (int i = 1; i < n; ++i) {
        b[i].tmp = mul(b[i].prev, b[i - 1].inv_lambda);
        M2 m = msub(b[i].cur, mul(b[i].tmp, b[i - 1].next));
        if (!inv(m, b[i].inv_lambda)) return false;
    }
    b[0].dx = b[0].C;
    for (int i = 1; i < n; ++i) b[i].dx = vsub(b[i].C, mul(b[i].tmp, b[i - 1].dx));
    b[n - 1].dx = mul(b[n - 1].inv_lambda, b[n - 1].dx);
    for (int i = n - 2; i >= 0; --i) b[i].dx = mul(b[i].inv_lambda, vsub(b[i].dx, mul(b[i].next, b[i + 1].dx)));
    return true;
}

/* manifold_ms.cpp:1234-1268 (Jakob & Marschner 2012) */
static Float invert_tridiagonal_geo(std::vector<MSBlock> &b) {
    auto inv = [](const M2 &A, M2 &Ai) {
        if (std::fabs(det(A)) == 0.f) return false;
        Ai = inverse(A);
        return true;
    };
    int n = (int)b.size();
    if (n == 0) return 0.f;
    M2 Li;
    if (!inv(b[0].cur, Li)) return 0.f;
    for (int i = 0; i < n - 2; ++i) {
        b[i].tmp = mul(Li, b[i].next);
        M2 m = msub(b[i + 1].cur, mul(b[i + 1].prev, b[i].tmp));
        if (!inv(m, Li)) return 0.f;
    }
    b[n - 2].inv_lambda = mul(mneg(Li), b[n - 2].next);
    for (int i = n - 3; i >= 0; --i) b[i].inv_lambda = mul(mneg(b[i].tmp), b[i + 1].inv_lambda);
    return std::fabs(det(mneg(b[0].inv_lambda)));
}

static void d_sph_pair(V3 w, V3 du, V3 dv, Float &a, Float &b, Float &c, Float &d) { d_sphcoords(w, du, dv, a, b, c, d); }

/* manifold_ms.cpp:631-857 (n_offset = (0,0,1), positional light) */
static bool ms_step_anglediff(V3 x0, V3 lp, const std::vector<MVertex> &v, std::vector<MSBlock> &b,
                              const std::vector<V3> *offs = nullptr) {
    size_t k = v.size();
    b.assign(k, MSBlock());
    bool success = true;
    for (size_t i = 0; i < k; ++i) {
        V3 xp = i == 0 ? x0 : v[i - 1].p, xn = i == k - 1 ? lp : v[i + 1].p, xc = v[i].p;
        V3 wo = xn - xc;
        Float ilo = norm(wo);
        if (ilo < 1e-3f) return false;
        ilo = 1.f / ilo; wo *= ilo;
        V3 dwo_du = (v[i].dp_du - wo * dot(wo, v[i].dp_du)) * -ilo;
        V3 dwo_dv = (v[i].dp_dv - wo * dot(wo, v[i].dp_dv)) * -ilo;
        V3 wi = xp - xc;
        Float ili = norm(wi);
        if (ili < 1e-3f) return false;
        ili = 1.f / ili; wi *= ili;
        V3 dwi_du = (v[i].dp_du - wi * dot(wi, v[i].dp_du)) * -ili;
        V3 dwi_dv = (v[i].dp_dv - wi * dot(wi, v[i].dp_dv)) * -ili;
        const MVertex &vi = v[i];
        V3 n = vi.n, dndu = vi.dn_du, dndv = vi.dn_dv;
        if (offs) {
            /* offset normal of vertex i (:707-717); no-ops for (0, 0, 1) */
            const V3 o = (*offs)[i];
            n = vi.s * o.x + vi.t * o.y + vi.n * o.z;
            dndu = vi.ds_du * o.x + vi.dt_du * o.y + vi.dn_du * o.z;
            dndv = vi.ds_dv * o.x + vi.dt_dv * o.y + vi.dn_dv * o.z;
        }
        auto transform = [&](V3 w, V3 &out) { return vi.eta == 1.f ? reflect(w, n, out) : refract(w, n, vi.eta, out); };
        auto d_transform = [&](V3 w, V3 du, V3 dv, V3 nd_u, V3 nd_v, V3 &ou, V3 &ov) {
            if (vi.eta == 1.f) d_reflect(w, du, dv, n, nd_u, nd_v, ou, ov);
            else d_refract(w, du, dv, n, nd_u, nd_v, vi.eta, ou, ov);
        };
        bool ok_i = false;
        V3 wio;
        if (transform(wi, wio)) {
            Float to, po, tio, pio;
            sphcoords(wo, to, po); sphcoords(wio, tio, pio);
            Float dt = to - tio, dp = po - pio;
            if (dp < -kPi) dp += 2.f * kPi; else if (dp > kPi) dp -= 2.f * kPi;
            b[i].C.x = dt; b[i].C.y = dp;
            Float a0, a1, a2, a3, c0, c1, c2, c3;
            if (i > 0) {
                V3 du = (v[i - 1].dp_du - wi * dot(wi, v[i - 1].dp_du)) * ili;
                V3 dv = (v[i - 1].dp_dv - wi * dot(wi, v[i - 1].dp_dv)) * ili;
                V3 ou, ov;
                d_transform(wi, du, dv, V3(0.f), V3(0.f), ou, ov);
                d_sph_pair(wio, ou, ov, c0, c1, c2, c3);
                b[i].prev.m[0][0] = -c0; b[i].prev.m[1][0] = -c1; b[i].prev.m[0][1] = -c2; b[i].prev.m[1][1] = -c3;
            }
            V3 ou, ov;
            d_transform(wi, dwi_du, dwi_dv, dndu, dndv, ou, ov);
            d_sph_pair(wo, dwo_du, dwo_dv, a0, a1, a2, a3);
            d_sph_pair(wio, ou, ov, c0, c1, c2, c3);
            b[i].cur.m[0][0] = a0 - c0; b[i].cur.m[1][0] = a1 - c1; b[i].cur.m[0][1] = a2 - c2; b[i].cur.m[1][1] = a3 - c3;
            if (i < k - 1) {
                V3 du = (v[i + 1].dp_du - wo * dot(wo, v[i + 1].dp_du)) * ilo;
                V3 dv = (v[i + 1].dp_dv - wo * dot(wo, v[i + 1].dp_dv)) * ilo;
                d_sph_pair(wo, du, dv, a0, a1, a2, a3);
                b[i].next.m[0][0] = a0; b[i].next.m[1][0] = a1; b[i].next.m[0][1] = a2; b[i].next.m[1][1] = a3;
            }
            ok_i = true;
        }
        V3 woi;
        if (transform(wo, woi) && !ok_i) {
            Float ti, pi, toi, poi;
            sphcoords(wi, ti, pi); sphcoords(woi, toi, poi);
            Float dt = ti - toi, dp = pi - poi;
            if (dp < -kPi) dp += 2.f * kPi; else if (dp > kPi) dp -= 2.f * kPi;
            b[i].C.x = dt; b[i].C.y = dp;
            Float a0, a1, a2, a3, c0, c1, c2, c3;
            if (i > 0) {
                V3 du = (v[i - 1].dp_du - wi * dot(wi, v[i - 1].dp_du)) * ili;
                V3 dv = (v[i - 1].dp_dv - wi * dot(wi, v[i - 1].dp_dv)) * ili;
                d_sph_pair(wi, du, dv, a0, a1, a2, a3);
                b[i].prev.m[0][0] = a0; b[i].prev.m[1][0] = a1; b[i].prev.m[0][1] = a2; b[i].prev.m[1][1] = a3;
            }
            V3 ou, ov;
            d_transform(wo, dwo_du, dwo_dv, dndu, dndv, ou, ov);
            d_sph_pair(wi, dwi_du, dwi_dv, a0, a1, a2, a3);
            d_sph_pair(woi, ou, ov, c0, c1, c2, c3);
            b[i].cur.m[0][0] = a0 - c0; b[i].cur.m[1][0] = a1 - c1; b[i].cur.m[0][1] = a2 - c2; b[i].cur.m[1][1] = a3 - c3;
            if (i < k - 1) {
                V3 du = (v[i + 1].dp_du - wo * dot(wo, v[i + 1].dp_du)) * ilo;
                V3 dv = (v[i + 1].dp_dv - wo * dot(wo, v[i + 1].dp_dv)) * ilo;
                d_transform(wo, du, dv, V3(0.f), V3(0.f), ou, ov);
                d_sph_pair(woi, ou, ov, c0, c1, c2, c3);
                b[i].next.m[0][0] = -c0; b[i].next.m[1][0] = -c1; b[i].next.m[0][1] = -c2; b[i].next.m[1][1] = -c3;
            }
            ok_i = true;
        }
        success = success && ok_i;
    }
    if (!success || !invert_tridiagonal_step(b)) return false;
    return true;
}

/* manifold_ms.cpp:500-629 */
static bool ms_step_halfvector(V3 x0, V3 lp, const std::vector<MVertex> &v, std::vector<MSBlock> &b,
                               const std::vector<V3> *offs = nullptr) {
    size_t k = v.size();
    b.assign(k, MSBlock());
    for (size_t i = 0; i < k; ++i) {
        V3 xp = i == 0 ? x0 : v[i - 1].p, xn = i == k - 1 ? lp : v[i + 1].p, xc = v[i].p;
        V3 wo = xn - xc;
        Float ilo = norm(wo);
        if (ilo < 1e-3f) return false;
        ilo = 1.f / ilo; wo *= ilo;
        V3 wi = xp - xc;
        Float ili = norm(wi);
        if (ili < 1e-3f) return false;
        ili = 1.f / ili; wi *= ili;
        Float eta = v[i].eta;
        if (dot(wi, v[i].gn) < 0.f) eta = 1.f / eta;
        V3 h = wi + wo * eta;
        if (eta != 1.f) h *= -1.f;
        Float ilh = 1.f / norm(h);
        h *= ilh;
        ilo *= eta * ilh;
        ili *= ilh;
        V3 du, dv;
        if (i > 0) {
            du = (v[i - 1].dp_du - wi * dot(wi, v[i - 1].dp_du)) * ili;
            dv = (v[i - 1].dp_dv - wi * dot(wi, v[i - 1].dp_dv)) * ili;
            du -= h * dot(du, h); dv -= h * dot(dv, h);
            if (eta != 1.f) { du *= -1.f; dv *= -1.f; }
            b[i].prev.m[0][0] = dot(v[i].s, du); b[i].prev.m[0][1] = dot(v[i].s, dv);
            b[i].prev.m[1][0] = dot(v[i].t, du); b[i].prev.m[1][1] = dot(v[i].t, dv);
        }
        du = -v[i].dp_du * (ili + ilo) + wi * (dot(wi, v[i].dp_du) * ili) + wo * (dot(wo, v[i].dp_du) * ilo);
        dv = -v[i].dp_dv * (ili + ilo) + wi * (dot(wi, v[i].dp_dv) * ili) + wo * (dot(wo, v[i].dp_dv) * ilo);
        du -= h * dot(du, h); dv -= h * dot(dv, h);
        if (eta != 1.f) { du *= -1.f; dv *= -1.f; }
        b[i].cur.m[0][0] = dot(v[i].ds_du, h) + dot(v[i].s, du);
        b[i].cur.m[0][1] = dot(v[i].ds_dv, h) + dot(v[i].s, dv);
        b[i].cur.m[1][0] = dot(v[i].dt_du, h) + dot(v[i].t, du);
        b[i].cur.m[1][1] = dot(v[i].dt_dv, h) + dot(v[i].t, dv);
        if (i < k - 1) {
            du = (v[i + 1].dp_du - wo * dot(wo, v[i + 1].dp_du)) * ilo;
            dv = (v[i + 1].dp_dv - wo * dot(wo, v[i + 1].dp_dv)) * ilo;
            du -= h * dot(du, h); dv -= h * dot(dv, h);
            if (eta != 1.f) { du *= -1.f; dv *= -1.f; }
            b[i].next.m[0][0] = dot(v[i].s, du); b[i].next.m[0][1] = dot(v[i].s, dv);
            b[i].next.m[1][0] = dot(v[i].t, du); b[i].next.m[1][1] = dot(v[i].t, dv);
        }
        b[i].C.x = dot(v[i].s, h);
        b[i].C.y = dot(v[i].t, h);
        if (offs) {   /* C = H - N (:618-621) */
            b[i].C.x = b[i].C.x - (*offs)[i].x;
            b[i].C.y = b[i].C.y - (*offs)[i].y;
        }
    }
    return invert_tridiagonal_step(b);
}

static bool is_chain_shape(const Scene &sc, int s) {
    uint32_t f = sc.shapes[s].flags;
    return (f & SMS_SHAPE_CAUSTIC_CASTER_MULTI) || (f & SMS_SHAPE_CAUSTIC_BOUNCER);
}

/* si.spawn_ray (interaction.h:58-62) */
static Ray spawn_ray(V3 p, V3 d) {
    Ray r; r.o = p; r.d = d; r.mint = (1.f + hmax_abs(p)) * kRayEps; r.maxt = kInf;
    return r;
}

/* Trace the specular chain from x0 toward x1 (sample_seed_path :280-408 with
 * first_path/template shapes, reproject :859-918).  template_shapes empty ->
 * any caster_multi/bouncer shape is allowed (first path). */
/* Offset normals of a rough chain (manifold_ms.cpp:356-375): draw (non-null)
 * holds the walk's 2 numbers per vertex; a rough vertex of a first path draws
 * a Beckmann offset from them (its density multiplies *pdf), a smooth one keeps
 * (0, 0, 1).  Otherwise offs holds the template's offsets (null: all smooth). */
struct ChainOffsets {
    std::vector<V3> *offs = nullptr;
    const V2 *draw = nullptr;
    Float *pdf = nullptr;
};

static bool ms_trace_chain(const Scene &sc, int bounces, V3 x0, V3 x1, const std::vector<int> &tmpl,
                           bool require_chain_flags, std::vector<MVertex> &path, bool straight = false,
                           ChainOffsets co = ChainOffsets()) {
    path.clear();
    if (co.draw) { co.offs->clear(); *co.pdf = 1.f; }
    V3 wo = normalize(x1 - x0);
    Ray ray; ray.o = x0; ray.d = wo;
    while ((int)path.size() < bounces) {
        int bounce = (int)path.size();
        SI si = ray_intersect(sc, ray);
        if (!si.valid()) return false;
        if (require_chain_flags && !is_chain_shape(sc, si.shape)) return false;
        if (!tmpl.empty() && si.shape != tmpl[bounce]) return false;
        MVertex v;
        vertex_from_si(sc, si, v);
        path.push_back(v);
        V3 m = v.n;
        if (co.draw) {
            V3 o(0.f, 0.f, 1.f);
            const sms_bsdf &bs = sc.shapes[si.shape].bsdf;
            if (is_rough(bs)) {
                Float p_o;
                o = beckmann_sample(bs.alpha, co.draw[bounce].x, co.draw[bounce].y, p_o);
                *co.pdf *= p_o;
            }
            co.offs->push_back(o);
        }
        if (co.offs && (int)co.offs->size() > bounce) {
            const V3 o = (*co.offs)[bounce];
            m = v.s * o.x + v.t * o.y + v.n * o.z;   /* :380-382, :894-897 */
        }
        V3 wi = -wo;
        bool ok = true;
        if (straight) { /* MNEE seed path: no scattering (manifold_ms.cpp:377-397) */ }
        else if (v.eta == 1.f) ok = reflect(wi, m, wo);
        else ok = refract(wi, m, v.eta, wo);
        if (!ok) return false;
        ray = spawn_ray(si.p, wo);
    }
    return true;
}

/* manifold_ms.cpp:410-498 */
static bool ms_newton(const Scene &sc, const sms_config &cfg, V3 x0, V3 lp, const std::vector<int> &tmpl,
                      std::vector<MVertex> &path, int &iters, std::vector<V3> *offs = nullptr) {
    bool success = false;
    int it = 0;
    Float beta = 1.f;
    bool needs_update = true;
    std::vector<MSBlock> b;
    while (it < cfg.max_iterations) {
        bool ok = true;
        if (needs_update)
            ok = cfg.halfvector_constraints ? ms_step_halfvector(x0, lp, path, b, offs)
                                            : ms_step_anglediff(x0, lp, path, b, offs);
        if (!ok) break;
        bool conv = true;
        for (const MSBlock &bl : b)
            if (std::sqrt(bl.C.x * bl.C.x + bl.C.y * bl.C.y) > cfg.solver_threshold) { conv = false; break; }
        if (conv) { success = true; break; }
        /* only the first proposed position drives the reprojection (:865-867) */
        const MVertex &v0 = path[0];
        V3 p0 = v0.p - (v0.dp_du * b[0].dx.x + v0.dp_dv * b[0].dx.y) * (cfg.step_scale * beta);
        std::vector<MVertex> prop;
        ChainOffsets co;
        co.offs = offs;
        bool proj = ms_trace_chain(sc, (int)path.size(), x0, p0, tmpl, false, prop, false, co) &&
                    prop.size() == tmpl.size();
        if (!proj) { beta = 0.5f * beta; needs_update = false; }
        else { beta = omin(1.f, 2.f * beta); path = prop; needs_update = true; }
        it++;
    }
    iters = it;
    if (!success) return false;
    size_t n = path.size();
    for (size_t i = 0; i < n; ++i) {
        V3 xp = i == 0 ? x0 : path[i - 1].p, xn = i == n - 1 ? lp : path[i + 1].p;
        V3 wi = normalize(xp - path[i].p), wo = normalize(xn - path[i].p);
        bool refraction = dot(path[i].gn, wi) * dot(path[i].gn, wo) < 0.f;
        bool reflection = !refraction;
        if ((path[i].eta == 1.f && !reflection) || (path[i].eta != 1.f && !refraction)) return false;
    }
    return true;
}

/* sample_path (:203-227): seed path + Newton.  seed_shapes: in = template
 * (empty for a first path), out = this walk's seed shapes. */
/* The offsets of an estimate's template (rough chains). */
struct MsOffsets {
    std::vector<V3> offs;   /* one per chain vertex */
    Float pdf = 1.f;
};

static bool ms_sample_path(const Scene &sc, const sms_config &cfg, int caster, const Query &q, V3 lp, V2 sample,
                           V3 p_start, std::vector<int> &tmpl, bool first_path, std::vector<MVertex> &path,
                           int &iters, bool &seed_ok, MsOffsets *mo = nullptr, const V2 *draw = nullptr) {
    iters = 0;
    seed_ok = false;
    V3 x1 = sample_position(sc.shapes[caster], sample);
    if (p_start.x != 0.f || p_start.y != 0.f || p_start.z != 0.f) x1 = p_start;
    static const std::vector<int> none;
    if (cfg.mnee_init) x1 = mnee_target(sc.shapes[caster], lp);
    /* a first path draws its own offsets; later walks follow the template's */
    std::vector<V3> own;
    Float own_pdf = 1.f;
    ChainOffsets co;
    if (mo) {
        if (first_path) { co.offs = &own; co.draw = draw; co.pdf = &own_pdf; }
        else co.offs = &mo->offs;
    }
    if (!ms_trace_chain(sc, cfg.bounces, q.p, x1, first_path ? none : tmpl, true, path, cfg.mnee_init != 0, co))
        return false;
    seed_ok = true;
    if (first_path) {
        tmpl.clear();
        for (const MVertex &v : path) tmpl.push_back(v.shape);
        if (mo) { mo->offs = own; mo->pdf = own_pdf; }
    }
    return ms_newton(sc, cfg, q.p, lp, tmpl, path, iters, mo ? &mo->offs : nullptr);
}

/* manifold_ms.cpp:920-1023.  At a rough vertex the reference computes the
 * glossy BSDF value in the half-vector domain (:963-985) but multiplies only
 * the delta branch's factor into the throughput (:1007), so a rough vertex
 * contributes 1; restated as is. */
static Float ms_specular_reflectance(const Scene &sc, V3 x0, V3 lp, const std::vector<MVertex> &path) {
    if (path.empty()) return 0.f;
    Ray ray; ray.o = x0; ray.d = normalize(path[0].p - x0);
    Float val = 1.f;
    SI si;
    for (size_t k = 0; k < path.size(); ++k) {
        si = ray_intersect(sc, ray);
        if (!si.valid()) return 0.f;
        V3 wo = k + 1 < path.size() ? normalize(path[k + 1].p - si.p) : normalize(lp - si.p);
        if (!is_rough(sc.shapes[si.shape].bsdf)) val *= specular_reflectance(sc, si, wo);
        ray = Ray(); ray.o = si.p; ray.d = wo;
    }
    Ray vis; vis.o = si.p; vis.d = normalize(lp - si.p);
    vis.mint = kRayEps * (1.f + hmax_abs(si.p));
    vis.maxt = norm(lp - si.p) * (1.f - kRayEps);
    if (ray_test(sc, vis)) return 0.f;
    return val;
}

/* manifold_ms.cpp:1025-1190 (positional endpoint) */
static Float ms_geometric_term(const MVertex &vx, const std::vector<MVertex> &path, const MVertex &vy) {
    std::vector<MVertex> v = path;
    v.push_back(vy);
    size_t k = v.size();
    std::vector<MSBlock> b(k);
    for (size_t i = 0; i + 1 < k; ++i) {
        V3 xc = v[i].p, xn = v[i + 1].p;
        V3 wo = xn - xc;
        Float ilo = norm(wo);
        if (ilo < 1e-3f) return 0.f;
        ilo = 1.f / ilo; wo *= ilo;
        V3 xp = i == 0 ? vx.p : v[i - 1].p;
        V3 wi = xp - xc;
        Float ili = norm(wi);
        if (ili < 1e-3f) return 0.f;
        ili = 1.f / ili; wi *= ili;
        Float eta = v[i].eta;
        if (dot(wi, v[i].gn) < 0.f) eta = 1.f / eta;
        V3 h = wi + wo * eta;
        if (eta != 1.f) h *= -1.f;
        Float ilh = 1.f / norm(h);
        h *= ilh;
        ilo *= eta * ilh;
        ili *= ilh;
        Float dpdu_n = dot(v[i].dp_du, v[i].n), dpdv_n = dot(v[i].dp_dv, v[i].n);
        V3 s = v[i].dp_du - v[i].n * dpdu_n, t = v[i].dp_dv - v[i].n * dpdv_n;
        V3 du, dv;
        if (i > 0) {
            du = (v[i - 1].dp_du - wi * dot(wi, v[i - 1].dp_du)) * ili;
            dv = (v[i - 1].dp_dv - wi * dot(wi, v[i - 1].dp_dv)) * ili;
            du -= h * dot(du, h); dv -= h * dot(dv, h);
            if (eta != 1.f) { du *= -1.f; dv *= -1.f; }
            b[i].prev.m[0][0] = dot(s, du); b[i].prev.m[0][1] = dot(s, dv);
            b[i].prev.m[1][0] = dot(t, du); b[i].prev.m[1][1] = dot(t, dv);
        }
        du = -v[i].dp_du * (ili + ilo) + wi * (dot(wi, v[i].dp_du) * ili) + wo * (dot(wo, v[i].dp_du) * ilo);
        dv = -v[i].dp_dv * (ili + ilo) + wi * (dot(wi, v[i].dp_dv) * ili) + wo * (dot(wo, v[i].dp_dv) * ilo);
        du -= h * dot(du, h); dv -= h * dot(dv, h);
        if (eta != 1.f) { du *= -1.f; dv *= -1.f; }
        Float hn = dot(h, v[i].n), hdu = dot(h, v[i].dn_du), hdv = dot(h, v[i].dn_dv);
        b[i].cur.m[0][0] = dot(du, s) - dot(v[i].dp_du, v[i].dn_du) * hn - dpdu_n * hdu;
        b[i].cur.m[0][1] = dot(dv, s) - dot(v[i].dp_du, v[i].dn_dv) * hn - dpdu_n * hdv;
        b[i].cur.m[1][0] = dot(du, t) - dot(v[i].dp_dv, v[i].dn_du) * hn - dpdv_n * hdu;
        b[i].cur.m[1][1] = dot(dv, t) - dot(v[i].dp_dv, v[i].dn_dv) * hn - dpdv_n * hdv;
        du = (v[i + 1].dp_du - wo * dot(wo, v[i + 1].dp_du)) * ilo;
        dv = (v[i + 1].dp_dv - wo * dot(wo, v[i + 1].dp_dv)) * ilo;
        du -= h * dot(du, h); dv -= h * dot(dv, h);
        if (eta != 1.f) { du *= -1.f; dv *= -1.f; }
        b[i].next.m[0][0] = dot(s, du); b[i].next.m[0][1] = dot(s, dv);
        b[i].next.m[1][0] = dot(t, du); b[i].next.m[1][1] = dot(t, dv);
    }
    Float dx1_dxend = invert_tridiagonal_geo(b);
    V3 d = vx.p - v[0].p;
    Float inv_r2 = 1.f / dot(d, d);
    d *= std::sqrt(inv_r2);
    return std::fabs(dot(d, v[0].gn)) * inv_r2 * dx1_dxend;
}

/* manifold_ms.cpp:229-278 */
static V3 ms_contribution(const Scene &sc, const Query &q, const EI &ei_in, const std::vector<MVertex> &path_in) {
    EI ei = ei_in;
    const MVertex &last = path_in.back();
    if (ei.is_point) {
        const Emitter &e = sc.emitters[ei.emitter];
        V3 d = e.p - last.p;
        Float dist = norm(d);
        Float inv = 1.f / dist;
        V3 spec = e.radiance * (inv * inv);
        Float emitter_pdf = ei.pdf;
        ei.p = e.p;
        ei.pdf = 1.f;
        ei.weight = (spec * dist) * dist;
        ei.pdf *= emitter_pdf;
        ei.weight = ei.weight * (1.f / emitter_pdf);
    }
    MVertex vy;
    if (!emitter_vertex(sc, ei, last.p, vy)) return V3(0.f);
    std::vector<MVertex> path = path_in;
    for (MVertex &v : path) make_orthonormal(v);
    MVertex vx;
    vx.p = q.p; vx.dp_du = q.dp_du; vx.dp_dv = q.dp_dv; vx.gn = q.n; vx.n = q.n;
    vx.dn_du = V3(0.f); vx.dn_dv = V3(0.f);
    make_orthonormal(vx);
    Float f = ms_specular_reflectance(sc, q.p, ei.p, path);
    f *= ms_geometric_term(vx, path, vy);
    return V3(f * ei.weight.x, f * ei.weight.y, f * ei.weight.z);
}

/* A chain shape (caster_multi or bouncer) with a rough BSDF: the estimate
 * samples offset normals (manifold_ms.cpp:356-375). */
static bool ms_rough_chain(const Scene &sc) {
    for (size_t s = 0; s < sc.shapes.size(); ++s)
        if (is_chain_shape(sc, (int)s) && is_rough(sc.shapes[s].bsdf)) return true;
    return false;
}

/* The random numbers of one walk.  Smooth chains: the seed position's 2 (the
 * reference's draw order).  Rough chains: every walk owns a fixed run of
 * 2 + 2 bounces numbers -- the seed position, then 2 per chain vertex for an
 * offset normal, used only by a first path at a rough vertex.  (The reference
 * draws those only when they are used, so later walks' positions in its
 * sampler depend on earlier walks' outcomes; the fixed run keeps walks
 * independent, as the batched device estimators need, with the same
 * expectation.) */
struct MsWalkDraws {
    V2 seed;
    V2 offs[8];
};
static MsWalkDraws ms_walk_draws(PCG32 &rng, bool rough, int bounces) {
    MsWalkDraws d;
    d.seed = rng.next_2d();
    if (rough)
        for (int b = 0; b < bounces; ++b) d.offs[b] = rng.next_2d();
    return d;
}

/* manifold_ms.cpp:27-201 */
static V3 ms_connect(const Scene &sc, const sms_config &cfg, const Query &q, PCG32 &rng, int &count_out,
                     int &walks_out, Stats &st) {
    count_out = 0; walks_out = 0;
    EI ei = sample_emitter_interaction(sc, sc.emitters_ms, q, rng);
    V3 result(0.f);
    if (sc.casters_ms.empty() || ei.emitter < 0) return result;
    st.connections++;
    const bool rough = ms_rough_chain(sc);
    for (int caster : sc.casters_ms) {
        V3 value(0.f);
        std::vector<int> tmpl;
        std::vector<MVertex> path;
        int it = 0;
        bool seed_ok;
        MsOffsets mo;
        MsOffsets *mop = rough ? &mo : nullptr;
        if (!cfg.biased) {
            count_out = 0;
            MsWalkDraws wd = ms_walk_draws(rng, rough, cfg.bounces);
            bool ok = ms_sample_path(sc, cfg, caster, q, ei.p, wd.seed, V3(0.f), tmpl, true, path, it, seed_ok, mop,
                                     wd.offs);
            walks_out++; st.walks++; st.newton += it;
            if (!ok) { st.failed++; continue; }
            st.succeeded++;
            V3 direction = normalize(path[0].p - q.p);
            V3 spec = ms_contribution(sc, q, ei, path);
            V3 bsdf = receiver_eval(sc, q, direction);
            Float inv_prob = 1.f;
            int iterations = 1;
            st.calls++;
            while (true) {
                std::vector<MVertex> tp;
                int it2 = 0;
                MsWalkDraws td = ms_walk_draws(rng, rough, cfg.bounces);
                bool ok2 = ms_sample_path(sc, cfg, caster, q, ei.p, td.seed, V3(0.f), tmpl, false, tp, it2, seed_ok,
                                          mop, td.offs);
                walks_out++; st.walks++; st.newton += it2;
                if (ok2 && std::fabs(dot(direction, normalize(tp[0].p - q.p)) - 1.f) < cfg.uniqueness_threshold) break;
                inv_prob += 1.f;
                iterations++;
                if (cfg.max_trials > 0 && iterations > cfg.max_trials) { inv_prob = 0.f; break; }
            }
            st.iters += (uint64_t)iterations;
            update_max(st.iters_max, (uint64_t)iterations);
            count_out = inv_prob == 0.f ? -1 : iterations;
            value = bsdf * spec * inv_prob;
        } else {
            std::vector<V3> solutions;
            for (int m = 0; m < cfg.max_trials; ++m) {
                bool first = tmpl.empty();
                MsWalkDraws wd = ms_walk_draws(rng, rough, cfg.bounces);
                bool ok = ms_sample_path(sc, cfg, caster, q, ei.p, wd.seed, V3(0.f), tmpl, first, path, it, seed_ok,
                                         mop, wd.offs);
                if (!seed_ok && first) tmpl.clear();
                walks_out++; st.walks++; st.newton += it;
                if (!ok) { st.failed++; continue; }
                st.succeeded++;
                V3 direction = normalize(path[0].p - q.p);
                bool dup = false;
                for (const V3 &s : solutions)
                    if (std::fabs(dot(direction, s) - 1.f) < cfg.uniqueness_threshold) { dup = true; break; }
                if (dup) continue;
                solutions.push_back(direction);
                V3 bsdf = receiver_eval(sc, q, direction);
                V3 spec = ms_contribution(sc, q, ei, path);
                value += bsdf * spec;
            }
            count_out += (int)solutions.size();
        }
        /* result += value / m_offset_normals_pdf (:198) */
        result += rough ? V3(value.x / mo.pdf, value.y / mo.pdf, value.z / mo.pdf) : value;
    }
    return result;
}


/* ====================================================================
 * Glints (src/librender/manifold_glints.cpp)
 * ==================================================================== */
struct GQuery {
    V3 p, n, dp_du, dp_dv, sensor;
    V2 uv, duv_dx, duv_dy;
};

static GQuery load_gquery(const float *q, uint32_t n, uint32_t i) {
    auto f = [&](int k) { return q[(size_t)k * n + i]; };
    GQuery r;
    r.p = V3(f(0), f(1), f(2)); r.n = V3(f(3), f(4), f(5));
    r.dp_du = V3(f(6), f(7), f(8)); r.dp_dv = V3(f(9), f(10), f(11));
    r.uv.x = f(12); r.uv.y = f(13); r.duv_dx.x = f(14); r.duv_dx.y = f(15);
    r.duv_dy.x = f(16); r.duv_dy.y = f(17);
    r.sensor = V3(f(18), f(19), f(20));
    return r;
}

/* bilinear setup of Normalmap::eval_normal (normalmap.h:62-104) at level 0
 * after the tiling wrap of NormalmapBSDF::slope (src/bsdfs/normalmap.cpp:305-316) */
static void nm_texels(const NormalMap &m, V2 uv_in, uint32_t idx[4], Float &wx, Float &wy) {
    Float u = uv_in.x * m.tiles, v = uv_in.y * m.tiles;
    u -= std::floor(u);
    v -= std::floor(v);
    Float res = (Float)m.res;
    Float duv = 1.f / res;
    Float px = (u - 0.5f * duv) * res, py = (v - 0.5f * duv) * res;
    px = omin(omax(px, 0.f), res - 1.f);
    py = omin(omax(py, 0.f), res - 1.f);
    uint32_t x0 = (uint32_t)std::floor(px), y0 = (uint32_t)std::floor(py);
    uint32_t x1 = omin(x0 + 1, m.res - 1), y1 = omin(y0 + 1, m.res - 1);
    x0 = omin(x0, m.res - 1); y0 = omin(y0, m.res - 1);
    idx[0] = y0 * m.res + x0; idx[1] = y0 * m.res + x1; idx[2] = y1 * m.res + x0; idx[3] = y1 * m.res + x1;
    wx = px - (Float)x0;
    wy = py - (Float)y0;
}

/* NormalmapBSDF::slope: (-n[0], -n[1]) of the bilinear slope normal */
static V2 nm_slope(const NormalMap &m, V2 uv) {
    uint32_t id[4]; Float wx, wy;
    nm_texels(m, uv, id, wx, wy);
    Float w0x = 1.f - wx, w0y = 1.f - wy;
    V2 r;
    Float a0 = w0x * m.sx[id[0]] + wx * m.sx[id[1]], a1 = w0x * m.sx[id[2]] + wx * m.sx[id[3]];
    Float b0 = w0x * m.sy[id[0]] + wx * m.sy[id[1]], b1 = w0x * m.sy[id[2]] + wx * m.sy[id[3]];
    r.x = w0y * a0 + wy * a1;
    r.y = w0y * b0 + wy * b1;
    return r;
}

/* NormalmapBSDF::slope_derivative (normalmap.cpp:318-336 with
 * normalmap.h:125-193): analytic bilinear derivative x res x tiles */
static void nm_slope_derivative(const NormalMap &m, V2 uv, V2 &du, V2 &dv) {
    uint32_t id[4]; Float wx, wy;
    nm_texels(m, uv, id, wx, wy);
    Float res = (Float)m.res;
    auto d = [&](const std::vector<Float> &c, Float &ou, Float &ov) {
        Float v00 = c[id[0]], v10 = c[id[1]], v01 = c[id[2]], v11 = c[id[3]];
        Float tmp = v01 + v10 - v11;
        ou = (v10 + v00 * (wy - 1.f) - tmp * wy) * res;
        ov = (v01 + v00 * (wx - 1.f) - tmp * wx) * res;
    };
    Float ux, vx_, uy, vy_;
    d(m.sx, ux, vx_);
    d(m.sy, uy, vy_);
    du.x = ux * m.tiles; du.y = uy * m.tiles;
    dv.x = vx_ * m.tiles; dv.y = vy_ * m.tiles;
}

/* manifold_glints.cpp:348-373 */
static bool glint_step(const NormalMap &m, V2 target, V2 uv, V2 &C, V2 &dX) {
    V2 cur = nm_slope(m, uv);
    C.x = cur.x - target.x; C.y = cur.y - target.y;
    V2 du, dv;
    nm_slope_derivative(m, uv, du, dv);
    M2 J;
    J.m[0][0] = du.x; J.m[1][0] = du.y; J.m[0][1] = dv.x; J.m[1][1] = dv.y;
    if (std::fabs(det(J)) < 1e-6f) return false;
    dX = mul(inverse(J), C);
    return true;
}

/* manifold_glints.h:162-194 */
static bool inside_triangle(V2 p, V2 a, V2 b, V2 c) {
    V2 v0{c.x - a.x, c.y - a.y}, v1{b.x - a.x, b.y - a.y}, v2{p.x - a.x, p.y - a.y};
    Float d00 = v0.x * v0.x + v0.y * v0.y, d01 = v0.x * v1.x + v0.y * v1.y, d02 = v0.x * v2.x + v0.y * v2.y,
          d11 = v1.x * v1.x + v1.y * v1.y, d12 = v1.x * v2.x + v1.y * v2.y;
    Float inv = 1.f / (d00 * d11 - d01 * d01);
    Float u = (d11 * d02 - d01 * d12) * inv, v = (d00 * d12 - d01 * d02) * inv;
    return u >= 0.f && v >= 0.f && u + v < 1.f;
}

/* manifold_glints.cpp:296-343 */
static bool glint_newton(const sms_config &cfg, const NormalMap &m, V2 target, V2 uv_init, const GQuery &q, V2 &uv_out,
                         int &iters) {
    V2 uv = uv_init;
    auto corner = [&](Float a, Float b) {
        V2 r; r.x = q.uv.x + a * q.duv_dx.x + b * q.duv_dy.x; r.y = q.uv.y + a * q.duv_dx.y + b * q.duv_dy.y;
        return r;
    };
    V2 fa = corner(0.5f, 0.5f), fb = corner(0.5f, -0.5f), fc = corner(-0.5f, -0.5f), fd = corner(-0.5f, 0.5f);
    bool success = false;
    int it = 0;
    Float beta = 1.f;
    while (it < cfg.max_iterations) {
        V2 C, step;
        if (!glint_step(m, target, uv, C, step)) break;
        if (std::sqrt(C.x * C.x + C.y * C.y) < cfg.solver_threshold) { success = true; break; }
        V2 prop;
        prop.x = uv.x - cfg.step_scale * beta * step.x;
        prop.y = uv.y - cfg.step_scale * beta * step.y;
        if (!(inside_triangle(prop, fa, fb, fc) || inside_triangle(prop, fa, fc, fd))) {
            beta = 0.5f * beta;
            it++;
            continue;
        }
        beta = omin(1.f, 2.f * beta);
        uv = prop;
        it++;
    }
    iters = it;
    uv_out = uv;
    return success;
}

static void base_frame(const GQuery &q, V3 &s, V3 &t) {
    s = normalize(q.dp_du - q.n * dot(q.n, q.dp_du));
    t = cross(q.n, s);
}

/* Inverse error function.  enoki's erfinv (the reference's) is not in the
 * checkout; this one starts from Winitzki's closed-form approximation (S.
 * Winitzki, "A handy approximation for the error function and its inverse",
 * 2008) and refines it with Newton steps on std::erf in double, so it is
 * accurate to double rounding before the final conversion. */
static double erfinv_double(double y) {
    if (!(y > -1.0)) return -std::numeric_limits<double>::infinity();
    if (!(y < 1.0)) return std::numeric_limits<double>::infinity();
    const double a = 0.147, pi = 3.14159265358979323846;
    const double l = std::log((1.0 - y) * (1.0 + y));
    const double b = 2.0 / (pi * a) + 0.5 * l;
    double x = std::copysign(std::sqrt(std::sqrt(b * b - l / a) - b), y);
    for (int i = 0; i < 4; ++i) {
        const double e = std::erf(x) - y;
        x -= e / (2.0 / std::sqrt(pi) * std::exp(-x * x));
    }
    return x;
}
static Float erfinv_f(Float y) {
    ORC_COUNT_FP64_OPS(1);
    return Float((float)erfinv_double((double)y));
}

/* Visible-normal sampling of an isotropic Beckmann distribution
 * (include/mitsuba/render/microfacet.h:287-314 with sample_visible_11,
 * :357-394, smith_g1 :331-355, Frame3f::sincos_phi frame.h:107-118): the
 * offset normal of a rough glinty surface (manifold_glints.cpp:56-64). */
static V3 beckmann_sample_visible(Float alpha, V3 wi, V2 u, Float &pdf) {
    V3 wp = normalize(V3(alpha * wi.x, alpha * wi.y, wi.z));
    Float st2 = wp.x * wp.x + wp.y * wp.y;
    Float sin_phi = 0.f, cos_phi = 1.f;
    if (!(std::fabs(st2) <= 4.f * std::numeric_limits<float>::epsilon())) {
        Float inv = 1.f / std::sqrt(st2);
        cos_phi = omin(1.f, omax(-1.f, wp.x * inv));
        sin_phi = omin(1.f, omax(-1.f, wp.y * inv));
    }
    const Float cos_i = wp.z;
    /* sample_visible_11, Beckmann */
    const Float tan_i = safe_sqrt(1.f - cos_i * cos_i) / cos_i;
    const Float cot_i = 1.f / tan_i;
    const Float maxval = std::erf(cot_i);
    V2 sm;
    sm.x = omax(omin(u.x, 1.f - 1e-6f), 1e-6f);
    sm.y = omax(omin(u.y, 1.f - 1e-6f), 1e-6f);
    const Float kInvSqrtPi = 0.56418958354775628695f;
    Float x = maxval - (maxval + 1.f) * std::erf(std::sqrt(-std::log(sm.x)));
    sm.x = sm.x * (1.f + maxval + kInvSqrtPi * tan_i * std::exp(-(cot_i * cot_i)));
    for (int i = 0; i < 3; ++i) {
        Float slope = erfinv_f(x);
        Float value = 1.f + x + kInvSqrtPi * tan_i * std::exp(-(slope * slope)) - sm.x;
        Float deriv = 1.f - slope * tan_i;
        x = x - value / deriv;
    }
    V2 sl;
    sl.x = erfinv_f(x);
    sl.y = erfinv_f(2.f * sm.y - 1.f);
    /* rotate and unstretch */
    V2 r;
    r.x = (cos_phi * sl.x - sin_phi * sl.y) * alpha;
    r.y = (sin_phi * sl.x + cos_phi * sl.y) * alpha;
    V3 m = normalize(V3(-r.x, -r.y, 1.f));
    pdf = beckmann_D(m, alpha) * beckmann_G1(wi, m, alpha) * std::fabs(dot(wi, m)) / wi.z;
    return m;
}

/* manifold_glints.cpp:225-265; no = the offset normal (local frame) */
static bool sample_glint(const sms_config &cfg, const NormalMap &m, const GQuery &q, V3 lp, V2 fp, V2 &uv_final,
                         V2 &uv_init, int &iters, V3 no = V3(0.f, 0.f, 1.f)) {
    iters = 0;
    V3 s, t;
    base_frame(q, s, t);
    V3 wiw = normalize(q.sensor - q.p), wow = normalize(lp - q.p);
    V3 wi(dot(wiw, s), dot(wiw, t), dot(wiw, q.n)), wo(dot(wow, s), dot(wow, t), dot(wow, q.n));
    if (wi.z <= 0.f || wo.z <= 0.f) return false;
    V3 h = normalize(wi + wo);
    V2 target;
    target.x = -h.x / h.z + (-no.x / no.z);
    target.y = -h.y / h.z + (-no.y / no.z);
    V2 duv;
    duv.x = (fp.x - 0.5f) * q.duv_dx.x + (fp.y - 0.5f) * q.duv_dy.x;
    duv.y = (fp.x - 0.5f) * q.duv_dx.y + (fp.y - 0.5f) * q.duv_dy.y;
    uv_init.x = q.uv.x + duv.x;
    uv_init.y = q.uv.y + duv.y;
    return glint_newton(cfg, m, target, uv_init, q, uv_final, iters);
}

/* normal-mapped shading frame and its derivative at uv (normalmap.cpp:218-290)
 * for a flat base surface (base frame derivative 0) */
static void glint_vertex(const NormalMap &m, const GQuery &q, V2 uv, MVertex &v) {
    V3 s, t;
    base_frame(q, s, t);
    V2 sl = nm_slope(m, uv);
    V2 du, dv;
    nm_slope_derivative(m, uv, du, dv);
    V3 nl(-sl.x, -sl.y, 1.f);
    V3 wn = s * nl.x + t * nl.y + q.n * nl.z;
    Float inv_len = 1.f / norm(wn);
    wn *= inv_len;
    /* eval_normal_derivatives returns (-d sx, -d sy, 0); the frame maps it to world */
    V3 dnu = (s * -du.x + t * -du.y) * inv_len;
    V3 dnv = (s * -dv.x + t * -dv.y) * inv_len;
    dnu -= wn * dot(dnu, wn);
    dnv -= wn * dot(dnv, wn);
    v = MVertex();
    v.p = q.p; v.dp_du = q.dp_du; v.dp_dv = q.dp_dv; v.gn = q.n; v.n = wn;
    v.dn_du = dnu; v.dn_dv = dnv; v.eta = 1.f;
    if (dot(v.n, v.gn) < 0.f) v.gn = -v.gn;
}

/* manifold_glints.cpp:411-554 (positional light) */
static Float glint_geometric_term(const MVertex &v0, const MVertex &v1, const MVertex &v2) {
    V3 wi = v0.p - v1.p;
    Float ili = norm(wi);
    if (ili < 1e-3f) return 0.f;
    ili = 1.f / ili; wi *= ili;
    V3 wo = v2.p - v1.p;
    Float ilo = norm(wo);
    if (ilo < 1e-3f) return 0.f;
    ilo = 1.f / ilo; wo *= ilo;
    V3 h = wi + wo;
    Float ilh = 1.f / norm(h);
    h *= ilh;
    ilo *= ilh;
    ili *= ilh;
    Float dpdu_n = dot(v1.dp_du, v1.n), dpdv_n = dot(v1.dp_dv, v1.n);
    V3 s = v1.dp_du - v1.n * dpdu_n, t = v1.dp_dv - v1.n * dpdv_n;
    V3 dh_du = -v1.dp_du * (ili + ilo) + wi * (dot(wi, v1.dp_du) * ili) + wo * (dot(wo, v1.dp_du) * ilo);
    V3 dh_dv = -v1.dp_dv * (ili + ilo) + wi * (dot(wi, v1.dp_dv) * ili) + wo * (dot(wo, v1.dp_dv) * ilo);
    dh_du -= h * dot(dh_du, h);
    dh_dv -= h * dot(dh_dv, h);
    Float hn = dot(h, v1.n), hdu = dot(h, v1.dn_du), hdv = dot(h, v1.dn_dv);
    M2 d11;
    d11.m[0][0] = dot(dh_du, s) - dot(v1.dp_du, v1.dn_du) * hn - dpdu_n * hdu;
    d11.m[0][1] = dot(dh_dv, s) - dot(v1.dp_du, v1.dn_dv) * hn - dpdu_n * hdv;
    d11.m[1][0] = dot(dh_du, t) - dot(v1.dp_dv, v1.dn_du) * hn - dpdv_n * hdu;
    d11.m[1][1] = dot(dh_dv, t) - dot(v1.dp_dv, v1.dn_dv) * hn - dpdv_n * hdv;
    dh_du = (v2.dp_du - wo * dot(wo, v2.dp_du)) * ilo;
    dh_dv = (v2.dp_dv - wo * dot(wo, v2.dp_dv)) * ilo;
    dh_du -= h * dot(dh_du, h);
    dh_dv -= h * dot(dh_dv, h);
    M2 d12;
    d12.m[0][0] = dot(dh_du, s); d12.m[0][1] = dot(dh_dv, s);
    d12.m[1][0] = dot(dh_du, t); d12.m[1][1] = dot(dh_dv, t);
    if (std::fabs(det(d11)) < 1e-6f) return 0.f;
    Float dx1_dx2 = std::fabs(det(mul(inverse(d11), d12)));
    V3 d = v0.p - v1.p;
    Float inv_r2 = 1.f / dot(d, d);
    d *= std::sqrt(inv_r2);
    Float G = std::fabs(dot(d, v1.gn)) * inv_r2 * dx1_dx2;
    return omin(1e-5f, G);
}

/* manifold_glints.cpp:375-409 (delta BSDF): Fresnel at the normal-mapped normal */
static Float glint_reflectance(const sms_bsdf &b, V3 n, V3 wo) {
    Float cos_theta = dot(n, wo);
    if (b.type == SMS_BSDF_CONDUCTOR && b.k != 0.f) return fresnel_conductor(std::fabs(cos_theta), b.eta, b.k);
    if (b.type == SMS_BSDF_DIELECTRIC || b.type == SMS_BSDF_CONDUCTOR) return fresnel(std::fabs(cos_theta), b.eta);
    return fresnel_conductor(std::fabs(cos_theta), 0.f, 1.f);
}

/* specular_reflectance (manifold_glints.cpp:375-409) of a rough glinty
 * surface: the BSDF value (NormalmapBSDF::eval, normalmap.cpp:172-181: the
 * nested rough BSDF in the normal-mapped frame at uv, wo kept only on the same
 * side of both frames) moved to the half-vector domain, x 4 |wo . h| in the
 * base frame. */
static Float glint_rough_reflectance(const Scene &sc, const GQuery &q, V2 uv, V3 wi_w, V3 wo_w) {
    const sms_bsdf &b = sc.shapes[sc.glinty_shape].bsdf;
    MVertex vt;
    glint_vertex(sc.nmap, q, uv, vt);
    V3 n = vt.n;
    V3 fs = normalize(q.dp_du - n * dot(n, q.dp_du));
    V3 ft = cross(n, fs);
    V3 wi(dot(wi_w, fs), dot(wi_w, ft), dot(wi_w, n)), wo(dot(wo_w, fs), dot(wo_w, ft), dot(wo_w, n));
    if (!(dot(wo_w, q.n) * wo.z > 0.f)) return 0.f;
    Float f = b.type == SMS_BSDF_CONDUCTOR ? roughconductor_eval(b.alpha, b.eta, b.k, wi, wo)
                                           : roughdielectric_eval(b.alpha, b.eta, wi, wo);
    V3 bs, bt;
    base_frame(q, bs, bt);
    V3 wil(dot(wi_w, bs), dot(wi_w, bt), dot(wi_w, q.n)), wol(dot(wo_w, bs), dot(wo_w, bt), dot(wo_w, q.n));
    V3 h = normalize(wil + wol);
    return f * 4.f * std::fabs(dot(wol, h));
}

/* manifold_glints.cpp:267-294 */
static Float glint_contribution(const Scene &sc, const GQuery &q, const EI &ei, V2 uv) {
    MVertex vy;
    if (!emitter_vertex(sc, ei, q.p, vy)) return 0.f;
    MVertex vx;
    vx.p = q.sensor;
    V3 dxv = normalize(q.p - q.sensor);
    vx.n = vx.gn = dxv;
    coordinate_system(vx.n, vx.dp_du, vx.dp_dv);
    MVertex vt;
    glint_vertex(sc.nmap, q, uv, vt);
    MVertex vt_o = vt;
    make_orthonormal(vt_o);
    const sms_bsdf &gb = sc.shapes[sc.glinty_shape].bsdf;
    Float f = is_rough(gb) ? glint_rough_reflectance(sc, q, uv, normalize(q.sensor - q.p), normalize(ei.p - q.p))
                           : glint_reflectance(gb, vt.n, normalize(ei.p - q.p));
    f *= glint_geometric_term(vx, vt_o, vy);
    return f;
}

/* manifold_glints.cpp:28-176: the SMS strategy, before the MIS weight and the
 * sensor importance (both applied by the integrator): sms_weight x ei.weight. */
static V3 glint_connect(const Scene &sc, const sms_config &cfg, const GQuery &q, PCG32 &rng, int &count_out,
                        int &walks_out, Stats &st) {
    count_out = 0; walks_out = 0;
    Query qq; qq.p = q.p;
    EI ei = sample_emitter_interaction(sc, sc.emitters_all, qq, rng);
    if (ei.emitter < 0 || sc.glinty_shape < 0 || sc.nmap.res == 0) return V3(0.f);
    st.connections++;
    V3 d = ei.p - q.p;
    Float dist = norm(d);
    d *= 1.f / dist;
    Ray r; r.o = q.p; r.d = d;
    r.mint = kRayEps * (1.f + hmax_abs(q.p));
    r.maxt = dist * (1.f - kRayEps);
    if (ray_test(sc, r)) return V3(0.f);
    /* offset normal of a rough glinty surface (:56-64): visible normals of the
       Beckmann distribution seen from the sensor direction */
    V3 no(0.f, 0.f, 1.f);
    Float p_off = 1.f;
    const sms_bsdf &gb = sc.shapes[sc.glinty_shape].bsdf;
    if (is_rough(gb)) {
        V3 bs, bt;
        base_frame(q, bs, bt);
        V3 wiw = normalize(q.sensor - q.p);
        no = beckmann_sample_visible(gb.alpha, V3(dot(wiw, bs), dot(wiw, bt), dot(wiw, q.n)), rng.next_2d(), p_off);
    }
    Float w = 0.f;
    V2 uvf, uvi;
    int it;
    if (!cfg.biased) {
        bool ok = sample_glint(cfg, sc.nmap, q, ei.p, rng.next_2d(), uvf, uvi, it, no);
        walks_out++; st.walks++; st.newton += it;
        if (!ok) { st.failed++; return V3(0.f); }
        st.succeeded++;
        Float spec = glint_contribution(sc, q, ei, uvf);
        Float inv_prob = 1.f;
        int iterations = 1;
        st.calls++;
        while (true) {
            V2 uvt, uvi2;
            int it2;
            bool ok2 = sample_glint(cfg, sc.nmap, q, ei.p, rng.next_2d(), uvt, uvi2, it2, no);
            walks_out++; st.walks++; st.newton += it2;
            Float dx = uvt.x - uvf.x, dy = uvt.y - uvf.y;
            if (ok2 && std::sqrt(dx * dx + dy * dy) < cfg.uniqueness_threshold) break;
            inv_prob += 1.f;
            iterations++;
            if (cfg.max_trials > 0 && iterations > cfg.max_trials) { inv_prob = 0.f; break; }
        }
        st.iters += (uint64_t)iterations;
        update_max(st.iters_max, (uint64_t)iterations);
        count_out = inv_prob == 0.f ? -1 : iterations;
        w = spec * inv_prob;
    } else {
        std::vector<V2> sols;
        for (int m = 0; m < cfg.max_trials; ++m) {
            bool ok = sample_glint(cfg, sc.nmap, q, ei.p, rng.next_2d(), uvf, uvi, it, no);
            walks_out++; st.walks++; st.newton += it;
            if (!ok) { st.failed++; continue; }
            st.succeeded++;
            bool dup = false;
            for (const V2 &u : sols) {
                Float dx = uvf.x - u.x, dy = uvf.y - u.y;
                if (std::sqrt(dx * dx + dy * dy) < cfg.uniqueness_threshold) { dup = true; break; }
            }
            if (dup) continue;
            sols.push_back(uvf);
            w += glint_contribution(sc, q, ei, uvf);
        }
        count_out = (int)sols.size();
    }
    w = w / p_off;   /* sms_weight /= p_offset (:141) */
    return V3(w * ei.weight.x, w * ei.weight.y, w * ei.weight.z);
}

/* ====================================================================
 * Path tracer around the SMS solvers: src/integrators/path.cpp:94-226,
 * path_sms_ss.cpp:69-251, path_sms_ms.cpp:172-330, MonteCarloIntegrator
 * (src/librender/integrator.cpp), perspective sensor, box filter.  One path at
 * a time, with the random-number layout of the library's sms_render: path p
 * draws from PCG32 stream p (state seed `seed`), its SMS call at bounce d from
 * stream p + d * 2^48 of state seed sms_seed(seed).
 * ==================================================================== */
static uint64_t sms_seed(uint64_t seed) {
    /* SplitMix64 (Steele, Lea and Flood 2014) */
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static Float mis_weight(Float a, Float b) {   /* path.cpp:227-231 */
    a *= a; b *= b;
    return a > 0.f ? a / (a + b) : Float(0.f);
}

static Float hmax_v(V3 v) { return omax(v.x, omax(v.y, v.z)); }

/* sh_frame of the surface interaction: tangent from dp_du (kdtree.h:2334-2366) */
static void pt_frame(const SI &si, V3 &s, V3 &t) {
    V3 n = si.shn;
    V3 a = si.dp_du - n * dot(n, si.dp_du);
    Float l2 = dot(a, a);
    if (l2 > 1e-20f) { s = a * (1.f / std::sqrt(l2)); t = cross(n, s); }
    else coordinate_system(n, s, t);
}

/* area.cpp eval: radiance from the front side of a sphere emitter */
static V3 pt_emitted(const Scene &sc, const Shape &s, V3 p, V3 d) {
    if (s.emitter < 0) return V3(0.f);
    V3 n = normalize(p - s.center);
    if (s.flip) n = -n;
    if (!(dot(n, -d) > 0.f)) return V3(0.f);
    return sc.emitters[s.emitter].radiance;
}

/* Sphere::pdf_direction x emitter pick (scene.cpp:206-220) */
static Float pt_emitter_pdf(const Scene &sc, const Shape &s, V3 x, V3 p, V3 d, Float dist) {
    V3 n = normalize(p - s.center);
    if (s.flip) n = -n;
    if (!(dot(d, n) < 0.f)) return 0.f;
    Float sin_a = s.radius / norm(s.center - x);
    Float cos_a = safe_sqrt(1.f - sin_a * sin_a);
    Float pdf;
    if (sin_a < 1.f - 5.9604644775390625e-08f) pdf = (0.5f * kInvPi) / (1.f - cos_a);
    else pdf = (1.f / (4.f * kPi * s.radius * s.radius)) * dist * dist / std::fabs(dot(d, n));
    return sc.emitters_all.size() > 1 ? pdf * (1.f / (Float)sc.emitters_all.size()) : pdf;
}

struct PtDir { V3 d, spec; Float dist = 0.f, pdf = 0.f; bool delta = false; };

/* Scene::sample_emitter_direction (scene.cpp:156-196), point.cpp and
 * area.cpp + Sphere::sample_direction (sphere.cpp) */
/* Scene::sample_emitter_direction over an emitter list (all emitters, or a
 * caustic list as path_filtered_teaser.cpp:331-378 picks them) */
static bool pt_sample_emitter_from(const Scene &sc, const std::vector<int> &list, V3 x, Float ux, Float uy,
                                   PtDir &ds) {
    const int ne = (int)list.size();
    if (ne == 0) return false;
    int idx = 0;
    if (ne > 1) {
        Float epdf = 1.f / (Float)ne;
        idx = (int)omin((uint32_t)(ux * (Float)ne), (uint32_t)ne - 1);
        ux = (ux - (Float)idx * epdf) * (Float)ne;
    }
    const Emitter &e = sc.emitters[list[idx]];
    if (e.kind == 0) {
        V3 d = e.p - x;
        ds.dist = norm(d);
        Float inv = 1.f / ds.dist;
        ds.d = d * inv; ds.pdf = 1.f; ds.delta = true;
        ds.spec = e.radiance * (inv * inv);
    } else {
        const Shape &s = sc.shapes[e.shape];
        V3 dc = s.center - x;
        Float dc2 = dot(dc, dc);
        Float r_adj = s.radius * (s.flip ? (1.f + kRayEps) : (1.f - kRayEps));
        V3 p, n;
        if (dc2 > r_adj * r_adj) {
            Float inv_dc = 1.f / std::sqrt(dc2);
            Float sin_max = s.radius * inv_dc, sin2_max = sin_max * sin_max, inv_sin_max = 1.f / sin_max;
            Float cos_max = safe_sqrt(1.f - sin2_max);
            Float a = (cos_max - 1.f) * ux + 1.f;
            Float sin2 = sin2_max > 0.00068523f ? 1.f - a * a : sin2_max * ux;
            Float cos_t = safe_sqrt(1.f - sin2);
            Float cos_al = sin2 * inv_sin_max + cos_t * safe_sqrt(1.f - sin2 * inv_sin_max * inv_sin_max);
            Float sin_al = safe_sqrt(1.f - cos_al * cos_al);
            Float ang = uy * (2.f * kPi);
            Float sp = std::sin(ang), cp = std::cos(ang);
            V3 fz = dc * -inv_dc, fs, ft;
            coordinate_system(fz, fs, ft);
            V3 dl = fs * (cp * sin_al) + ft * (sp * sin_al) + fz * cos_al;
            p = dl * s.radius + s.center; n = dl;
            V3 dv = p - x;
            ds.dist = norm(dv);
            ds.d = dv * (1.f / ds.dist);
            ds.pdf = ds.dist == 0.f ? Float(0.f) : (0.5f * kInvPi) / (1.f - cos_max);
        } else {
            V3 dl = square_to_uniform_sphere(V2{ux, uy});
            p = dl * s.radius + s.center; n = dl;
            V3 dv = p - x;
            Float dist2 = dot(dv, dv);
            ds.dist = std::sqrt(dist2);
            ds.d = dv * (1.f / ds.dist);
            ds.pdf = (1.f / (4.f * kPi * s.radius * s.radius)) * dist2 / std::fabs(dot(ds.d, n));
        }
        if (s.flip) n = -n;
        ds.delta = false;
        if (!(dot(ds.d, n) < 0.f && ds.pdf != 0.f)) return false;
        ds.spec = e.radiance * (1.f / ds.pdf);
    }
    if (ne > 1) { ds.pdf *= 1.f / (Float)ne; ds.spec = ds.spec * (Float)ne; }
    return ds.pdf != 0.f;
}
static bool pt_sample_emitter(const Scene &sc, V3 x, Float ux, Float uy, PtDir &ds) {
    return pt_sample_emitter_from(sc, sc.emitters_all, x, ux, uy, ds);
}

/* warp.h:54-90 concentric disk, lifted to the cosine hemisphere (warp.h:332-340) */
static V3 pt_cosine_hemisphere(Float u1, Float u2) {
    Float x = 2.f * u1 - 1.f, y = 2.f * u2 - 1.f, r, phi;
    if (x == 0.f && y == 0.f) { r = 0.f; phi = 0.f; }
    else if (std::fabs(x) < std::fabs(y)) { r = y; phi = 0.5f * kPi - (x / y) * (0.25f * kPi); }
    else { r = x; phi = (y / x) * (0.25f * kPi); }
    Float px = r * std::cos(phi), py = r * std::sin(phi);
    return V3(px, py, safe_sqrt(1.f - px * px - py * py));
}

struct PtBsdf {
    V3 wo, weight;
    Float pdf = 0.f, eta = 1.f;
    bool delta = false;
    bool transmit = false;   /* BSDFFlags::Transmission of the sampled lobe */
};

/* density of pt_rough_sample for (wi, wo): D(m) cos(theta_m) x the Jacobian
 * of reflection / refraction (roughconductor.cpp / roughdielectric.cpp pdf
 * with normals drawn from D cos instead of the visible normals) */
static Float pt_rough_pdf(const sms_bsdf &b, V3 wi, V3 wo) {
    const Float ci = wi.z, co = wo.z;
    if (b.type == SMS_BSDF_CONDUCTOR) {
        if (!(ci > 0.f && co > 0.f)) return 0.f;
        V3 h = normalize(wo + wi);
        return beckmann_D(h, b.alpha) * h.z / (4.f * dot(wo, h));
    }
    if (ci == 0.f) return 0.f;
    const bool reflect = ci * co > 0.f;
    const Float eta = ci > 0.f ? b.eta : 1.f / b.eta;
    V3 m = normalize(wi + wo * (reflect ? Float(1.f) : eta));
    if (m.z < 0.f) m = -m;
    if (dot(wi, m) * ci <= 0.f || dot(wo, m) * co <= 0.f) return 0.f;
    const Float F = fresnel(dot(wi, m), b.eta);
    const Float pm = beckmann_D(m, b.alpha) * m.z;
    if (reflect) return F * pm / (4.f * std::fabs(dot(wo, m)));
    const Float den = dot(wi, m) + eta * dot(wo, m);
    return (1.f - F) * pm * eta * eta * std::fabs(dot(wo, m)) / (den * den);
}

/* diffuse.cpp eval, roughconductor.cpp / roughdielectric.cpp eval (value x
 * |cos_theta_o|); delta BSDFs give 0 */
static V3 pt_bsdf_eval(const sms_bsdf &b, V3 wi, V3 wo) {
    if (b.type == SMS_BSDF_DIFFUSE) {
        if (!(wi.z > 0.f && wo.z > 0.f)) return V3(0.f);
        return V3(b.albedo[0], b.albedo[1], b.albedo[2]) * (kInvPi * wo.z);
    }
    if (!(b.alpha > 0.f)) return V3(0.f);
    return V3(b.type == SMS_BSDF_CONDUCTOR ? roughconductor_eval(b.alpha, b.eta, b.k, wi, wo)
                                           : roughdielectric_eval(b.alpha, b.eta, wi, wo));
}

static Float pt_bsdf_pdf(const sms_bsdf &b, V3 wi, V3 wo) {
    if (b.type == SMS_BSDF_DIFFUSE) return (wi.z > 0.f && wo.z > 0.f) ? kInvPi * wo.z : Float(0.f);
    return b.alpha > 0.f ? pt_rough_pdf(b, wi, wo) : Float(0.f);
}

/* rough sampling: m ~ D cos (microfacet.h, sample_visible = false), then
 * reflection, or for a dielectric reflection / refraction by the Fresnel
 * reflectance at m (roughdielectric.cpp sample); weight = value / density */
static bool pt_rough_sample(const sms_bsdf &b, V3 wi, Float u1, Float u2, Float u3, PtBsdf &bs) {
    const Float ci = wi.z;
    Float pm;
    const V3 m = beckmann_sample(b.alpha, u2, u3, pm);
    bs.delta = false;
    bs.eta = 1.f;
    if (b.type == SMS_BSDF_CONDUCTOR) {
        if (!(ci > 0.f)) return false;
        bs.wo = m * (2.f * dot(wi, m)) - wi;
        if (!(bs.wo.z > 0.f)) return false;
    } else {
        Float cos_t;
        const Float F = fresnel(dot(wi, m), b.eta, &cos_t);
        const bool outside = dot(wi, m) >= 0.f;
        const Float eta_it = outside ? b.eta : 1.f / b.eta, eta_ti = outside ? 1.f / b.eta : b.eta;
        if (u1 <= F) {
            bs.wo = m * (2.f * dot(wi, m)) - wi;
            if (!(bs.wo.z * ci > 0.f)) return false;
        } else {
            bs.wo = m * (dot(wi, m) * eta_ti + cos_t) - wi * eta_ti;
            if (!(bs.wo.z * ci < 0.f)) return false;
            bs.eta = eta_it;
        }
    }
    bs.pdf = pt_rough_pdf(b, wi, bs.wo);
    if (!(bs.pdf > 0.f)) return false;
    bs.weight = pt_bsdf_eval(b, wi, bs.wo) * (1.f / bs.pdf);
    return true;
}

/* diffuse.cpp / dielectric.cpp / conductor.cpp sample() (smooth, radiance) */
static bool pt_bsdf_sample(const sms_bsdf &b, V3 wi, Float u1, Float u2, Float u3, PtBsdf &bs) {
    const Float ci = wi.z;
    if (b.type != SMS_BSDF_DIFFUSE && b.alpha > 0.f) return pt_rough_sample(b, wi, u1, u2, u3, bs);
    if (b.type == SMS_BSDF_DIFFUSE) {
        if (!(ci > 0.f)) return false;
        bs.wo = pt_cosine_hemisphere(u2, u3);
        bs.pdf = kInvPi * bs.wo.z; bs.eta = 1.f; bs.delta = false;
        bs.weight = V3(b.albedo[0], b.albedo[1], b.albedo[2]);
        return bs.pdf > 0.f;
    }
    if (b.type == SMS_BSDF_DIELECTRIC) {
        Float cos_t_abs;
        Float r = fresnel(ci, b.eta, &cos_t_abs);
        bool outside = ci >= 0.f;
        Float eta_it = outside ? b.eta : 1.f / b.eta, eta_ti = outside ? 1.f / b.eta : b.eta;
        Float cos_t = outside ? -std::fabs(cos_t_abs) : std::fabs(cos_t_abs);
        bs.delta = true;
        if (u1 <= r) {
            bs.wo = V3(-wi.x, -wi.y, wi.z); bs.pdf = r; bs.eta = 1.f; bs.weight = V3(1.f);
        } else {
            bs.wo = V3(-eta_ti * wi.x, -eta_ti * wi.y, cos_t); bs.pdf = 1.f - r; bs.eta = eta_it;
            bs.weight = V3(eta_ti * eta_ti);
        }
        return true;
    }
    if (!(ci > 0.f)) return false;
    bs.wo = V3(-wi.x, -wi.y, wi.z); bs.pdf = 1.f; bs.eta = 1.f; bs.delta = true;
    bs.weight = V3(fresnel_conductor(ci, b.eta, b.k));
    return true;
}

/* ---- LEAN mapping for the glints integrator ---------------------------
 * Level 0 from the slope map with the base variance 0.5 * 1e-4^2 of
 * normalmap.cpp:36-40; each coarser level the 2x2 box average of the finer one
 * (Bitmap::resample with a box filter at exactly half the size). */
static void build_lean(NormalMap &m) {
    if (!m.lean.empty() || m.res == 0) return;
    const Float base_sigma_2 = 0.5f * 0.0001f * 0.0001f;
    std::vector<Float> l0(5 * (size_t)m.res * m.res);
    for (size_t i = 0; i < (size_t)m.res * m.res; ++i) {
        Float x = m.sx[i], y = m.sy[i];
        l0[5 * i] = x; l0[5 * i + 1] = y;
        l0[5 * i + 2] = x * x + base_sigma_2; l0[5 * i + 3] = y * y + base_sigma_2; l0[5 * i + 4] = x * y;
    }
    m.lean.push_back(std::move(l0));
    uint32_t res = m.res;
    while (res > 1) {
        uint32_t r2 = res / 2;
        const std::vector<Float> &src = m.lean.back();
        std::vector<Float> dst(5 * (size_t)r2 * r2);
        for (uint32_t y = 0; y < r2; ++y)
            for (uint32_t x = 0; x < r2; ++x)
                for (int c = 0; c < 5; ++c) {
                    Float a = src[5 * ((size_t)(2 * y) * res + 2 * x) + c] + src[5 * ((size_t)(2 * y) * res + 2 * x + 1) + c];
                    Float b = src[5 * ((size_t)(2 * y + 1) * res + 2 * x) + c] +
                              src[5 * ((size_t)(2 * y + 1) * res + 2 * x + 1) + c];
                    dst[5 * ((size_t)y * r2 + x) + c] = 0.25f * (a + b);
                }
        m.lean.push_back(std::move(dst));
        res = r2;
    }
}

/* NormalmapBSDF::mipmap_level (normalmap.cpp:374-388); a footprint finer than
 * a texel (negative level) takes level 0 */
static int lean_level(const NormalMap &m, V2 duv_dx, V2 duv_dy) {
    const int L = (int)m.lean.size();
    Float w = 2.f * omax(omax(std::fabs(m.tiles * duv_dx.x), std::fabs(m.tiles * duv_dx.y)),
                             omax(std::fabs(m.tiles * duv_dy.x), std::fabs(m.tiles * duv_dy.y)));
    Float lv = std::ceil((Float)(L - 1) + std::log2(omax(w, 1e-8f)));
    if (!(lv > 0.f)) return 0;
    return (int)omin(lv, (Float)(L - 1));
}

/* Bilinear LEAN lookup (normalmap.h:62-104, 199-233): mean slope mu and
 * covariance (a, c; c, b) at the tiled uv on level l */
static void lean_lookup(const NormalMap &m, V2 uv_in, int l, V2 &mu, Float &sa, Float &sb, Float &sc) {
    uint32_t res = m.res >> l;
    Float u = uv_in.x * m.tiles, v = uv_in.y * m.tiles;
    u -= std::floor(u); v -= std::floor(v);
    Float fr = (Float)res, duv = 1.f / fr;
    Float px = omin(omax((u - 0.5f * duv) * fr, 0.f), fr - 1.f);
    Float py = omin(omax((v - 0.5f * duv) * fr, 0.f), fr - 1.f);
    uint32_t x0 = (uint32_t)std::floor(px), y0 = (uint32_t)std::floor(py);
    uint32_t x1 = omin(x0 + 1, res - 1), y1 = omin(y0 + 1, res - 1);
    x0 = omin(x0, res - 1); y0 = omin(y0, res - 1);
    Float wx = px - (Float)x0, wy = py - (Float)y0;
    const std::vector<Float> &d = m.lean[l];
    Float vv[5];
    for (int c = 0; c < 5; ++c) {
        Float v00 = d[5 * ((size_t)y0 * res + x0) + c], v10 = d[5 * ((size_t)y0 * res + x1) + c];
        Float v01 = d[5 * ((size_t)y1 * res + x0) + c], v11 = d[5 * ((size_t)y1 * res + x1) + c];
        Float a = (1.f - wx) * v00 + wx * v10, b = (1.f - wx) * v01 + wx * v11;
        vv[c] = (1.f - wy) * a + wy * b;
    }
    mu.x = vv[0]; mu.y = vv[1];
    sa = omax(0.f, vv[2] - vv[0] * vv[0]);
    sb = omax(0.f, vv[3] - vv[1] * vv[1]);
    sc = omax(0.f, vv[4] - vv[0] * vv[1]);
}

/* LEAN/LEADR distribution (include/mitsuba/render/lean.h, after Dupuy's
 * reference implementation): parameters from the LEAN moments plus a base
 * Beckmann roughness, visible-normal density, shadowing. */
struct LeanP { V3 n; Float ax, ay, rho, srho, tx, ty; };
static LeanP lean_params(V2 mu, Float sa, Float sb, Float sc, Float alpha) {
    Float e1 = mu.x, e2 = mu.y;
    Float lax = std::sqrt(2.f * sa), lay = std::sqrt(2.f * sb);
    Float rho = 2.f * sc / (lax * lay);
    Float e3 = 0.5f * lax * lax + e1 * e1 + 0.5f * alpha * alpha;
    Float e4 = 0.5f * lay * lay + e2 * e2 + 0.5f * alpha * alpha;
    Float e5 = 0.5f * rho * lax * lay + e1 * e2;
    LeanP p;
    p.tx = e1; p.ty = e2;
    p.ax = std::sqrt(2.f * omax(0.f, e3 - e1 * e1));
    p.ay = std::sqrt(2.f * omax(0.f, e4 - e2 * e2));
    p.rho = 2.f * (e5 - e1 * e2) / (p.ax * p.ay);
    p.srho = std::sqrt(1.f - p.rho * p.rho);
    p.n = normalize(V3(-p.tx, -p.ty, 1.f));
    return p;
}
static Float lean_sigma_std(Float ct) {
    if (ct == 1.f) return 1.f;
    Float st = std::sqrt(1.f - ct * ct), nu = ct / st;
    Float tmp = std::exp(-nu * nu) * 0.56418958354775628695f;   /* 1 / sqrt(pi) */
    return 0.5f * (ct * (1.f + std::erf(nu)) + st * tmp);
}
static Float lean_sigma(V3 k, const LeanP &p) {
    Float a = k.x * p.ax + k.y * p.ay * p.rho, b = k.y * p.ay * p.srho, c = k.z - k.x * p.tx - k.y * p.ty;
    Float nrm = std::sqrt(a * a + b * b + c * c);
    return nrm * lean_sigma_std(c / nrm);
}
static Float lean_g1(V3 k, const LeanP &p) { return dot(k, p.n) > 0.f ? k.z / lean_sigma(k, p) : Float(0.f); }
static Float lean_ndf(V3 h, const LeanP &p) {
    if (!(h.z > 5.9604644775390625e-08f)) return 0.f;
    Float t1 = h.z * h.z, t2 = t1 * t1;
    Float sx = -h.x / h.z - p.tx, sy = -h.y / h.z - p.ty;
    Float nrm = p.ax * p.ay * p.srho;
    Float x = sx / p.ax, y = (p.ax * sy - p.rho * p.ay * sx) / (p.ax * p.ay * p.srho);
    return kInvPi * std::exp(-(x * x + y * y)) / nrm / t2;
}
/* SpecularManifoldGlints::lean_pdf (manifold_glints.cpp:557-579), local frame */
static Float glint_lean_pdf(const NormalMap &m, V2 uv, V2 duv_dx, V2 duv_dy, V3 wi, V3 wo) {
    if (wi.z < 0.f || wo.z < 0.f) return 0.f;
    V2 mu; Float sa, sb, sc;
    lean_lookup(m, uv, lean_level(m, duv_dx, duv_dy), mu, sa, sb, sc);
    LeanP p = lean_params(mu, sa, sb, sc, 0.f);
    V3 h = normalize(wo + wi);
    Float G = lean_g1(wo, p) * lean_g1(wi, p);   /* LEAN::gaf: G1 ignores h */
    if (!(G > 0.f)) return 0.f;
    Float dp = dot(wi, h);
    Float vndf = dp > 0.f ? dp * lean_ndf(h, p) / lean_sigma(wi, p) : Float(0.f);
    return vndf / (4.f * dot(wi, h));
}

/* NormalmapBSDF's LEAN fallback (normalmap.cpp:80-112, 142-170, 187-203):
 * the glossy LEAN distribution of the top pyramid level widened by the base
 * roughness alpha, Fresnel of eta + i k (dielectric when k = 0).  Visible
 * slopes by LEAN::sample_vndf (include/mitsuba/render/lean.h): qf2 inverts the
 * standard distribution's visible-slope CDF by Newton steps kept inside a
 * bisection bracket in the erf domain, qf1 = erfinv(2u - 1), then the
 * Cholesky map to the surface's slope distribution. */
static Float lean_qf2(Float u, Float ct, Float st) {
    const Float kInvSqrtPi = 0.56418958354775628695f;
    const Float cot = ct / st, tan_t = st / ct;
    Float a = -1.f, c = std::erf(cot);
    u = omax(u, Float(1e-6f));
    const Float fit = 1.f + ct * (-0.876f + ct * (0.4265f - 0.0594f * ct));
    Float b = c - (1.f + c) * std::pow(1.f - u, fit);
    const Float norm_cdf = 1.f / (1.f + c + kInvSqrtPi * tan_t * std::exp(-cot * cot));
    int it = 0;
    while (++it < 10) {
        if (!(b >= a && b <= c)) b = 0.5f * (a + c);
        const Float ie = erfinv_f(b);
        const Float value = norm_cdf * (1.f + b + kInvSqrtPi * tan_t * std::exp(-ie * ie)) - u;
        const Float deriv = norm_cdf * (1.f - ie * tan_t);
        if (std::fabs(value) < 1e-5f) break;
        if (value > 0.f) c = b;
        else a = b;
        b -= value / deriv;
    }
    return erfinv_f(omax(Float(-0.9999f), b));
}
static V2 lean_sample_vp22_std(V3 wi, Float u0, Float u1) {
    const Float ct = wi.z;
    const Float st = ct < 1.f ? std::sqrt(1.f - ct * ct) : Float(0.f);
    const Float tx = lean_qf2(u0, ct, st);
    const Float ty = erfinv_f(2.f * u1 - 1.f);
    if (st == 0.f) return V2{tx, ty};
    const Float nrm = 1.f / std::sqrt(wi.x * wi.x + wi.y * wi.y);
    const Float cp = wi.x * nrm, sp = wi.y * nrm;
    return V2{cp * tx - sp * ty, sp * tx + cp * ty};
}
static V3 lean_sample_vndf(V3 wi, Float u0, Float u1, const LeanP &p) {
    const Float a = wi.x * p.ax + wi.y * p.ay * p.rho, b = wi.y * p.ay * p.srho;
    const Float c = wi.z - wi.x * p.tx - wi.y * p.ty;
    const V3 ws = normalize(V3(a, b, c));
    if (!(ws.z > 0.f)) return V3(0.f, 0.f, 1.f);
    const V2 t = lean_sample_vp22_std(ws, u0, u1);
    const Float txh = p.ax * t.x + p.tx;
    const Float chol = p.rho * t.x + p.srho * t.y;
    const Float tyh = p.ay * chol + p.ty;
    return normalize(V3(-txh, -tyh, 1.f));
}
static Float lean_vndf(V3 h, V3 wi, const LeanP &p) {
    const Float dp = dot(wi, h);
    return dp > 0.f ? dp * lean_ndf(h, p) / lean_sigma(wi, p) : Float(0.f);
}
static Float lean_gaf(V3 a, V3 b, const LeanP &p) {   /* LEAN::gaf: the product of the two G1 */
    const Float g = lean_g1(a, p) * lean_g1(b, p);
    return g > 0.f ? g : Float(0.f);
}
static LeanP lean_fb_params(const NormalMap &m, const LeanFallback &f) {
    V2 mu; Float sa, sb, sc;
    lean_lookup(m, V2{0.f, 0.f}, (int)m.lean.size() - 1, mu, sa, sb, sc);
    return lean_params(mu, sa, sb, sc, f.alpha);
}
static Float lean_fb_fresnel(const LeanFallback &f, Float c) {
    return f.k == 0.f ? fresnel(c, f.eta) : fresnel_conductor(c, f.eta, f.k);
}
static bool lean_fb_sample(const NormalMap &m, const LeanFallback &f, V3 wi, Float u0, Float u1, V3 &wo,
                           Float &weight, Float &pdf) {
    if (!(wi.z > 0.f)) return false;
    const LeanP p = lean_fb_params(m, f);
    const V3 mm = lean_sample_vndf(wi, u0, u1, p);
    const Float dm = dot(wi, mm);
    wo = mm * (2.f * dm) - wi;
    const Float G = lean_gaf(wo, wi, p);
    if (!(G > 0.f && wo.z > 0.f)) return false;
    pdf = lean_vndf(mm, wi, p) / (4.f * dm);
    weight = lean_fb_fresnel(f, dm) * G / lean_g1(wi, p);
    return true;
}
static Float lean_fb_eval(const NormalMap &m, const LeanFallback &f, V3 wi, V3 wo) {
    if (!(wi.z > 0.f && wo.z > 0.f)) return 0.f;
    const LeanP p = lean_fb_params(m, f);
    const V3 h = normalize(wo + wi);
    return lean_fb_fresnel(f, dot(wi, h)) * lean_ndf(h, p) * lean_gaf(wi, wo, p) / (4.f * wi.z);
}
static Float lean_fb_pdf(const NormalMap &m, const LeanFallback &f, V3 wi, V3 wo) {
    const LeanP p = lean_fb_params(m, f);
    const V3 h = normalize(wo + wi);
    return lean_gaf(wo, wi, p) > 0.f ? lean_vndf(h, wi, p) / (4.f * dot(wi, h)) : Float(0.f);
}

/* NormalmapBSDF::frame (normalmap.cpp:236-257) at level 0: the base shading
 * frame (n, tangent from dp_du) tilted to the bilinear slope normal */
static void nm_frame(const NormalMap &m, V3 n, V3 dp_du, V2 uv, V3 &pn, V3 &ps, V3 &pt) {
    V3 bs = normalize(dp_du - n * dot(n, dp_du)), bt = cross(n, bs);
    V2 sl = nm_slope(m, uv);
    pn = normalize(bs * -sl.x + bt * -sl.y + n);
    ps = normalize(dp_du - pn * dot(pn, dp_du));
    pt = cross(pn, ps);
}

/* NormalmapBSDF::sample with a smooth conductor inside (normalmap.cpp:
 * 116-139, conductor.cpp sample): reflection about the perturbed normal,
 * world-space directions; weight = Fresnel. */
static bool nm_conductor_sample(const NormalMap &m, const sms_bsdf &b, V3 n, V3 dp_du, V2 uv, V3 wi_w,
                                V3 &wo_w, Float &weight) {
    V3 pn, ps, pt;
    nm_frame(m, n, dp_du, uv, pn, ps, pt);
    Float ci = dot(wi_w, pn);
    if (!(ci > 0.f)) return false;
    wo_w = pn * (2.f * ci) - wi_w;
    if (!(dot(wo_w, n) * dot(wo_w, pn) > 0.f)) return false;
    weight = fresnel_conductor(ci, b.eta, b.k);
    return true;
}

/* ---- roughplastic (src/bsdfs/roughplastic.cpp) */

/* Gauss-Legendre nodes and weights on [-1, 1] (quad::gauss_legendre): the
 * roots of P_n by Newton's method from the Tricomi initial guesses */
static void gauss_legendre_nodes(int n, std::vector<double> &x, std::vector<double> &w) {
    x.assign(n, 0.0); w.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(3.14159265358979323846 * (i + 0.75) / (n + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) { const double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k; p0 = p1; p1 = p2; }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-15) break;
        }
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

/* eval_transmittance / eval_reflectance (microfacet.h:454-551): visible
 * normals drawn at the Gauss-Legendre nodes mapped to [0, 1]^2 (32 x 32 when
 * eta > 1, else 128 x 128), weighted by G1 of the refracted / reflected
 * direction and by 1 - F / F; the weight sum of 4 is divided out */
static Float rp_eval_coating(Float alpha, Float eta, V3 wi, bool transmit) {
    const int res = eta > 1.f ? 32 : 128;
    std::vector<double> gx, gw;
    gauss_legendre_nodes(res, gx, gw);
    Float acc = 0.f;
    for (int j = 0; j < res; ++j)
        for (int k = 0; k < res; ++k) {
            V2 u; u.x = Float(gx[j] * 0.5 + 0.5); u.y = Float(gx[k] * 0.5 + 0.5);
            Float pdf;
            const V3 m = beckmann_sample_visible(alpha, wi, u, pdf);
            Float cos_t;
            const Float dm = dot(wi, m);
            const Float F = fresnel(dm, eta, &cos_t);
            Float val;
            if (transmit) {
                const Float eta_ti = dm >= 0.f ? 1.f / eta : eta;
                const V3 wo = m * (dm * eta_ti + cos_t) - wi * eta_ti;
                val = wo.z * wi.z >= 0.f ? Float(0.f) : beckmann_G1(wo, m, alpha) * (1.f - F);
            } else {
                const V3 wo = m * (2.f * dm) - wi;
                val = (wo.z <= 0.f || wi.z <= 0.f) ? Float(0.f) : beckmann_G1(wo, m, alpha) * F;
            }
            acc += val * Float(gw[j] * gw[k]);
        }
    return acc * 0.25f;
}

/* parameters_changed (roughplastic.cpp:364-396) */
static void rp_init(Shape &sh) {
    if (sh.bsdf.type != SMS_BSDF_ROUGHPLASTIC) return;
    const sms_bsdf &b = sh.bsdf;
    Float rsum = 0.f;
    for (int i = 0; i < kRoughPlasticRes; ++i) {
        const Float mu = omax(Float(1e-6f), Float(i) / Float(kRoughPlasticRes - 1));
        const V3 wi(std::sqrt(1.f - mu * mu), 0.f, mu);
        sh.rp.t[i] = rp_eval_coating(b.alpha, b.eta, wi, true);
        rsum += rp_eval_coating(b.alpha, 1.f / b.eta, wi, false) * mu;
    }
    sh.rp.fdr = rsum / Float(kRoughPlasticRes) * 2.f;
    const Float d_mean = (b.albedo[0] + b.albedo[1] + b.albedo[2]) / 3.f;
    sh.rp.ws = 1.f / (d_mean + 1.f);
}

/* lerp_gather (roughplastic.cpp:299-310) */
static Float rp_transmittance(const RoughPlastic &rp, Float c) {
    const Float x = c * Float(kRoughPlasticRes - 1);
    const int i = std::min((int)x, kRoughPlasticRes - 2);
    return rp.t[i] + (rp.t[i + 1] - rp.t[i]) * (x - Float(i));
}
static Float rp_prob_specular(const RoughPlastic &rp, Float ci) {
    const Float t_i = rp_transmittance(rp, ci);
    const Float ps = (1.f - t_i) * rp.ws, pd = t_i * (1.f - rp.ws);
    return ps / (ps + pd);
}

/* eval (roughplastic.cpp:245-297), value x cos_theta_o */
static V3 rp_eval(const Shape &sh, V3 wi, V3 wo) {
    const sms_bsdf &b = sh.bsdf;
    const Float ci = wi.z, co = wo.z;
    if (!(ci > 0.f && co > 0.f)) return V3(0.f);
    const V3 h = normalize(wo + wi);
    const Float F = fresnel(dot(wi, h), b.eta);
    const Float G = beckmann_G1(wi, h, b.alpha) * beckmann_G1(wo, h, b.alpha);
    const Float spec = F * beckmann_D(h, b.alpha) * G / (4.f * ci);
    const Float t_i = rp_transmittance(sh.rp, ci), t_o = rp_transmittance(sh.rp, co);
    V3 diff(b.albedo[0], b.albedo[1], b.albedo[2]);
    if (b.nonlinear)
        diff = V3(diff.x / (1.f - diff.x * sh.rp.fdr), diff.y / (1.f - diff.y * sh.rp.fdr),
                  diff.z / (1.f - diff.z * sh.rp.fdr));
    else
        diff = diff * (1.f / (1.f - sh.rp.fdr));
    return V3(spec) + diff * (kInvPi * (1.f / (b.eta * b.eta)) * co * t_i * t_o);
}

/* pdf (roughplastic.cpp:312-353), microfacet normals drawn from D cos */
static Float rp_pdf(const Shape &sh, V3 wi, V3 wo) {
    const Float ci = wi.z, co = wo.z;
    if (!(ci > 0.f && co > 0.f)) return 0.f;
    const Float ps = rp_prob_specular(sh.rp, ci);
    const V3 h = normalize(wo + wi);
    return beckmann_D(h, sh.bsdf.alpha) * h.z / (4.f * dot(wo, h)) * ps + (1.f - ps) * kInvPi * co;
}

/* sample (roughplastic.cpp:185-243) */
static bool rp_sample(const Shape &sh, V3 wi, Float u1, Float u2, Float u3, PtBsdf &bs) {
    const Float ci = wi.z;
    if (!(ci > 0.f)) return false;
    if (u1 < rp_prob_specular(sh.rp, ci)) {
        Float pm;
        const V3 m = beckmann_sample(sh.bsdf.alpha, u2, u3, pm);
        bs.wo = m * (2.f * dot(wi, m)) - wi;
    } else {
        bs.wo = pt_cosine_hemisphere(u2, u3);
    }
    bs.delta = false;
    bs.eta = 1.f;
    bs.pdf = rp_pdf(sh, wi, bs.wo);
    if (!(bs.pdf > 0.f)) return false;
    bs.weight = rp_eval(sh, wi, bs.wo) * (1.f / bs.pdf);
    return true;
}

/* the path tracers' BSDF of a shape: roughplastic or the plain BSDFs */
static V3 shape_bsdf_eval(const Shape &sh, V3 wi, V3 wo) {
    return sh.bsdf.type == SMS_BSDF_ROUGHPLASTIC ? rp_eval(sh, wi, wo) : pt_bsdf_eval(sh.bsdf, wi, wo);
}
static Float shape_bsdf_pdf(const Shape &sh, V3 wi, V3 wo) {
    return sh.bsdf.type == SMS_BSDF_ROUGHPLASTIC ? rp_pdf(sh, wi, wo) : pt_bsdf_pdf(sh.bsdf, wi, wo);
}
static bool shape_bsdf_sample(const Shape &sh, V3 wi, Float u1, Float u2, Float u3, PtBsdf &bs) {
    return sh.bsdf.type == SMS_BSDF_ROUGHPLASTIC ? rp_sample(sh, wi, u1, u2, u3, bs)
                                                 : pt_bsdf_sample(sh.bsdf, wi, u1, u2, u3, bs);
}

/* NormalmapBSDF::sample (normalmap.cpp:118-135) around any smooth nested BSDF:
 * sampled in the perturbed frame at uv, the direction taken back to the
 * shading frame (fs, ft, n) and kept when it lies on the same side of both
 * frames' normals. */
static bool nm_bsdf_sample(const NormalMap &m, const sms_bsdf &b, V3 fs, V3 ft, V3 n, V3 dp_du, V2 uv, V3 wi_w,
                           Float u1, Float u2, Float u3, PtBsdf &bs) {
    V3 pn, ps, pt;
    nm_frame(m, n, dp_du, uv, pn, ps, pt);
    const V3 wi(dot(wi_w, ps), dot(wi_w, pt), dot(wi_w, pn));
    if (!pt_bsdf_sample(b, wi, u1, u2, u3, bs)) return false;
    bs.transmit = bs.wo.z * wi.z < 0.f;
    const V3 wo_w = ps * bs.wo.x + pt * bs.wo.y + pn * bs.wo.z;
    const V3 wo(dot(wo_w, fs), dot(wo_w, ft), dot(wo_w, n));
    if (!(bs.wo.z * wo.z > 0.f)) return false;
    bs.wo = wo;
    return true;
}

/* PerspectiveCamera::importance (perspective.cpp:224-276) x film size for the
 * world-space direction d from the camera */
static Float pt_importance(const sms_camera &cam, const double tm[2], V3 d) {
    const float *M = cam.to_world;
    V3 dl(M[0] * d.x + M[4] * d.y + M[8] * d.z, M[1] * d.x + M[5] * d.y + M[9] * d.z,
          M[2] * d.x + M[6] * d.y + M[10] * d.z);
    if (!(dl.z > 0.f)) return 0.f;
    Float ic = 1.f / dl.z;
    Float px = dl.x * ic, py = dl.y * ic;
    Float tx = (Float)tm[0], ty = (Float)tm[1];
    if (!(px >= -tx && px <= tx && py >= -ty && py <= ty)) return 0.f;
    Float norm_ = 1.f / (4.f * tx * ty);
    return norm_ * ic * ic * ic * (Float)cam.width * (Float)cam.height;
}

/* One camera sample (path id g) of the integrator; returns its radiance. */
static V3 pt_sample(const Scene &sc, const sms_config &cfg, const sms_camera &cam, const sms_render_options &opt,
                    const double tm[2], uint64_t g, Stats &st) {
    const uint64_t wh = (uint64_t)cam.width * (uint64_t)cam.height;
    const uint32_t pix = (uint32_t)(g % wh);
    const uint32_t px = pix % (uint32_t)cam.width, py = pix / (uint32_t)cam.width;
    PCG32 rng;
    rng.seed(opt.seed, g);
    Float ux = rng.next_f32(), uy = rng.next_f32();
    (void)rng.next_f32();
    Float sx = ((Float)px + ux) / (Float)cam.width, sy = ((Float)py + uy) / (Float)cam.height;
    V3 dc = normalize(V3((Float)tm[0] * (1.f - 2.f * sx), (Float)tm[1] * (1.f - 2.f * sy), 1.f));
    Float inv_z = 1.f / dc.z;
    const float *M = cam.to_world;
    Ray ray;
    ray.o = V3(M[3], M[7], M[11]);
    ray.d = normalize(V3(M[0] * dc.x + M[1] * dc.y + M[2] * dc.z, M[4] * dc.x + M[5] * dc.y + M[6] * dc.z,
                         M[8] * dc.x + M[9] * dc.y + M[10] * dc.z));
    Float near_clip = cam.near_clip > 0.f ? cam.near_clip : 1e-2f;
    Float far_clip = cam.far_clip > near_clip ? cam.far_clip : 1e4f;
    ray.mint = near_clip * inv_z; ray.maxt = far_clip * inv_z;
    /* ray differentials (perspective.cpp:198-220), scaled by
       max(1/sqrt(spp), glint_diff_scale_factor_clamp) (integrator.cpp:164-165) */
    V3 rdx, rdy;
    {
        auto cam_dir = [&](Float ax, Float ay) {
            V3 c = normalize(V3((Float)tm[0] * (1.f - 2.f * ax), (Float)tm[1] * (1.f - 2.f * ay), 1.f));
            return normalize(V3(M[0] * c.x + M[1] * c.y + M[2] * c.z, M[4] * c.x + M[5] * c.y + M[6] * c.z,
                                M[8] * c.x + M[9] * c.y + M[10] * c.z));
        };
        Float scale = omax(1.f / std::sqrt((Float)opt.spp), opt.glint_diff_scale_factor_clamp);
        rdx = ray.d + (cam_dir(sx + 1.f / (Float)cam.width, sy) - ray.d) * scale;
        rdy = ray.d + (cam_dir(sx, sy + 1.f / (Float)cam.height) - ray.d) * scale;
    }
    SI si = ray_intersect(sc, ray);
    V3 L(0.f), thr(1.f);
    Float eta = 1.f;
    if (si.valid()) L += pt_emitted(sc, sc.shapes[si.shape], si.p, ray.d);
    bool spec_cam = true, prev_receiver = false;
    V3 prev_p;
    const int integ = opt.integrator;
    const bool filtered_ss = integ == SMS_INTEGRATOR_PATH_FILTERED_SS, filtered_ms = integ == SMS_INTEGRATOR_PATH_FILTERED_MS;
    /* path_sms_teaser (path_sms_teaser.cpp:120-320): caustics with cfg, glints
       with opt.glints run biased (:347-350); its SMS calls draw from their own
       state seeds: single scatter sms_seed(seed), multi scatter sms_seed(seed + 1),
       glints sms_seed(seed + 2) */
    const bool teaser = integ == SMS_INTEGRATOR_PATH_SMS_TEASER;
    sms_config gcfg = opt.glints;
    gcfg.biased = 1;
    const int bounces = (integ == SMS_INTEGRATOR_PATH_SMS_MS || filtered_ms || integ == SMS_INTEGRATOR_PATH_FILTERED_TEASER)
                            ? cfg.bounces : 1;
    /* PathRecord of path_filtered_ms.cpp:219-301 (state 0 default, 1 receiver,
       2 caster, 3 emitter; chain bounce count), after the camera ray */
    int rec = (si.valid() && (sc.shapes[si.shape].flags & SMS_SHAPE_CAUSTIC_RECEIVER)) ? 1 : 0, rec_b = 0;
    /* PathRecord of path_filtered_teaser.cpp:36-43, 334-410 (state 0 default,
       1 receiver, 2 single caster, 3 single emitter, 4 multi caster, 5 multi
       emitter; chain bounce count in rec_b), after the camera ray */
    const bool filtered_teaser = integ == SMS_INTEGRATOR_PATH_FILTERED_TEASER;
    int tf = rec == 1 ? 1 : 0;
    /* MNEEHelper of path_sms_ms.cpp:54-142 for unbiased MNEE: the same states
       in rec / rec_b, plus the receiver point and the specular vertices */
    const bool mnee_ms = integ == SMS_INTEGRATOR_PATH_SMS_MS && cfg.mnee_init && !opt.biased_mnee;
    V3 mnee_end = rec == 1 ? si.p : V3(0.f);
    int mnee_shape = -1;
    std::vector<V3> mnee_pos;
    for (int depth = 1;; ++depth) {
        if (!si.valid()) break;
        if (depth > opt.rr_depth) {
            Float q = omin(hmax_v(thr) * eta * eta, 0.95f);
            Float u = rng.next_f32();
            if (integ == SMS_INTEGRATOR_PATH ? !(u < q) : (u > q)) break;
            thr = thr * (1.f / q);
        }
        if ((uint32_t)depth >= (uint32_t)opt.max_depth) break;
        const Shape &s = sc.shapes[si.shape];
        V3 fs, ft;
        pt_frame(si, fs, ft);
        V3 wiw = -ray.d;
        /* a twosided BSDF seen from the back (cos_theta(wi) <= 0) works in the
           local frame with its normal reflected (twosided.cpp) */
        V3 n_sh = (s.bsdf.twosided && !(dot(wiw, si.shn) > 0.f)) ? -si.shn : si.shn;
        V3 wi(dot(wiw, fs), dot(wiw, ft), dot(wiw, n_sh));
        const bool receiver = (s.flags & SMS_SHAPE_CAUSTIC_RECEIVER) != 0;
        bool on_caster = false;
        if (teaser)
            on_caster = (s.flags & (SMS_SHAPE_CAUSTIC_CASTER_SINGLE | SMS_SHAPE_CAUSTIC_CASTER_MULTI |
                                    SMS_SHAPE_CAUSTIC_BOUNCER)) != 0;
        else if (integ == SMS_INTEGRATOR_PATH_SMS_SS) on_caster = (s.flags & SMS_SHAPE_CAUSTIC_CASTER_SINGLE) != 0;
        else if (integ == SMS_INTEGRATOR_PATH_SMS_MS || filtered_ms)
            on_caster = (s.flags & (SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER)) != 0;
        else if (filtered_ss)
            on_caster = (s.flags & (SMS_SHAPE_CAUSTIC_CASTER_SINGLE | SMS_SHAPE_CAUSTIC_CASTER_MULTI)) != 0;
        else if (filtered_teaser)
            on_caster = (s.flags & (SMS_SHAPE_CAUSTIC_CASTER_SINGLE | SMS_SHAPE_CAUSTIC_CASTER_MULTI |
                                    SMS_SHAPE_CAUSTIC_BOUNCER)) != 0;
        const bool glint_case = depth == 1 && !opt.disable_reflected_emitters;
        /* path_filtered_ss.cpp:109-110; light_connection_valid (path_filtered_ms.cpp:240-242) */
        const bool valid_conn = filtered_ss ? on_caster && (prev_receiver || glint_case)
                                            : filtered_ms && rec == 2 && rec_b == bounces;
        const Float caustic_eta = bsdf_eta(s.bsdf);
        const bool diffuse = s.bsdf.type == SMS_BSDF_DIFFUSE;
        /* the normal-mapped shape (glinty, or a caster / bouncer) carries the
           normalmap BSDF around its smooth conductor or dielectric */
        const bool nmapped = si.shape == sc.glinty_shape && sc.nmap.res > 0;
        /* with the LEAN fallback the normalmap BSDF is also glossy; it takes
           the fallback where the interaction has no uv partials, i.e. after
           the camera's first hit (normalmap.cpp:80, 142, 187) */
        const bool lean_fb = nmapped && sc.lean_fb.on;
        const bool lean_now = lean_fb && depth > 1;
        const bool smooth = (!nmapped && (diffuse || is_rough(s.bsdf))) || lean_fb;   /* BSDFFlags::Smooth */
        const bool on_glinty = (integ == SMS_INTEGRATOR_PATH_SMS_GLINTS || (teaser && opt.glints_enabled)) &&
                               depth == 1 && nmapped && (s.flags & SMS_SHAPE_GLINTY);
        const sms_config &glint_cfg = teaser ? gcfg : cfg;
        if (on_glinty) {
            /* SurfaceInteraction::compute_partials (interaction.h:216-248) */
            Float dn = dot(si.n, si.p);
            V3 dp_dx = ray.o + rdx * ((dn - dot(si.n, ray.o)) / dot(si.n, rdx)) - si.p;
            V3 dp_dy = ray.o + rdy * ((dn - dot(si.n, ray.o)) / dot(si.n, rdy)) - si.p;
            Float a00 = dot(si.dp_du, si.dp_du), a01 = dot(si.dp_du, si.dp_dv), a11 = dot(si.dp_dv, si.dp_dv);
            Float inv_det = 1.f / (a00 * a11 - a01 * a01);
            if (!std::isfinite(inv_det)) inv_det = 0.f;
            Float b0x = dot(si.dp_du, dp_dx), b1x = dot(si.dp_dv, dp_dx);
            Float b0y = dot(si.dp_du, dp_dy), b1y = dot(si.dp_dv, dp_dy);
            GQuery gq;
            gq.p = si.p; gq.n = si.shn; gq.dp_du = si.dp_du; gq.dp_dv = si.dp_dv; gq.sensor = ray.o; gq.uv = si.uv;
            gq.duv_dx.x = (a11 * b0x - a01 * b1x) * inv_det; gq.duv_dx.y = (a00 * b1x - a01 * b0x) * inv_det;
            gq.duv_dy.x = (a11 * b0y - a01 * b1y) * inv_det; gq.duv_dy.y = (a00 * b1y - a01 * b0y) * inv_det;
            V3 fs0 = normalize(si.dp_du - si.shn * dot(si.shn, si.dp_du)), ft0 = cross(si.shn, fs0);
            auto local = [&](V3 w) { return V3(dot(w, fs0), dot(w, ft0), dot(w, si.shn)); };
            const V3 wi_l = local(-ray.d);
            /* SMS strategy (manifold_glints.cpp:40-176) */
            const uint64_t gseed = sms_seed(opt.seed + (teaser ? 2 : 0));
            PCG32 grng;
            grng.seed(gseed, g + (1ull << 48));
            int gc = 0, gw = 0;
            V3 gv = glint_connect(sc, glint_cfg, gq, grng, gc, gw, st);
            if (gv.x != 0.f || gv.y != 0.f || gv.z != 0.f) {
                PCG32 r2;
                r2.seed(gseed, g + (1ull << 48));
                Query qq; qq.p = si.p;
                EI ei = sample_emitter_interaction(sc, sc.emitters_all, qq, r2);
                V3 ed = ei.p - si.p;
                Float edist = norm(ed);
                ed *= 1.f / edist;
                Float p_sms = 1.f;
                if (!ei.is_point) p_sms = pt_emitter_pdf(sc, sc.shapes[sc.emitters[ei.emitter].shape], si.p, ei.p, ed, edist);
                Float p_bsdf = glint_lean_pdf(sc.nmap, gq.uv, gq.duv_dx, gq.duv_dy, local(normalize(gq.sensor - si.p)),
                                              local(ed)) + 1.f;
                Float mis = (cfg.bsdf_strategy_only && !teaser) ? Float(0.f) : mis_weight(p_sms, p_bsdf);
                Float We = pt_importance(cam, tm, normalize(si.p - ray.o));
                L += thr * gv * (mis * We);
            }
            /* BSDF strategy inside the footprint (manifold_glints.cpp:178-220) */
            V2 fp = rng.next_2d();
            (void)rng.next_f32(); (void)rng.next_2d();
            V2 uvo;
            uvo.x = si.uv.x + (fp.x - 0.5f) * gq.duv_dx.x + (fp.y - 0.5f) * gq.duv_dy.x;
            uvo.y = si.uv.y + (fp.x - 0.5f) * gq.duv_dx.y + (fp.y - 0.5f) * gq.duv_dy.y;
            V3 bwo; Float bw;
            if (nm_conductor_sample(sc.nmap, s.bsdf, si.shn, si.dp_du, uvo, -ray.d, bwo, bw)) {
                Ray br; br.o = si.p; br.d = bwo; br.mint = kRayEps * (1.f + hmax_abs(si.p)); br.maxt = kInf;
                SI sb = ray_intersect(sc, br);
                if (sb.valid() && sc.shapes[sb.shape].emitter >= 0) {
                    const Shape &es = sc.shapes[sb.shape];
                    V3 ep = br.o + br.d * sb.t;
                    V3 Le = pt_emitted(sc, es, ep, br.d);
                    Float p_bsdf = glint_lean_pdf(sc.nmap, uvo, gq.duv_dx, gq.duv_dy, wi_l, local(bwo)) + 1.f;
                    Float p_sms = pt_emitter_pdf(sc, es, si.p, ep, bwo, sb.t);
                    Float mis = (cfg.sms_strategy_only && !teaser) ? Float(0.f) : mis_weight(p_bsdf, p_sms);
                    L += thr * Le * (mis * bw);
                }
            }
        }
        V3 albedo(s.bsdf.albedo[0], s.bsdf.albedo[1], s.bsdf.albedo[2]);
        /* the teaser's caustics at a receiver (path_sms_teaser.cpp:152-162):
           single scatter if depth + 1 < max_depth, multi scatter if depth +
           bounces < max_depth, both with cfg */
        /* any receiver whose BSDF has a non-delta lobe takes SMS queries
           (path_sms_ss.cpp:120-124; a delta BSDF's eval toward the chain is
           zero); a diffuse one passes its albedo, any other its shape and
           the incident direction in the frame coordinate_system(n_sh) */
        const bool sms_receiver = receiver && smooth && !nmapped;
        if (!diffuse) {
            V3 os, ot;
            coordinate_system(n_sh, os, ot);
            albedo = V3(-1.f - (Float)si.shape, dot(wiw, os), dot(wiw, ot));
        }
        if (teaser && opt.caustics_enabled && sms_receiver) {
            Query q;
            q.p = si.p; q.n = n_sh; q.dp_du = si.dp_du; q.dp_dv = si.dp_dv; q.albedo = albedo; q.cos_i = wi.z;
            int c = 0, w = 0;
            if (opt.max_depth < 0 || depth + 1 < opt.max_depth) {
                PCG32 srng;
                srng.seed(sms_seed(opt.seed), g + ((uint64_t)depth << 48));
                L += thr * ss_connect(sc, cfg, q, srng, c, w, st);
            }
            if (opt.max_depth < 0 || depth + cfg.bounces < opt.max_depth) {
                PCG32 srng;
                srng.seed(sms_seed(opt.seed + 1), g + ((uint64_t)depth << 48));
                L += thr * ms_connect(sc, cfg, q, srng, c, w, st);
            }
        }
        /* SMS at a receiver (path_sms_ss.cpp:115-121, path_sms_ms.cpp:226-232) */
        if (integ != SMS_INTEGRATOR_PATH && !teaser && !filtered_ss && !filtered_ms && !filtered_teaser && receiver &&
            !on_caster && sms_receiver &&
            (opt.max_depth < 0 || depth + bounces < opt.max_depth)) {
            Query q;
            q.p = si.p; q.n = n_sh; q.dp_du = si.dp_du; q.dp_dv = si.dp_dv; q.albedo = albedo; q.cos_i = wi.z;
            PCG32 srng;
            srng.seed(sms_seed(opt.seed), g + ((uint64_t)depth << 48));
            int c = 0, w = 0;
            V3 v = integ == SMS_INTEGRATOR_PATH_SMS_MS ? ms_connect(sc, cfg, q, srng, c, w, st)
                                                       : ss_connect(sc, cfg, q, srng, c, w, st);
            L += thr * v;
        }
        /* emitter sampling */
        bool nee = smooth && !on_caster && !on_glinty;
        if (integ == SMS_INTEGRATOR_PATH_SMS_SS) nee = nee || (depth == 1 && !opt.disable_reflected_emitters);
        if (teaser) nee = smooth && !on_caster && opt.non_sms_paths_enabled;   /* :185 */
        if (filtered_ss || filtered_ms) nee = smooth && (!on_caster || valid_conn);
        if (filtered_teaser) nee = smooth;   /* path_filtered_teaser.cpp:108 */
        if (nee) {
            Float ex = rng.next_f32(), ey = rng.next_f32();
            PtDir ds;
            bool got;
            if (filtered_teaser && on_caster) {
                /* sample_filtered_emitter_direction (:331-378) */
                const bool single_em = tf == 2 && rec_b == 1, multi_em = tf == 4 && rec_b == bounces;
                got = (single_em || multi_em) &&
                      pt_sample_emitter_from(sc, single_em ? sc.emitters_ss : sc.emitters_ms, si.p, ex, ey, ds);
            } else {
                got = pt_sample_emitter(sc, si.p, ex, ey, ds);
            }
            if (got) {
                Ray sr; sr.o = si.p; sr.d = ds.d;
                sr.mint = kRayEps * (1.f + hmax_abs(si.p)); sr.maxt = ds.dist * (1.f - kShadowEps);
                if (!ray_test(sc, sr) && smooth) {
                    V3 wo(dot(ds.d, fs), dot(ds.d, ft), dot(ds.d, n_sh));
                    /* with uv partials the normalmap BSDF evaluates its smooth
                       nested BSDF: nothing */
                    V3 bv = lean_now  ? V3(lean_fb_eval(sc.nmap, sc.lean_fb, wi, wo))
                            : nmapped ? V3(0.f)
                                      : shape_bsdf_eval(s, wi, wo);
                    if (bv.x != 0.f || bv.y != 0.f || bv.z != 0.f) {
                        const Float bp = lean_now ? lean_fb_pdf(sc.nmap, sc.lean_fb, wi, wo) : shape_bsdf_pdf(s, wi, wo);
                        Float w = ds.delta ? Float(1.f) : mis_weight(ds.pdf, bp);
                        /* path_filtered_ss.cpp:127-142 / path_filtered_ms.cpp:137-150 */
                        if (valid_conn && (filtered_ms || depth > 1)) {
                            const bool refraction = wo.z * wi.z < 0.f;
                            if (caustic_eta == 1.f ? refraction : !refraction) w = 0.f;
                        }
                        /* path_filtered_teaser.cpp:131-150 */
                        if (filtered_teaser) {
                            const bool refraction = wo.z * wi.z < 0.f;
                            if (on_caster ? (caustic_eta == 1.f ? refraction : !refraction) : !opt.non_sms_paths_enabled)
                                w = 0.f;
                        }
                        L += thr * bv * ds.spec * w;
                    }
                }
            }
        }
        /* BSDF sampling */
        Float u1 = rng.next_f32(), u2 = rng.next_f32(), u3 = rng.next_f32();
        PtBsdf bs;
        if (lean_now) {
            /* the LEAN fallback (normalmap.cpp:80-112): glossy reflection */
            V3 lwo;
            Float lw, lpdf;
            if (!lean_fb_sample(sc.nmap, sc.lean_fb, wi, u2, u3, lwo, lw, lpdf)) break;
            bs.wo = lwo;
            bs.weight = V3(lw);
            bs.pdf = lpdf;
            bs.eta = 1.f;
            bs.delta = false;
            bs.transmit = false;
        } else if (nmapped) {
            /* the normal-mapped BSDF at the hit's own uv */
            if (!nm_bsdf_sample(sc.nmap, s.bsdf, fs, ft, n_sh, si.dp_du, si.uv, wiw, u1, u2, u3, bs)) break;
        } else {
            if (!shape_bsdf_sample(s, wi, u1, u2, u3, bs)) break;
            bs.transmit = bs.wo.z * wi.z < 0.f;
        }
        thr = thr * bs.weight;
        eta *= bs.eta;
        if (!bs.delta) spec_cam = false;
        if (thr.x == 0.f && thr.y == 0.f && thr.z == 0.f) break;
        Ray nr;
        nr.o = si.p; nr.d = fs * bs.wo.x + ft * bs.wo.y + n_sh * bs.wo.z;
        nr.mint = kRayEps * (1.f + hmax_abs(si.p)); nr.maxt = kInf;
        SI si2 = ray_intersect(sc, nr);
        if (filtered_ms) {
            /* PathRecord::state_transition (path_filtered_ms.cpp:244-300) */
            const bool nv = si2.valid();
            const uint32_t nf = nv ? sc.shapes[si2.shape].flags : 0u;
            if (nv && (nf & SMS_SHAPE_CAUSTIC_RECEIVER)) { rec = 1; rec_b = 0; }
            else if (rec == 1) {
                if (nv && (nf & SMS_SHAPE_CAUSTIC_CASTER_MULTI)) { rec = 2; rec_b = 1; }
                else { rec = 0; rec_b = 0; }
            } else if (rec == 2) {
                if (rec_b < bounces && nv && (nf & (SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER))) {
                    if (caustic_eta == 1.f ? bs.transmit : !bs.transmit) { rec = 0; rec_b = 0; }
                    else rec_b++;
                } else if (rec_b == bounces && nv && sc.shapes[si2.shape].emitter >= 0 &&
                           std::find(sc.emitters_ms.begin(), sc.emitters_ms.end(), sc.shapes[si2.shape].emitter) !=
                               sc.emitters_ms.end()) {
                    rec = 3;
                } else { rec = 0; rec_b = 0; }
            } else { rec = 0; rec_b = 0; }
        }
        if (filtered_teaser) {
            /* PathRecord::state_transition (path_filtered_teaser.cpp:334-410) */
            const bool nv = si2.valid();
            const uint32_t nf = nv ? sc.shapes[si2.shape].flags : 0u;
            const int em = nv ? sc.shapes[si2.shape].emitter : -1;
            auto in = [&](const std::vector<int> &l) { return em >= 0 && std::find(l.begin(), l.end(), em) != l.end(); };
            const bool wrong = caustic_eta == 1.f ? bs.transmit : !bs.transmit;
            if (nv && (nf & SMS_SHAPE_CAUSTIC_RECEIVER)) { tf = 1; rec_b = 0; }
            else if (tf == 1) {
                if (nv && (nf & SMS_SHAPE_CAUSTIC_CASTER_SINGLE)) { tf = 2; rec_b = 1; }
                else if (nv && (nf & SMS_SHAPE_CAUSTIC_CASTER_MULTI)) { tf = 4; rec_b = 1; }
                else { tf = 0; rec_b = 0; }
            } else if (tf == 2) {
                if (!wrong && rec_b == 1 && in(sc.emitters_ss)) tf = 3;
                else { tf = 0; rec_b = 0; }
            } else if (tf == 4) {
                if (wrong) { tf = 0; rec_b = 0; }
                else if (rec_b < bounces && nv && (nf & (SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER))) rec_b++;
                else if (rec_b == bounces && in(sc.emitters_ms)) tf = 5;
                else { tf = 0; rec_b = 0; }
            } else { tf = 0; rec_b = 0; }
        }
        if (mnee_ms) {
            /* MNEEHelper::state_transition (path_sms_ms.cpp:84-140) */
            const bool nv = si2.valid();
            const uint32_t nf = nv ? sc.shapes[si2.shape].flags : 0u;
            if (nv && (nf & SMS_SHAPE_CAUSTIC_RECEIVER)) {
                rec = 1; rec_b = 0; mnee_end = si2.p; mnee_pos.clear();
            } else if (rec == 1) {
                if (nv && (nf & SMS_SHAPE_CAUSTIC_CASTER_MULTI)) {
                    rec = 2; rec_b = 1; mnee_shape = si2.shape; mnee_pos.assign(1, si2.p);
                } else { rec = 0; rec_b = 0; }
            } else if (rec == 2) {
                if (rec_b < bounces && nv && (nf & (SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER))) {
                    mnee_pos.push_back(si2.p);
                    rec_b++;
                } else if (rec_b == bounces && nv && sc.shapes[si2.shape].emitter >= 0 &&
                           std::find(sc.emitters_ms.begin(), sc.emitters_ms.end(), sc.shapes[si2.shape].emitter) !=
                               sc.emitters_ms.end()) {
                    rec = 3;
                } else { rec = 0; rec_b = 0; }
            } else { rec = 0; rec_b = 0; }
        }
        if (si2.valid() && sc.shapes[si2.shape].emitter >= 0) {
            const Shape &es = sc.shapes[si2.shape];
            V3 ep = nr.o + nr.d * si2.t;
            V3 Le = pt_emitted(sc, es, ep, nr.d);
            bool allow = true;
            if (integ == SMS_INTEGRATOR_PATH_SMS_SS) allow = !on_caster || (depth == 1 && !opt.disable_reflected_emitters);
            else if (integ == SMS_INTEGRATOR_PATH_SMS_MS) allow = !on_caster || spec_cam;
            else if (integ == SMS_INTEGRATOR_PATH_SMS_GLINTS) allow = !on_glinty;
            else if (teaser) allow = !on_caster && opt.non_sms_paths_enabled && !on_glinty;   /* :276 */
            else if (filtered_ss)   /* path_filtered_ss.cpp:166-172 */
                allow = !on_caster || (prev_receiver && (caustic_eta == 1.f ? !bs.transmit : bs.transmit)) || glint_case;
            else if (filtered_ms)   /* light_hit_valid (path_filtered_ms.cpp:191) */
                allow = !on_caster || (rec == 3 && rec_b == bounces) || spec_cam;
            else if (filtered_teaser)   /* filtered_emitter_hit_valid (:380-393), :186-195 */
                allow = on_caster ? (((tf == 3 && rec_b == 1) || (tf == 5 && rec_b == bounces)) &&
                                     std::find(sc.emitters_ms.begin(), sc.emitters_ms.end(), es.emitter) !=
                                         sc.emitters_ms.end())
                                  : opt.non_sms_paths_enabled != 0;
            if (allow) {
                Float epdf = bs.delta ? Float(0.f) : pt_emitter_pdf(sc, es, si.p, ep, nr.d, si2.t);
                L += thr * Le * mis_weight(bs.pdf, epdf);
            } else if (mnee_ms && rec == 3 && rec_b == bounces) {
                /* path_sms_ms.cpp:323-360: the MNEE walk from the receiver point */
                Query q;
                q.p = mnee_end;
                std::vector<int> tmpl;
                std::vector<MVertex> path;
                int it = 0;
                bool seed_ok = false;
                bool found = ms_sample_path(sc, cfg, mnee_shape, q, ep, V2{0.5f, 0.5f}, V3(0.f), tmpl, true, path, it,
                                            seed_ok);
                for (size_t k = 0; found && k < path.size(); ++k)
                    if (!(norm(path[k].p - mnee_pos[k]) < 1e-5f)) found = false;
                if (!found) L += thr * Le;
            } else if (integ == SMS_INTEGRATOR_PATH_SMS_SS && cfg.mnee_init && !opt.biased_mnee && prev_receiver &&
                       std::find(sc.emitters_ss.begin(), sc.emitters_ss.end(), es.emitter) != sc.emitters_ss.end()) {
                /* path_sms_ss.cpp:207-241: the MNEE walk from the previous vertex */
                Query q;
                q.p = prev_p;
                EI ei;
                ei.p = ep;
                SI sf, s0;
                int it = 0;
                sms_config c1 = cfg;
                c1.twostage = 0;   /* the library refuses twostage with this check */
                bool found = sample_path(sc, c1, si.shape, q, ei, V2{0.5f, 0.5f}, V3(0.f), sf, s0, it);
                if (found) {
                    V3 dpt = normalize(si.p - prev_p), dmn = normalize(sf.p - prev_p);
                    found = std::fabs(dot(dpt, dmn) - 1.f) < cfg.uniqueness_threshold;
                }
                if (!found) L += thr * Le;
            }
        }
        prev_p = si.p;
        prev_receiver = receiver;
        ray = nr;
        si = si2;
    }
    return L;
}

static Scene *as_scene(void *p) { return reinterpret_cast<Scene *>(p); }

} // namespace orc

using namespace orc;

extern "C" {

/* Which scalar type this build computes with: 0 float, 1 double, 2 counting float. */
int oracle_build_kind() {
#if defined(ORC_OPCOUNT)
    return 2;
#elif defined(ORC_DOUBLE)
    return 1;
#else
    return 0;
#endif
}

/* Operation counts since the last reset, summed over every thread: add/sub,
 * mul, div, sqrt, transcendental, BVH box tests, triangle tests, FLOPs inside
 * the box tests, FLOPs inside the triangle tests, ray casts; zeros unless
 * ORC_OPCOUNT. */
void oracle_opcount_read(uint64_t *out) {
#if defined(ORC_OPCOUNT)
    orc_opcount::read_counters(out);
#else
    for (int i = 0; i < 10; ++i) out[i] = 0;
#endif
}
void oracle_opcount_reset() {
#if defined(ORC_OPCOUNT)
    orc_opcount::reset_counters();
#endif
}

void *oracle_scene_create() { return new Scene(); }
void oracle_scene_destroy(void *s) { delete as_scene(s); }

int oracle_scene_add_sphere(void *s, const float *c, float r, int flip, const sms_bsdf *b,
                            uint32_t flags) {
    Scene *sc = as_scene(s);
    Shape sh;
    sh.kind = 0; sh.center = V3(c[0], c[1], c[2]); sh.radius = std::fabs(r);
    sh.flip = (flip != 0) != (r <= 0.f);
    sh.bsdf = *b; sh.flags = flags;
    rp_init(sh);
    sh.bbox_center = sh.center;
    sc->shapes.push_back(sh);
    sc->finalized = false;
    return (int)sc->shapes.size() - 1;
}

int oracle_scene_add_mesh(void *s, const float *P, const float *N, const float *UV, uint32_t nv,
                          const uint32_t *F, uint32_t nf, const sms_bsdf *b, uint32_t flags) {
    Scene *sc = as_scene(s);
    Shape sh;
    sh.kind = 1;
    sh.P.resize(nv);
    for (uint32_t i = 0; i < nv; ++i) sh.P[i] = V3(P[3 * i], P[3 * i + 1], P[3 * i + 2]);
    if (N) { sh.N.resize(nv); for (uint32_t i = 0; i < nv; ++i) sh.N[i] = V3(N[3 * i], N[3 * i + 1], N[3 * i + 2]); }
    if (UV) { sh.UV.resize(nv); for (uint32_t i = 0; i < nv; ++i) { sh.UV[i].x = UV[2 * i]; sh.UV[i].y = UV[2 * i + 1]; } }
    sh.F.assign(F, F + 3 * (size_t)nf);
    {
        V3 lo(kInf), hi(-kInf);
        for (const V3 &p : sh.P) {
            lo = V3(std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z));
            hi = V3(std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z));
        }
        sh.bbox_center = (lo + hi) * 0.5f;
    }
    /* mesh.cpp:505-528 + distr_1d.h:60-88: double accumulation, float storage */
    sh.pmf.resize(nf); sh.cdf.resize(nf);
    double sum = 0.0;
    bool first = true;
    for (uint32_t f = 0; f < nf; ++f) {
        V3 p0 = sh.P[F[3 * f]], p1 = sh.P[F[3 * f + 1]], p2 = sh.P[F[3 * f + 2]];
        float a = 0.5f * norm(cross(p1 - p0, p2 - p0));
        sh.pmf[f] = a;
        sum += (double)a;
        sh.cdf[f] = (float)sum;
        if (a > 0.f) { if (first) { sh.valid_lo = f; first = false; } sh.valid_hi = f; }
    }
    sh.area_sum = (float)sum;
    sh.area_norm = (float)(1.0 / sum);
    sh.bsdf = *b; sh.flags = flags;
    rp_init(sh);
    sc->shapes.push_back(sh);
    sc->finalized = false;
    return (int)sc->shapes.size() - 1;
}

int oracle_scene_add_point_emitter(void *s, const float *p, const float *I, uint32_t flags) {
    Scene *sc = as_scene(s);
    Emitter e; e.kind = 0; e.p = V3(p[0], p[1], p[2]); e.radiance = V3(I[0], I[1], I[2]); e.flags = flags;
    sc->emitters.push_back(e);
    return (int)sc->emitters.size() - 1;
}

int oracle_scene_add_area_emitter(void *s, int shape, const float *L, uint32_t flags) {
    Scene *sc = as_scene(s);
    if (shape < 0 || shape >= (int)sc->shapes.size() || sc->shapes[shape].kind != 0) return -1;
    Emitter e; e.kind = 1; e.shape = shape; e.radiance = V3(L[0], L[1], L[2]); e.flags = flags;
    sc->emitters.push_back(e);
    sc->shapes[shape].emitter = (int)sc->emitters.size() - 1;
    return (int)sc->emitters.size() - 1;
}

void oracle_scene_finalize(void *s) {
    Scene *sc = as_scene(s);
    sc->tri_shape.clear(); sc->tri_face.clear(); sc->nodes.clear();
    sc->casters_ss.clear(); sc->casters_ms.clear(); sc->bouncers.clear();
    sc->emitters_ss.clear(); sc->emitters_ms.clear();
    std::vector<uint32_t> idx;
    for (size_t i = 0; i < sc->shapes.size(); ++i) {
        const Shape &sh = sc->shapes[i];
        if (sh.flags & SMS_SHAPE_CAUSTIC_CASTER_SINGLE) sc->casters_ss.push_back((int)i);
        if (sh.flags & SMS_SHAPE_CAUSTIC_CASTER_MULTI) sc->casters_ms.push_back((int)i);
        if (sh.flags & SMS_SHAPE_CAUSTIC_BOUNCER) sc->bouncers.push_back((int)i);
        if (sh.kind == 1)
            for (uint32_t f = 0; f < sh.F.size() / 3; ++f) {
                sc->tri_shape.push_back((uint32_t)i); sc->tri_face.push_back(f);
            }
    }
    sc->emitters_all.clear();
    for (size_t i = 0; i < sc->emitters.size(); ++i) {
        sc->emitters_all.push_back((int)i);
        if (sc->emitters[i].flags & SMS_EMITTER_CAUSTIC_SINGLE) sc->emitters_ss.push_back((int)i);
        if (sc->emitters[i].flags & SMS_EMITTER_CAUSTIC_MULTI) sc->emitters_ms.push_back((int)i);
    }
    size_t np = sc->tri_shape.size();
    if (np) {
        std::vector<uint32_t> order(np);
        std::vector<Float> cen(3 * np);
        for (uint32_t i = 0; i < np; ++i) {
            order[i] = i;
            Float lo[3], hi[3], c[3];
            bvh_bounds(*sc, i, lo, hi, c);
            for (int k = 0; k < 3; ++k) cen[3 * i + k] = c[k];
        }
        bvh_build_rec(*sc, order, cen, 0, (uint32_t)np, sc->nodes);
        std::vector<uint32_t> ts(np), tf(np);
        for (size_t i = 0; i < np; ++i) { ts[i] = sc->tri_shape[order[i]]; tf[i] = sc->tri_face[order[i]]; }
        sc->tri_shape.swap(ts); sc->tri_face.swap(tf);
    }
    sc->finalized = true;
}

/* Per-walk sample_path with explicit ei.p and start point (SoA in/out as in
 * include/sms_gb300.h sms_ss_walk_batch; with cfg.twostage walk_in carries
 * SMS_SS_WALK_IN_FIELDS_TWOSTAGE rows, the last two the slope sample).
 * n_final is the solution vertex's normal (the normal map's, on a
 * normal-mapped caster). */
int oracle_ss_walk_batch(void *s, const sms_config *cfg, int caster, const float *queries,
                         const float *walk_in, uint32_t n, float *out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    for (uint32_t i = 0; i < n; ++i) {
        Query q = load_query(queries, n, i);
        auto w = [&](int k) { return walk_in[(size_t)k * n + i]; };
        EI ei; ei.p = V3(w(0), w(1), w(2)); ei.is_point = true;
        V3 ps(w(3), w(4), w(5));
        V2 smp; smp.x = w(6); smp.y = w(7);
        V2 g;
        if (cfg->twostage) { g.x = w(8); g.y = w(9); }
        SI sf, s0;
        int it = 0;
        bool ok = sample_path(*sc, *cfg, caster, q, ei, smp, ps, sf, s0, it, V3(0.f, 0.f, 1.f), g);
        MVertex vf;
        if (ok) vertex_from_si(*sc, sf, vf);
        float vals[SMS_WALK_OUT_FIELDS] = {ok ? 1.f : 0.f, (float)it, (float)sf.p.x, (float)sf.p.y,
                                           (float)sf.p.z, (float)s0.p.x, (float)s0.p.y, (float)s0.p.z,
                                           (float)vf.n.x, (float)vf.n.y, (float)vf.n.z};
        if (!ok) { for (int k = 2; k < 5; ++k) vals[k] = 0.f; for (int k = 8; k < 11; ++k) vals[k] = 0.f; }
        if (!s0.valid()) for (int k = 5; k < 8; ++k) vals[k] = 0.f;
        for (int k = 0; k < SMS_WALK_OUT_FIELDS; ++k) out[(size_t)k * n + i] = vals[k];
    }
    return 0;
}

/* SpecularManifoldSingleScatter::specular_manifold_sampling over n queries on
 * nthreads host threads (blocks of queries, like the reference's TBB loop). */
int oracle_ss_connect_batch(void *s, const sms_config *cfg, const float *queries, uint32_t n,
                            uint64_t seed, uint64_t stream_offset, float *value, int32_t *count,
                            int32_t *walks, int nthreads, uint64_t *stats_out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    Stats st;
    if (nthreads < 1) nthreads = 1;
    std::atomic<uint32_t> next{0};
    const uint32_t block = 64;
    auto worker = [&]() {
        while (true) {
            uint32_t b = next.fetch_add(block);
            if (b >= n) break;
            uint32_t e = std::min(n, b + block);
            for (uint32_t i = b; i < e; ++i) {
                Query q = load_query(queries, n, i);
                PCG32 rng;
                rng.seed(seed, (uint64_t)i + stream_offset);
                int c = 0, w = 0;
                V3 v = ss_connect(*sc, *cfg, q, rng, c, w, st);
                value[i] = v.x; value[(size_t)n + i] = v.y; value[2 * (size_t)n + i] = v.z;
                count[i] = c; walks[i] = w;
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
    worker();
    for (auto &t : th) t.join();
    if (stats_out) {
        stats_out[0] = st.succeeded; stats_out[1] = st.failed; stats_out[2] = st.calls;
        stats_out[3] = st.iters; stats_out[4] = st.iters_max; stats_out[5] = st.walks;
        stats_out[6] = st.newton; stats_out[7] = st.connections;
    }
    return 0;
}

/* Constraint and Jacobian of one single-scatter Newton step at the point of
 * `shape` with uv (u, v) (sphere: sphere.cpp:322-373 parametrization; mesh:
 * texture coordinates), for a
 * shading point x and light point lp: out = ok, C (2), J (2x2, row-major:
 * rows the constraint components, columns d/du, d/dv).  Test hook for the
 * finite-difference check of compute_step_anglediff / _halfvector. */
int oracle_ss_step_at(void *s, int shape, int halfvector, float u, float v, const float *x, const float *lp,
                      float *out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    for (int k = 0; k < 7; ++k) out[k] = 0.f;
    if (shape < 0 || shape >= (int)sc->shapes.size()) return 1;
    const Shape &sh = sc->shapes[shape];
    Ray r;
    if (sh.kind == 0) {
        const float th = kPi * v, ph = 2.f * kPi * u;
        V3 dir(std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th));
        r.o = sh.center + dir * (3.f * sh.radius);
        r.d = -dir;
    } else {
        /* mesh: (u, v) are texture coordinates; find the face holding them */
        if (sh.UV.empty()) return 1;
        bool found = false;
        for (size_t f = 0; f < sh.F.size() / 3 && !found; ++f) {
            V2 a = sh.UV[sh.F[3 * f]], b = sh.UV[sh.F[3 * f + 1]], c = sh.UV[sh.F[3 * f + 2]];
            float d = (b.x - a.x) * (c.y - a.y) - (c.x - a.x) * (b.y - a.y);
            if (d == 0.f) continue;
            float b1 = ((u - a.x) * (c.y - a.y) - (c.x - a.x) * (v - a.y)) / d;
            float b2 = ((b.x - a.x) * (v - a.y) - (u - a.x) * (b.y - a.y)) / d;
            if (b1 < 0.f || b2 < 0.f || b1 + b2 > 1.f) continue;
            V3 p0 = sh.P[sh.F[3 * f]], p1 = sh.P[sh.F[3 * f + 1]], p2 = sh.P[sh.F[3 * f + 2]];
            V3 pt = p0 * (1.f - b1 - b2) + p1 * b1 + p2 * b2;
            V3 gn = normalize(cross(p1 - p0, p2 - p0));
            r.o = pt + gn * 0.5f;
            r.d = -gn;
            found = true;
        }
        if (!found) return 2;
    }
    SI si = ray_intersect(*sc, r);
    if (!si.valid() || si.shape != shape) return 2;
    MVertex vtx;
    vertex_from_si(*sc, si, vtx);
    EI ei;
    ei.p = V3(lp[0], lp[1], lp[2]);
    ei.is_point = true;
    V2 C, dX;
    M2 J;
    bool ok = halfvector ? step_halfvector(V3(x[0], x[1], x[2]), vtx, ei, C, dX, &J)
                         : step_anglediff(V3(x[0], x[1], x[2]), vtx, ei, C, dX, &J);
    out[0] = ok ? 1.f : 0.f;
    out[1] = C.x; out[2] = C.y;
    out[3] = J.m[0][0]; out[4] = J.m[0][1]; out[5] = J.m[1][0]; out[6] = J.m[1][1];
    return 0;
}

/* The emitter interaction the single-scatter estimator draws first for each
 * query (stream (seed, stream_offset + i), manifold.h:204-260): out rows
 * ei.p (3), valid (1). */
int oracle_ss_emitter_batch(void *s, const float *queries, uint32_t n, uint64_t seed, uint64_t stream_offset,
                            float *out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    for (uint32_t i = 0; i < n; ++i) {
        Query q = load_query(queries, n, i);
        PCG32 rng;
        rng.seed(seed, (uint64_t)i + stream_offset);
        EI ei = sample_emitter_interaction(*sc, sc->emitters_ss, q, rng);
        out[i] = ei.p.x; out[(size_t)n + i] = ei.p.y; out[2 * (size_t)n + i] = ei.p.z;
        out[3 * (size_t)n + i] = ei.emitter >= 0 ? 1.f : 0.f;
    }
    return 0;
}

/* Unbiased single scatter with a learned proposal on caster `shape`: mix is
 * the processed mixture per query (40 x n, as sms_proposal_eval with
 * mixture = 1), frame = kind, org (3), ax_u (3), ax_v (3). */
int oracle_ss_connect_learned_batch(void *s, const sms_config *cfg, const float *queries, uint32_t n,
                                    uint64_t seed, uint64_t stream_offset, int shape, float defensive,
                                    const float *frame, const float *mix, float *value, int32_t *count,
                                    int32_t *walks, int nthreads, uint64_t *stats_out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    Stats st;
    if (nthreads < 1) nthreads = 1;
    std::atomic<uint32_t> next{0};
    const uint32_t block = 64;
    auto worker = [&]() {
        while (true) {
            uint32_t b = next.fetch_add(block);
            if (b >= n) break;
            uint32_t e = std::min(n, b + block);
            for (uint32_t i = b; i < e; ++i) {
                Learned L;
                L.shape = shape;
                L.defensive = defensive;
                L.kind = (int)frame[0];
                L.org = V3(frame[1], frame[2], frame[3]);
                L.ax_u = V3(frame[4], frame[5], frame[6]);
                L.ax_v = V3(frame[7], frame[8], frame[9]);
                L.mix = mix + i;
                L.stride = n;
                Query q = load_query(queries, n, i);
                PCG32 rng;
                rng.seed(seed, (uint64_t)i + stream_offset);
                int c = 0, w = 0;
                V3 v = ss_connect(*sc, *cfg, q, rng, c, w, st, &L);
                value[i] = v.x; value[(size_t)n + i] = v.y; value[2 * (size_t)n + i] = v.z;
                count[i] = c; walks[i] = w;
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
    worker();
    for (auto &t : th) t.join();
    if (stats_out) {
        stats_out[0] = st.succeeded; stats_out[1] = st.failed; stats_out[2] = st.calls;
        stats_out[3] = st.iters; stats_out[4] = st.iters_max; stats_out[5] = st.walks;
        stats_out[6] = st.newton; stats_out[7] = st.connections;
    }
    return 0;
}

/* Multi-scatter per-walk: first-path sample_path with explicit light point and
 * start point (walk_in rows: ei.p (3), p_start (3), sample (2)); out rows: ok,
 * iterations, p of the first vertex (3), p of the last vertex (3), seed ok. */
int oracle_ms_walk_batch(void *s, const sms_config *cfg, int caster, const float *queries, const float *walk_in,
                         uint32_t n, float *out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    for (uint32_t i = 0; i < n; ++i) {
        Query q = load_query(queries, n, i);
        auto w = [&](int k) { return walk_in[(size_t)k * n + i]; };
        V3 lp(w(0), w(1), w(2)), ps(w(3), w(4), w(5));
        V2 smp; smp.x = w(6); smp.y = w(7);
        std::vector<int> tmpl;
        std::vector<MVertex> path;
        int it = 0;
        bool seed_ok = false;
        bool ok = ms_sample_path(*sc, *cfg, caster, q, lp, smp, ps, tmpl, true, path, it, seed_ok);
        float vals[9] = {ok ? 1.f : 0.f, (float)it, 0, 0, 0, 0, 0, 0, seed_ok ? 1.f : 0.f};
        if (ok) {
            vals[2] = path[0].p.x; vals[3] = path[0].p.y; vals[4] = path[0].p.z;
            vals[5] = path.back().p.x; vals[6] = path.back().p.y; vals[7] = path.back().p.z;
        }
        for (int k = 0; k < 9; ++k) out[(size_t)k * n + i] = vals[k];
    }
    return 0;
}

int oracle_ms_connect_batch(void *s, const sms_config *cfg, const float *queries, uint32_t n, uint64_t seed,
                            uint64_t stream_offset, float *value, int32_t *count, int32_t *walks, int nthreads,
                            uint64_t *stats_out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    Stats st;
    if (nthreads < 1) nthreads = 1;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        while (true) {
            uint32_t b = next.fetch_add(16);
            if (b >= n) break;
            for (uint32_t i = b; i < std::min(n, b + 16); ++i) {
                Query q = load_query(queries, n, i);
                PCG32 rng;
                rng.seed(seed, (uint64_t)i + stream_offset);
                int c = 0, w = 0;
                V3 v = ms_connect(*sc, *cfg, q, rng, c, w, st);
                value[i] = v.x; value[(size_t)n + i] = v.y; value[2 * (size_t)n + i] = v.z;
                count[i] = c; walks[i] = w;
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
    worker();
    for (auto &t : th) t.join();
    if (stats_out) {
        stats_out[0] = st.succeeded; stats_out[1] = st.failed; stats_out[2] = st.calls;
        stats_out[3] = st.iters; stats_out[4] = st.iters_max; stats_out[5] = st.walks;
        stats_out[6] = st.newton; stats_out[7] = st.connections;
    }
    return 0;
}

int oracle_scene_set_normalmap(void *s, int shape, const uint16_t *slopes_half, uint32_t res, float tiles) {
    Scene *sc = as_scene(s);
    if (shape < 0 || shape >= (int)sc->shapes.size() || res == 0) return -1;
    auto h2f = [](uint16_t h) {
        uint32_t sign = (uint32_t)(h >> 15) << 31, e = (h >> 10) & 0x1f, m = h & 0x3ff, bits;
        if (e == 0) {
            if (m == 0) bits = sign;
            else { /* subnormal */
                int shift = 0;
                while (!(m & 0x400)) { m <<= 1; ++shift; }
                m &= 0x3ff;
                bits = sign | ((uint32_t)(127 - 15 - shift + 1) << 23) | (m << 13);
            }
        } else if (e == 31) {
            bits = sign | 0x7f800000u | (m << 13);
        } else {
            bits = sign | ((e - 15 + 127) << 23) | (m << 13);
        }
        float f;
        std::memcpy(&f, &bits, 4);
        return f;
    };
    sc->nmap.res = res;
    sc->nmap.tiles = tiles;
    size_t n = (size_t)res * res;
    sc->nmap.sx.resize(n);
    sc->nmap.sy.resize(n);
    for (size_t i = 0; i < n; ++i) { sc->nmap.sx[i] = h2f(slopes_half[2 * i]); sc->nmap.sy[i] = h2f(slopes_half[2 * i + 1]); }
    sc->nmap.lean.clear();
    sc->glinty_shape = shape;
    const uint32_t chain = SMS_SHAPE_CAUSTIC_CASTER_SINGLE | SMS_SHAPE_CAUSTIC_CASTER_MULTI | SMS_SHAPE_CAUSTIC_BOUNCER;
    if (!(sc->shapes[shape].flags & chain)) sc->shapes[shape].flags |= SMS_SHAPE_GLINTY;
    else build_lean(sc->nmap);   /* the two-stage solver's smoothed frames read its top level */
    return 0;
}

int oracle_scene_set_lean_fallback(void *s, float alpha, float eta, float k) {
    Scene *sc = as_scene(s);
    if (sc->nmap.res == 0) return -1;
    sc->lean_fb.on = true;
    sc->lean_fb.alpha = alpha;
    sc->lean_fb.eta = eta;
    sc->lean_fb.k = k;
    build_lean(sc->nmap);
    return 0;
}

/* The LEAN fallback BSDF of the scene's normal map, for n local-frame pairs
 * (SoA, 3 x n each): out rows eval, pdf. */
int oracle_lean_fb_eval(void *s, const float *wi, const float *wo, uint32_t n, float *out) {
    Scene *sc = as_scene(s);
    if (!sc->lean_fb.on) return -1;
    for (uint32_t i = 0; i < n; ++i) {
        const V3 a(wi[i], wi[n + i], wi[2 * n + i]), b(wo[i], wo[n + i], wo[2 * n + i]);
        out[i] = (float)lean_fb_eval(sc->nmap, sc->lean_fb, a, b);
        out[n + i] = (float)lean_fb_pdf(sc->nmap, sc->lean_fb, a, b);
    }
    return 0;
}

/* ... and its sampling from local wi (3 x n) with numbers u (2 x n): out rows
 * ok, wo (3), weight, pdf. */
int oracle_lean_fb_sample(void *s, const float *wi, const float *u, uint32_t n, float *out) {
    Scene *sc = as_scene(s);
    if (!sc->lean_fb.on) return -1;
    for (uint32_t i = 0; i < n; ++i) {
        const V3 a(wi[i], wi[n + i], wi[2 * n + i]);
        V3 wo(0.f);
        Float w = 0.f, pdf = 0.f;
        const bool ok = lean_fb_sample(sc->nmap, sc->lean_fb, a, u[i], u[n + i], wo, w, pdf);
        out[i] = ok ? 1.f : 0.f;
        out[n + i] = (float)wo.x; out[2 * n + i] = (float)wo.y; out[3 * n + i] = (float)wo.z;
        out[4 * n + i] = (float)w; out[5 * n + i] = (float)pdf;
    }
    return 0;
}

/* A shape's BSDF as the path tracers see it, for local-frame pairs wi, wo
 * (3 x n): out rows eval (BSDF x cos_o, 3), pdf. */
int oracle_shape_bsdf_eval(void *s, int shape, const float *wi, const float *wo, uint32_t n, float *out) {
    Scene *sc = as_scene(s);
    if (shape < 0 || shape >= (int)sc->shapes.size()) return -1;
    const Shape &sh = sc->shapes[shape];
    for (uint32_t i = 0; i < n; ++i) {
        const V3 a(wi[i], wi[n + i], wi[2 * n + i]), b(wo[i], wo[n + i], wo[2 * n + i]);
        const V3 f = shape_bsdf_eval(sh, a, b);
        out[i] = (float)f.x; out[n + i] = (float)f.y; out[2 * n + i] = (float)f.z;
        out[3 * n + i] = (float)shape_bsdf_pdf(sh, a, b);
    }
    return 0;
}

/* ... and its sampling from local wi (3 x n) with numbers u (3 x n): out rows
 * ok, wo (3), weight (3), pdf. */
int oracle_shape_bsdf_sample(void *s, int shape, const float *wi, const float *u, uint32_t n, float *out) {
    Scene *sc = as_scene(s);
    if (shape < 0 || shape >= (int)sc->shapes.size()) return -1;
    const Shape &sh = sc->shapes[shape];
    for (uint32_t i = 0; i < n; ++i) {
        const V3 a(wi[i], wi[n + i], wi[2 * n + i]);
        PtBsdf bs;
        const bool ok = shape_bsdf_sample(sh, a, u[i], u[n + i], u[2 * n + i], bs);
        out[i] = ok ? 1.f : 0.f;
        out[n + i] = ok ? (float)bs.wo.x : 0.f; out[2 * n + i] = ok ? (float)bs.wo.y : 0.f;
        out[3 * n + i] = ok ? (float)bs.wo.z : 0.f;
        out[4 * n + i] = ok ? (float)bs.weight.x : 0.f; out[5 * n + i] = ok ? (float)bs.weight.y : 0.f;
        out[6 * n + i] = ok ? (float)bs.weight.z : 0.f; out[7 * n + i] = ok ? (float)bs.pdf : 0.f;
    }
    return 0;
}

/* A roughplastic shape's precomputed terms: out = transmittance (64),
 * internal reflectance, specular sampling weight. */
int oracle_roughplastic_tables(void *s, int shape, float *out) {
    Scene *sc = as_scene(s);
    if (shape < 0 || shape >= (int)sc->shapes.size()) return -1;
    const Shape &sh = sc->shapes[shape];
    if (sh.bsdf.type != SMS_BSDF_ROUGHPLASTIC) return -1;
    for (int i = 0; i < kRoughPlasticRes; ++i) out[i] = (float)sh.rp.t[i];
    out[kRoughPlasticRes] = (float)sh.rp.fdr;
    out[kRoughPlasticRes + 1] = (float)sh.rp.ws;
    return 0;
}

/* sample_glint with an explicit footprint sample (xi_start, :225-265) and
 * light point: out rows ok, iterations, uv_final (2), uv_init (2). */
int oracle_glint_walk_batch(void *s, const sms_config *cfg, const float *queries, const float *walk_in, uint32_t n,
                            float *out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    for (uint32_t i = 0; i < n; ++i) {
        GQuery q = load_gquery(queries, n, i);
        auto w = [&](int k) { return walk_in[(size_t)k * n + i]; };
        V3 lp(w(0), w(1), w(2));
        V2 fp; fp.x = w(3); fp.y = w(4);
        V2 uvf, uvi;
        int it = 0;
        bool ok = sample_glint(*cfg, sc->nmap, q, lp, fp, uvf, uvi, it);
        float vals[6] = {ok ? 1.f : 0.f, (float)it, (float)uvf.x, (float)uvf.y, (float)uvi.x, (float)uvi.y};
        for (int k = 0; k < 6; ++k) out[(size_t)k * n + i] = vals[k];
    }
    return 0;
}

int oracle_glint_connect_batch(void *s, const sms_config *cfg, const float *queries, uint32_t n, uint64_t seed,
                               uint64_t stream_offset, float *value, int32_t *count, int32_t *walks, int nthreads,
                               uint64_t *stats_out) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    Stats st;
    if (nthreads < 1) nthreads = 1;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        while (true) {
            uint32_t b = next.fetch_add(64);
            if (b >= n) break;
            for (uint32_t i = b; i < std::min(n, b + 64); ++i) {
                GQuery q = load_gquery(queries, n, i);
                PCG32 rng;
                rng.seed(seed, (uint64_t)i + stream_offset);
                int c = 0, w = 0;
                V3 v = glint_connect(*sc, *cfg, q, rng, c, w, st);
                value[i] = v.x; value[(size_t)n + i] = v.y; value[2 * (size_t)n + i] = v.z;
                count[i] = c; walks[i] = w;
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
    worker();
    for (auto &t : th) t.join();
    if (stats_out) {
        stats_out[0] = st.succeeded; stats_out[1] = st.failed; stats_out[2] = st.calls;
        stats_out[3] = st.iters; stats_out[4] = st.iters_max; stats_out[5] = st.walks;
        stats_out[6] = st.newton; stats_out[7] = st.connections;
    }
    return 0;
}

/* Known-answer hooks for the dependency pins (fresnel.h:34-120, warp.h). */
float oracle_fresnel(float cos_i, float eta, float *cos_t) {
    Float ct = 0.f;
    const Float r = fresnel(cos_i, eta, cos_t ? &ct : nullptr);
    if (cos_t) *cos_t = (float)ct;
    return (float)r;
}
float oracle_fresnel_conductor(float cos_i, float eta, float k) { return (float)fresnel_conductor(cos_i, eta, k); }
/* Image of spp samples per pixel (height x width x 3, row-major), the
 * library's sms_render restated path by path; nthreads host threads. */
int oracle_render(void *s, const sms_config *cfg, const sms_camera *cam, const sms_render_options *opt,
                  float *image, int nthreads) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    if (opt->integrator == SMS_INTEGRATOR_PATH_SMS_GLINTS || (opt->integrator == SMS_INTEGRATOR_PATH_SMS_TEASER && opt->glints_enabled && sc->nmap.res > 0))
        build_lean(sc->nmap);
    const uint64_t wh = (uint64_t)cam->width * (uint64_t)cam->height;
    const double aspect = (double)cam->width / (double)cam->height;
    const double t = std::tan(0.5 * (double)cam->fov * 3.14159265358979323846 / 180.0);
    double tx = t;
    if (cam->fov_axis == SMS_FOV_Y) tx = t * aspect;
    else if (cam->fov_axis == SMS_FOV_DIAGONAL) tx = t / std::sqrt(1.0 + 1.0 / (aspect * aspect));
    else if (cam->fov_axis == SMS_FOV_SMALLER) tx = aspect >= 1.0 ? t * aspect : t;
    else if (cam->fov_axis == SMS_FOV_LARGER) tx = aspect >= 1.0 ? t : t * aspect;
    const double tm[2] = {(double)(float)tx, (double)(float)(tx / aspect)};
    const uint64_t total = wh * (uint64_t)opt->spp;
    std::vector<float> Ls(3 * total);
    Stats st;
    if (nthreads < 1) nthreads = 1;
    std::atomic<uint64_t> next{0};
    auto worker = [&]() {
        while (true) {
            uint64_t b = next.fetch_add(16);
            if (b >= total) break;
            for (uint64_t g = b; g < std::min(total, b + 16); ++g) {
                V3 L = pt_sample(*sc, *cfg, *cam, *opt, tm, g, st);
                Ls[3 * g] = L.x; Ls[3 * g + 1] = L.y; Ls[3 * g + 2] = L.z;
            }
        }
    };
    std::vector<std::thread> th;
    for (int k = 1; k < nthreads; ++k) th.emplace_back(worker);
    worker();
    for (auto &x : th) x.join();
    if (opt->rfilter == SMS_RFILTER_GAUSSIAN) {
        /* the Gaussian reconstruction filter (gaussian.cpp; radius 4 stddev),
           tabulated at 32 points (rfilter.cpp:9-20); every sample splats onto
           n pixels per axis (ImageBlock::put, imageblock.cpp:111-160) and each
           pixel is its weighted mean */
        const int R = 31;
        const float sd = opt->rfilter_stddev, r = 4.f * sd, alpha = -1.f / (2.f * sd * sd);
        const float bias = std::exp(alpha * r * r);
        float table[32];
        for (int i = 0; i < R; ++i) {
            const float x = (r * (float)i) / (float)R;
            table[i] = std::max(0.f, std::exp(alpha * (x * x)) - bias);
        }
        table[R] = 0.f;
        const float scale = (float)R / r;
        const int n = (int)std::ceil((r - 2.f * (float)kRayEps) * 2.f);
        std::vector<float> img(3 * wh, 0.f), wsum(wh, 0.f);
        const int W = cam->width, H = cam->height;
        for (uint64_t g = 0; g < total; ++g) {
            const uint64_t p = g % wh;
            const int px = (int)(p % (uint64_t)W), py = (int)(p / (uint64_t)W);
            PCG32 rng;
            rng.seed(opt->seed, g);   /* the camera sample's position (pt_sample) */
            const float ux = (float)rng.next_f32(), uy = (float)rng.next_f32();
            const float sx = ((float)px + ux) / (float)W, sy = ((float)py + uy) / (float)H;
            const float pos[2] = {sx * (float)W - 0.5f, sy * (float)H - 0.5f};
            int lo[2];
            float w[2][64];
            int cnt[2];
            for (int a = 0; a < 2; ++a) {
                lo[a] = (int)std::ceil(pos[a] - r);
                const int hi = (int)std::floor(pos[a] + r);
                cnt[a] = std::min(n, hi - lo[a] + 1);
                const float base = (float)lo[a] - pos[a];
                for (int i = 0; i < cnt[a]; ++i)
                    w[a][i] = table[std::min((int)std::fabs((base + (float)i) * scale), R)];
            }
            for (int yr = 0; yr < cnt[1]; ++yr) {
                const int y = lo[1] + yr;
                if (y < 0 || y >= H) continue;
                for (int xr = 0; xr < cnt[0]; ++xr) {
                    const int x = lo[0] + xr;
                    if (x < 0 || x >= W) continue;
                    const float wt = w[1][yr] * w[0][xr];
                    const uint64_t d = (uint64_t)y * W + x;
                    for (int c = 0; c < 3; ++c) img[3 * d + c] += Ls[3 * g + c] * wt;
                    wsum[d] += wt;
                }
            }
        }
        for (uint64_t p = 0; p < wh; ++p) {
            const float sc = wsum[p] != 0.f ? 1.f / wsum[p] : 0.f;
            for (int c = 0; c < 3; ++c) image[3 * p + c] = img[3 * p + c] * sc;
        }
        return 0;
    }
    for (uint64_t p = 0; p < wh; ++p) {
        float acc[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < opt->spp; ++k)
            for (int c = 0; c < 3; ++c) acc[c] += Ls[3 * ((uint64_t)k * wh + p) + c];
        for (int c = 0; c < 3; ++c) image[3 * p + c] = acc[c] * (1.f / (float)opt->spp);
    }
    return 0;
}

/* LEAN density of the glints integrator's MIS (glint_lean_pdf) for tests:
 * duv = (duv_dx, duv_dy), wi / wo in the local frame of the glinty shape. */
float oracle_glint_lean_pdf(void *s, float u, float v, const float *duv, const float *wi, const float *wo) {
    Scene *sc = as_scene(s);
    if (!sc->finalized) oracle_scene_finalize(s);
    build_lean(sc->nmap);
    V2 uv; uv.x = u; uv.y = v;
    V2 dx; dx.x = duv[0]; dx.y = duv[1];
    V2 dy; dy.x = duv[2]; dy.y = duv[3];
    return glint_lean_pdf(sc->nmap, uv, dx, dy, V3(wi[0], wi[1], wi[2]), V3(wo[0], wo[1], wo[2]));
}

/* The two-stage solver's slope sample (sample_gaussian) for tests: mu (2),
 * sigma = (a, c; c, b), u (2); out = the slope. */
void oracle_sample_slope_gaussian(const float *mu, float a, float b, float c, const float *u, float *out) {
    V2 m; m.x = mu[0]; m.y = mu[1];
    V2 uu; uu.x = u[0]; uu.y = u[1];
    V2 r = sample_slope_gaussian(m, a, b, c, uu);
    out[0] = r.x; out[1] = r.y;
}

void oracle_uniform_sphere(float u, float v, float *out) {
    V2 s; s.x = u; s.y = v;
    V3 r = square_to_uniform_sphere(s);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void oracle_pcg32(uint64_t initstate, uint64_t initseq, uint32_t n, uint32_t *out) {
    PCG32 r; r.seed(initstate, initseq);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.next_u32();
}
void oracle_nm_slope(void *s, float u, float v, float *out) {
    Scene *sc = as_scene(s);
    V2 uv; uv.x = u; uv.y = v;
    V2 sl = nm_slope(sc->nmap, uv), du, dv;
    nm_slope_derivative(sc->nmap, uv, du, dv);
    out[0] = sl.x; out[1] = sl.y; out[2] = du.x; out[3] = du.y; out[4] = dv.x; out[5] = dv.y;
}
void oracle_pcg32_f32(uint64_t initstate, uint64_t initseq, uint32_t n, float *out) {
    PCG32 r; r.seed(initstate, initseq);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.next_f32();
}

} // extern "C"
