// sms_device.cuh -- device-side building blocks of the SMS walks on sm_103a.
//
// Geometry (BVH over all mesh triangles + analytic spheres), the manifold vertex
// rebuilt after every accepted Newton step, the specular constraints and their
// 2x2 Jacobians, Fresnel terms and the generalized geometric term.  All FP32.
//
// Reference behaviour restated here (paths relative to the reference project):
//   manifold vertex            include/mitsuba/render/manifold.h:50-141
//   reflect/refract/sphcoords  include/mitsuba/render/manifold.h:348-443
//   anglediff / halfvector     src/librender/manifold_ss.cpp:407-636
//   geometric term             src/librender/manifold_ss.cpp:695-857
//   shading frame derivative   include/mitsuba/core/frame.h:197-240
//   sphere                     src/shapes/sphere.cpp:153-170,275-382
//   triangles                  include/mitsuba/render/mesh.h:203-228,
//                              src/librender/mesh.cpp:541-586,618-765
//   Fresnel                    include/mitsuba/render/fresnel.h:34-120
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

// Every helper here is host+device so that the host-side tests can run the
// exact traversal and vertex code the kernels run.
#define SMS_HD __host__ __device__ __forceinline__

namespace sms {

template <typename T>
SMS_HD T sms_ldg(const T *p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}
SMS_HD int sms_as_int(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_int(f);
#else
    int i;
    std::memcpy(&i, &f, 4);
    return i;
#endif
}
SMS_HD float sms_as_float(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}
SMS_HD uint32_t sms_rotr(uint32_t x, uint32_t r) {
#ifdef __CUDA_ARCH__
    return __funnelshift_r(x, x, r);
#else
    return (x >> (r & 31u)) | (x << ((32u - r) & 31u));
#endif
}

// ------------------------------------------------------------------ constants
// include/mitsuba/core/math.h:37-38 (float epsilon / 2 * 1500, x10 for shadows)
constexpr float kRayEps = 5.9604644775390625e-08f * 1500.f;
constexpr float kShadowEps = kRayEps * 10.f;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr int kStackDepth = 32;
constexpr int kMaxCasters = 8;
constexpr int kMaxEmitters = 16;
constexpr int kMaxSpheres = 16;
constexpr int kMaxLeanLevels = 20;

// Device error flags (bitwise or-ed into DevCounters::error).
constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrTrialLimit = 2u;
constexpr uint32_t kErrSolutionOverflow = 4u;
constexpr uint32_t kErrBadQuery = 8u;   // a query names a receiver shape outside the scene

// ------------------------------------------------------------------- vectors
struct f3 { float x, y, z; };
SMS_HD f3 mk(float x, float y, float z) { return {x, y, z}; }
SMS_HD f3 splat(float a) { return {a, a, a}; }
SMS_HD f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
SMS_HD f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
SMS_HD f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
SMS_HD f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
SMS_HD f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
SMS_HD float dot(f3 a, f3 b) {
    // Plain multiply-add order; contraction into FMA is left to the compiler.
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
SMS_HD f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
SMS_HD float length(f3 a) { return sqrtf(dot(a, a)); }
SMS_HD f3 normalize(f3 a) { return a * (1.f / sqrtf(dot(a, a))); }
SMS_HD float safe_sqrt(float v) { return sqrtf(fmaxf(v, 0.f)); }
SMS_HD float clamp1(float v) { return fminf(1.f, fmaxf(-1.f, v)); }

struct M2 { float a, b, c, d; };  // [[a b] [c d]]
SMS_HD float det2(M2 m) { return m.a * m.d - m.b * m.c; }

// Duff et al. 2017 orthonormal basis (include/mitsuba/core/vector.h:116-135).
SMS_HD void onb(f3 n, f3 &s, f3 &t) {
    float sign = copysignf(1.f, n.z);
    float a = -1.f / (sign + n.z);
    float b = n.x * n.y * a;
    s = mk(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    t = mk(b, sign + n.y * n.y * a, -n.y);
}

// --------------------------------------------------------------------- PCG32
// O'Neill's PCG32 (XSH-RR 64/32); one stream per query.
struct Pcg32 {
    uint64_t state, inc;
    SMS_HD uint32_t next_u32() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return sms_rotr(xs, rot);
    }
    SMS_HD void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next_u32();
        state += initstate;
        next_u32();
    }
    SMS_HD float next_f32() {
        return sms_as_float((next_u32() >> 9) | 0x3f800000u) - 1.f;
    }
    // Skip `delta` outputs in O(log delta): the LCG step x -> a x + c applied
    // k times is x -> A_k x + C_k, composed by binary powering (Brown 1994,
    // "Random number generation with arbitrary strides").
    SMS_HD void advance(uint64_t delta) {
        uint64_t cur_mult = 6364136223846793005ULL, cur_plus = inc;
        uint64_t acc_mult = 1u, acc_plus = 0u;
        while (delta > 0) {
            if (delta & 1u) {
                acc_mult *= cur_mult;
                acc_plus = acc_plus * cur_mult + cur_plus;
            }
            cur_plus = (cur_mult + 1u) * cur_plus;
            cur_mult *= cur_mult;
            delta >>= 1u;
        }
        state = acc_mult * state + acc_plus;
    }
};

// --------------------------------------------------------------- scene data
enum : int { kShapeSphere = 0, kShapeMesh = 1 };
// shape flags (same bits as SMS_SHAPE_* in sms_gb300.h)
constexpr uint32_t kShapeFlagReceiver = 1u << 0;
constexpr uint32_t kShapeFlagCasterSingle = 1u << 1;
constexpr uint32_t kShapeFlagCasterMulti = 1u << 2;
constexpr uint32_t kShapeFlagBouncer = 1u << 3;
constexpr uint32_t kShapeFlagGlinty = 1u << 4;
enum : int { kBsdfDiffuse = 0, kBsdfDielectric = 1, kBsdfConductor = 2, kBsdfRoughPlastic = 3 };
constexpr int kRoughPlasticRes = 64;   // MTS_ROUGH_TRANSMITTANCE_RES (roughplastic.cpp)

struct DevShape {
    int kind;
    uint32_t flags;
    int bsdf_type;
    float eta, k;          // ior (eta + i k)
    float spec_eta;        // manifold-vertex eta (manifold.h:94-96)
    // sphere
    float cx, cy, cz, radius;
    int flip;
    // mesh: offsets into the concatenated mesh arrays
    uint32_t v_off, f_off, n_faces;
    int has_normals, has_uvs;
    uint32_t cdf_off;
    float area_sum, area_norm;
    uint32_t valid_lo, valid_hi;
    int emitter;
    float bcx, bcy, bcz;   // bounding-box centre
    int reflective;        // complex ior: MNEE initialisation aims at the box centre
    float albedo[3];       // diffuse reflectance (path tracer)
    float alpha;           // Beckmann roughness of a rough dielectric / conductor (0: smooth)
    int nmap_frames;       // manifold vertices on this shape use its normal map (a caster / bouncer)
    int twosided;          // the path tracer reflects the local frame at back-side hits (twosided.cpp)
    // roughplastic: the coating's external transmittance at kRoughPlasticRes
    // cosines, the base's internal diffuse reflectance, the specular
    // sampling weight and the nonlinear switch (roughplastic.cpp:355-399)
    float rp_t[kRoughPlasticRes];
    float rp_fdr, rp_ws;
    int rp_nonlinear;
};

// Target of the MNEE initialisation (manifold_ss.cpp:229-241,
// manifold_ms.cpp:305-316): the shape's bounding-box centre for reflecting
// (complex-ior) BSDFs, the light sample otherwise.
SMS_HD f3 mnee_target(const DevShape &s, f3 lp) { return s.reflective ? mk(s.bcx, s.bcy, s.bcz) : lp; }

struct DevEmitter {
    int kind;              // 0 point, 1 area on a sphere shape
    float px, py, pz;      // point position
    float r, g, b;         // intensity / radiance
    int shape;
};

// BVH2 node: both children's boxes in one 64-byte record.
//   n0 = (l.lo.x, l.lo.y, l.lo.z, l.hi.x)
//   n1 = (l.hi.y, l.hi.z, r.lo.x, r.lo.y)
//   n2 = (r.lo.z, r.hi.x, r.hi.y, r.hi.z)
//   n3 = (left, right, left_count, right_count) as ints; count > 0 -> leaf
//        whose triangles start at the child index.
struct DevScene {
    const float4 *nodes;       // 4 float4 per node
    const float4 *tris;        // 3 float4 per triangle: p0|shape, e1|face, e2
    uint32_t n_nodes, n_tris;
    const DevShape *shapes;
    int n_shapes;
    const float *mesh_P;       // xyz per vertex (all meshes)
    const float *mesh_N;
    const float *mesh_UV;
    const uint32_t *mesh_F;    // 3 indices per face, local to the mesh
    const float *cdf;          // face-area CDFs (unnormalized), per mesh
    const float *pmf;
    // analytic spheres (all of them are tested for every ray)
    int n_spheres;
    int sphere_shape[kMaxSpheres];
    float4 sphere[kMaxSpheres];  // center xyz, radius
    // caustic lists (scene.cpp:95-112)
    int n_casters_ss, casters_ss[kMaxCasters];
    uint32_t casters_ss_rough;   // bit c: single-scatter caster c is rough (alpha > 0)
    uint32_t casters_ss_nm;      // bit c: single-scatter caster c carries the normal map
    int ms_nm;                   // a multi-scatter chain shape carries the normal map
    int ms_rough;                // a multi-scatter chain shape is rough (alpha > 0)
    int n_emitters_ss, emitters_ss[kMaxEmitters];
    int n_casters_ms, casters_ms[kMaxCasters];
    int n_emitters_ms, emitters_ms[kMaxEmitters];
    int n_emitters_all, emitters_all[kMaxEmitters];
    // glints: FP16 (sx, sy) slope map of the glinty shape, res x res texels
    const uint32_t *nmap;      // one __half2 per texel
    uint32_t nmap_res;
    float nmap_tiles;
    int glinty_shape;           // the shape carrying the slope map
    int nmap_shape;             // same id: normal-mapped manifold-vertex frames
    // LEAN mip pyramid of the slope map (glints integrator): level l starts at
    // lean + lean_off[l] (floats), 5 floats per texel, (nmap_res >> l)^2 texels
    const float *lean;
    uint32_t lean_off[kMaxLeanLevels];
    int lean_levels;
    // the normal map's LEAN fallback BSDF (glossy reflection of the top LEAN
    // level widened by lf_alpha, Fresnel of lf_eta + i lf_k) at vertices
    // without uv partials; 0 = off
    int lean_fb;
    float lf_alpha, lf_eta, lf_k;
    const DevEmitter *emitters;
    // The first n_tnodes node records (the top levels of the tree: records are
    // stored breadth first) are also held in the launching kernel's dynamic
    // shared memory (sms_tree_smem), filled by tree_smem_fill; 0 = none.
    uint32_t n_tnodes;
};

#ifdef __CUDACC__
// Dynamic shared memory of a kernel that stages the top of the tree.
extern __shared__ __align__(16) float4 sms_tree_smem[];

// Copy the first sc.n_tnodes node records into sms_tree_smem (all threads of
// the block call it before any traversal).
__device__ __forceinline__ void tree_smem_fill(const DevScene &sc) {
    if (sc.n_tnodes == 0) return;
    for (uint32_t i = threadIdx.x; i < 4 * sc.n_tnodes; i += blockDim.x) sms_tree_smem[i] = __ldg(sc.nodes + i);
    __syncthreads();
}
#endif

// ------------------------------------------------------------------ hits
struct Hit {
    float t;
    int shape;       // -1: miss
    uint32_t prim;
    float u, v;      // triangle barycentrics
    uint32_t nodes;  // BVH nodes fetched by this ray (64 B each)
    uint32_t tests;  // triangles fetched by this ray (48 B each)
};

// Robust FP32 ray-sphere intersection (the reference solves the quadratic in
// FP64, sphere.cpp:275-297).  The discriminant is formed from the vector to the
// closest approach instead of b^2 - 4ac, which keeps FP32 accurate at the
// distances of these scenes.  Same [mint, maxt] / inside-segment rules.
SMS_HD bool sphere_hit(float4 s, f3 o, f3 d, float mint, float maxt, float &t_out) {
    f3 oc = o - mk(s.x, s.y, s.z);
    float a = dot(d, d);
    float b = dot(oc, d);                 // half of the reference's B
    f3 qv = oc - d * (b / a);
    float r2 = s.w * s.w;
    float disc = a * (r2 - dot(qv, qv));
    if (!(disc >= 0.f)) return false;
    float c = dot(oc, oc) - r2;
    float q = -(b + copysignf(sqrtf(disc), b));
    float t0 = c / q, t1 = q / a;
    if (q == 0.f) { t0 = t1 = 0.f; }
    float nt = fminf(t0, t1), ft = fmaxf(t0, t1);
    bool out_bounds = !(nt <= maxt && ft >= mint);
    bool in_bounds = nt < mint && ft > maxt;
    if (out_bounds || in_bounds) return false;
    t_out = nt < mint ? ft : nt;
    return true;
}

// Moller-Trumbore in the reference's operation order (mesh.h:203-228).
SMS_HD bool tri_hit(float4 a, float4 b, float4 c, f3 o, f3 d, float mint,
                                        float maxt, float &t, float &u, float &v) {
    f3 p0 = mk(a.x, a.y, a.z), e1 = mk(b.x, b.y, b.z), e2 = mk(c.x, c.y, c.z);
    f3 pvec = cross(d, e2);
    const float det = dot(e1, pvec);
    f3 tvec = o - p0;
    const float un = dot(tvec, pvec);
    // The same bounds on the numerators, scaled by |det| and widened by a
    // relative 1e-6 (more than the rounding of the quotients), reject most
    // triangles before the reciprocal (the first barycentric before the
    // second cross product); the test on the quotients decides.
    const float sg = det < 0.f ? -1.f : 1.f, ad = fabsf(det);
    const float us = un * sg;
    const float hi = ad * (1.f + 1e-6f);
    if (!(us >= 0.f && us <= hi)) return false;
    f3 qvec = cross(tvec, e1);
    const float vn = dot(d, qvec), tn = dot(e2, qvec);
    const float vs = vn * sg, ts = tn * sg;
    if (!(vs >= 0.f && us + vs <= hi && ts >= mint * ad * (1.f - 1e-6f) && ts <= maxt * hi)) return false;
    const float inv_det = 1.f / det;
    u = un * inv_det;
    v = vn * inv_det;
    t = tn * inv_det;
    return u >= 0.f && u <= 1.f && v >= 0.f && u + v <= 1.f && t >= mint && t <= maxt;
}

// Slab test of one box; inv the reciprocal direction, oi = o * inv, so that
// each slab distance (lo - o) / d is one FMA.
SMS_HD bool box2(float lox, float loy, float loz, float hix, float hiy, float hiz,
                                     f3 inv, f3 oi, float tmin, float tmax, float &tn) {
    float tx0 = fmaf(lox, inv.x, -oi.x), tx1 = fmaf(hix, inv.x, -oi.x);
    float ty0 = fmaf(loy, inv.y, -oi.y), ty1 = fmaf(hiy, inv.y, -oi.y);
    float tz0 = fmaf(loz, inv.z, -oi.z), tz1 = fmaf(hiz, inv.z, -oi.z);
    float t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    float t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    tn = t0;
    return t0 <= t1;
}

// Closest hit (any_hit = false) or occlusion test (any_hit = true) against the
// whole scene; one traversal loop serves both so that lanes of a warp casting
// different kinds of rays still traverse together.  kTree: the launching
// kernel holds the top sc.n_tnodes node records in shared memory (a separate
// instantiation, so that kernels without it keep the plain fetch).  Returns false and sets *err on stack overflow (treated as miss).
template <bool kTree = false>
SMS_HD bool trace(const DevScene &sc, f3 o, f3 d, float mint, float maxt, bool any_hit, Hit &hit,
                  uint32_t &err) {
    hit.t = maxt; hit.shape = -1; hit.prim = 0; hit.u = hit.v = 0.f;
    hit.nodes = 0; hit.tests = 0;
    // A NaN origin or direction (a Newton step through a NaN Jacobian, which
    // the reference's |det| < 1e-6 test lets pass) can hit nothing: every
    // comparison in the sphere and triangle tests is false.  Return the miss
    // now instead of letting NaN slabs open every box of the tree.
    if (!(fabsf(o.x) + fabsf(o.y) + fabsf(o.z) + fabsf(d.x) + fabsf(d.y) + fabsf(d.z) < INFINITY))
        return false;
    bool found = false;
    for (int i = 0; i < sc.n_spheres; ++i) {
        float t;
        if (sphere_hit(sc.sphere[i], o, d, mint, hit.t, t) && (!found || t < hit.t)) {
            hit.t = t; hit.shape = sc.sphere_shape[i]; found = true;
            if (any_hit) return true;
        }
    }
    if (sc.n_tris == 0) return found;
    bool tri_best = false;
    // Reciprocal direction, a zero component replaced by 1e-20 of its sign so
    // that every slab distance is finite (a slab the ray runs inside then
    // spans about +-1e20 and constrains nothing).
    auto rcp_dir = [](float x) { return 1.f / (fabsf(x) > 1e-20f ? x : copysignf(1e-20f, x)); };
    const f3 inv = mk(rcp_dir(d.x), rcp_dir(d.y), rcp_dir(d.z));
    const f3 oi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
    int stack[kStackDepth];
    int sp = 0;
    int node = 0;
    // The loop ends: the host accepts only trees whose inner children come
    // after their parents (validate_bvh), and a node is reached only from its
    // parent's single visit, so every node is visited at most once.
    while (true) {
        hit.nodes++;
        float4 n0, n1, n2;
        int4 n3;
#ifdef __CUDA_ARCH__
        if (kTree && (uint32_t)node < sc.n_tnodes) {
            const float4 *sp = sms_tree_smem + 4 * node;
            n0 = sp[0]; n1 = sp[1]; n2 = sp[2];
            n3 = *reinterpret_cast<const int4 *>(sp + 3);
        } else
#endif
        {
            const float4 *np = sc.nodes + 4 * (size_t)node;
            n0 = sms_ldg(np); n1 = sms_ldg(np + 1); n2 = sms_ldg(np + 2);
            n3 = sms_ldg(reinterpret_cast<const int4 *>(np + 3));
        }
        float tl, tr;
        bool hl = box2(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, inv, oi, mint, hit.t, tl);
        bool hr = box2(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, inv, oi, mint, hit.t, tr);
        // Leaves are processed right away, the triangles of both hit leaf
        // children in one loop (left first), so that lanes whose leaves sit on
        // different sides test their triangles together; inner children are
        // pushed.
        int next = -1;
        const int c0 = hl ? n3.z : 0, nt = c0 + (hr ? n3.w : 0);
        hit.tests += (uint32_t)nt;
        for (int k = 0; k < nt; ++k) {
            const int ti = k < c0 ? n3.x + k : n3.y + (k - c0);
            const float4 *tp = sc.tris + 3 * (size_t)ti;
            float4 a = sms_ldg(tp), b = sms_ldg(tp + 1), c = sms_ldg(tp + 2);
            float t, u, v;
            if (tri_hit(a, b, c, o, d, mint, hit.t, t, u, v)) {
                const int shape = sms_as_int(a.w);
                const uint32_t prim = (uint32_t)sms_as_int(b.w);
                // Equal distances (a ray through a shared edge) go to the lower
                // (shape, face) index, so the hit does not depend on the tree.
                if (!found || t < hit.t ||
                    (t == hit.t && tri_best && (shape < hit.shape || (shape == hit.shape && prim < hit.prim)))) {
                    hit.t = t; hit.u = u; hit.v = v;
                    hit.shape = shape;
                    hit.prim = prim;
                    found = true;
                    tri_best = true;
                    if (any_hit) return true;
                }
            }
        }
        bool il = hl && n3.z == 0, ir = hr && n3.w == 0;
        if (il && ir) {
            int near = tl <= tr ? n3.x : n3.y, far = tl <= tr ? n3.y : n3.x;
            if (sp >= kStackDepth) { err |= kErrStackOverflow; return false; }
            stack[sp++] = far;
            next = near;
        } else if (il) {
            next = n3.x;
        } else if (ir) {
            next = n3.y;
        }
        if (next < 0) {
            if (sp == 0) break;
            next = stack[--sp];
        }
        node = next;
    }
    return found;
}

// ------------------------------------------------------- surface interaction
struct SurfPt {
    f3 p, n, shn, dp_du, dp_dv;
    float u, v;     // uv
};

// sphere.cpp:322-373 (no rotation in to_world)
SMS_HD void sphere_surface(const DevShape &s, f3 o, f3 d, float t, SurfPt &si) {
    f3 c = mk(s.cx, s.cy, s.cz);
    f3 n = normalize(o + d * t - c);
    si.p = n * s.radius + c;
    f3 l = (si.p - c) * (1.f / s.radius);
    float rd2 = l.x * l.x + l.y * l.y;
    float sz = copysignf(1.f, l.z);
    f3 w = mk(l.x, l.y, l.z - sz);
    float tmp = 2.f * asinf(fminf(1.f, 0.5f * length(w)));
    float theta = l.z >= 0.f ? tmp : kPi - tmp;
    float phi = atan2f(l.y, l.x);
    if (phi < 0.f) phi += 2.f * kPi;
    si.u = phi * (0.5f / kPi);
    si.v = theta * (1.f / kPi);
    float rd = sqrtf(rd2), inv_rd = 1.f / rd;
    f3 dpdu = mk(-l.y, l.x, 0.f);
    f3 dpdv = mk(l.z * (l.x * inv_rd), l.z * (l.y * inv_rd), -rd);
    if (rd == 0.f) dpdv = mk(1.f, 0.f, 0.f);
    si.dp_du = dpdu * (s.radius * 2.f * kPi);
    si.dp_dv = dpdv * (s.radius * kPi);
    if (s.flip) n = -n;
    si.n = n;
    si.shn = n;
}

SMS_HD f3 ld3(const float *a, uint32_t i) {
    return mk(sms_ldg(a + 3 * i), sms_ldg(a + 3 * i + 1), sms_ldg(a + 3 * i + 2));
}

struct MeshTri {
    f3 p0, p1, p2, n0, n1, n2;
    float u0, v0, u1, v1, u2, v2;
};

SMS_HD void load_tri(const DevScene &sc, const DevShape &s, uint32_t f, MeshTri &m) {
    const uint32_t *F = sc.mesh_F + 3 * (size_t)(s.f_off + f);
    uint32_t i0 = s.v_off + sms_ldg(F), i1 = s.v_off + sms_ldg(F + 1), i2 = s.v_off + sms_ldg(F + 2);
    m.p0 = ld3(sc.mesh_P, i0); m.p1 = ld3(sc.mesh_P, i1); m.p2 = ld3(sc.mesh_P, i2);
    if (s.has_normals) {
        m.n0 = ld3(sc.mesh_N, i0); m.n1 = ld3(sc.mesh_N, i1); m.n2 = ld3(sc.mesh_N, i2);
    }
    if (s.has_uvs) {
        m.u0 = sms_ldg(sc.mesh_UV + 2 * i0); m.v0 = sms_ldg(sc.mesh_UV + 2 * i0 + 1);
        m.u1 = sms_ldg(sc.mesh_UV + 2 * i1); m.v1 = sms_ldg(sc.mesh_UV + 2 * i1 + 1);
        m.u2 = sms_ldg(sc.mesh_UV + 2 * i2); m.v2 = sms_ldg(sc.mesh_UV + 2 * i2 + 1);
    } else {
        m.u0 = 0.f; m.v0 = 0.f; m.u1 = 1.f; m.v1 = 0.f; m.u2 = 0.f; m.v2 = 1.f;
    }
}

// mesh.cpp:618-687
SMS_HD void mesh_surface(const MeshTri &m, int has_normals, float b1, float b2,
                                             SurfPt &si) {
    float b0 = 1.f - b1 - b2;
    f3 dp0 = m.p1 - m.p0, dp1 = m.p2 - m.p0;
    si.p = m.p0 * b0 + m.p1 * b1 + m.p2 * b2;
    f3 n = normalize(cross(dp0, dp1));
    si.n = n;
    f3 dpdu, dpdv;
    si.u = m.u0 * b0 + m.u1 * b1 + m.u2 * b2;
    si.v = m.v0 * b0 + m.v1 * b1 + m.v2 * b2;
    float du0 = m.u1 - m.u0, dv0 = m.v1 - m.v0, du1 = m.u2 - m.u0, dv1 = m.v2 - m.v0;
    float dt = du0 * dv1 - dv0 * du1;
    if (dt != 0.f) {
        float inv = 1.f / dt;
        dpdu = (dp0 * dv1 - dp1 * dv0) * inv;
        dpdv = (dp1 * du0 - dp0 * du1) * inv;
    } else {
        onb(n, dpdu, dpdv);   // degenerate uv parameterization
    }
    if (has_normals) n = normalize(m.n0 * b0 + m.n1 * b1 + m.n2 * b2);
    si.shn = n;
    si.dp_du = dpdu;
    si.dp_dv = dpdv;
}

// mesh.cpp:693-765 (without vertex normals: flat, like the rectangle shape)
SMS_HD void mesh_dn(const MeshTri &m, int has_normals, f3 p, f3 &dndu, f3 &dndv) {
    if (!has_normals) { dndu = splat(0.f); dndv = splat(0.f); return; }
    f3 rel = p - m.p0, du = m.p1 - m.p0, dv = m.p2 - m.p0;
    float b1 = dot(du, rel), b2 = dot(dv, rel), a11 = dot(du, du), a12 = dot(du, dv), a22 = dot(dv, dv);
    float inv_det = 1.f / (a11 * a22 - a12 * a12);
    float u = (a22 * b1 - a12 * b2) * inv_det, v = (a11 * b2 - a12 * b1) * inv_det, w = 1.f - u - v;
    f3 N = m.n1 * u + m.n2 * v + m.n0 * w;
    float il = 1.f / sqrtf(dot(N, N));
    N = N * il;
    f3 a = (m.n1 - m.n0) * il, b = (m.n2 - m.n0) * il;
    a = a - N * dot(N, a);
    b = b - N * dot(N, b);
    float du1 = m.u1 - m.u0, dv1 = m.v1 - m.v0, du2 = m.u2 - m.u0, dv2 = m.v2 - m.v0;
    float id = 1.f / (du1 * dv2 - dv1 * du2);
    dndu = (a * dv2 - b * dv1) * id;
    dndv = (b * du1 - a * du2) * id;
}

// ------------------------------------------------------------ manifold vertex
// The fields the Newton step, the admissibility test and the contribution
// read.  The tangent frame (s, t and their derivatives) is rebuilt from n,
// dp_du and dn_du/dn_dv only where the half-vector constraint needs it.
struct Vtx {
    f3 p, dp_du, dp_dv, n, dn_du, dn_dv, gn;
    f3 n0;   // shading normal before the normal map (n where there is none)
    float eta;
    int shape;
};

// ManifoldVertex(si) (manifold.h:89-113) from a closest hit.
SMS_HD float2 nm_texel(const DevScene &sc, uint32_t idx) {
#ifdef __CUDA_ARCH__
    uint32_t bits = __ldg(sc.nmap + idx);
    __half2 h = *reinterpret_cast<__half2 *>(&bits);
    return __half22float2(h);
#else
    (void)sc; (void)idx;
    return make_float2(0.f, 0.f);
#endif
}

// Bilinear slope at level 0 after the tiling wrap (normalmap.cpp:305-316).
SMS_HD float2 nm_slope0(const DevScene &sc, float u_in, float v_in) {
    float u = u_in * sc.nmap_tiles, v = v_in * sc.nmap_tiles;
    u -= floorf(u);
    v -= floorf(v);
    const uint32_t R = sc.nmap_res;
    float res = (float)R, duv = 1.f / res;
    float px = fminf(fmaxf((u - 0.5f * duv) * res, 0.f), res - 1.f);
    float py = fminf(fmaxf((v - 0.5f * duv) * res, 0.f), res - 1.f);
    uint32_t x0 = (uint32_t)floorf(px), y0 = (uint32_t)floorf(py);
    uint32_t x1 = min(x0 + 1, R - 1), y1 = min(y0 + 1, R - 1);
    x0 = min(x0, R - 1);
    y0 = min(y0, R - 1);
    float wx = px - (float)x0, wy = py - (float)y0;
    float2 t00 = nm_texel(sc, y0 * R + x0), t10 = nm_texel(sc, y0 * R + x1), t01 = nm_texel(sc, y1 * R + x0),
           t11 = nm_texel(sc, y1 * R + x1);
    float w0x = 1.f - wx, w0y = 1.f - wy;
    return make_float2(w0y * (w0x * t00.x + wx * t10.x) + wy * (w0x * t01.x + wx * t11.x),
                       w0y * (w0x * t00.y + wx * t10.y) + wy * (w0x * t01.y + wx * t11.y));
}

// Bilinear slope at level 0 and its uv derivative x res x tiles
// (normalmap.h:125-193 with the tiling scale of normalmap.cpp:270-273).
SMS_HD float2 nm_slope0_d(const DevScene &sc, float u_in, float v_in, float2 &du, float2 &dv) {
    float u = u_in * sc.nmap_tiles, v = v_in * sc.nmap_tiles;
    u -= floorf(u);
    v -= floorf(v);
    const uint32_t R = sc.nmap_res;
    float res = (float)R, duv = 1.f / res;
    float px = fminf(fmaxf((u - 0.5f * duv) * res, 0.f), res - 1.f);
    float py = fminf(fmaxf((v - 0.5f * duv) * res, 0.f), res - 1.f);
    uint32_t x0 = (uint32_t)floorf(px), y0 = (uint32_t)floorf(py);
    uint32_t x1 = min(x0 + 1, R - 1), y1 = min(y0 + 1, R - 1);
    x0 = min(x0, R - 1);
    y0 = min(y0, R - 1);
    float wx = px - (float)x0, wy = py - (float)y0;
    float2 t00 = nm_texel(sc, y0 * R + x0), t10 = nm_texel(sc, y0 * R + x1), t01 = nm_texel(sc, y1 * R + x0),
           t11 = nm_texel(sc, y1 * R + x1);
    float w0x = 1.f - wx, w0y = 1.f - wy;
    float tmpx = t01.x + t10.x - t11.x, tmpy = t01.y + t10.y - t11.y;
    du = make_float2((t10.x + t00.x * (wy - 1.f) - tmpx * wy) * res * sc.nmap_tiles,
                     (t10.y + t00.y * (wy - 1.f) - tmpy * wy) * res * sc.nmap_tiles);
    dv = make_float2((t01.x + t00.x * (wx - 1.f) - tmpx * wx) * res * sc.nmap_tiles,
                     (t01.y + t00.y * (wx - 1.f) - tmpy * wx) * res * sc.nmap_tiles);
    return make_float2(w0y * (w0x * t00.x + wx * t10.x) + wy * (w0x * t01.x + wx * t11.x),
                       w0y * (w0x * t00.y + wx * t10.y) + wy * (w0x * t01.y + wx * t11.y));
}

// Mean slope and covariance of the whole map: the top level of the LEAN
// pyramid (the lookup of a surface point without uv partials,
// normalmap.cpp:374-377, as the two-stage solver's lean() call makes it).
SMS_HD void nm_top_lean(const DevScene &sc, float &mx, float &my, float &sa, float &sb, float &scv) {
    const float *t = sc.lean + sc.lean_off[sc.lean_levels - 1];
    mx = t[0];
    my = t[1];
    sa = fmaxf(0.f, t[2] - t[0] * t[0]);
    sb = fmaxf(0.f, t[3] - t[1] * t[1]);
    scv = fmaxf(0.f, t[4] - t[0] * t[1]);
}

// ManifoldVertex frame of a normal-mapped shape (NormalmapBSDF::frame /
// frame_derivative, normalmap.cpp:236-290): the base shading frame (n0,
// tangent from dp_du) and its derivative (frame.h:197-240) applied to the
// slope normal (-s_x, -s_y, 1) and its uv derivative.  coarse: the two-stage
// solver's smoothing = 1, i.e. the top LEAN level (mean slope, no derivative).
SMS_HD void nm_vertex_frame(const DevScene &sc, f3 p, f3 dp_du, f3 n0, f3 dn0_du, f3 dn0_dv, float u, float v,
                            bool coarse, f3 &n, f3 &dn_du, f3 &dn_dv) {
    (void)p;
    f3 s0 = dp_du - n0 * dot(n0, dp_du);
    const float inv_len = 1.f / length(s0);
    s0 = s0 * inv_len;
    const f3 t0 = cross(n0, s0);
    f3 ds_du = (-dn0_du * dot(n0, dp_du) - n0 * dot(dn0_du, dp_du)) * inv_len;
    f3 ds_dv = (-dn0_dv * dot(n0, dp_du) - n0 * dot(dn0_dv, dp_du)) * inv_len;
    ds_du = ds_du - s0 * dot(ds_du, s0);
    ds_dv = ds_dv - s0 * dot(ds_dv, s0);
    const f3 dt_du = cross(dn0_du, s0) + cross(n0, ds_du), dt_dv = cross(dn0_dv, s0) + cross(n0, ds_dv);
    f3 nl, dl_du, dl_dv;
    if (coarse) {
        float mx, my, sa, sb, scv;
        nm_top_lean(sc, mx, my, sa, sb, scv);
        nl = mk(-mx, -my, 1.f);
        dl_du = splat(0.f);
        dl_dv = splat(0.f);
    } else {
        float2 du, dv;
        const float2 sl = nm_slope0_d(sc, u, v, du, dv);
        nl = mk(-sl.x, -sl.y, 1.f);
        dl_du = mk(-du.x, -du.y, 0.f);
        dl_dv = mk(-dv.x, -dv.y, 0.f);
    }
    f3 wn = s0 * nl.x + t0 * nl.y + n0 * nl.z;
    const float il = 1.f / length(wn);
    wn = wn * il;
    f3 a = (s0 * dl_du.x + t0 * dl_du.y + n0 * dl_du.z + ds_du * nl.x + dt_du * nl.y + dn0_du * nl.z) * il;
    f3 b = (s0 * dl_dv.x + t0 * dl_dv.y + n0 * dl_dv.z + ds_dv * nl.x + dt_dv * nl.y + dn0_dv * nl.z) * il;
    n = wn;
    dn_du = a - wn * dot(a, wn);
    dn_dv = b - wn * dot(b, wn);
}

// kNM: apply the scene's normal map where the shape carries it (false: the
// caller knows no normal-mapped shape is involved, and the check is compiled
// away); nm_coarse: the two-stage solver's smoothed frame.
template <bool kNM = true>
SMS_HD void vertex_from_hit(const DevScene &sc, f3 o, f3 d, const Hit &h, Vtx &v,
                                                SurfPt *si_out = nullptr, bool nm_coarse = false) {
    const DevShape &s = sc.shapes[h.shape];
    SurfPt si;
    f3 dndu, dndv;
    if (s.kind == kShapeSphere) {
        sphere_surface(s, o, d, h.t, si);
        float inv_r = (s.flip ? -1.f : 1.f) / s.radius;
        dndu = si.dp_du * inv_r;
        dndv = si.dp_dv * inv_r;
    } else {
        MeshTri m;
        load_tri(sc, s, h.prim, m);
        mesh_surface(m, s.has_normals, h.u, h.v, si);
        mesh_dn(m, s.has_normals, si.p, dndu, dndv);
    }
    v.p = si.p; v.dp_du = si.dp_du; v.dp_dv = si.dp_dv;
    v.n = si.shn; v.gn = si.n; v.dn_du = dndu; v.dn_dv = dndv;
    v.n0 = si.shn;
    if (kNM && h.shape == sc.nmap_shape && sc.nmap_res > 0 && s.nmap_frames)
        nm_vertex_frame(sc, si.p, si.dp_du, si.shn, dndu, dndv, si.u, si.v, nm_coarse, v.n, v.dn_du, v.dn_dv);
    v.eta = s.spec_eta;
    v.shape = h.shape;
    if (dot(v.n, v.gn) < 0.f) v.gn = -v.gn;
    if (si_out) *si_out = si;
}

// manifold.h:115-126
SMS_HD void make_orthonormal(f3 &dp_du, f3 &dp_dv, f3 &dn_du, f3 &dn_dv) {
    float inv = 1.f / length(dp_du);
    dp_du = dp_du * inv; dn_du = dn_du * inv;
    float dp = dot(dp_du, dp_dv);
    f3 a = dp_dv - dp_du * dp, b = dn_dv - dn_du * dp;
    inv = 1.f / length(a);
    dp_dv = a * inv; dn_dv = b * inv;
}

// ------------------------------------------------------ specular transforms
SMS_HD void d_reflect(f3 w, f3 dwdu, f3 dwdv, f3 n, f3 dndu, f3 dndv, f3 &ou, f3 &ov) {
    float dwn = dot(w, n);
    ou = (n * (dot(dwdu, n) + dot(w, dndu)) + dndu * dwn) * 2.f - dwdu;
    ov = (n * (dot(dwdv, n) + dot(w, dndv)) + dndv * dwn) * 2.f - dwdv;
}

SMS_HD bool refract(f3 w, f3 n, float eta_, f3 &out) {
    float eta = 1.f / eta_;
    if (dot(w, n) < 0.f) { eta = 1.f / eta; n = -n; }
    float dwn = dot(w, n);
    float root = 1.f - eta * eta * (1.f - dwn * dwn);
    if (root < 0.f) return false;
    out = -(w - n * dwn) * eta - n * sqrtf(root);
    return true;
}

SMS_HD void d_refract(f3 w, f3 dwdu, f3 dwdv, f3 n, f3 dndu, f3 dndv, float eta_,
                                          f3 &ou, f3 &ov) {
    float eta = 1.f / eta_;
    if (dot(w, n) < 0.f) { eta = 1.f / eta; n = -n; dndu = -dndu; dndv = -dndv; }
    float dwn = dot(w, n);
    float root = sqrtf(1.f - eta * eta * (1.f - dwn * dwn));
    float su = dot(dwdu, n) + dot(w, dndu), sv = dot(dwdv, n) + dot(w, dndv);
    float k = 1.f / (2.f * root);
    f3 au = -(dwdu - (n * su + dndu * dwn)) * eta;
    f3 bu = -(dndu * root + n * k * (-eta * eta * (-2.f * dwn * su)));
    f3 av = -(dwdv - (n * sv + dndv * dwn)) * eta;
    f3 bv = -(dndv * root + n * k * (-eta * eta * (-2.f * dwn * sv)));
    ou = au + bu;
    ov = av + bv;
}

SMS_HD void sphcoords(f3 w, float &theta, float &phi) {
    theta = acosf(clamp1(w.z));
    phi = atan2f(w.y, w.x);
    if (phi < 0.f) phi += 2.f * kPi;
}

SMS_HD void d_sphcoords(f3 w, f3 du, f3 dv, float &dtu, float &dpu, float &dtv,
                                            float &dpv) {
    float d_acos = -1.f / safe_sqrt(1.f - w.z * w.z);
    dtu = d_acos * du.z;
    dtv = d_acos * dv.z;
    float yx = w.y / w.x;
    float d_atan = 1.f / (1.f + yx * yx);
    float inv = 1.f / (w.x * w.x);
    dpu = d_atan * (w.x * du.y - w.y * du.x) * inv;
    dpv = d_atan * (w.x * dv.y - w.y * dv.x) * inv;
    if (w.x == 0.f) { dpu = 0.f; dpv = 0.f; }
}

// Angle-difference constraint and Newton step (manifold_ss.cpp:494-636) with
// n_offset = (0, 0, 1).  Returns false when the step is invalid.
SMS_HD void frame_and_derivative(const Vtx &v, f3 &s, f3 &t, f3 &dsdu, f3 &dsdv, f3 &dtdu, f3 &dtdv);

// Angle-difference constraint and Newton step (manifold_ss.cpp:494-636).  `no`
// is the offset normal in the shading frame (manifold_ss.cpp:560-569): the
// specular transform uses m = s no.x + t no.y + n no.z and its derivatives;
// (0, 0, 1) leaves n untouched.
SMS_HD bool step_anglediff(f3 x, const Vtx &v, f3 lp, float &c0, float &c1,
                                               float &dx0, float &dx1, f3 no = f3{0.f, 0.f, 1.f}) {
    f3 wi = x - v.p;
    float ili = length(wi);
    if (ili < 1e-3f) return false;
    ili = 1.f / ili; wi = wi * ili;
    f3 wo = lp - v.p;
    float ilo = length(wo);
    if (ilo < 1e-3f) return false;
    ilo = 1.f / ilo; wo = wo * ilo;
    f3 dwi_du = (v.dp_du - wi * dot(wi, v.dp_du)) * -ili;
    f3 dwi_dv = (v.dp_dv - wi * dot(wi, v.dp_dv)) * -ili;
    f3 dwo_du = (v.dp_du - wo * dot(wo, v.dp_du)) * -ilo;
    f3 dwo_dv = (v.dp_dv - wo * dot(wo, v.dp_dv)) * -ilo;
    const bool refl = v.eta == 1.f;
    f3 nn = v.n, nn_du = v.dn_du, nn_dv = v.dn_dv;
    if (no.x != 0.f || no.y != 0.f) {
        f3 fs, ft, fsdu, fsdv, ftdu, ftdv;
        frame_and_derivative(v, fs, ft, fsdu, fsdv, ftdu, ftdv);
        nn = fs * no.x + ft * no.y + v.n * no.z;
        nn_du = fsdu * no.x + ftdu * no.y + v.dn_du * no.z;
        nn_dv = fsdv * no.x + ftdv * no.y + v.dn_dv * no.z;
    }
    // Try the transform of wi first, then of wo (manifold_ss.cpp:573-624).
    f3 a = wi, a_du = dwi_du, a_dv = dwi_dv;   // transformed
    f3 b = wo, b_du = dwo_du, b_dv = dwo_dv;   // compared against
    bool ok = false;
    f3 t;
    #pragma unroll 1
    for (int pass = 0; pass < 2 && !ok; ++pass) {
        if (pass == 1) {
            a = wo; a_du = dwo_du; a_dv = dwo_dv;
            b = wi; b_du = dwi_du; b_dv = dwi_dv;
        }
        if (refl) {
            t = nn * (2.f * dot(a, nn)) - a;
            ok = true;
        } else {
            ok = refract(a, nn, v.eta, t);
        }
    }
    if (!ok) return false;
    f3 t_du, t_dv;
    if (refl) d_reflect(a, a_du, a_dv, nn, nn_du, nn_dv, t_du, t_dv);
    else d_refract(a, a_du, a_dv, nn, nn_du, nn_dv, v.eta, t_du, t_dv);
    float tb, pb, tt, pt;
    sphcoords(b, tb, pb);
    sphcoords(t, tt, pt);
    float dt = tb - tt, dp = pb - pt;
    if (dp < -kPi) dp += 2.f * kPi; else if (dp > kPi) dp -= 2.f * kPi;
    c0 = dt; c1 = dp;
    float bu0, bu1, bv0, bv1, tu0, tu1, tv0, tv1;
    d_sphcoords(b, b_du, b_dv, bu0, bu1, bv0, bv1);
    d_sphcoords(t, t_du, t_dv, tu0, tu1, tv0, tv1);
    M2 J{bu0 - tu0, bv0 - tv0, bu1 - tu1, bv1 - tv1};
    float dj = det2(J);
    if (fabsf(dj) < 1e-6f) return false;
    float id = 1.f / dj;
    // inverse(J) * C
    dx0 = (J.d * id) * c0 + (-J.b * id) * c1;
    dx1 = (-J.c * id) * c0 + (J.a * id) * c1;
    return true;
}

// Shading frame and its derivative (frame.h:197-240).
SMS_HD void frame_and_derivative(const Vtx &v, f3 &s, f3 &t, f3 &dsdu, f3 &dsdv,
                                                     f3 &dtdu, f3 &dtdv) {
    f3 n = v.n;
    f3 s0 = v.dp_du - n * dot(n, v.dp_du);
    float inv_len = 1.f / length(s0);
    s0 = s0 * inv_len;
    s = s0;
    t = cross(n, s0);
    f3 a = (-v.dn_du * dot(n, v.dp_du) - n * dot(v.dn_du, v.dp_du)) * inv_len;
    f3 b = (-v.dn_dv * dot(n, v.dp_du) - n * dot(v.dn_dv, v.dp_du)) * inv_len;
    a = a - s0 * dot(a, s0);
    b = b - s0 * dot(b, s0);
    dsdu = a; dsdv = b;
    dtdu = cross(v.dn_du, s0) + cross(n, a);
    dtdv = cross(v.dn_dv, s0) + cross(n, b);
}

// Half-vector constraint and Newton step (manifold_ss.cpp:407-492).
// `no`: offset normal; the constraint is H_st - no_xy (manifold_ss.cpp:485-488).
SMS_HD bool step_halfvector(f3 x, const Vtx &v, f3 lp, float &c0, float &c1,
                                                float &dx0, float &dx1, f3 no = f3{0.f, 0.f, 1.f}) {
    f3 wo = lp - v.p;
    float ilo = length(wo);
    if (ilo < 1e-3f) return false;
    ilo = 1.f / ilo; wo = wo * ilo;
    f3 wi = x - v.p;
    float ili = length(wi);
    if (ili < 1e-3f) return false;
    ili = 1.f / ili; wi = wi * ili;
    float eta = v.eta;
    if (dot(wi, v.gn) < 0.f) eta = 1.f / eta;
    f3 h = wi + wo * eta;
    if (eta != 1.f) h = h * -1.f;
    float ilh = 1.f / length(h);
    h = h * ilh;
    ilo *= eta * ilh;
    ili *= ilh;
    f3 dh_du = -v.dp_du * (ili + ilo) + wi * (dot(wi, v.dp_du) * ili) + wo * (dot(wo, v.dp_du) * ilo);
    f3 dh_dv = -v.dp_dv * (ili + ilo) + wi * (dot(wi, v.dp_dv) * ili) + wo * (dot(wo, v.dp_dv) * ilo);
    dh_du = dh_du - h * dot(dh_du, h);
    dh_dv = dh_dv - h * dot(dh_dv, h);
    if (eta != 1.f) { dh_du = dh_du * -1.f; dh_dv = dh_dv * -1.f; }
    f3 s, t, dsdu, dsdv, dtdu, dtdv;
    frame_and_derivative(v, s, t, dsdu, dsdv, dtdu, dtdv);
    M2 J{dot(dsdu, h) + dot(s, dh_du), dot(dsdv, h) + dot(s, dh_dv),
         dot(dtdu, h) + dot(t, dh_du), dot(dtdv, h) + dot(t, dh_dv)};
    float dj = det2(J);
    if (fabsf(dj) < 1e-6f) return false;
    c0 = dot(s, h) - no.x; c1 = dot(t, h) - no.y;
    float id = 1.f / dj;
    dx0 = (J.d * id) * c0 + (-J.b * id) * c1;
    dx1 = (-J.c * id) * c0 + (J.a * id) * c1;
    return true;
}

// ---------------------------------------------------------------- Fresnel
SMS_HD float fresnel_dielectric(float cos_i, float eta) {
    bool outside = cos_i >= 0.f;
    float rcp_eta = 1.f / eta;
    float eta_it = outside ? eta : rcp_eta, eta_ti = outside ? rcp_eta : eta;
    float ct2 = 1.f - (1.f - cos_i * cos_i) * (eta_ti * eta_ti);
    float ci = fabsf(cos_i), ct = safe_sqrt(ct2);
    float a_s = (ci - eta_it * ct) / (ci + eta_it * ct);
    float a_p = (ct - eta_it * ci) / (ct + eta_it * ci);
    float r = 0.5f * (a_s * a_s + a_p * a_p);
    if (eta == 1.f) r = 0.f;
    else if (ci == 0.f) r = 1.f;
    return r;
}

SMS_HD float fresnel_conductor(float cos_i, float er, float ek) {
    float c2 = cos_i * cos_i, s2 = 1.f - c2, s4 = s2 * s2;
    float t1 = er * er - ek * ek - s2;
    float a2pb2 = safe_sqrt(t1 * t1 + 4.f * ek * ek * er * er);
    float a = safe_sqrt(0.5f * (a2pb2 + t1));
    float term1 = a2pb2 + c2, term2 = 2.f * cos_i * a;
    float rs = (term1 - term2) / (term1 + term2);
    float term3 = a2pb2 * c2 + s4, term4 = term2 * s2;
    float rp = rs * (term3 - term4) / (term3 + term4);
    return 0.5f * (rs + rp);
}

// ------------------------------------------------- Beckmann microfacets
// Isotropic Beckmann distribution (include/mitsuba/render/microfacet.h): D(m)
// with the same underflow cut-off, Smith's G1 through Walter et al. 2007's
// rational approximation (eq. 27 of "Microfacet Models for Refraction through
// Rough Surfaces"), and sampling of m with density D(m) cos(theta_m).
SMS_HD float beckmann_D(f3 m, float alpha) {
    float c2 = m.z * m.z;
    float r = expf(-((m.x * m.x + m.y * m.y) / (alpha * alpha)) / c2) / (kPi * alpha * alpha * c2 * c2);
    return r * m.z > 1e-20f ? r : 0.f;
}

SMS_HD float beckmann_G1(f3 v, f3 m, float alpha) {
    float xy = alpha * alpha * (v.x * v.x + v.y * v.y);
    float r;
    if (xy == 0.f) {
        r = 1.f;
    } else {
        float a = 1.f / sqrtf(xy / (v.z * v.z)), a2 = a * a;
        r = a >= 1.6f ? 1.f : (3.535f * a + 2.181f * a2) / (1.f + 2.276f * a + 2.577f * a2);
    }
    return dot(v, m) * v.z <= 0.f ? 0.f : r;
}

SMS_HD f3 beckmann_sample(float alpha, float u0, float u1, float &pdf) {
    float sp, cp;
#ifdef __CUDA_ARCH__
    sincosf(2.f * kPi * u1, &sp, &cp);
#else
    sp = std::sin(2.f * kPi * u1); cp = std::cos(2.f * kPi * u1);
#endif
    float ct = 1.f / sqrtf(1.f - alpha * alpha * logf(1.f - u0));
    float c2 = ct * ct;
    pdf = (1.f - u0) / (kPi * alpha * alpha * fmaxf(c2 * ct, 1e-20f));
    float st = sqrtf(1.f - c2);
    return mk(cp * st, sp * st, ct);
}

// Rough conductor BSDF value times cos(theta_o) (roughconductor.cpp eval), local frame.
SMS_HD float roughconductor_eval(float alpha, float er, float ek, f3 wi, f3 wo) {
    if (!(wi.z > 0.f && wo.z > 0.f)) return 0.f;
    f3 h = normalize(wo + wi);
    float D = beckmann_D(h, alpha);
    if (D == 0.f) return 0.f;
    float G = beckmann_G1(wi, h, alpha) * beckmann_G1(wo, h, alpha);
    return D * G / (4.f * wi.z) * fresnel_conductor(dot(wi, h), er, ek);
}

// Rough dielectric BSDF value times |cos(theta_o)| (roughdielectric.cpp eval,
// radiance transport), local frame.
SMS_HD float roughdielectric_eval(float alpha, float eta_, f3 wi, f3 wo) {
    const float ci = wi.z, co = wo.z;
    if (ci == 0.f) return 0.f;
    const bool reflect = ci * co > 0.f;
    const float eta = ci > 0.f ? eta_ : 1.f / eta_, inv_eta = ci > 0.f ? 1.f / eta_ : eta_;
    f3 m = normalize(wi + wo * (reflect ? 1.f : eta));
    if (m.z < 0.f) m = -m;
    float D = beckmann_D(m, alpha);
    float F = fresnel_dielectric(dot(wi, m), eta_);
    float G = beckmann_G1(wi, m, alpha) * beckmann_G1(wo, m, alpha);
    if (reflect) return F * D * G / (4.f * fabsf(ci));
    float den = dot(wi, m) + eta * dot(wo, m);
    return fabsf((inv_eta * inv_eta) * (1.f - F) * D * G * eta * eta * dot(wi, m) * dot(wo, m) /
                 (ci * den * den));
}

// specular_reflectance for smooth BSDFs (manifold_ss.cpp:638-693).
SMS_HD float specular_reflectance(const DevShape &s, f3 shn, f3 wo) {
    float cos_t = dot(shn, wo);
    if (s.bsdf_type == kBsdfConductor && s.k != 0.f) return fresnel_conductor(fabsf(cos_t), s.eta, s.k);
    if (s.bsdf_type == kBsdfDielectric || s.bsdf_type == kBsdfConductor) {
        float eta = s.eta;
        if (cos_t < 0.f) eta = 1.f / eta;
        return (1.f - fresnel_dielectric(cos_t, eta)) * eta * eta;
    }
    return fresnel_conductor(fabsf(cos_t), 0.f, 1.f);
}

// specular_reflectance of a rough BSDF (manifold_ss.cpp:648-669): the BSDF
// value for wi (toward the shading point) and wo (toward the light) in the
// shading frame (n, tangent from dp_du), turned into the half-vector domain.
// nm: the shape carries the normal map, n is its perturbed normal and n0 the
// shading normal under it -- NormalmapBSDF::eval (normalmap.cpp:172-181)
// evaluates the nested BSDF in the perturbed frame and keeps wo only on the
// same side of both normals, while the half-vector factor flips eta by the
// side of wi in the unperturbed frame.
SMS_HD float specular_reflectance_rough(const DevShape &s, f3 n, f3 dp_du, f3 wi_w, f3 wo_w, f3 n0 = f3{0.f, 0.f, 0.f},
                                        bool nm = false) {
    f3 fs = dp_du - n * dot(n, dp_du);
    fs = normalize(fs);
    f3 ft = cross(n, fs);
    f3 wi = mk(dot(wi_w, fs), dot(wi_w, ft), dot(wi_w, n));
    f3 wo = mk(dot(wo_w, fs), dot(wo_w, ft), dot(wo_w, n));
    if (nm && !(dot(wo_w, n0) * wo.z > 0.f)) return 0.f;
    const bool complex_ior = s.bsdf_type == kBsdfConductor && s.k != 0.f;
    if (complex_ior) {
        float f = roughconductor_eval(s.alpha, s.eta, s.k, wi, wo);
        f3 h = normalize(wi + wo);
        return f * 4.f * fabsf(dot(wo, h));
    }
    float f = s.bsdf_type == kBsdfConductor ? roughconductor_eval(s.alpha, s.eta, s.k, wi, wo)
                                            : roughdielectric_eval(s.alpha, s.eta, wi, wo);
    float eta = s.eta;
    if ((nm ? dot(wi_w, n0) : wi.z) < 0.f) eta = 1.f / eta;
    f3 h = -normalize(wi + wo * eta);
    float a = dot(wi, h) + eta * dot(wo, h);
    return f * a * a / (eta * eta * fabsf(dot(wo, h)));
}

// Generalized geometric term for a positional endpoint (manifold_ss.cpp:695-857,
// the !fixed_direction branch).  v0: shading point (orthonormal, flat),
// v1: specular vertex (orthonormal), v2: emitter vertex (orthonormal).
SMS_HD float geometric_term(f3 x, const Vtx &v1, f3 yp, f3 y_du, f3 y_dv) {
    f3 wi = x - v1.p;
    float ili = length(wi);
    if (ili < 1e-3f) return 0.f;
    ili = 1.f / ili; wi = wi * ili;
    f3 wo = yp - v1.p;
    float ilo = length(wo);
    if (ilo < 1e-3f) return 0.f;
    ilo = 1.f / ilo; wo = wo * ilo;
    float eta = v1.eta;
    if (dot(wi, v1.gn) < 0.f) eta = 1.f / eta;
    f3 h = wi + wo * eta;
    if (eta != 1.f) h = h * -1.f;
    float ilh = 1.f / length(h);
    h = h * ilh;
    ilo *= eta * ilh;
    ili *= ilh;
    float dpdu_n = dot(v1.dp_du, v1.n), dpdv_n = dot(v1.dp_dv, v1.n);
    f3 s = v1.dp_du - v1.n * dpdu_n, t = v1.dp_dv - v1.n * dpdv_n;
    f3 dh_du = -v1.dp_du * (ili + ilo) + wi * (dot(wi, v1.dp_du) * ili) + wo * (dot(wo, v1.dp_du) * ilo);
    f3 dh_dv = -v1.dp_dv * (ili + ilo) + wi * (dot(wi, v1.dp_dv) * ili) + wo * (dot(wo, v1.dp_dv) * ilo);
    dh_du = dh_du - h * dot(dh_du, h);
    dh_dv = dh_dv - h * dot(dh_dv, h);
    if (eta != 1.f) { dh_du = dh_du * -1.f; dh_dv = dh_dv * -1.f; }
    float hn = dot(h, v1.n), hdu = dot(h, v1.dn_du), hdv = dot(h, v1.dn_dv);
    M2 A{dot(dh_du, s) - dot(v1.dp_du, v1.dn_du) * hn - dpdu_n * hdu,
         dot(dh_dv, s) - dot(v1.dp_du, v1.dn_dv) * hn - dpdu_n * hdv,
         dot(dh_du, t) - dot(v1.dp_dv, v1.dn_du) * hn - dpdv_n * hdu,
         dot(dh_dv, t) - dot(v1.dp_dv, v1.dn_dv) * hn - dpdv_n * hdv};
    dh_du = (y_du - wo * dot(wo, y_du)) * ilo;
    dh_dv = (y_dv - wo * dot(wo, y_dv)) * ilo;
    dh_du = dh_du - h * dot(dh_du, h);
    dh_dv = dh_dv - h * dot(dh_dv, h);
    if (eta != 1.f) { dh_du = dh_du * -1.f; dh_dv = dh_dv * -1.f; }
    M2 B{dot(dh_du, s), dot(dh_dv, s), dot(dh_du, t), dot(dh_dv, t)};
    float dA = det2(A);
    if (fabsf(dA) < 1e-6f) return 0.f;
    float id = 1.f / dA;
    M2 Ai{A.d * id, -A.b * id, -A.c * id, A.a * id};
    M2 P{Ai.a * B.a + Ai.b * B.c, Ai.a * B.b + Ai.b * B.d, Ai.c * B.a + Ai.d * B.c, Ai.c * B.b + Ai.d * B.d};
    float dx1_dx2 = fminf(fabsf(det2(P)), 1.f);
    f3 dd = x - v1.p;
    float inv_r2 = 1.f / dot(dd, dd);
    dd = dd * sqrtf(inv_r2);
    return fabsf(dot(dd, v1.gn)) * inv_r2 * dx1_dx2;
}

// Uniform point on a shape (sphere.cpp:153-170, mesh.cpp:541-586 with
// DiscreteDistribution::sample_reuse, distr_1d.h:144-201).
SMS_HD f3 sample_position(const DevScene &sc, const DevShape &s, float sx, float sy,
                                              f3 *n_out = nullptr) {
    if (s.kind == kShapeSphere) {
        float z = 1.f - 2.f * sy;
        float r = safe_sqrt(1.f - z * z);
        float sn, cs;
        sincosf(2.f * kPi * sx, &sn, &cs);
        f3 l = mk(r * cs, r * sn, z);
        if (n_out) *n_out = s.flip ? -l : l;
        return l * s.radius + mk(s.cx, s.cy, s.cz);
    }
    const float *cdf = sc.cdf + s.cdf_off;
    float value = sy * s.area_sum;
    uint32_t lo = s.valid_lo, hi = s.valid_hi;
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        if (sms_ldg(cdf + mid) < value) lo = mid + 1; else hi = mid;
    }
    uint32_t f = lo;
    float pmf = sms_ldg(sc.pmf + s.cdf_off + f) * s.area_norm;
    float cprev = f > 0 ? sms_ldg(cdf + f - 1) * s.area_norm : 0.f;
    float y = (sy - cprev) / pmf;
    float tq = safe_sqrt(1.f - sx);
    float bx = 1.f - tq, by = tq * y;
    MeshTri m;
    load_tri(sc, s, f, m);
    f3 e0 = m.p1 - m.p0, e1 = m.p2 - m.p0;
    if (n_out) {
        if (s.has_normals) *n_out = normalize(m.n0 * (1.f - bx - by) + m.n1 * bx + m.n2 * by);
        else *n_out = normalize(cross(e0, e1));
    }
    return m.p0 + e0 * bx + e1 * by;
}

// Counters shared by all kernels of a context (one record per context).
// Profiling phases (one per kernel family), after the reference's profiler
// phases SMSCaustics / SMSCausticsBernoulliTrials / SMSGlints
// (include/mitsuba/core/profiler.h:25-28).
enum : int { kPhaseSsFirst = 0, kPhaseSsTrials = 1, kPhaseSsBiased = 2, kPhaseSsWalk = 3, kPhaseMs = 4,
             kPhaseGlints = 5, kPhaseMsWalk = 6, kPhaseGlintWalk = 7, kPhases = 8 };

struct DevCounters {
    unsigned long long phase_rays[kPhases], phase_nodes[kPhases], phase_tris[kPhases];
    unsigned long long solver_succeeded, solver_failed, bernoulli_calls, bernoulli_iters,
        bernoulli_max, walks, newton_iters, connections, rays, bvh_nodes, tri_tests, speculative_walks;
    unsigned int trial_count;  // queries appended to the Bernoulli-trial queue
    unsigned int trial_head;   // next queue entry (must follow trial_count)
    unsigned int queue_head;   // general persistent-kernel work queue
    unsigned int error;
};

}  // namespace sms
