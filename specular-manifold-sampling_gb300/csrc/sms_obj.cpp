// sms_obj.cpp -- Wavefront OBJ reader for caster / receiver meshes (host).
//
// Restates the reference's OBJ shape plugin (src/shapes/obj.cpp:90-330):
//   * "v x y z", "vn x y z", "vt u v" (v flipped to 1 - v unless
//     flip_tex_coords is false, :188-199);
//   * "f" with v, v/vt, v//vn or v/vt/vn references (1-based, positive);
//     every distinct (v, vt, vn) triple becomes one output vertex, numbered
//     in order of first use (:206-256);
//   * polygons are fan-triangulated: (a, b, c), then (a, c, d), ... (:258-266);
//   * without "vn" lines (and face_normals off) vertex normals are recomputed
//     with the angle-weighted scheme of Thuermer and Wuethrich
//     (src/librender/mesh.cpp:420-470); face_normals drops vertex normals.
// Other statements (o, g, s, usemtl, mtllib, #, ...) are ignored.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sms_gb300.h"
#include "sms_kernels.h"

namespace {

struct Key {
    uint32_t v, t, n;
    bool operator==(const Key &o) const { return v == o.v && t == o.t && n == o.n; }
};
struct KeyHash {
    size_t operator()(const Key &k) const {
        return (size_t)k.v * 73856093u ^ (size_t)k.t * 19349663u ^ (size_t)k.n * 83492791u;
    }
};

sms_status obj_fail(const std::string &msg) { return (sms_status)set_last_error_impl((int)SMS_ERR_PARSE, msg.c_str()); }

// angle between unit vectors a and b, computed without acos near 0 / pi
// (the reference's unit_angle, include/mitsuba/core/vector.h:116-135)
float unit_angle(const float a[3], const float b[3]) {
    float d = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    if (d < 0.f) {
        float s[3] = {a[0] + b[0], a[1] + b[1], a[2] + b[2]};
        return (float)M_PI - 2.f * std::asin(std::fmin(1.f, 0.5f * std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2])));
    }
    float s[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    return 2.f * std::asin(std::fmin(1.f, 0.5f * std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2])));
}

void normalize3(float v[3]) {
    float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l > 0.f) { v[0] /= l; v[1] /= l; v[2] /= l; }
}

}  // namespace

extern "C" sms_status sms_obj_load(const char *path, int32_t face_normals, int32_t flip_tex_coords,
                                   sms_mesh_data *out) {
    if (!path || !out) return obj_fail("sms_obj_load: null argument");
    std::memset(out, 0, sizeof(*out));
    FILE *f = std::fopen(path, "rb");
    if (!f) return obj_fail(std::string("sms_obj_load: cannot open ") + path);
    std::vector<float> V, VN, VT;
    std::vector<uint32_t> F;
    std::vector<Key> keys;
    std::unordered_map<Key, uint32_t, KeyHash> ids;
    char buf[4096];
    size_t line_no = 0;
    sms_status st = SMS_OK;
    while (st == SMS_OK && std::fgets(buf, sizeof(buf), f)) {
        ++line_no;
        const char *c = buf;
        while (*c == ' ' || *c == '\t') ++c;
        auto floats = [&](const char *p, int n, std::vector<float> &dst) {
            for (int k = 0; k < n; ++k) {
                char *e;
                float x = std::strtof(p, &e);
                if (e == p) return false;
                dst.push_back(x);
                p = e;
            }
            return true;
        };
        if (c[0] == 'v' && (c[1] == ' ' || c[1] == '\t')) {
            if (!floats(c + 2, 3, V)) st = obj_fail("could not parse line " + std::to_string(line_no));
        } else if (c[0] == 'v' && c[1] == 'n' && (c[2] == ' ' || c[2] == '\t')) {
            if (!floats(c + 3, 3, VN)) st = obj_fail("could not parse line " + std::to_string(line_no));
        } else if (c[0] == 'v' && c[1] == 't' && (c[2] == ' ' || c[2] == '\t')) {
            if (!floats(c + 3, 2, VT)) st = obj_fail("could not parse line " + std::to_string(line_no));
            else if (flip_tex_coords) VT.back() = 1.f - VT.back();
        } else if (c[0] == 'f' && (c[1] == ' ' || c[1] == '\t')) {
            const char *p = c + 2;
            uint32_t poly[3] = {0, 0, 0};
            int nv = 0;
            while (true) {
                while (*p == ' ' || *p == '\t') ++p;
                if (*p == '\0' || *p == '\n' || *p == '\r') break;
                Key k{0, 0, 0};
                uint32_t *slot[3] = {&k.v, &k.t, &k.n};
                int ti = 0;
                char *e;
                unsigned long x = std::strtoul(p, &e, 10);
                if (e == p) { st = obj_fail("could not parse line " + std::to_string(line_no)); break; }
                *slot[0] = (uint32_t)x;
                p = e;
                while (*p == '/') {
                    ++ti;
                    ++p;
                    if (ti > 2) break;
                    x = std::strtoul(p, &e, 10);
                    if (e != p) { *slot[ti] = (uint32_t)x; p = e; }
                }
                if (ti > 2) { st = obj_fail("could not parse line " + std::to_string(line_no)); break; }
                if (k.v == 0 || (size_t)k.v > V.size() / 3) {
                    st = obj_fail("reference to invalid vertex " + std::to_string(k.v) + " on line " +
                                  std::to_string(line_no));
                    break;
                }
                if (k.t && (size_t)k.t > VT.size() / 2) {
                    st = obj_fail("reference to invalid texture coordinate " + std::to_string(k.t));
                    break;
                }
                if (k.n && (size_t)k.n > VN.size() / 3) {
                    st = obj_fail("reference to invalid normal " + std::to_string(k.n));
                    break;
                }
                auto it = ids.find(k);
                uint32_t id;
                if (it != ids.end()) {
                    id = it->second;
                } else {
                    id = (uint32_t)keys.size();
                    ids.emplace(k, id);
                    keys.push_back(k);
                }
                if (nv < 3) {
                    poly[nv] = id;
                } else {
                    poly[1] = poly[2];
                    poly[2] = id;
                }
                ++nv;
                if (nv >= 3) F.insert(F.end(), poly, poly + 3);
            }
        }
    }
    std::fclose(f);
    if (st != SMS_OK) return st;
    if (F.empty()) return obj_fail(std::string("sms_obj_load: no faces in ") + path);
    const uint32_t nv = (uint32_t)keys.size(), nf = (uint32_t)(F.size() / 3);
    bool has_uv = !VT.empty(), has_n = !face_normals;
    float *P = (float *)std::malloc(sizeof(float) * 3 * nv);
    float *N = has_n ? (float *)std::malloc(sizeof(float) * 3 * nv) : nullptr;
    float *UV = has_uv ? (float *)std::malloc(sizeof(float) * 2 * nv) : nullptr;
    uint32_t *FF = (uint32_t *)std::malloc(sizeof(uint32_t) * 3 * nf);
    if (!P || (has_n && !N) || (has_uv && !UV) || !FF) {
        std::free(P); std::free(N); std::free(UV); std::free(FF);
        return obj_fail("sms_obj_load: out of memory");
    }
    std::memcpy(FF, F.data(), sizeof(uint32_t) * 3 * nf);
    bool file_normals = !VN.empty();
    for (uint32_t i = 0; i < nv; ++i) {
        const Key &k = keys[i];
        for (int a = 0; a < 3; ++a) P[3 * i + a] = V[3 * (k.v - 1) + a];
        if (has_uv) {
            UV[2 * i] = k.t ? VT[2 * (k.t - 1)] : 0.f;
            UV[2 * i + 1] = k.t ? VT[2 * (k.t - 1) + 1] : 0.f;
        }
        if (has_n && file_normals)
            for (int a = 0; a < 3; ++a) N[3 * i + a] = k.n ? VN[3 * (k.n - 1) + a] : 0.f;
    }
    if (has_n && !file_normals) {
        // mesh.cpp:420-470: face normals weighted by the face angle at each
        // vertex, accumulated in float like the reference
        std::vector<float> acc(3 * (size_t)nv, 0.f);
        for (uint32_t t = 0; t < nf; ++t) {
            const float *v[3] = {&P[3 * FF[3 * t]], &P[3 * FF[3 * t + 1]], &P[3 * FF[3 * t + 2]]};
            float s0[3], s1[3], n[3];
            for (int a = 0; a < 3; ++a) { s0[a] = v[1][a] - v[0][a]; s1[a] = v[2][a] - v[0][a]; }
            n[0] = s0[1] * s1[2] - s0[2] * s1[1];
            n[1] = s0[2] * s1[0] - s0[0] * s1[2];
            n[2] = s0[0] * s1[1] - s0[1] * s1[0];
            float l2 = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
            if (!(l2 > 0.f)) continue;
            normalize3(n);
            for (int j = 0; j < 3; ++j) {
                float e1[3], e2[3];
                for (int a = 0; a < 3; ++a) {
                    e1[a] = v[(j + 1) % 3][a] - v[j][a];
                    e2[a] = v[(j + 2) % 3][a] - v[j][a];
                }
                normalize3(e1);
                normalize3(e2);
                float ang = unit_angle(e1, e2);
                for (int a = 0; a < 3; ++a) acc[3 * (size_t)FF[3 * t + j] + a] += n[a] * ang;
            }
        }
        for (uint32_t i = 0; i < nv; ++i) {
            float n[3] = {acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]};
            float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            if (l != 0.f) { n[0] /= l; n[1] /= l; n[2] /= l; }
            else { n[0] = 1.f; n[1] = 0.f; n[2] = 0.f; }
            for (int a = 0; a < 3; ++a) N[3 * i + a] = n[a];
        }
    }
    out->n_vertices = nv;
    out->n_faces = nf;
    out->positions = P;
    out->normals = N;
    out->texcoords = UV;
    out->faces = FF;
    return SMS_OK;
}

extern "C" void sms_mesh_data_free(sms_mesh_data *m) {
    if (!m) return;
    std::free(m->positions);
    std::free(m->normals);
    std::free(m->texcoords);
    std::free(m->faces);
    std::memset(m, 0, sizeof(*m));
}
