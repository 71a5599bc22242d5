// sms_bvh.cpp -- binned-SAH BVH2 builder (host).  See sms_bvh.h.
#include "sms_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace sms {
namespace {

struct Box {
    float lo[3], hi[3];
    Box() { for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; } }
    void grow(const Box &b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    void grow(const float *p) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    float area() const {
        float d[3];
        for (int k = 0; k < 3; ++k) d[k] = std::max(0.f, hi[k] - lo[k]);
        return 2.f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

struct TNode {
    Box box;
    int left = -1, right = -1;
    uint32_t first = 0, count = 0;
};

constexpr int kMaxLeaf = 2;
constexpr int kMaxDepth = 31;   // below the device traversal stack depth (32)
constexpr int kBins = 16;

struct Builder {
    std::vector<Box> boxes;
    std::vector<float> cen;
    std::vector<uint32_t> idx;
    std::vector<TNode> nodes;
    int max_depth = 0, max_leaf = 0;

    int build(uint32_t first, uint32_t count, int depth) {
        TNode node;
        Box cb;
        for (uint32_t i = first; i < first + count; ++i) {
            node.box.grow(boxes[idx[i]]);
            cb.grow(&cen[3 * idx[i]]);
        }
        int id = (int)nodes.size();
        nodes.push_back(node);
        max_depth = std::max(max_depth, depth);
        if ((int)count <= kMaxLeaf || depth >= kMaxDepth) {
            nodes[id].first = first;
            nodes[id].count = count;
            max_leaf = std::max(max_leaf, (int)count);
            return id;
        }
        float best_cost = INFINITY;
        int best_axis = -1, best_split = -1;
        for (int axis = 0; axis < 3; ++axis) {
            float ext = cb.hi[axis] - cb.lo[axis];
            if (!(ext > 0.f)) continue;
            Box bb[kBins];
            int bc[kBins] = {0};
            float scale = kBins / ext;
            for (uint32_t i = first; i < first + count; ++i) {
                int b = std::min(kBins - 1, (int)((cen[3 * idx[i] + axis] - cb.lo[axis]) * scale));
                bc[b]++;
                bb[b].grow(boxes[idx[i]]);
            }
            float la[kBins], ra[kBins];
            int lc[kBins], rc[kBins];
            Box acc;
            int c = 0;
            for (int b = 0; b < kBins; ++b) { acc.grow(bb[b]); c += bc[b]; la[b] = acc.area(); lc[b] = c; }
            acc = Box();
            c = 0;
            for (int b = kBins - 1; b >= 0; --b) { acc.grow(bb[b]); c += bc[b]; ra[b] = acc.area(); rc[b] = c; }
            for (int b = 0; b < kBins - 1; ++b) {
                if (lc[b] == 0 || rc[b + 1] == 0) continue;
                float cost = la[b] * lc[b] + ra[b + 1] * rc[b + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = axis; best_split = b; }
            }
        }
        uint32_t mid;
        if (best_axis < 0) {
            mid = first + count / 2;  // coincident centroids
        } else {
            float scale = kBins / (cb.hi[best_axis] - cb.lo[best_axis]);
            auto it = std::partition(idx.begin() + first, idx.begin() + first + count, [&](uint32_t p) {
                int b = std::min(kBins - 1, (int)((cen[3 * p + best_axis] - cb.lo[best_axis]) * scale));
                return b <= best_split;
            });
            mid = (uint32_t)(it - idx.begin());
            if (mid == first || mid == first + count) mid = first + count / 2;
        }
        int l = build(first, mid - first, depth + 1);
        int r = build(mid, first + count - mid, depth + 1);
        nodes[id].left = l;
        nodes[id].right = r;
        return id;
    }
};

// Pad so float rounding in the slab test never culls a triangle that the
// exact triangle test accepts.
void pad_box(Box &b) {
    for (int k = 0; k < 3; ++k) {
        float m = std::max(1.f, std::max(std::fabs(b.lo[k]), std::fabs(b.hi[k])));
        b.lo[k] -= 2e-6f * m;
        b.hi[k] += 2e-6f * m;
    }
}

float4 pack_ids(int a, int b, int c, int d) {
    int4 ids = make_int4(a, b, c, d);
    float4 f;
    std::memcpy(&f, &ids, 16);
    return f;
}

}  // namespace

bool build_bvh(const std::vector<BvhInputTri> &in, BvhResult &out, std::string &err) {
    out = BvhResult();
    if (in.empty()) { err = "no triangles"; return false; }
    Builder b;
    size_t n = in.size();
    b.boxes.resize(n);
    b.cen.resize(3 * n);
    b.idx.resize(n);
    for (size_t i = 0; i < n; ++i) {
        b.boxes[i].grow(in[i].p0);
        b.boxes[i].grow(in[i].p1);
        b.boxes[i].grow(in[i].p2);
        for (int k = 0; k < 3; ++k) {
            if (!std::isfinite(b.boxes[i].lo[k]) || !std::isfinite(b.boxes[i].hi[k])) {
                err = "non-finite vertex position";
                return false;
            }
            b.cen[3 * i + k] = 0.5f * (b.boxes[i].lo[k] + b.boxes[i].hi[k]);
        }
        b.idx[i] = (uint32_t)i;
    }
    b.build(0, (uint32_t)n, 0);
    out.max_depth = b.max_depth;
    out.max_leaf = b.max_leaf;
    // triangles in leaf order
    out.tris.resize(3 * n);
    for (size_t k = 0; k < n; ++k) {
        const BvhInputTri &t = in[b.idx[k]];
        float fs, ff;
        std::memcpy(&fs, &t.shape, 4);
        std::memcpy(&ff, &t.face, 4);
        out.tris[3 * k] = make_float4(t.p0[0], t.p0[1], t.p0[2], fs);
        out.tris[3 * k + 1] = make_float4(t.p1[0] - t.p0[0], t.p1[1] - t.p0[1], t.p1[2] - t.p0[2], ff);
        out.tris[3 * k + 2] = make_float4(t.p2[0] - t.p0[0], t.p2[1] - t.p0[1], t.p2[2] - t.p0[2], 0.f);
    }
    auto is_leaf = [&](int i) { return b.nodes[i].left < 0; };
    if (is_leaf(0)) {
        // single leaf: root with the leaf as left child and an empty right child
        Box L = b.nodes[0].box;
        pad_box(L);
        out.nodes.push_back(make_float4(L.lo[0], L.lo[1], L.lo[2], L.hi[0]));
        out.nodes.push_back(make_float4(L.hi[1], L.hi[2], 0.f, 0.f));
        out.nodes.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
        out.nodes.push_back(pack_ids((int)b.nodes[0].first, 0, (int)b.nodes[0].count, -1));
        return true;
    }
    // breadth-first numbering of inner nodes: children always after parents
    std::vector<int> queue{0}, out_id(b.nodes.size(), -1);
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        int i = queue[qi];
        out_id[i] = (int)qi;
        for (int ch : {b.nodes[i].left, b.nodes[i].right})
            if (!is_leaf(ch)) queue.push_back(ch);
    }
    out.nodes.resize(4 * queue.size());
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        const TNode &t = b.nodes[queue[qi]];
        Box L = b.nodes[t.left].box, R = b.nodes[t.right].box;
        pad_box(L);
        pad_box(R);
        int li, ri, lc, rc;
        if (is_leaf(t.left)) { li = (int)b.nodes[t.left].first; lc = (int)b.nodes[t.left].count; }
        else { li = out_id[t.left]; lc = 0; }
        if (is_leaf(t.right)) { ri = (int)b.nodes[t.right].first; rc = (int)b.nodes[t.right].count; }
        else { ri = out_id[t.right]; rc = 0; }
        out.nodes[4 * qi] = make_float4(L.lo[0], L.lo[1], L.lo[2], L.hi[0]);
        out.nodes[4 * qi + 1] = make_float4(L.hi[1], L.hi[2], R.lo[0], R.lo[1]);
        out.nodes[4 * qi + 2] = make_float4(R.lo[2], R.hi[0], R.hi[1], R.hi[2]);
        out.nodes[4 * qi + 3] = pack_ids(li, ri, lc, rc);
    }
    return true;
}

bool validate_bvh(const BvhResult &bvh, std::string &err) {
    size_t nn = bvh.nodes.size() / 4, nt = bvh.tris.size() / 3;
    for (size_t i = 0; i < nn; ++i) {
        int4 ids;
        std::memcpy(&ids, &bvh.nodes[4 * i + 3], 16);
        int ch[2] = {ids.x, ids.y}, cn[2] = {ids.z, ids.w};
        for (int k = 0; k < 2; ++k) {
            if (cn[k] < 0) continue;  // empty child
            if (cn[k] == 0) {
                if (ch[k] <= (int)i || (size_t)ch[k] >= nn) { err = "child index out of range"; return false; }
            } else if (ch[k] < 0 || (size_t)ch[k] + (size_t)cn[k] > nt) {
                err = "leaf range out of range";
                return false;
            }
        }
    }
    return true;
}

}  // namespace sms
