// sms_bvh.h -- host-side BVH builder for the device traversal in sms_device.cuh.
//
// The reference ray-casts through a SAH kd-tree (include/mitsuba/render/
// kdtree.h); any exact closest-hit structure gives the same answers.  This one
// is a binned-SAH BVH2 flattened so that each 64-byte node holds both
// children's boxes (layout documented at DevScene in sms_device.cuh).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace sms {

struct BvhInputTri {
    float p0[3], p1[3], p2[3];
    int shape;
    int face;
};

struct BvhResult {
    std::vector<float4> nodes;   // 4 per node
    std::vector<float4> tris;    // 3 per triangle: (p0|shape) (e1|face) (e2|0)
    int max_depth = 0;
    int max_leaf = 0;
};

// Build over all triangles; false + err on failure.
bool build_bvh(const std::vector<BvhInputTri> &in, BvhResult &out, std::string &err);
// Structural check: child indices move forward, leaf ranges are in bounds.
bool validate_bvh(const BvhResult &bvh, std::string &err);

}  // namespace sms
