// Host BVH construction for the device traversal in trace.cuh.
#pragma once
#include <vector>
#include "common.cuh"

namespace drmlt {

// triP: per triangle p0, e1 = p1 - p0, e2 = p2 - p0 (9 floats). Produces the
// node array (root = node 0) and the triangles in leaf order.
void BuildBvh(const float *triP, const int *triShape, int numTris, std::vector<BvhNode> &nodes,
              std::vector<Tri> &tris);

}  // namespace drmlt
