// Host SBVH builder for the render path.
//
// Builds the reference's binary SBVH (src/intersect/accel/sbvh/detail/
// generator.cu:17-713): full-sort SAH object splits on each axis, optional
// binned spatial splits when the best object split's child overlap exceeds
// overlap_threshold of the root area, leaf when base_cost / area +
// traversal_per_intersect_cost >= n.  Subtrees are built in parallel with
// OpenMP tasks and then laid out in the reference's depth-first node order,
// so the node array, extra index array and permutation are identical to the
// reference's serial build.
#pragma once

#include "geom.h"

#include <vector>

namespace pg {

// bvh::Node (include/intersect/accel/detail/bvh/node.h:14-127): two 32-bit
// words with a tag in bit 31 of each, plus the box.  Split: w0 = left | tag,
// w1 = right.  Items: w0 = start, w1 = end | (is_for_extra ? tag : 0).
struct BinaryNode {
  uint32_t w0, w1;
  box aabb;
};

struct BinaryBVH {
  std::vector<BinaryNode> nodes;
  std::vector<uint32_t> extra_idxs;
  std::vector<uint32_t> permutation; // BVH position -> input index
  uint32_t max_leaf_size = 0;
  uint32_t depth = 0;
};

struct SBVHSettings {
  float overlap_threshold = 1e-5f;
  bool use_spatial_splits = false;
  float traversal_per_intersect_cost = 0.5f;
  uint32_t target_objects = 4;
};

constexpr uint32_t kNodeTag = 1u << 31;

BinaryBVH build_sbvh(const f3 *v0, const f3 *v1, const f3 *v2, size_t n,
                     const SBVHSettings &settings);

// ClippedTriangle::new_bounds (include/intersect/accel/detail/
// clipped_triangle_impl.h:13-124): box of the triangle clipped to the slab
// [left, right] on axis, within the current bounds
box clipped_bounds(f3 a, f3 b, f3 c, box bounds, float left, float right,
                   int axis);

} // namespace pg
