// Compressed 8-wide BVH built from the binary SBVH.
//
// Each wide node takes the children of a binary node and repeatedly opens the
// internal child with the largest surface area until it has eight children
// (or no internal child can be opened without exceeding 32 leaf triangles);
// this is the greedy collapse used for wide BVHs in Ylitie, Karras and Laine,
// "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs"
// (HPG 2017), whose 80-byte quantised node this layout follows.  Leaves keep
// the binary leaves' triangles (duplicates from spatial splits included), so
// the closest hit found through the wide BVH is the one the binary BVH finds,
// up to the order in which equal-distance candidates are met.
#pragma once

#include "devtypes.h"
#include "sbvh.h"

#include <vector>

namespace pg {

struct WideBVH {
  std::vector<WideNode> nodes;
  std::vector<uint32_t> tri_index; // wide-leaf slot -> BVH-order triangle
  uint32_t depth = 0;
};

WideBVH build_wide(const BinaryBVH &bvh);

// decoded child box of a wide node in float arithmetic (for tests)
box wide_child_box(const WideNode &n, int slot);

} // namespace pg
