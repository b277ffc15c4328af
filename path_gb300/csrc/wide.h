// Compressed 8-wide BVH built from the binary SBVH.
//
// The binary tree is collapsed by the surface-area cost optimisation of
// Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs
// Through Compressed Wide BVHs" (HPG 2017, section 3.1): bottom-up, the
// cheapest way to represent every binary subtree as a forest of at most i
// slots (i = 1..8) of its parent -- leaf slots of at most four triangles,
// a wide node of its own, or a split of the slots between its two children
// -- then top-down, every wide node takes the best forest of eight slots of
// its binary node's children.  The 80-byte quantised node follows the same
// paper.  Leaves keep the binary leaves' triangles (duplicates from spatial
// splits included), so the closest hit found through the wide BVH is the one
// the binary BVH finds, up to the order in which equal-distance candidates
// are met; a binary leaf of more than a node's 32 triangles continues in a
// child node with the same box.
#pragma once

#include "devtypes.h"
#include "sbvh.h"

#include <vector>

namespace pg {

// depth down to which the nodes are laid out breadth first (see build_wide)
constexpr uint32_t kBfsDepth = 3;

struct WideBVH {
  std::vector<WideNode> nodes;
  std::vector<uint32_t> tri_index; // wide-leaf slot -> BVH-order triangle
  uint32_t depth = 0;
  // nodes [0, n_top) are the nodes of depth <= kBfsDepth in breadth-first
  // order (root, its internal children, theirs, ...)
  uint32_t n_top = 0;
};

WideBVH build_wide(const BinaryBVH &bvh);

// decoded child box of a wide node in float arithmetic (for tests)
box wide_child_box(const WideNode &n, int slot);

} // namespace pg
