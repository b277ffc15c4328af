// 8-wide BVH built on the GPU (gpu_build.cu).
#pragma once

#include "renderer.h"

namespace pg {

struct GpuWideBVH {
  DeviceBuffer perm;      // [n] BVH order -> input triangle
  DeviceBuffer nodes;     // WideNode, n_nodes used
  DeviceBuffer wide_tris; // [n_wide_tris][12] floats: v0, e1, e2, BVH-order index bits
  uint32_t n_nodes = 0;
  uint32_t n_wide_tris = 0; // n, or more with split references
  uint32_t depth = 0;     // deepest wide node (root 0)
};

// t9: [n][9] world-space vertices (device); lo, hi: a box holding every
// triangle's centroid; split: triangles much smaller than their boxes are
// split into references first (spatial splits)
Status gpu_build_wide(const float *t9, uint32_t n, const float *lo, const float *hi, bool split,
                      cudaStream_t s, GpuWideBVH &out);

} // namespace pg
