// Data layout of the render path in device memory.
//
//  * BVH-order triangles: 3 x float4 = 48 B, (v0.xyz, e1.x) (e1.yz, e2.xy)
//    (e2.z, -, -, -) with e1 = v1 - v0, e2 = v2 - v0 precomputed (the same
//    subtraction Triangle::intersect performs, so the bits are unchanged).
//  * shading data: 3 x float4 = 48 B, the three vertex normals and the
//    material index (scene::TriangleData, include/scene/triangle_data.h).
//  * binary SBVH nodes: 2 x uint4 = 32 B in the reference's node layout.
//  * compressed 8-wide nodes: 5 x uint4 = 80 B (layout below), children's
//    boxes quantised to 8 bits per plane relative to the node's origin with
//    a power-of-two scale per axis, rounded outward.
//  * wide-leaf triangles: 3 x float4 = 48 B with the BVH-order index in the
//    fourth lane of the last float4.
#pragma once

#include <stdint.h>

namespace pg {

// bsdf::UnionBSDF + emission (include/scene/material.h) with the values the
// reference's BSDF constructors precompute.
struct DevMaterial {
  uint32_t type;
  float diffuse[3];
  float specular[3];
  float shininess;
  float ior;
  float w_d;
  float w_g;
  float roughness;
  float emission[3];
  float glossy_norm;      // (shininess + 2) / (2 pi)      glossy.h:19-23
  float inv_shininess_p1; // 1 / (shininess + 1)
  float r0;               // ((ior - 1) / (ior + 1))^2     dielectric_refractive.h
  float cont_inclusive0;  // w_d / (w_d + w_g)              combined.h:22-47
  float pad[5];
};
static_assert(sizeof(DevMaterial) == 96, "DevMaterial is 96 bytes");

// 80-byte compressed wide node.
//   word 0-2 : origin p (float x3)
//   word 3   : exponent bytes ex, ey, ez (scale = 2^(e - 127)), imask
//   word 4   : child_base  (index of the first internal child)
//   word 5   : tri_base    (index of the first wide-leaf triangle)
//   word 6-7 : meta[8]: internal child -> rank among internal children;
//              leaf child -> (count << 5) | triangle offset; 0 -> empty
//   word 8-19: qlo_x[8] qlo_y[8] qlo_z[8] qhi_x[8] qhi_y[8] qhi_z[8]
struct WideNode {
  float p[3];
  uint8_t e[3];
  uint8_t imask;
  uint32_t child_base;
  uint32_t tri_base;
  uint8_t meta[8];
  uint8_t qlo[3][8];
  uint8_t qhi[3][8];
};
static_assert(sizeof(WideNode) == 80, "WideNode is 80 bytes");

constexpr uint32_t kMaxLeafTris = 7;      // 3-bit count in meta
constexpr uint32_t kMaxNodeTris = 32;     // 5-bit offset in meta
// node groups a wide traversal keeps waiting: at most one per tree level
constexpr uint32_t kWideStackDepth = 64;
// most top nodes the streaming trace kernel stages in shared memory (40 KB)
constexpr uint32_t kMaxStagedNodes = 512;

// Feature set of a path kernel, a template parameter: bit t allows BSDF
// type t (0 Diffuse, 1 Glossy, 2 DiffuseGlossy, 3 DiffuseMirror, 4 Mirror,
// 5 DielectricRefractive, 6 GGX), and the flag bits fix termination to
// NIters, direction sampling to the BSDF sampler and light sampling to
// RandomTriangle.  A kernel specialised to a scene's features carries none
// of the other code (the shade kernel's largest stall is instruction
// fetch); the host only launches a specialisation whose feature set covers
// the scene and the settings.
constexpr uint32_t kFeatAllMats = 0x7fu;
constexpr uint32_t kFeatNIters = 1u << 8;
constexpr uint32_t kFeatBsdfDir = 1u << 9;
constexpr uint32_t kFeatLightTri = 1u << 10;
constexpr uint32_t kFeatAll = kFeatAllMats; // every choice made at run time
// Diffuse, GGX and dielectric materials under NIters, the BSDF sampler and
// RandomTriangle: the large-mesh, batched and Cornell workloads
constexpr uint32_t kFeatPlain = (1u << 0) | (1u << 5) | (1u << 6) | kFeatNIters |
                                kFeatBsdfDir | kFeatLightTri;
// whether a kernel compiled for `kernel` may run work whose features are
// `need` (the material types it shades and the fixed choices it assumes)
inline constexpr bool feat_covers(uint32_t kernel, uint32_t need) {
  return (need & kFeatAllMats & ~kernel) == 0 &&
         (kernel & ~kFeatAllMats & ~need) == 0;
}

// device status word codes (first error wins)
enum DeviceStatus : uint32_t {
  kStatusOk = 0,
  kStatusStackOverflow = 1,
  kStatusObjectsOverflow = 2,
  kStatusBadNode = 3,
  kStatusPathTooLong = 4,
  kStatusPassCount = 5, // a light-only pass met a path with an extension ray
};

// Safety bound on the vertices of one path.  The reference loops until the
// termination draw ends the path; a bound keeps a kernel from spinning if a
// termination setting never ends a path.  No path of the built settings
// comes near it (NIters ends a path after iters + 1 vertices).
constexpr uint32_t kMaxPathVertices = 4096;
// most path steps of an OutputPerStep render
constexpr uint32_t kMaxOutputSteps = 64;

} // namespace pg
