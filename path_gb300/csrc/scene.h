// Scene model of the render path (host side).
//
// Mirrors scene::Scene (include/scene/scene.h:29-130): meshes of triangles
// with per-vertex normals and a material index, instances (object-to-world
// transforms of meshes), emissive clusters and materials.  flatten()
// restates intersectable_scene::flat_triangle::Generator::gen
// (include/intersectable_scene/flat_triangle/flat_triangle.h:79-146) and the
// light table of light_sampler::RandomTriangle::gen
// (include/integrate/light_sampler/random_triangle/random_triangle.h:120-161).
#pragma once

#include "geom.h"
#include "path_gb300.h"

#include <string>
#include <vector>

namespace pg {

struct Scene {
  std::vector<float> tris;      // [n][3][3] object space
  std::vector<float> normals;   // [n][3][3]
  std::vector<uint32_t> tri_material;
  std::vector<uint32_t> mesh_ends;
  std::vector<uint32_t> cluster_ends_per_mesh;
  std::vector<affine> instances;
  std::vector<uint32_t> instance_mesh;
  std::vector<uint32_t> clusters; // [c][3] material, start, end
  std::vector<path_material> materials;
  uint64_t version = 0;          // geometry (and material list) edits
  uint64_t material_version = 0; // in-place material parameter edits
  uint64_t id = 0;

  uint32_t n_tris() const { return (uint32_t)tri_material.size(); }
};

// world-space scene ready for accel build and upload
struct FlatScene {
  std::vector<f3> v0, v1, v2;       // world-space vertices
  std::vector<f3> n0, n1, n2;       // world-space vertex normals
  std::vector<uint32_t> material;
  std::vector<f3> light_v0, light_v1, light_v2;
  std::vector<float> light_cdf;
};

bool is_emissive(const path_material &m);
affine identity_affine();
FlatScene flatten(const Scene &s);

// scene::get_camera_transform (src/scene/camera.cpp:4-27)
affine camera_transform(f3 look, f3 up, f3 pos, float height_angle_deg,
                        float width_height_ratio);

// CS123 XML + OBJ/MTL loader (src/scene/scenefile_compat/scenefile_loader.cpp)
bool load_scene_xml(const std::string &path, float width_height_ratio,
                    Scene &out, affine &film_to_world, std::string &err);

} // namespace pg
