// Scene flattening, light table and camera transform (host side).
#include "scene.h"

#include <cmath>

namespace pg {

bool is_emissive(const path_material &m) {
  // TriangleConstructor::add_material (src/scene/triangle_constructor.cpp:6)
  float e2 = (m.emission[0] * m.emission[0] + m.emission[1] * m.emission[1]) +
             m.emission[2] * m.emission[2];
  return e2 > 1e-9f;
}

affine identity_affine() {
  affine a;
  const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  for (int i = 0; i < 12; ++i) {
    a.m[i] = id[i];
  }
  return a;
}

static f3 load3(const float *p) { return mk(p[0], p[1], p[2]); }

static uint32_t range_start(const std::vector<uint32_t> &ends, uint32_t i) {
  return i == 0 ? 0u : ends[i - 1];
}

FlatScene flatten(const Scene &s) {
  FlatScene out;
  size_t total = 0;
  for (size_t i = 0; i < s.instances.size(); ++i) {
    uint32_t mesh = s.instance_mesh[i];
    total += s.mesh_ends[mesh] - range_start(s.mesh_ends, mesh);
  }
  out.v0.reserve(total);
  out.v1.reserve(total);
  out.v2.reserve(total);
  out.n0.reserve(total);
  out.n1.reserve(total);
  out.n2.reserve(total);
  out.material.reserve(total);
  float cumulative = 0.f;
  for (size_t i = 0; i < s.instances.size(); ++i) {
    uint32_t mesh = s.instance_mesh[i];
    const affine &xf = s.instances[i];
    // the reference bounds this loop by mesh_ends[instance]
    // (flat_triangle.h:93-94); the mesh's own end is the intended bound and
    // the two agree whenever each mesh has one instance
    for (uint32_t j = range_start(s.mesh_ends, mesh); j < s.mesh_ends[mesh]; ++j) {
      const float *t = &s.tris[9 * (size_t)j];
      const float *n = &s.normals[9 * (size_t)j];
      out.v0.push_back(xf.point(load3(t)));
      out.v1.push_back(xf.point(load3(t + 3)));
      out.v2.push_back(xf.point(load3(t + 6)));
      out.n0.push_back(normalize(xf.vector(load3(n))));
      out.n1.push_back(normalize(xf.vector(load3(n + 3))));
      out.n2.push_back(normalize(xf.vector(load3(n + 6))));
      out.material.push_back(s.tri_material[j]);
    }
    // RandomTriangle::gen: area x emission-sum weights, in cluster order
    uint32_t c0 = range_start(s.cluster_ends_per_mesh, mesh);
    for (uint32_t c = c0; c < s.cluster_ends_per_mesh[mesh]; ++c) {
      uint32_t mat = s.clusters[3 * c];
      const path_material &m = s.materials[mat];
      float esum = (m.emission[0] + m.emission[1]) + m.emission[2];
      for (uint32_t j = s.clusters[3 * c + 1]; j < s.clusters[3 * c + 2]; ++j) {
        const float *t = &s.tris[9 * (size_t)j];
        f3 a = xf.point(load3(t));
        f3 b = xf.point(load3(t + 3));
        f3 c3 = xf.point(load3(t + 6));
        f3 scaled = cross(b - a, c3 - a) * 0.5f;
        cumulative += length(scaled) * esum;
        out.light_v0.push_back(a);
        out.light_v1.push_back(b);
        out.light_v2.push_back(c3);
        out.light_cdf.push_back(cumulative);
      }
    }
  }
  for (float &w : out.light_cdf) {
    w /= cumulative;
  }
  return out;
}

// camera.cpp:4-27: film_to_world = (scale * view)^-1, computed here in
// double precision and rounded once to float
affine camera_transform(f3 look, f3 up, f3 pos, float height_angle_deg,
                        float width_height_ratio) {
  f3 f = normalize(look);
  f3 u0 = normalize(up);
  f3 s = cross(f, u0);
  f3 u = cross(s, f);
  double view[4][4] = {
      {s.x, s.y, s.z, -(double)dot(s, pos)},
      {u.x, u.y, u.z, -(double)dot(u, pos)},
      {-f.x, -f.y, -f.z, (double)dot(f, pos)},
      {0, 0, 0, 1},
  };
  float half = (float)M_PI * height_angle_deg / 360.f;
  double tan_h = std::tan((double)half);
  double tan_w = (double)width_height_ratio * tan_h;
  double sx = 1.0 / tan_w, sy = 1.0 / tan_h;
  // M = scale * view: rows 0 and 1 scaled.  The inverse of [R t; 0 1] with
  // R = diag(sx, sy, 1) * V3 is [R^-1, -R^-1 t]; V3 is orthonormal so
  // R^-1 = V3^T diag(1/sx, 1/sy, 1).
  double r[3][3], t[3];
  for (int i = 0; i < 3; ++i) {
    double sc = i == 0 ? sx : (i == 1 ? sy : 1.0);
    for (int j = 0; j < 3; ++j) {
      r[i][j] = view[i][j] * sc;
    }
    t[i] = view[i][3] * sc;
  }
  // general 3x3 inverse (cofactors), so non-orthonormal input still works
  double det = r[0][0] * (r[1][1] * r[2][2] - r[1][2] * r[2][1]) -
               r[0][1] * (r[1][0] * r[2][2] - r[1][2] * r[2][0]) +
               r[0][2] * (r[1][0] * r[2][1] - r[1][1] * r[2][0]);
  double inv[3][3];
  inv[0][0] = (r[1][1] * r[2][2] - r[1][2] * r[2][1]) / det;
  inv[0][1] = (r[0][2] * r[2][1] - r[0][1] * r[2][2]) / det;
  inv[0][2] = (r[0][1] * r[1][2] - r[0][2] * r[1][1]) / det;
  inv[1][0] = (r[1][2] * r[2][0] - r[1][0] * r[2][2]) / det;
  inv[1][1] = (r[0][0] * r[2][2] - r[0][2] * r[2][0]) / det;
  inv[1][2] = (r[0][2] * r[1][0] - r[0][0] * r[1][2]) / det;
  inv[2][0] = (r[1][0] * r[2][1] - r[1][1] * r[2][0]) / det;
  inv[2][1] = (r[0][1] * r[2][0] - r[0][0] * r[2][1]) / det;
  inv[2][2] = (r[0][0] * r[1][1] - r[0][1] * r[1][0]) / det;
  affine out;
  for (int i = 0; i < 3; ++i) {
    double ti = -(inv[i][0] * t[0] + inv[i][1] * t[1] + inv[i][2] * t[2]);
    for (int j = 0; j < 3; ++j) {
      out.m[4 * i + j] = (float)inv[i][j];
    }
    out.m[4 * i + 3] = (float)ti;
  }
  return out;
}

} // namespace pg
