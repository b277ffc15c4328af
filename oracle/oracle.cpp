// CPU oracle for the render hot path -- TEST INFRASTRUCTURE ONLY.
// See oracle.h for what this library is and who may use it.  Each function
// names the reference file:line it restates.  Build flags: -O2
// -ffp-contract=off -fopenmp (no -ffast-math: subnormals and IEEE division
// must behave exactly as on the GPU).

#include "oracle.h"

#include "../path_gb300/csrc/pmath.h"

#include <curand.h>
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <iterator>
#include <limits>
#include <optional>
#include <random>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace {

// Transcendental functions of the integrator.  The default build shares
// path_gb300/csrc/pmath.h with the kernels, so that CPU and GPU round every
// bounce direction identically.  Built with -DORACLE_LIBM (liboracle_libm.so)
// the oracle calls the C library's sinf / cosf / asinf / acosf / powf where
// the reference calls std::sin, std::cos, std::asin, std::acos and std::pow
// (include/bsdf/diffuse.h:30-45, glossy.h:26-49, lib/projection.h:9-32,
// dielectric_refractive.h:24-33, multiplier_func.h:19-30): the two builds
// measure how far the shared polynomials move an image from the C library's
// arithmetic.
namespace om {
#ifdef ORACLE_LIBM
inline float sin(float x) { return ::sinf(x); }
inline float cos(float x) { return ::cosf(x); }
inline float asin(float x) { return ::asinf(x); }
inline float acos(float x) { return ::acosf(x); }
inline float pow(float x, float y) { return ::powf(x, y); }
#else
inline float sin(float x) { return pm::sin(x); }
inline float cos(float x) { return pm::cos(x); }
inline float asin(float x) { return pm::asin(x); }
inline float acos(float x) { return pm::acos(x); }
inline float pow(float x, float y) { return pm::pow(x, y); }
#endif
} // namespace om

constexpr float kFloatMax = std::numeric_limits<float>::max();
constexpr float kFloatLowest = std::numeric_limits<float>::lowest();

// ---------------------------------------------------------------------------
// vector arithmetic: Eigen's Vector3f restated with an explicit evaluation
// order (left to right), no contraction.
struct V3 {
  float x, y, z;
  float &operator[](unsigned i) { return i == 0 ? x : (i == 1 ? y : z); }
  float operator[](unsigned i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 cmul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 cmin(V3 a, V3 b) {
  return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)};
}
inline V3 cmax(V3 a, V3 b) {
  return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)};
}
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float squared_norm(V3 a) { return dot(a, a); }
inline float norm(V3 a) { return pm::sqrt(squared_norm(a)); }
// Eigen's normalized(): unchanged when the squared norm is zero
inline V3 normalized(V3 a) {
  float n2 = squared_norm(a);
  if (n2 > 0.f) {
    return a / pm::sqrt(n2);
  }
  return a;
}
inline float max_coeff(V3 a) { return std::max(a.x, std::max(a.y, a.z)); }
inline float min_coeff(V3 a) { return std::min(a.x, std::min(a.y, a.z)); }

struct RGB {
  float r, g, b;
};
inline RGB operator+(RGB a, RGB b) { return {a.r + b.r, a.g + b.g, a.b + b.b}; }
inline RGB operator*(RGB a, RGB b) { return {a.r * b.r, a.g * b.g, a.b * b.b}; }
inline RGB operator*(RGB a, float s) { return {a.r * s, a.g * s, a.b * s}; }
inline RGB operator/(RGB a, float s) { return {a.r / s, a.g / s, a.b / s}; }
inline RGB operator/(RGB a, RGB b) { return {a.r / b.r, a.g / b.g, a.b / b.b}; }
inline RGB rgb_zero() { return {0.f, 0.f, 0.f}; }
inline float rgb_sum(RGB a) { return (a.r + a.g) + a.b; }

// affine 3x4 row-major: out = L v + t, each row ((m0 x + m1 y) + m2 z) + t
struct Affine {
  float m[12];
  V3 apply(V3 v) const {
    return {((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3],
            ((m[4] * v.x + m[5] * v.y) + m[6] * v.z) + m[7],
            ((m[8] * v.x + m[9] * v.y) + m[10] * v.z) + m[11]};
  }
  V3 linear(V3 v) const {
    return {(m[0] * v.x + m[1] * v.y) + m[2] * v.z,
            (m[4] * v.x + m[5] * v.y) + m[6] * v.z,
            (m[8] * v.x + m[9] * v.y) + m[10] * v.z};
  }
  V3 translation() const { return {m[3], m[7], m[11]}; }
};

struct Ray {
  V3 o;
  V3 d;
};

// ---------------------------------------------------------------------------
// include/intersect/accel/aabb.h:16-131
struct AABB {
  V3 lo, hi;
  static AABB empty() {
    return {{kFloatMax, kFloatMax, kFloatMax},
            {kFloatLowest, kFloatLowest, kFloatLowest}};
  }
  AABB union_other(const AABB &o) const {
    return {cmin(lo, o.lo), cmax(hi, o.hi)};
  }
  AABB union_point(V3 p) const { return {cmin(lo, p), cmax(hi, p)}; }
  AABB intersection_other(const AABB &o) const {
    return {cmax(lo, o.lo), cmin(hi, o.hi)};
  }
  bool contains(V3 p) const {
    return lo.x <= p.x && lo.y <= p.y && lo.z <= p.z && hi.x >= p.x &&
           hi.y >= p.y && hi.z >= p.z;
  }
  float surface_area() const {
    V3 d = hi - lo;
    if (d.x < 0.f || d.y < 0.f || d.z < 0.f) {
      return 0.f;
    }
    return 2 * (d.x * d.y + d.z * d.y + d.z * d.x);
  }
  V3 centroid() const { return (lo + hi) / 2.f; }
  bool solve(V3 p, V3 inv, float *t_min, float *t_max) const {
    V3 t0 = cmul(lo - p, inv);
    V3 t1 = cmul(hi - p, inv);
    float tmin = max_coeff(cmin(t0, t1));
    float tmax = min_coeff(cmax(t0, t1));
    if (tmin <= tmax) {
      *t_min = tmin;
      *t_max = tmax;
      return true;
    }
    return false;
  }
};

// aabb.h:16-28
inline V3 inv_direction(V3 d) {
  for (unsigned i = 0; i < 3; ++i) {
    if (d[i] == 0.0f) {
      d[i] = 1e-20f;
    }
  }
  return {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
}

// include/intersect/triangle.h, triangle_impl.h
struct Tri {
  V3 v[3];
  V3 normal_raw() const { return cross(v[1] - v[0], v[2] - v[0]); }
  V3 normal_scaled_by_area() const { return 0.5f * normal_raw(); }
  V3 normal() const { return normalized(normal_raw()); }
  AABB bounds() const {
    AABB out = AABB::empty();
    for (const V3 &p : v) {
      out.lo = cmin(out.lo, p);
      out.hi = cmax(out.hi, p);
    }
    return out;
  }
  V3 baryo_to_point(float s, float t) const {
    V3 e0 = v[1] - v[0];
    V3 e1 = v[2] - v[0];
    return (e0 * s + e1 * t) + v[0];
  }
  // triangle_impl.h:55-72
  void interpolation_values(V3 point, float w[3]) const {
    V3 p0 = v[1] - v[0];
    V3 p1 = v[2] - v[0];
    V3 p2 = point - v[0];
    float d00 = dot(p0, p0);
    float d01 = dot(p0, p1);
    float d11 = dot(p1, p1);
    float d20 = dot(p2, p0);
    float d21 = dot(p2, p1);
    float denom = d00 * d11 - d01 * d01;
    float vv = (d11 * d20 - d01 * d21) / denom;
    float ww = (d00 * d21 - d01 * d20) / denom;
    float uu = (float)((1. - (double)vv) - (double)ww); // double literal 1.
    w[0] = uu;
    w[1] = vv;
    w[2] = ww;
  }
};

struct Hit {
  bool ok = false;
  float t = 0.f;
  bool back = false;
  unsigned idx = 0;
};

// triangle_impl.h:9-39 (literal double-precision comparisons kept)
inline Hit tri_intersect(const Tri &tri, const Ray &ray) {
  V3 edge1 = tri.v[1] - tri.v[0];
  V3 edge2 = tri.v[2] - tri.v[0];
  V3 h = cross(ray.d, edge2);
  float a = dot(edge1, h);
  if ((double)std::fabs(a) < 1e-7) {
    return {};
  }
  float f = (float)(1. / (double)a);
  V3 s = ray.o - tri.v[0];
  float u = f * dot(s, h);
  if (u < 0.f || u > 1.f) {
    return {};
  }
  V3 q = cross(s, edge1);
  float v = f * dot(ray.d, q);
  if (v < 0.f || u + v > 1.f) {
    return {};
  }
  float t = f * dot(edge2, q);
  if ((double)t > 1e-5) {
    return {true, t, a < 0.f, 0};
  }
  return {};
}

// optional_min fold (include/intersect/optional_min.h:10-26): on equal
// distance the later candidate wins
inline void fold_min(Hit &best, Hit cand) {
  if (!cand.ok) {
    return;
  }
  if (!best.ok) {
    best = cand;
    return;
  }
  if (best.t < cand.t) {
    return;
  }
  best = cand;
}

// ---------------------------------------------------------------------------
// include/intersect/accel/detail/bvh/node.h:14-127
constexpr uint32_t kTagBit = 1u << 31;
struct Node {
  uint32_t w0, w1; // PackedBoolUnsigned pair
  AABB aabb;
  bool is_split() const { return (w0 & kTagBit) != 0; }
  uint32_t first() const { return w0 & ~kTagBit; }
  uint32_t second() const { return w1 & ~kTagBit; }
  bool is_for_extra() const { return (w1 & kTagBit) != 0; }
  static Node split(uint32_t l, uint32_t r, AABB b) {
    return {l | kTagBit, r, b};
  }
  static Node items(uint32_t s, uint32_t e, bool extra, AABB b) {
    return {s, e | (extra ? kTagBit : 0u), b};
  }
};

// src/intersect/accel/sbvh/detail/generator.cu and
// include/intersect/accel/detail/clipped_triangle_impl.h
struct ClippedTriangle {
  Tri triangle;
  AABB bounds;

  // clipped_triangle_impl.h:13-124
  AABB new_bounds(float left_bound, float right_bound, unsigned axis) const {
    AABB nb = bounds;
    nb.lo[axis] = std::max(nb.lo[axis], left_bound);
    nb.hi[axis] = std::min(nb.hi[axis], right_bound);
    for (unsigned ax = 0; ax < 3; ++ax) {
      if (nb.lo[ax] == nb.hi[ax]) {
        nb.lo[ax] = (float)((double)nb.lo[ax] - 1.);
        nb.hi[ax] = (float)((double)nb.hi[ax] + 1.);
      }
    }
    AABB out = AABB::empty();
    for (const V3 &vert : triangle.v) {
      if (nb.contains(vert)) {
        out = out.union_point(vert);
      }
    }
    const unsigned edges[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (unsigned e = 0; e < 3; ++e) {
      unsigned start = edges[e][0], end = edges[e][1];
      V3 dir = triangle.v[end] - triangle.v[start];
      for (float sign : {-1.f, 1.f}) {
        V3 dir_sign = dir * sign;
        V3 inv = inv_direction(dir_sign);
        float tmin, tmax;
        if (nb.solve(triangle.v[start], inv, &tmin, &tmax)) {
          out = out.union_point(dir_sign * tmin + triangle.v[start]);
        }
      }
    }
    for (unsigned pd = 0; pd < 3; ++pd) {
      for (bool is_min_next : {false, true}) {
        for (bool is_min_next_next : {false, true}) {
          unsigned na = (pd + 1) % 3;
          unsigned nna = (pd + 2) % 3;
          float px = (is_min_next ? nb.lo : nb.hi)[na];
          float py = (is_min_next_next ? nb.lo : nb.hi)[nna];
          V3 d01 = triangle.v[1] - triangle.v[0];
          V3 d02 = triangle.v[2] - triangle.v[0];
          float v0x = triangle.v[0][na], v0y = triangle.v[0][nna];
          float v1x = triangle.v[1][na], v1y = triangle.v[1][nna];
          float v2x = triangle.v[2][na], v2y = triangle.v[2][nna];
          float area_inner = (((-v1y) * v2x + v0y * ((-v1x) + v2x)) +
                              v0x * (v1y - v2y)) +
                             v1x * v2y;
          float area = (float)(0.5 * (double)area_inner);
          float inv2a = 1 / (2 * area);
          float s = inv2a * (((v0y * v2x - v0x * v2y) + (v2y - v0y) * px) +
                             (v0x - v2x) * py);
          float t = inv2a * (((v0x * v1y - v0y * v1x) + (v0y - v1y) * px) +
                             (v1x - v0x) * py);
          if (s >= 0 && t >= 0 && (1 - s - t) > 0) {
            out = out.union_point((d01 * s + d02 * t) + triangle.v[0]);
          }
        }
      }
    }
    return out;
  }
};

struct SplitCandidate {
  float base_cost = kFloatMax;
  bool is_spatial = false;
  // object split
  std::vector<unsigned> perm;
  unsigned split_point = 0;
  float intersection_surface_area = 0.f;
  // spatial split
  std::vector<unsigned> left_triangles, right_triangles;
  std::vector<AABB> left_bounds, right_bounds;
};

struct SBVHBuilder {
  float overlap_threshold;
  bool use_spatial_splits;
  float traversal_cost;
  float root_surface_area = 0.f;
  std::vector<Node> nodes;
  std::vector<unsigned> extra_idxs;

  // generator.cu:406-438
  std::vector<unsigned> sort_by_axis(std::vector<ClippedTriangle> &tris,
                                     unsigned axis) {
    struct ValueIdx {
      float value;
      unsigned idx;
    };
    std::vector<ValueIdx> to_sort(tris.size());
    for (unsigned i = 0; i < tris.size(); ++i) {
      to_sort[i] = {tris[i].bounds.centroid()[axis], i};
    }
    std::sort(to_sort.begin(), to_sort.end(),
              [](ValueIdx l, ValueIdx r) { return l.value < r.value; });
    std::vector<unsigned> out(tris.size());
    std::vector<ClippedTriangle> old = tris;
    for (unsigned i = 0; i < tris.size(); ++i) {
      out[i] = to_sort[i].idx;
      tris[i] = old[to_sort[i].idx];
    }
    return out;
  }

  // generator.cu:343-404
  SplitCandidate best_object_split(const ClippedTriangle *in, size_t n,
                                   unsigned axis) {
    std::vector<ClippedTriangle> tris(in, in + n);
    std::vector<unsigned> sort_perm = sort_by_axis(tris, axis);
    std::vector<AABB> backward(n);
    AABB running_back = AABB::empty();
    for (size_t i = n; i-- > 0;) {
      running_back = running_back.union_other(tris[i].bounds);
      backward[i] = running_back;
    }
    float best_base_cost = kFloatMax;
    float best_isa = 0.f;
    unsigned best_split = 0;
    AABB running = AABB::empty();
    for (unsigned i = 0; i < n; ++i) {
      const AABB &left = running;
      const AABB &right = backward[i];
      float isa = left.intersection_other(right).surface_area();
      float sl = left.surface_area();
      float sr = right.surface_area();
      float base_cost = (float)i * sl + (float)(n - i) * sr;
      if (base_cost < best_base_cost) {
        best_base_cost = base_cost;
        best_isa = isa;
        best_split = i;
      }
      running = running.union_other(tris[i].bounds);
    }
    SplitCandidate out;
    out.base_cost = best_base_cost;
    out.is_spatial = false;
    out.perm = std::move(sort_perm);
    out.split_point = best_split;
    out.intersection_surface_area = best_isa;
    return out;
  }

  // generator.cu:440-713
  SplitCandidate best_spatial_split(const ClippedTriangle *tris, size_t n,
                                    unsigned axis) {
    AABB overall = AABB::empty();
    for (size_t i = 0; i < n; ++i) {
      overall = overall.union_other(tris[i].bounds);
    }
    unsigned num_divisions = (unsigned)n * 2;
    unsigned num_inside_edges = num_divisions - 1;
    float total = overall.hi[axis] - overall.lo[axis];
    struct BinInfo {
      AABB aabb = AABB::empty();
      unsigned entries = 0;
      unsigned exits = 0;
    };
    std::vector<BinInfo> bins(num_divisions);
    std::vector<std::vector<unsigned>> crossing(num_inside_edges);
    auto split_point = [&](unsigned loc) -> float {
      float frac = (float)loc / (float)num_divisions;
      if (loc == num_divisions) {
        return overall.hi[axis];
      }
      return frac * total + overall.lo[axis];
    };
    for (unsigned ti = 0; ti < n; ++ti) {
      const ClippedTriangle &tri = tris[ti];
      AABB b = tri.bounds;
      float min_axis = b.lo[axis];
      float max_axis = b.hi[axis];
      float min_prop = (min_axis - overall.lo[axis]) / total;
      float max_prop = (max_axis - overall.lo[axis]) / total;
      unsigned min_loc =
          std::min((unsigned)std::floor(min_prop * (float)num_divisions),
                   num_divisions - 1);
      unsigned max_loc =
          std::min((unsigned)std::floor(max_prop * (float)num_divisions),
                   num_divisions - 1);
      if (split_point(min_loc) > b.lo[axis]) {
        --min_loc;
      }
      if (split_point(max_loc + 1) < b.hi[axis]) {
        ++max_loc;
      }
      if (min_loc != max_loc) {
        if (split_point(max_loc) >= max_axis) {
          --max_loc;
        }
        if (split_point(min_loc + 1) <= min_axis) {
          ++min_loc;
        }
      }
      ++bins[min_loc].entries;
      ++bins[max_loc].exits;
      for (unsigned loc = min_loc; loc <= max_loc; ++loc) {
        if (loc != max_loc) {
          crossing[loc].push_back(ti);
        }
        bins[loc].aabb = bins[loc].aabb.union_other(
            tri.new_bounds(split_point(loc), split_point(loc + 1), axis));
      }
    }
    std::vector<AABB> backward(bins.size());
    AABB running_back = AABB::empty();
    for (size_t i = bins.size(); i-- > 0;) {
      running_back = running_back.union_other(bins[i].aabb);
      backward[i] = running_back;
    }
    float best_base_cost = kFloatMax;
    unsigned best_edge = 0;
    std::unordered_set<unsigned> best_left_only, best_right_only;
    unsigned total_left_overall = 0;
    unsigned total_right_overall = (unsigned)n;
    AABB running = AABB::empty();
    for (unsigned edge = 0; edge < num_divisions - 1; ++edge) {
      unsigned loc_left = edge;
      unsigned loc_right = edge + 1;
      total_left_overall += bins[loc_left].entries;
      total_right_overall -= bins[loc_left].exits;
      unsigned total_left = total_left_overall;
      unsigned total_right = total_right_overall;
      running = running.union_other(bins[loc_left].aabb);
      AABB left_aabb = running;
      AABB right_aabb = backward[loc_right];
      float sl = left_aabb.surface_area();
      float sr = right_aabb.surface_area();
      float base_cost = (float)total_left * sl + (float)total_right * sr;
      std::unordered_set<unsigned> left_only, right_only;
      for (unsigned ti : crossing[edge]) {
        const ClippedTriangle &tri = tris[ti];
        AABB lo_b = left_aabb.union_other(tri.bounds);
        AABB ro_b = right_aabb.union_other(tri.bounds);
        float cost_left_only =
            (float)total_left * lo_b.surface_area() + (float)(total_right - 1) * sr;
        float cost_right_only =
            (float)(total_left - 1) * sl + (float)total_right * ro_b.surface_area();
        if (std::min(cost_left_only, cost_right_only) < base_cost) {
          if (cost_left_only < cost_right_only) {
            total_right -= 1;
            base_cost = cost_left_only;
            sl = lo_b.surface_area();
            left_aabb = lo_b;
            left_only.insert(ti);
          } else {
            total_left -= 1;
            base_cost = cost_right_only;
            sr = ro_b.surface_area();
            right_aabb = ro_b;
            right_only.insert(ti);
          }
        }
      }
      if (base_cost < best_base_cost) {
        best_base_cost = base_cost;
        best_edge = edge;
        best_left_only = left_only;
        best_right_only = right_only;
      }
    }
    AABB left_aabb = AABB::empty();
    AABB right_aabb = AABB::empty();
    SplitCandidate out;
    out.is_spatial = true;
    for (unsigned ti = 0; ti < n; ++ti) {
      const ClippedTriangle &tri = tris[ti];
      if (best_left_only.count(ti)) {
        left_aabb = left_aabb.union_other(tri.bounds);
        out.left_bounds.push_back(tri.bounds);
        out.left_triangles.push_back(ti);
        continue;
      }
      if (best_right_only.count(ti)) {
        right_aabb = right_aabb.union_other(tri.bounds);
        out.right_bounds.push_back(tri.bounds);
        out.right_triangles.push_back(ti);
        continue;
      }
      float sp = split_point(best_edge + 1);
      bool to_left = tri.bounds.lo[axis] < sp;
      bool to_right = tri.bounds.hi[axis] > sp;
      bool on_split = !to_left && !to_right;
      if (to_left || on_split) {
        AABB nb = tri.new_bounds(kFloatLowest, sp, axis);
        left_aabb = left_aabb.union_other(nb);
        out.left_bounds.push_back(nb);
        out.left_triangles.push_back(ti);
      }
      if (to_right) {
        AABB nb = tri.new_bounds(sp, kFloatMax, axis);
        right_aabb = right_aabb.union_other(nb);
        out.right_bounds.push_back(nb);
        out.right_triangles.push_back(ti);
      }
    }
    out.base_cost = (float)out.left_triangles.size() * left_aabb.surface_area() +
                    (float)out.right_triangles.size() * right_aabb.surface_area();
    return out;
  }

  // generator.cu:68-341.  tris/idxs/finals are views into the caller's
  // arrays and are reordered in place, as in the reference.
  Node create_node(ClippedTriangle *tris, unsigned *idxs,
                   std::optional<unsigned> *finals, size_t n,
                   unsigned start_idx, bool is_root) {
    AABB overall = AABB::empty();
    for (size_t i = 0; i < n; ++i) {
      overall = overall.union_other(tris[i].bounds);
    }
    if (is_root) {
      root_surface_area = overall.surface_area();
    }
    SplitCandidate best;
    for (unsigned axis = 0; axis < 3; ++axis) {
      SplitCandidate c = best_object_split(tris, n, axis);
      if (c.base_cost < best.base_cost) {
        best = std::move(c);
      }
    }
    float isa = best.intersection_surface_area;
    if (use_spatial_splits && isa / root_surface_area > overlap_threshold) {
      for (unsigned axis = 0; axis < 3; ++axis) {
        SplitCandidate c = best_spatial_split(tris, n, axis);
        if (c.base_cost < best.base_cost) {
          best = std::move(c);
        }
      }
    }
    float sa = overall.surface_area();
    float best_cost = best.base_cost / sa + traversal_cost;
    if (best_cost >= (float)n) {
      std::vector<unsigned> actual(n);
      unsigned running_idx = start_idx;
      for (size_t i = 0; i < n; ++i) {
        if (finals[i].has_value()) {
          actual[i] = *finals[i];
        } else {
          actual[i] = running_idx++;
        }
      }
      bool use_start_end = true;
      for (size_t i = 0; i + 1 < n; ++i) {
        use_start_end = use_start_end && actual[i + 1] > actual[i] &&
                        actual[i + 1] - actual[i] == 1;
      }
      if (!use_start_end) {
        for (unsigned a : actual) {
          extra_idxs.push_back(a);
        }
        return Node::items((unsigned)(extra_idxs.size() - actual.size()),
                           (unsigned)extra_idxs.size(), true, overall);
      }
      return Node::items(actual[0], actual[0] + (unsigned)n, false, overall);
    }

    nodes.resize(nodes.size() + 2);
    unsigned left_idx = (unsigned)nodes.size() - 2;
    unsigned right_idx = (unsigned)nodes.size() - 1;
    std::vector<ClippedTriangle> old_tris(tris, tris + n);
    std::vector<unsigned> old_idxs(idxs, idxs + n);
    std::vector<std::optional<unsigned>> old_finals(finals, finals + n);

    if (!best.is_spatial) {
      for (size_t i = 0; i < n; ++i) {
        unsigned p = best.perm[i];
        tris[i] = old_tris[p];
        idxs[i] = old_idxs[p];
        finals[i] = old_finals[p];
      }
      unsigned sp = best.split_point;
      unsigned num_in_order = 0;
      for (unsigned i = 0; i < sp; ++i) {
        if (!finals[i].has_value()) {
          ++num_in_order;
        }
      }
      Node l = create_node(tris, idxs, finals, sp, start_idx, false);
      nodes[left_idx] = l;
      Node r = create_node(tris + sp, idxs + sp, finals + sp, n - sp,
                           start_idx + num_in_order, false);
      nodes[right_idx] = r;
    } else {
      const auto &lt = best.left_triangles;
      const auto &rt = best.right_triangles;
      for (size_t i = 0; i < lt.size(); ++i) {
        unsigned p = lt[i];
        tris[i] = old_tris[p];
        tris[i].bounds = best.left_bounds[i];
        idxs[i] = old_idxs[p];
        finals[i] = old_finals[p];
      }
      unsigned sp = (unsigned)lt.size();
      Node l = create_node(tris, idxs, finals, sp, start_idx, false);
      nodes[left_idx] = l;

      std::unordered_set<unsigned> dups;
      std::set_intersection(lt.begin(), lt.end(), rt.begin(), rt.end(),
                            std::inserter(dups, dups.begin()));
      std::unordered_map<unsigned, unsigned> dup_idx_to_right_idx;
      for (unsigned i = 0; i < rt.size(); ++i) {
        unsigned actual_idx = rt[i];
        if (dups.count(actual_idx)) {
          dup_idx_to_right_idx.insert({old_idxs[actual_idx], i});
        }
      }
      std::vector<ClippedTriangle> tris_right(rt.size());
      std::vector<unsigned> idxs_right(rt.size());
      std::vector<std::optional<unsigned>> finals_right(rt.size());
      for (unsigned i = 0; i < rt.size(); ++i) {
        unsigned p = rt[i];
        tris_right[i] = old_tris[p];
        tris_right[i].bounds = best.right_bounds[i];
        idxs_right[i] = i;
        finals_right[i] = old_finals[p];
      }
      unsigned num_in_order = 0;
      for (unsigned i = 0; i < lt.size(); ++i) {
        unsigned idx = idxs[i];
        auto it = dup_idx_to_right_idx.find(idx);
        if (it != dup_idx_to_right_idx.end()) {
          unsigned ri = it->second;
          if (!finals_right[ri].has_value()) {
            finals_right[ri] = start_idx + num_in_order;
          }
        }
        if (!finals[i].has_value()) {
          ++num_in_order;
        }
      }
      Node r = create_node(tris_right.data(), idxs_right.data(),
                           finals_right.data(), rt.size(),
                           start_idx + num_in_order, false);
      nodes[right_idx] = r;
      unsigned overall_idx = (unsigned)lt.size();
      for (unsigned i = 0; i < rt.size(); ++i) {
        unsigned prev = idxs_right[i];
        if (dups.count(rt[prev])) {
          continue;
        }
        idxs[overall_idx] = old_idxs[rt[prev]];
        finals[overall_idx] = old_finals[rt[prev]];
        ++overall_idx;
      }
    }
    return Node::split(left_idx, right_idx, overall);
  }
};

struct BVH {
  std::vector<Node> nodes;
  std::vector<unsigned> extra_idxs;
  std::vector<unsigned> permutation; // BVH position -> original index
  std::vector<Tri> tris;             // in BVH order
  unsigned target_objects = 4;
};

// generator.cu:17-66
BVH build_bvh(const std::vector<Tri> &in, float overlap_threshold,
              bool use_spatial_splits, float traversal_cost,
              unsigned target_objects) {
  BVH out;
  out.target_objects = target_objects;
  if (in.empty()) {
    return out;
  }
  std::vector<ClippedTriangle> tris(in.size());
  std::vector<unsigned> idxs(in.size());
  for (unsigned i = 0; i < in.size(); ++i) {
    tris[i] = {in[i], in[i].bounds()};
    idxs[i] = i;
  }
  std::vector<std::optional<unsigned>> finals(in.size());
  SBVHBuilder b;
  b.overlap_threshold = overlap_threshold;
  b.use_spatial_splits = use_spatial_splits;
  b.traversal_cost = traversal_cost;
  b.nodes.resize(1);
  Node root = b.create_node(tris.data(), idxs.data(), finals.data(), tris.size(),
                            0, true);
  b.nodes[0] = root;
  out.nodes = std::move(b.nodes);
  out.extra_idxs = std::move(b.extra_idxs);
  out.permutation = idxs;
  out.tris.resize(in.size());
  for (unsigned i = 0; i < in.size(); ++i) {
    out.tris[i] = in[out.permutation[i]];
  }
  return out;
}

// include/intersect/accel/detail/bvh/bvh_impl.h:12-89 (stack of 64 nodes,
// candidate batch of up to 10 triangles)
// order_independent: the closest hit of the GPU's 8-wide traversal instead
// of the reference's tie rule -- at equal distance the smallest BVH-order
// index wins, and a box is pruned only when the best distance is strictly
// below its entry distance, so that no equal-distance candidate is skipped.
// Results then do not depend on the order nodes are visited in.
Hit bvh_intersect(const BVH &bvh, const Ray &ray, bool order_independent = false) {
  Hit best;
  if (bvh.nodes.empty()) {
    return best;
  }
  V3 inv = inv_direction(ray.d);
  unsigned stack[64];
  unsigned sp = 0;
  stack[sp++] = 0;
  unsigned objects[10];
  unsigned n_obj = 0;
  while (sp != 0) {
    while (n_obj < bvh.target_objects && sp != 0) {
      const Node &node = bvh.nodes[stack[--sp]];
      float tmin, tmax;
      if (node.aabb.solve(ray.o, inv, &tmin, &tmax) &&
          (!best.ok || best.t > tmin || (order_independent && best.t == tmin))) {
        if (node.is_split()) {
          stack[sp++] = node.second();
          stack[sp++] = node.first();
        } else {
          for (unsigned i = node.first(); i < node.second(); ++i) {
            objects[n_obj++] = node.is_for_extra() ? bvh.extra_idxs[i] : i;
          }
        }
      }
    }
    if (n_obj == 0) {
      break;
    }
    for (unsigned k = 0; k < n_obj; ++k) {
      Hit h = tri_intersect(bvh.tris[objects[k]], ray);
      h.idx = objects[k];
      if (!order_independent) {
        fold_min(best, h);
      } else if (h.ok && (!best.ok || h.t < best.t || (h.t == best.t && h.idx < best.idx))) {
        best = h;
      }
    }
    n_obj = 0;
  }
  return best;
}

float sah_cost_impl(const BVH &bvh, float trav, unsigned idx) {
  const Node &n = bvh.nodes[idx];
  if (!n.is_split()) {
    return (float)(n.second() - n.first());
  }
  auto child = [&](unsigned c) {
    return sah_cost_impl(bvh, trav, c) * bvh.nodes[c].aabb.surface_area() /
           n.aabb.surface_area();
  };
  return trav + child(n.first()) + child(n.second());
}

// ---------------------------------------------------------------------------
// include/lib/projection.h:9-32: rotation by an angle about an axis
// (Rodrigues' formula v c + (a x v) s + a (a.v)(1 - c))
V3 rotate_axis_angle(V3 v, float angle, V3 axis) {
  float c = om::cos(angle);
  float s = om::sin(angle);
  V3 term0 = v * c;
  V3 term1 = cross(axis, v) * s;
  V3 term2 = axis * ((1.f - c) * dot(axis, v));
  return (term0 + term1) + term2;
}

V3 rotate_to(V3 inp, V3 target, float sign) {
  float angle = om::acos(dot(inp, target));
  V3 axis = normalized(cross(inp, target));
  return rotate_axis_angle(inp, sign * angle, axis);
}

// projection.h:24-32
V3 find_relative_vec(V3 vec, float phi, float theta) {
  float sin_theta = om::sin(theta);
  V3 local = {sin_theta * om::cos(phi), sin_theta * om::sin(phi),
              om::cos(theta)};
  V3 z = {0.f, 0.f, 1.f};
  float angle = om::acos(dot(vec, z));
  V3 axis = normalized(cross(vec, z));
  return normalized(rotate_axis_angle(local, -angle, axis));
}

// bsdf/utils.h:10-36
V3 reflect_over_normal(V3 vec, V3 normal) {
  float k = 2.0f * -dot(vec, normal);
  return normalized(vec + normal * k);
}

V3 refract_by_normal(float ior, V3 vec, V3 normal) {
  float cos_to_normal = -dot(vec, normal);
  bool exiting = cos_to_normal < 0.f;
  float frac = exiting ? ior : 1 / ior;
  float in_sqrt = 1 - frac * frac * (1 - cos_to_normal * cos_to_normal);
  V3 n_eff = exiting ? -normal : normal;
  if (in_sqrt > 0.f) {
    float angle = om::acos(pm::sqrt(in_sqrt));
    V3 axis = normalized(cross(vec, n_eff));
    return normalized(rotate_axis_angle(-n_eff, angle, axis));
  }
  return reflect_over_normal(vec, normal);
}

// ---------------------------------------------------------------------------
// RNG: include/rng/rng_from_sequence_gen.h:26-107, include/lib/fnv.h:5-14
uint32_t fnv_hash(uint32_t in) {
  const uint32_t prime = 16777619u;
  uint32_t h = 2166136261u;
  for (unsigned i = 0; i < 4; ++i) {
    h ^= (in >> (8 * i)) & 0xffu;
    h *= prime;
  }
  return h;
}

struct SobolTable {
  unsigned dimension_bound = 256;
  unsigned initial_dimension_bound = 64;
  std::vector<float> vals;
};

// Sobol point for (dimension, offset): Gray-code ordered scrambled Sobol
// point x = c_d ^ XOR_{bit j of g} v_{d,j}, g = offset ^ (offset >> 1), mapped
// to (0, 1] as (x + 1/2) 2^-32 and with 1.0 replaced by 0.0
// (src/rng/sobel/sobel.cu:59-70, include/lib/cuda/curand_utils.h:58-66)
float sobol_value(const uint32_t *v, uint32_t scramble, uint32_t offset) {
  uint32_t g = offset ^ (offset >> 1);
  uint32_t x = scramble;
  for (unsigned j = 0; j < 32; ++j) {
    if ((g >> j) & 1u) {
      x ^= v[j];
    }
  }
  float f = (float)x * 0x1p-32f + 0x1p-33f;
  return f == 1.0f ? 0.0f : f;
}

bool sobol_table(unsigned dimension_bound, unsigned count, SobolTable &out) {
  curandDirectionVectors32_t *vecs = nullptr;
  unsigned *scr = nullptr;
  if (curandGetDirectionVectors32(
          &vecs, CURAND_SCRAMBLED_DIRECTION_VECTORS_32_JOEKUO6) !=
          CURAND_STATUS_SUCCESS ||
      curandGetScrambleConstants32(&scr) != CURAND_STATUS_SUCCESS) {
    return false;
  }
  out.dimension_bound = dimension_bound;
  out.initial_dimension_bound = std::min(64u, dimension_bound);
  out.vals.resize((size_t)dimension_bound * count);
  for (unsigned i = 0; i < count; ++i) {
    for (unsigned d = 0; d < dimension_bound; ++d) {
      out.vals[(size_t)i * dimension_bound + d] =
          sobol_value(vecs[d], scr[d], i);
    }
  }
  return true;
}

// Sobel (table) or Uniform: include/rng/uniform/uniform.h:18-76 on the CPU
// execution model, std::mt19937 seeded with sample + location x samples_per
// and std::uniform_real_distribution<float>(0, 1).  (The reference's GPU
// execution model draws cuRAND XORWOW for Uniform, so its two models give
// different images; they agree in expectation.)
struct RngState {
  const SobolTable *table;
  unsigned sample;
  unsigned dim;
  bool uniform = false;
  std::mt19937 gen;
  std::uniform_real_distribution<float> dist{0.f, 1.f};
  float next() {
    if (uniform) {
      return dist(gen);
    }
    float out = table->vals[(size_t)sample * table->dimension_bound + dim];
    ++dim;
    dim %= table->dimension_bound;
    return out;
  }
};

void get_generator(const SobolTable &t, unsigned sample_idx, unsigned location,
                   RngState &out) {
  out.table = &t;
  out.sample = sample_idx;
  out.dim = fnv_hash(location) % t.initial_dimension_bound;
}

void get_uniform_generator(unsigned sample_idx, unsigned location, unsigned samples_per,
                           RngState &out) {
  out.uniform = true;
  out.gen.seed(sample_idx + location * samples_per);
}

// ---------------------------------------------------------------------------
// BSDFs: include/bsdf/*.h (+ GGX, new)
enum BSDFType : uint32_t {
  kDiffuse = 0,
  kGlossy = 1,
  kDiffuseGlossy = 2,
  kDiffuseMirror = 3,
  kMirror = 4,
  kDielectric = 5,
  kGGX = 6,
};

struct Material {
  uint32_t type;
  RGB diffuse, specular, emission;
  float shininess, ior, w_d, w_g, roughness;
  // derived (constructors of Glossy, DielectricRefractive, Combined)
  float glossy_norm, inv_shininess_p_1, r0, cont_inclusive0;
};

Material make_material(const oracle_material &m) {
  Material o;
  o.type = m.type;
  o.diffuse = {m.diffuse[0], m.diffuse[1], m.diffuse[2]};
  o.specular = {m.specular[0], m.specular[1], m.specular[2]};
  o.emission = {m.emission[0], m.emission[1], m.emission[2]};
  o.shininess = m.shininess;
  o.ior = m.ior;
  o.w_d = m.diffuse_weight;
  o.w_g = m.glossy_weight;
  o.roughness = m.roughness;
  // glossy.h:19-23
  o.glossy_norm = (o.shininess + 2.f) / (2.f * (float)M_PI);
  o.inv_shininess_p_1 = 1.f / (o.shininess + 1.f);
  // dielectric_refractive.h:15-19
  float r0 = (o.ior - 1) / (o.ior + 1);
  o.r0 = r0 * r0;
  // combined.h:22-47: inclusive continuous weight normalised by the total
  o.cont_inclusive0 = o.w_d / (o.w_d + o.w_g);
  return o;
}

bool is_brdf(const Material &m) { return m.type != kDielectric; }

// union_bsdf.h:47-60 / combined.h:89-104
float prob_continuous(const Material &m) {
  switch (m.type) {
  case kDiffuse:
  case kGlossy:
  case kDiffuseGlossy:
  case kGGX:
    return 1.0f;
  case kMirror:
  case kDielectric:
    return 0.0f;
  default: // DiffuseMirror: fixed probability of the continuous lobe
    return m.w_d;
  }
}

const float kInvPi = (float)(1 / M_PI);

RGB diffuse_eval(RGB albedo) { return albedo * kInvPi; }

RGB glossy_eval(const Material &m, RGB spec, V3 in, V3 out, V3 n) {
  float c = std::max(dot(reflect_over_normal(in, n), out), 0.0f);
  return (spec * m.glossy_norm) * om::pow(c, m.shininess);
}

// GGX microfacet reflection (Walter et al. 2007, "Microfacet Models for
// Refraction through Rough Surfaces"): D GGX, separable Smith G, Schlick F.
float ggx_g1(float c, float a2) {
  return (2.f * c) / (c + pm::sqrt(a2 + (1.f - a2) * (c * c)));
}

RGB schlick(RGB f0, float c) {
  float m = 1.f - c;
  float m2 = m * m;
  float m5 = (m2 * m2) * m;
  return {f0.r + (1.f - f0.r) * m5, f0.g + (1.f - f0.g) * m5,
          f0.b + (1.f - f0.b) * m5};
}

// GGX normal distribution D(h) = a2 / (pi ((n.h)^2 (a2 - 1) + 1)^2)
// (Walter et al. 2007, eq. 33)
float ggx_d(float ch, float a2) {
  float dd = (ch * ch) * (a2 - 1.f) + 1.f;
  return a2 / (((float)M_PI * dd) * dd);
}

RGB ggx_eval(const Material &m, V3 in, V3 out, V3 n) {
  V3 wo = -in;
  if (dot(wo, n) < 0.f) {
    n = -n;
  }
  float co = dot(wo, n);
  float ci = dot(out, n);
  if (!(co > 0.f) || !(ci > 0.f)) {
    return rgb_zero();
  }
  float a = m.roughness;
  float a2 = a * a;
  V3 h = normalized(wo + out);
  float ch = dot(h, n);
  float d = ggx_d(ch, a2);
  float g = ggx_g1(co, a2) * ggx_g1(ci, a2);
  RGB f = schlick(m.specular, dot(wo, h));
  float scale = (d * g) / ((4.f * ci) * co);
  return f * scale;
}

RGB continuous_eval(const Material &m, V3 in, V3 out, V3 n) {
  switch (m.type) {
  case kDiffuse:
    return diffuse_eval(m.diffuse);
  case kGlossy:
    return glossy_eval(m, m.specular, in, out, n);
  case kDiffuseGlossy: {
    // combined.h:68-87: weights are differences of the inclusive sums
    float w0 = m.cont_inclusive0 - 0.f;
    float w1 = 1.f - m.cont_inclusive0;
    return diffuse_eval(m.diffuse) * w0 + glossy_eval(m, m.specular, in, out, n) * w1;
  }
  case kDiffuseMirror:
    return diffuse_eval(m.diffuse) * (1.f - 0.f);
  case kGGX:
    return ggx_eval(m, in, out, n);
  default:
    return rgb_zero();
  }
}

struct BSDFSample {
  V3 dir;
  RGB mult;
};

BSDFSample diffuse_sample(RGB albedo, V3 in, V3 n, RngState &rng) {
  float v0 = rng.next();
  float v1 = rng.next();
  float phi = (float)(2 * M_PI * (double)v0);
  float theta = om::asin(pm::sqrt(v1));
  V3 aligned = n;
  if (dot(in, n) > 0.f) {
    aligned = -n;
  }
  return {find_relative_vec(aligned, phi, theta), albedo};
}

BSDFSample glossy_sample(const Material &m, V3 in, V3 n, RngState &rng) {
  float v0 = rng.next();
  float v1 = rng.next();
  V3 reflection = reflect_over_normal(in, n);
  float phi = (float)(2 * M_PI * (double)v0);
  float psi = om::acos(om::pow(v1, m.inv_shininess_p_1));
  return {find_relative_vec(reflection, phi, psi), m.specular};
}

// orthonormal basis around n (Duff et al. 2017, "Building an Orthonormal
// Basis, Revisited")
void onb(V3 n, V3 &b1, V3 &b2) {
  float sign = n.z >= 0.f ? 1.f : -1.f;
  float a = -1.f / (sign + n.z);
  float b = n.x * n.y * a;
  b1 = {1.f + sign * n.x * n.x * a, sign * b, -sign * n.x};
  b2 = {b, sign + n.y * n.y * a, -n.y};
}

// GGX sampling of the normal distribution D(h)(n.h) (Walter et al. 2007)
BSDFSample ggx_sample(const Material &m, V3 in, V3 n, RngState &rng) {
  float u0 = rng.next();
  float u1 = rng.next();
  V3 wo = -in;
  if (dot(wo, n) < 0.f) {
    n = -n;
  }
  float a = m.roughness;
  float a2 = a * a;
  float phi = (float)(2 * M_PI * (double)u0);
  float tan2 = (a2 * u1) / (1.f - u1);
  float cos_t = 1.f / pm::sqrt(1.f + tan2);
  float sin_t = pm::sqrt(std::max(0.f, 1.f - cos_t * cos_t));
  V3 b1, b2;
  onb(n, b1, b2);
  V3 h = normalized((b1 * (sin_t * om::cos(phi)) + b2 * (sin_t * om::sin(phi))) +
                    n * cos_t);
  float k = 2.f * dot(wo, h);
  V3 wi = normalized(h * k - wo);
  float co = dot(wo, n);
  float ci = dot(wi, n);
  float ch = dot(h, n);
  float oh = dot(wo, h);
  if (!(ci > 0.f) || !(co > 0.f) || !(ch > 0.f) || !(oh > 0.f)) {
    return {wi, rgb_zero()};
  }
  float g = ggx_g1(co, a2) * ggx_g1(ci, a2);
  RGB f = schlick(m.specular, oh);
  float w = (g * oh) / (co * ch);
  return {wi, f * w};
}

BSDFSample continuous_sample(const Material &m, V3 in, V3 n, RngState &rng) {
  switch (m.type) {
  case kDiffuse:
    return diffuse_sample(m.diffuse, in, n, rng);
  case kGlossy:
    return glossy_sample(m, in, n, rng);
  case kDiffuseGlossy: {
    // combined.h:106-121: lobe choice by one draw
    float loc = rng.next();
    if (loc <= m.cont_inclusive0) {
      return diffuse_sample(m.diffuse, in, n, rng);
    }
    return glossy_sample(m, in, n, rng);
  }
  case kDiffuseMirror: {
    (void)rng.next(); // one continuous lobe: the choice draw is still made
    return diffuse_sample(m.diffuse, in, n, rng);
  }
  case kGGX:
    return ggx_sample(m, in, n, rng);
  default:
    return {in, rgb_zero()};
  }
}

BSDFSample discrete_sample(const Material &m, V3 in, V3 n, RngState &rng) {
  switch (m.type) {
  case kMirror:
    return {reflect_over_normal(in, n), m.specular};
  case kDiffuseMirror:
    (void)rng.next(); // combined.h:123-137: one discrete lobe
    return {reflect_over_normal(in, n), m.specular};
  case kDielectric: {
    // dielectric_refractive.h:21-34
    float cos_to_normal = std::fabs(dot(in, n));
    double x = (double)(1 - cos_to_normal);
    double x2 = x * x;
    double p5 = (x2 * x2) * x;
    float prop = (float)((double)m.r0 + (double)(1 - m.r0) * p5);
    if (rng.next() < prop) {
      return {reflect_over_normal(in, n), m.specular};
    }
    return {refract_by_normal(m.ior, in, n), m.specular};
  }
  default:
    return {in, rgb_zero()};
  }
}

// ---------------------------------------------------------------------------
// scene flattening (include/intersectable_scene/flat_triangle/flat_triangle.h
// :79-146) and the light sampler (random_triangle.h:120-161)
struct TriData {
  V3 n[3];
  uint32_t material;
  V3 get_normal(V3 point, const Tri &tri) const {
    float w[3];
    tri.interpolation_values(point, w);
    return normalized((n[0] * w[0] + n[1] * w[1]) + n[2] * w[2]);
  }
};

struct FlatScene {
  std::vector<Tri> tris;         // world space, original order
  std::vector<TriData> data;
  std::vector<Material> materials;
  std::vector<Tri> light_tris;
  std::vector<float> light_cdf;
};

Affine read_affine(const float *p) {
  Affine a;
  std::memcpy(a.m, p, sizeof(a.m));
  return a;
}

V3 read_v3(const float *p) { return {p[0], p[1], p[2]}; }

FlatScene flatten(const oracle_scene &s) {
  FlatScene out;
  for (uint32_t i = 0; i < s.n_materials; ++i) {
    out.materials.push_back(make_material(s.materials[i]));
  }
  for (uint32_t inst = 0; inst < s.n_instances; ++inst) {
    uint32_t mesh = s.instance_mesh[inst];
    Affine xf = read_affine(s.instance_xforms + 12 * inst);
    uint32_t start = mesh == 0 ? 0 : s.mesh_ends[mesh - 1];
    // the reference bounds this loop by mesh_ends[inst]; the mesh's own end
    // is used here (identical when every mesh has one instance)
    uint32_t end = s.mesh_ends[mesh];
    for (uint32_t j = start; j < end; ++j) {
      Tri t;
      TriData d;
      for (int k = 0; k < 3; ++k) {
        t.v[k] = xf.apply(read_v3(s.triangles + 9 * j + 3 * k));
        d.n[k] = normalized(xf.linear(read_v3(s.normals + 9 * j + 3 * k)));
      }
      d.material = s.tri_material[j];
      out.tris.push_back(t);
      out.data.push_back(d);
    }
    // random_triangle.h:129-151
    uint32_t cstart = mesh == 0 ? 0 : s.cluster_ends_per_mesh[mesh - 1];
    uint32_t cend = s.cluster_ends_per_mesh[mesh];
    for (uint32_t c = cstart; c < cend; ++c) {
      uint32_t mat = s.clusters[3 * c + 0];
      for (uint32_t ti = s.clusters[3 * c + 1]; ti < s.clusters[3 * c + 2];
           ++ti) {
        Tri t;
        for (int k = 0; k < 3; ++k) {
          t.v[k] = xf.apply(read_v3(s.triangles + 9 * ti + 3 * k));
        }
        out.light_tris.push_back(t);
        out.light_cdf.push_back(0.f);
      }
      (void)mat;
    }
  }
  // cumulative weights, then normalised
  float cumulative = 0.f;
  size_t li = 0;
  for (uint32_t inst = 0; inst < s.n_instances; ++inst) {
    uint32_t mesh = s.instance_mesh[inst];
    uint32_t cstart = mesh == 0 ? 0 : s.cluster_ends_per_mesh[mesh - 1];
    uint32_t cend = s.cluster_ends_per_mesh[mesh];
    for (uint32_t c = cstart; c < cend; ++c) {
      uint32_t mat = s.clusters[3 * c + 0];
      for (uint32_t ti = s.clusters[3 * c + 1]; ti < s.clusters[3 * c + 2];
           ++ti) {
        float area = norm(out.light_tris[li].normal_scaled_by_area());
        cumulative += area * rgb_sum(out.materials[mat].emission);
        out.light_cdf[li] = cumulative;
        ++li;
      }
    }
  }
  for (float &w : out.light_cdf) {
    w /= cumulative;
  }
  return out;
}

struct LightSample {
  V3 dir;
  float mult;
  float target_distance;
};

// random_triangle.h:35-90
bool sample_light(const FlatScene &sc, V3 position, const Material &mat, V3 normal,
                  RngState &rng, LightSample &out) {
  if (sc.light_cdf.empty()) {
    return false;
  }
  float search_value = rng.next();
  unsigned idx = 0;
  unsigned n = (unsigned)sc.light_cdf.size();
  for (idx = 0; idx < n; ++idx) {
    if (sc.light_cdf[idx] >= search_value) {
      break;
    }
  }
  const Tri &tri = sc.light_tris[idx];
  float s = rng.next();
  float t = rng.next();
  if (s + t > 1.f) {
    s = 1 - s;
    t = 1 - t;
  }
  V3 point = tri.baryo_to_point(s, t);
  V3 dir_un = point - position;
  if (is_brdf(mat) && dot(dir_un, normal) <= 0.f) {
    return false;
  }
  V3 dir = normalized(dir_un);
  V3 tn = tri.normal_scaled_by_area();
  float prob = sc.light_cdf[idx] - (idx == 0 ? 0.f : sc.light_cdf[idx - 1]);
  float nw = std::fabs(dot(normal, dir) * dot(tn, dir));
  if ((double)nw < 1e-8) {
    return false;
  }
  float weight = nw / squared_norm(dir_un);
  out = {dir, prob / weight, norm(dir_un)};
  return true;
}

// term_prob/*: Constant, NIters, MultiplierFunc, Normalize
float term_prob(const oracle_settings &st, unsigned iters, RGB mult) {
  switch (st.term_prob) {
  case 0:
    return st.term_prob_prob;
  case 1:
    return iters >= st.term_prob_iters ? 1.0f : 0.0f;
  case 2: {
    RGB q = {mult.r / (mult.r + 1), mult.g / (mult.g + 1), mult.b / (mult.b + 1)};
    q = q * 0.57f;
    float sq = std::clamp((q.r * q.r + q.g * q.g) + q.b * q.b, 0.0f, 1.0f);
    float p = std::fabs(om::pow(1 - sq, st.term_prob_exp));
    return std::max(p, st.term_prob_min_prob);
  }
  default: {
    float p = 1.f - 1.f / (rgb_sum(mult) / 3.f);
    return std::clamp(p, st.term_prob_min_prob, 1.f);
  }
  }
}

// uniform_direction_sample.h / dir_sampler/uniform/uniform.h
BSDFSample uniform_dir_sample(const Material &m, V3 in, V3 n, RngState &rng) {
  float v0 = rng.next();
  float v1 = rng.next();
  bool whole = !is_brdf(m);
  float phi = (float)(2 * M_PI * (double)v0);
  float theta = om::acos(whole ? 2 * v1 - 1 : v1);
  V3 dir = find_relative_vec(n, phi, theta);
  float inv_prob = (float)((whole ? 4 : 2) * M_PI);
  RGB f = continuous_eval(m, in, dir, n);
  return {dir, (f * dot(dir, n)) * inv_prob};
}

struct Intersector {
  const BVH *bvh;
  Hit intersect(const Ray &r) const { return bvh_intersect(*bvh, r); }
};

// include/render/detail/integrate_image/initial_ray_sample.h:16-56
Ray initial_ray(float x, float y, unsigned x_dim, unsigned y_dim,
                const Affine &f2w) {
  V3 film = {(2.0f * x) / (float)x_dim - 1.0f, (-2.0f * y) / (float)y_dim + 1.0f,
             -1.0f};
  V3 world = f2w.apply(film);
  Ray r;
  r.o = f2w.translation();
  r.d = normalized(world - r.o);
  return r;
}

Ray read_ray(const float *p);

struct RenderCtx {
  const FlatScene *scene;
  const BVH *bvh;
  const oracle_settings *st;
  const SobolTable *sobol;
  Affine f2w;
  unsigned x_dim, y_dim;
  const float *rays = nullptr; // InitialRays / InitialIdxAndDir: one ray per location
  const unsigned *idxs = nullptr; // InitialIdxAndDir: BVH-order hit triangle per location
  unsigned n_steps = 0;           // OutputPerStep: steps per path, 0 = off
  unsigned spp = 0;               // samples per location (Uniform RNG seed)
  unsigned sample_offset = 0;     // Sobol row of sample s is s + sample_offset
};

// rendering_equation.h:27-129 + rendering_equation_iteration.h:9-153 for one
// camera sample, with one light sample per vertex (RandomTriangle) or none.
// With OutputPerStep (steps != nullptr) the radiance gathered in pass k is
// added to steps[k] and the path stops after c.n_steps passes
// (rendering_equation.h:61-124).
RGB integrate_sample(const RenderCtx &c, unsigned sample_idx, unsigned x,
                     unsigned y, RGB *steps = nullptr) {
  const FlatScene &sc = *c.scene;
  const oracle_settings &st = *c.st;
  unsigned location = x + y * c.x_dim;
  RngState rng;
  if (st.rng == 1) {
    // a progressive frame seeds as the kernels do: sample + location x spp
    // + offset x locations (the reference's seed for offset 0)
    get_uniform_generator(sample_idx + c.sample_offset * (c.x_dim * c.y_dim), location, c.spp,
                          rng);
  } else {
    get_generator(*c.sobol, sample_idx + c.sample_offset, location, rng);
  }
  Ray ray;
  if (c.rays != nullptr) {
    // initial_ray_sample.h:47-48: the caller's ray, no RNG draw
    ray = read_ray(c.rays + 6 * (size_t)x);
  } else {
    float xo = rng.next();
    float yo = rng.next();
    ray = initial_ray((float)x + xo, (float)y + yo, c.x_dim, c.y_dim, c.f2w);
  }

  unsigned iters = 0;
  bool count_emission = true;
  bool has_next = true;
  RGB multiplier = {1.f, 1.f, 1.f};
  bool has_light = false;
  Ray light_ray{};
  RGB light_mult = rgb_zero();
  float light_target = 0.f;
  RGB total = rgb_zero();
  const bool performs_samples = st.light_sampler == 0;

  auto include_lighting = [&](const Hit &h) {
    return !st.back_cull_emission || !h.back;
  };
  unsigned step = 0;
  auto end_pass = [&]() {
    if (steps != nullptr) {
      steps[step] = steps[step] + total;
      total = rgb_zero();
    }
    ++step;
  };

  while (true) {
    if (steps != nullptr && step >= c.n_steps) {
      return total;
    }
    // safety bound shared with the kernels (no counterpart in the reference;
    // no path of the tested settings reaches it)
    if (iters >= 4096) {
      return total;
    }
    // intersect all pending rays (light ray first, then the next ray)
    Hit light_hit, next_hit;
    if (has_light) {
      light_hit = bvh_intersect(*c.bvh, light_ray, st.tie_rule != 0);
    }
    if (has_next) {
      if (step == 0 && c.idxs != nullptr) {
        // initial_ray_sample.h:58-74: the caller's hit, distance 1, front
        next_hit.ok = true;
        next_hit.t = 1.f;
        next_hit.back = false;
        next_hit.idx = c.idxs[x];
      } else {
        next_hit = bvh_intersect(*c.bvh, ray, st.tie_rule != 0);
      }
    }
    if (has_light) {
      if (light_hit.ok &&
          (double)std::fabs(light_target - light_hit.t) < 1e-6 &&
          include_lighting(light_hit)) {
        const TriData &d = sc.data[c.bvh->permutation[light_hit.idx]];
        total = total + sc.materials[d.material].emission * light_mult;
      }
    }
    if (!has_next || !next_hit.ok) {
      end_pass();
      return total;
    }
    V3 point = ray.o + ray.d * next_hit.t;
    unsigned orig = c.bvh->permutation[next_hit.idx];
    const TriData &td = sc.data[orig];
    const Material &mat = sc.materials[td.material];
    if ((!performs_samples || count_emission) && include_lighting(next_hit)) {
      total = total + multiplier * mat.emission;
    }
    V3 normal = td.get_normal(point, c.bvh->tris[next_hit.idx]);

    bool new_has_light = false;
    RGB new_light_mult = rgb_zero();
    float new_light_target = 0.f;
    Ray new_light_ray{};
    float pc = prob_continuous(mat);
    if (pc > 0.f && performs_samples) {
      LightSample ls;
      if (sample_light(sc, point, mat, normal, rng, ls)) {
        RGB f = continuous_eval(mat, ray.d, ls.dir, normal);
        new_light_mult = ((multiplier * f) * pc) / ls.mult;
        new_light_target = ls.target_distance;
        new_light_ray = {point, ls.dir};
        new_has_light = true;
      }
    }
    // dir sampler: ref_from_continuous_sampler.h:10-44
    BSDFSample smp;
    bool is_discrete;
    bool take_discrete;
    if (pc == 0.f) {
      take_discrete = true;
    } else if (pc == 1.f) {
      take_discrete = false;
    } else {
      take_discrete = pc < rng.next();
    }
    if (take_discrete) {
      smp = discrete_sample(mat, ray.d, normal, rng);
      is_discrete = true;
    } else {
      smp = st.dir_sampler == 0 ? continuous_sample(mat, ray.d, normal, rng)
                                : uniform_dir_sample(mat, ray.d, normal, rng);
      is_discrete = false;
    }
    RGB new_multiplier = multiplier * smp.mult;
    float p = term_prob(st, iters, new_multiplier);
    bool next = rng.next() > p;
    iters += 1;
    count_emission = is_discrete;
    has_light = new_has_light;
    light_mult = new_light_mult;
    light_target = new_light_target;
    light_ray = new_light_ray;
    if (next) {
      new_multiplier = new_multiplier / (1.0f - p);
      multiplier = new_multiplier;
      ray = {point, smp.dir};
      has_next = true;
    } else {
      has_next = false;
      if (!has_light) {
        end_pass();
        return total;
      }
    }
    end_pass();
  }
}

// ---------------------------------------------------------------------------
// src/kernel/work_division.cpp:12-69, include/kernel/work_division_impl.h
unsigned closest_power_of_2(unsigned n) {
  if (n == 0) {
    return 1;
  }
  unsigned place = 31 - (unsigned)__builtin_clz(n);
  unsigned smaller = 1u << place;
  if (place == 31) {
    return smaller;
  }
  unsigned larger = smaller << 1;
  return (n - smaller <= larger - n) ? smaller : larger;
}

bool power_of_2(unsigned n) { return n != 0 && (n & (n - 1)) == 0; }

bool make_division(const oracle_work_division_settings &s, unsigned spp,
                   unsigned x_dim, unsigned y_dim, oracle_work_division &o) {
  o.block_size = s.block_size;
  if (o.block_size % 32 != 0 || !power_of_2(o.block_size) ||
      !power_of_2(s.target_x_block_size)) {
    return false;
  }
  double target;
  if (s.force_target_samples) {
    target = s.forced_target_samples_per_thread;
  } else {
    double total = ((double)spp * x_dim) * y_dim;
    double ratio = total / s.base_num_threads;
    double base = std::pow(ratio, (double)s.samples_per_thread_scaling_power);
    target = std::min(base, (double)s.max_samples_per_thread);
  }
  unsigned n_threads =
      closest_power_of_2((unsigned)std::round((double)spp / target));
  o.base_samples_per_thread = spp / n_threads;
  o.n_threads_per_unit_extra = spp - o.base_samples_per_thread * n_threads;
  o.sample_block_size = std::min(n_threads, o.block_size);
  unsigned xy = o.block_size / o.sample_block_size;
  o.x_block_size = std::min(xy, s.target_x_block_size);
  o.y_block_size = xy / o.x_block_size;
  o.num_sample_blocks = n_threads / o.sample_block_size;
  o.num_x_blocks = (x_dim + o.x_block_size - 1) / o.x_block_size;
  o.num_y_blocks = (y_dim + o.y_block_size - 1) / o.y_block_size;
  o.x_dim = x_dim;
  o.y_dim = y_dim;
  return true;
}

struct ThreadInfo {
  unsigned start, end, x, y;
  bool exit;
};

ThreadInfo thread_info(const oracle_work_division &w, unsigned block_idx,
                       unsigned thread_idx) {
  unsigned bs = block_idx % w.num_sample_blocks;
  unsigned bl = block_idx / w.num_sample_blocks;
  unsigned bx = bl % w.num_x_blocks;
  unsigned by = bl / w.num_x_blocks;
  unsigned ts = thread_idx % w.sample_block_size;
  unsigned tl = thread_idx / w.sample_block_size;
  unsigned tx = tl % w.x_block_size;
  unsigned ty = tl / w.x_block_size;
  unsigned sample_idx = ts + bs * w.sample_block_size;
  ThreadInfo o;
  o.x = tx + bx * w.x_block_size;
  o.y = ty + by * w.y_block_size;
  unsigned before = sample_idx * w.base_samples_per_thread;
  unsigned extra_before = std::min(w.n_threads_per_unit_extra, sample_idx);
  o.start = before + extra_before;
  unsigned n = w.base_samples_per_thread +
               (sample_idx < w.n_threads_per_unit_extra ? 1 : 0);
  o.end = o.start + n;
  o.exit = o.x >= w.x_dim || o.y >= w.y_dim;
  return o;
}

unsigned total_blocks(const oracle_work_division &w) {
  return w.num_sample_blocks * w.num_x_blocks * w.num_y_blocks;
}

// GPU shuffle-tree order of sub_block_reduce (include/lib/cuda/reduce.cuh:
// 35-102): val = shuffle_down(val) + val per step; cross-warp through shared
template <typename T, typename Add>
T tree_reduce(const T *vals, unsigned block_size, unsigned sub_block_size,
              unsigned thread_idx, Add add) {
  // emulate every lane of the block, then read the lane we need
  std::vector<T> v(vals, vals + block_size);
  unsigned width = std::min(sub_block_size, 32u);
  auto warp_reduce = [&](std::vector<T> &lanes, unsigned w) {
    for (unsigned off = w / 2; off > 0; off /= 2) {
      std::vector<T> next = lanes;
      for (unsigned l = 0; l < lanes.size(); ++l) {
        unsigned seg_lane = l % w;
        T other = (seg_lane + off < w) ? lanes[l + off] : lanes[l];
        next[l] = add(other, lanes[l]);
      }
      lanes = next;
    }
  };
  // per warp (lanes segmented by width inside each warp)
  warp_reduce(v, width);
  if (sub_block_size <= 32) {
    return v[thread_idx];
  }
  unsigned n_warps = block_size / 32;
  std::vector<T> shared(n_warps);
  for (unsigned w = 0; w < n_warps; ++w) {
    shared[w] = v[w * 32];
  }
  unsigned per_group = sub_block_size / 32;
  std::vector<T> v2 = v;
  for (unsigned t = 0; t < block_size; ++t) {
    unsigned sbt = t % sub_block_size;
    unsigned sbi = t / sub_block_size;
    unsigned lane = t % 32;
    if (sbt < per_group) {
      v2[t] = shared[lane + sbi * per_group];
    }
  }
  // final reduce of width per_group, inside each warp
  for (unsigned off = per_group / 2; off > 0; off /= 2) {
    std::vector<T> next = v2;
    for (unsigned l = 0; l < block_size; ++l) {
      unsigned lane = l % 32;
      unsigned seg_lane = lane % per_group;
      T other = (seg_lane + off < per_group) ? v2[l + off] : v2[l];
      next[l] = add(other, v2[l]);
    }
    v2 = next;
  }
  return v2[thread_idx];
}

struct Reducer {
  unsigned reduction_factor;
  unsigned order;
};

// one "kernel launch" of the CPU execution model
// (include/kernel/kernel_launch_impl_cpu.h:10-26): blocks in parallel,
// threads of a block in order; each thread yields n_vals values, each
// reduced over reduction_factor lanes (runtime_constants_reducer.h:46-62
// for CPU order) and handed to out_fn(block, info, value index, total)
template <typename ThreadFn, typename OutFn>
void run_blocks_n(const oracle_work_division &w, unsigned n_threads_omp,
                  unsigned order, unsigned n_vals, ThreadFn thread_fn, OutFn out_fn) {
  unsigned nb = total_blocks(w);
  int nt = n_threads_omp ? (int)n_threads_omp : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (unsigned block = 0; block < nb; ++block) {
    // vals[k * block_size + t]: value k of thread t
    std::vector<RGB> vals((size_t)n_vals * w.block_size, rgb_zero());
    std::vector<RGB> mine(n_vals);
    std::vector<ThreadInfo> infos(w.block_size);
    for (unsigned t = 0; t < w.block_size; ++t) {
      infos[t] = thread_info(w, block, t);
      if (!infos[t].exit) {
        std::fill(mine.begin(), mine.end(), rgb_zero());
        thread_fn(block, infos[t], mine.data());
        for (unsigned k = 0; k < n_vals; ++k) {
          vals[(size_t)k * w.block_size + t] = mine[k];
        }
      }
    }
    unsigned rf = w.sample_block_size;
    auto add = [](RGB a, RGB b) { return a + b; };
    for (unsigned k = 0; k < n_vals; ++k) {
      const RGB *v = vals.data() + (size_t)k * w.block_size;
      for (unsigned t = 0; t < w.block_size; t += rf) {
        if (infos[t].exit) {
          continue;
        }
        RGB total;
        if (order == 0) {
          total = v[t];
          for (unsigned j = 1; j < rf; ++j) {
            total = add(total, v[t + j]);
          }
        } else {
          total = tree_reduce(v, w.block_size, rf, t, add);
        }
        out_fn(block, infos[t], k, total);
      }
    }
  }
}

template <typename ThreadFn, typename OutFn>
void run_blocks(const oracle_work_division &w, unsigned n_threads_omp,
                unsigned order, ThreadFn thread_fn, OutFn out_fn) {
  run_blocks_n(
      w, n_threads_omp, order, 1,
      [&](unsigned block, const ThreadInfo &ti, RGB *out) { out[0] = thread_fn(block, ti); },
      [&](unsigned block, const ThreadInfo &ti, unsigned, RGB total) {
        out_fn(block, ti, total);
      });
}

struct RenderOut {
  std::vector<RGB> rgb; // x_dim * y_dim
};

// include/render/detail/integrate_image/assign_output.h:11-31 and
// mega_kernel/reduce_float_rgb_impl.h:17-63
struct SpecExtras {
  const float *rays = nullptr;      // InitialRays / InitialIdxAndDir
  const uint32_t *idxs = nullptr;   // InitialIdxAndDir, scene-order triangles
  unsigned n_steps = 0;             // OutputPerStep
};

// The flattened scene and its SBVH, built once for renders that share the
// scene and the accel settings (flat_triangle.h:79-146, generator.cu:17-66).
struct Prepared {
  FlatScene sc;
  BVH bvh;
  oracle_settings st; // the settings the BVH and light table were built with
};

void prepare(const oracle_scene &scene, const oracle_settings &st, Prepared &out) {
  out.sc = flatten(scene);
  if (st.light_sampler != 0) {
    out.sc.light_tris.clear();
    out.sc.light_cdf.clear();
  }
  out.bvh = build_bvh(out.sc.tris, st.overlap_threshold, st.use_spatial_splits != 0,
                      st.traversal_per_intersect_cost, st.target_objects);
  out.st = st;
}

// which rows of the image a render covers: row_start, row_start + stride, ...
// below row_end
struct RowSet {
  unsigned start = 0, end = 0, stride = 1;
  bool has(unsigned y) const {
    return y >= start && y < end && (y - start) % stride == 0;
  }
};

bool render_prepared(const Prepared &pr, const oracle_settings &st, unsigned spp,
                     unsigned x_dim, unsigned y_dim, const float *f2w, RowSet rows,
                     unsigned sample_offset, RenderOut &out, double *seconds,
                     const SpecExtras &ex = SpecExtras());

bool render_image(const oracle_scene &scene, const oracle_settings &st,
                  unsigned spp, unsigned x_dim, unsigned y_dim,
                  const float *f2w, unsigned row_start, unsigned row_end,
                  RenderOut &out, double *seconds, const SpecExtras &ex = SpecExtras()) {
  Prepared pr;
  prepare(scene, st, pr);
  RowSet rows;
  rows.start = row_start;
  rows.end = row_end;
  return render_prepared(pr, st, spp, x_dim, y_dim, f2w, rows, 0, out, seconds, ex);
}

bool render_prepared(const Prepared &pr, const oracle_settings &st, unsigned spp,
                     unsigned x_dim, unsigned y_dim, const float *f2w, RowSet rows,
                     unsigned sample_offset, RenderOut &out, double *seconds,
                     const SpecExtras &ex) {
  const FlatScene &sc = pr.sc;
  const BVH &bvh = pr.bvh;
  SobolTable sobol;
  if (!sobol_table(st.max_sample_size, sample_offset + spp, sobol)) {
    return false;
  }
  oracle_work_division w;
  if (!make_division(st.render_wd, spp, x_dim, y_dim, w)) {
    return false;
  }
  float identity[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  std::vector<unsigned> bvh_idxs;
  if (ex.idxs != nullptr) {
    std::vector<unsigned> orig_to_bvh(bvh.permutation.size());
    for (size_t i = 0; i < bvh.permutation.size(); ++i) {
      orig_to_bvh[bvh.permutation[i]] = (unsigned)i;
    }
    bvh_idxs.resize(x_dim);
    for (unsigned i = 0; i < x_dim; ++i) {
      if (ex.idxs[i] >= orig_to_bvh.size()) {
        return false;
      }
      bvh_idxs[i] = orig_to_bvh[ex.idxs[i]];
    }
  }
  RenderCtx ctx{&sc,    &bvh,  &st, &sobol, read_affine(f2w ? f2w : identity), x_dim, y_dim,
                ex.rays, ex.idxs ? bvh_idxs.data() : nullptr, ex.n_steps, spp, sample_offset};
  const unsigned n_out = ex.n_steps ? ex.n_steps : 1;
  const size_t n_pix = (size_t)x_dim * y_dim;
  auto t0 = std::chrono::steady_clock::now();
  unsigned nsb = w.num_sample_blocks;
  // partial[k][...]: output step k (one image unless OutputPerStep)
  std::vector<std::vector<RGB>> partial(n_out,
                                        std::vector<RGB>((size_t)nsb * n_pix, rgb_zero()));
  run_blocks_n(
      w, st.n_threads, st.reduce_order, n_out,
      [&](unsigned, const ThreadInfo &ti, RGB *vals) {
        if (!rows.has(ti.y)) {
          return;
        }
        if (ex.n_steps) {
          for (unsigned s = ti.start; s < ti.end; ++s) {
            integrate_sample(ctx, s, ti.x, ti.y, vals);
          }
          return;
        }
        RGB total = rgb_zero();
        for (unsigned s = ti.start; s < ti.end; ++s) {
          total = total + integrate_sample(ctx, s, ti.x, ti.y);
        }
        vals[0] = total;
      },
      [&](unsigned block, const ThreadInfo &ti, unsigned k, RGB total) {
        unsigned sb = block % nsb;
        size_t idx = sb + (size_t)nsb * (ti.x + ti.y * x_dim);
        if (nsb == 1) {
          total = total / (float)spp;
        }
        partial[k][idx] = total;
      });
  out.rgb.assign(n_out * n_pix, rgb_zero());
  for (unsigned k = 0; k < n_out; ++k) {
    // ReduceFloatRGB: repeated WorkDivision over the partial sums
    unsigned reduction_factor = nsb;
    std::vector<RGB> in = partial[k];
    while (reduction_factor != 1) {
      unsigned xd = (unsigned)(in.size() / reduction_factor);
      oracle_work_division rw;
      if (!make_division(st.reduce_wd, reduction_factor, xd, 1, rw)) {
        return false;
      }
      unsigned rnsb = rw.num_sample_blocks;
      std::vector<RGB> next((size_t)xd * rnsb, rgb_zero());
      run_blocks(
          rw, st.n_threads, st.reduce_order,
          [&](unsigned, const ThreadInfo &ti) -> RGB {
            RGB total = rgb_zero();
            for (unsigned i = ti.start; i < ti.end; ++i) {
              total = total + in[i + (size_t)ti.x * reduction_factor];
            }
            return total;
          },
          [&](unsigned block, const ThreadInfo &ti, RGB total) {
            unsigned sb = block % rnsb;
            size_t idx = sb + (size_t)rnsb * ti.x;
            if (rnsb == 1) {
              total = total / (float)spp;
            }
            next[idx] = total;
          });
      reduction_factor = rnsb;
      in.swap(next);
    }
    for (size_t i = 0; i < n_pix; ++i) {
      out.rgb[k * n_pix + i] = in[i];
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) {
    *seconds = std::chrono::duration<double>(t1 - t0).count();
  }
  return true;
}

// selected rows in order
std::vector<unsigned> row_list(RowSet rows) {
  std::vector<unsigned> out;
  for (unsigned y = rows.start; y < rows.end; y += rows.stride) {
    out.push_back(y);
  }
  return out;
}

// Per-pixel loop shared by the FP64 and per-sample modes: fn(ctx, x, y, row
// index) for every pixel of the selected rows, pixels in parallel.
template <typename PixelFn>
bool for_pixels(const Prepared &pr, const oracle_settings &st, unsigned spp, unsigned x_dim,
                unsigned y_dim, const float *f2w, RowSet rows, unsigned sample_offset,
                double *seconds, PixelFn fn) {
  SobolTable sobol;
  if (!sobol_table(st.max_sample_size, sample_offset + spp, sobol)) {
    return false;
  }
  RenderCtx ctx{&pr.sc, &pr.bvh, &st, &sobol, read_affine(f2w), x_dim, y_dim};
  ctx.spp = spp;
  ctx.sample_offset = sample_offset;
  std::vector<unsigned> ys = row_list(rows);
  const long n = (long)ys.size() * x_dim;
  int nt = st.n_threads ? (int)st.n_threads : omp_get_max_threads();
  auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
  for (long i = 0; i < n; ++i) {
    unsigned r = (unsigned)(i / x_dim);
    unsigned x = (unsigned)(i % x_dim);
    fn(ctx, x, ys[r], r);
  }
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) {
    *seconds = std::chrono::duration<double>(t1 - t0).count();
  }
  return true;
}

bool settings_match_prepared(const Prepared &pr, const oracle_settings &st) {
  return pr.st.overlap_threshold == st.overlap_threshold &&
         pr.st.use_spatial_splits == st.use_spatial_splits &&
         pr.st.traversal_per_intersect_cost == st.traversal_per_intersect_cost &&
         pr.st.target_objects == st.target_objects && pr.st.light_sampler == st.light_sampler;
}

std::vector<Tri> read_tris(const float *p, size_t n) {
  std::vector<Tri> out(n);
  for (size_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      out[i].v[k] = read_v3(p + 9 * i + 3 * k);
    }
  }
  return out;
}

Ray read_ray(const float *p) { return {read_v3(p), read_v3(p + 3)}; }

} // namespace

// ---------------------------------------------------------------------------
extern "C" {

void oracle_pmath(int fn, const float *x, const float *y, float *out,
                  size_t n) {
  for (size_t i = 0; i < n; ++i) {
    switch (fn) {
    case 0:
      out[i] = pm::sin(x[i]);
      break;
    case 1:
      out[i] = pm::cos(x[i]);
      break;
    case 2:
      out[i] = pm::asin(x[i]);
      break;
    case 3:
      out[i] = pm::acos(x[i]);
      break;
    default:
      out[i] = pm::pow(x[i], y[i]);
      break;
    }
  }
}

void oracle_triangle_intersect(const float *tris, const float *rays, size_t n,
                               float *t_out, int32_t *is_back_out) {
  std::vector<Tri> t = read_tris(tris, n);
  for (size_t i = 0; i < n; ++i) {
    Hit h = tri_intersect(t[i], read_ray(rays + 6 * i));
    t_out[i] = h.ok ? h.t : std::numeric_limits<float>::quiet_NaN();
    is_back_out[i] = h.ok ? (h.back ? 1 : 0) : -1;
  }
}

// include/intersect/accel/loop_all/loop_all.h:15-42
void oracle_loop_all(const float *tris, uint32_t n_tris, const float *rays,
                     size_t n_rays, int32_t *idx_out, float *t_out) {
  std::vector<Tri> t = read_tris(tris, n_tris);
#pragma omp parallel for schedule(static)
  for (size_t r = 0; r < n_rays; ++r) {
    Ray ray = read_ray(rays + 6 * r);
    Hit best;
    for (uint32_t i = 0; i < n_tris; ++i) {
      Hit h = tri_intersect(t[i], ray);
      h.idx = i;
      fold_min(best, h);
    }
    idx_out[r] = best.ok ? (int32_t)best.idx : -1;
    t_out[r] = best.ok ? best.t : std::numeric_limits<float>::quiet_NaN();
  }
}

void *oracle_sbvh_build(const float *tris, uint32_t n_tris,
                        float overlap_threshold, uint32_t use_spatial_splits,
                        float traversal_per_intersect_cost,
                        uint32_t target_objects) {
  BVH *b = new BVH(build_bvh(read_tris(tris, n_tris), overlap_threshold,
                             use_spatial_splits != 0,
                             traversal_per_intersect_cost, target_objects));
  return b;
}

void oracle_sbvh_free(void *h) { delete static_cast<BVH *>(h); }

void oracle_sbvh_sizes(void *h, uint32_t *sizes) {
  BVH *b = static_cast<BVH *>(h);
  sizes[0] = (uint32_t)b->nodes.size();
  sizes[1] = (uint32_t)b->extra_idxs.size();
  sizes[2] = (uint32_t)b->permutation.size();
}

void oracle_sbvh_export(void *h, uint32_t *node_words, float *node_aabbs,
                        uint32_t *extra_idxs, uint32_t *permutation) {
  BVH *b = static_cast<BVH *>(h);
  for (size_t i = 0; i < b->nodes.size(); ++i) {
    node_words[2 * i] = b->nodes[i].w0;
    node_words[2 * i + 1] = b->nodes[i].w1;
    const AABB &a = b->nodes[i].aabb;
    float v[6] = {a.lo.x, a.lo.y, a.lo.z, a.hi.x, a.hi.y, a.hi.z};
    std::memcpy(node_aabbs + 6 * i, v, sizeof(v));
  }
  std::copy(b->extra_idxs.begin(), b->extra_idxs.end(), extra_idxs);
  std::copy(b->permutation.begin(), b->permutation.end(), permutation);
}

void oracle_bvh_intersect(void *h, const float *rays, size_t n_rays,
                          int32_t *idx_out, float *t_out) {
  BVH *b = static_cast<BVH *>(h);
#pragma omp parallel for schedule(static)
  for (size_t r = 0; r < n_rays; ++r) {
    Hit best = bvh_intersect(*b, read_ray(rays + 6 * r));
    idx_out[r] = best.ok ? (int32_t)b->permutation[best.idx] : -1;
    t_out[r] = best.ok ? best.t : std::numeric_limits<float>::quiet_NaN();
  }
}

float oracle_sah_cost(void *h, float traversal_per_intersect_cost) {
  BVH *b = static_cast<BVH *>(h);
  if (b->nodes.empty()) {
    return 0.f;
  }
  return sah_cost_impl(*b, traversal_per_intersect_cost, 0);
}

void oracle_clipped_new_bounds(const float *tri, const float *bounds,
                               float left, float right, uint32_t axis,
                               float *out) {
  ClippedTriangle ct;
  ct.triangle = read_tris(tri, 1)[0];
  ct.bounds = {read_v3(bounds), read_v3(bounds + 3)};
  AABB r = ct.new_bounds(left, right, axis);
  float v[6] = {r.lo.x, r.lo.y, r.lo.z, r.hi.x, r.hi.y, r.hi.z};
  std::memcpy(out, v, sizeof(v));
}

void oracle_rotate_to(const float *inp, const float *target, float *out) {
  V3 r = rotate_to(read_v3(inp), read_v3(target), 1.f);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
}

void oracle_find_relative_vec(const float *vec, float phi, float theta,
                              float *out) {
  V3 r = find_relative_vec(read_v3(vec), phi, theta);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
}

int oracle_work_division_make(const oracle_work_division_settings *s,
                              uint32_t samples_per, uint32_t x_dim,
                              uint32_t y_dim, oracle_work_division *out) {
  return make_division(*s, samples_per, x_dim, y_dim, *out) ? 0 : 1;
}

void oracle_work_division_thread_info(const oracle_work_division *wd,
                                      uint32_t block_idx, uint32_t thread_idx,
                                      uint32_t *out) {
  ThreadInfo t = thread_info(*wd, block_idx, thread_idx);
  out[0] = t.start;
  out[1] = t.end;
  out[2] = t.x;
  out[3] = t.y;
  out[4] = t.exit ? 1 : 0;
}

void oracle_sub_block_reduce(const float *vals, uint32_t n_blocks,
                             uint32_t block_size, uint32_t sub_block_size,
                             uint32_t order, float *out) {
  auto add = [](float a, float b) { return a + b; };
  for (uint32_t b = 0; b < n_blocks; ++b) {
    const float *v = vals + (size_t)b * block_size;
    for (uint32_t t = 0; t < block_size; t += sub_block_size) {
      float total;
      if (order == 0) {
        total = v[t];
        for (uint32_t k = 1; k < sub_block_size; ++k) {
          total = add(total, v[t + k]);
        }
      } else {
        total = tree_reduce(v, block_size, sub_block_size, t, add);
      }
      out[((size_t)b * block_size + t) / sub_block_size] = total;
    }
  }
}

int oracle_sobol_table(uint32_t dimension_bound, uint32_t count, float *out) {
  SobolTable t;
  if (!sobol_table(dimension_bound, count, t)) {
    return 1;
  }
  std::copy(t.vals.begin(), t.vals.end(), out);
  return 0;
}

int oracle_render(const oracle_scene *scene, const oracle_settings *settings,
                  uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                  const float *film_to_world, uint32_t row_start,
                  uint32_t row_end, float *out, double *seconds) {
  RenderOut r;
  if (!render_image(*scene, *settings, samples_per, x_dim, y_dim,
                    film_to_world, row_start, row_end, r, seconds)) {
    return 1;
  }
  for (size_t i = 0; i < r.rgb.size(); ++i) {
    unsigned y = (unsigned)(i / x_dim);
    if (y < row_start || y >= row_end) {
      continue;
    }
    out[3 * i] = r.rgb[i].r;
    out[3 * i + 1] = r.rgb[i].g;
    out[3 * i + 2] = r.rgb[i].b;
  }
  return 0;
}

// include/lib/bgra_32.h:12-31 with tone_map v / (v + 1)
// InitialRays (idxs == NULL) and InitialIdxAndDir sample specs: location x
// renders entry x (x_dim = n_rays, y_dim = 1, mega_kernel/run_impl.h:56-67).
// n_steps == 0: out = [n_rays][3]; OutputPerStep: out = [n_steps][n_rays][3]
int oracle_render_rays(const oracle_scene *scene, const oracle_settings *settings,
                       uint32_t samples_per, const float *rays, const uint32_t *idxs,
                       uint32_t n_rays, uint32_t n_steps, float *out) {
  RenderOut r;
  SpecExtras ex;
  ex.rays = rays;
  ex.idxs = idxs;
  ex.n_steps = n_steps;
  if (!render_image(*scene, *settings, samples_per, n_rays, 1, nullptr, 0, 1, r, nullptr, ex)) {
    return 1;
  }
  for (size_t i = 0; i < r.rgb.size(); ++i) {
    out[3 * i] = r.rgb[i].r;
    out[3 * i + 1] = r.rgb[i].g;
    out[3 * i + 2] = r.rgb[i].b;
  }
  return 0;
}

// OutputPerStep of a square image: out = [n_steps][y_dim * x_dim][3]
int oracle_render_steps(const oracle_scene *scene, const oracle_settings *settings,
                        uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                        const float *film_to_world, uint32_t n_steps, float *out) {
  RenderOut r;
  SpecExtras ex;
  ex.n_steps = n_steps;
  if (n_steps == 0 || !render_image(*scene, *settings, samples_per, x_dim, y_dim,
                                    film_to_world, 0, y_dim, r, nullptr, ex)) {
    return 1;
  }
  for (size_t i = 0; i < r.rgb.size(); ++i) {
    out[3 * i] = r.rgb[i].r;
    out[3 * i + 1] = r.rgb[i].g;
    out[3 * i + 2] = r.rgb[i].b;
  }
  return 0;
}

int oracle_render_bgra(const oracle_scene *scene,
                       const oracle_settings *settings, uint32_t samples_per,
                       uint32_t x_dim, uint32_t y_dim,
                       const float *film_to_world, uint8_t *out) {
  RenderOut r;
  if (!render_image(*scene, *settings, samples_per, x_dim, y_dim,
                    film_to_world, 0, y_dim, r, nullptr)) {
    return 1;
  }
  for (size_t i = 0; i < r.rgb.size(); ++i) {
    RGB v = r.rgb[i];
    RGB tm = {v.r / (v.r + 1), v.g / (v.g + 1), v.b / (v.b + 1)};
    out[4 * i + 0] = (uint8_t)(tm.b * 255.0f);
    out[4 * i + 1] = (uint8_t)(tm.g * 255.0f);
    out[4 * i + 2] = (uint8_t)(tm.r * 255.0f);
    out[4 * i + 3] = 0;
  }
  return 0;
}

// src/scene/camera.cpp:4-27: film_to_world = (scale * view)^-1 with
// s = f x up, u = s x f, view rows (s, -s.pos), (u, -u.pos), (-f, f.pos),
// scale = diag(1 / tan_w, 1 / tan_h, 1); evaluated in double from the float
// vectors and rounded to float (Eigen's float 4x4 inverse is not restated).
void oracle_camera_transform(const float *look, const float *up, const float *pos,
                             float height_angle_deg, float width_height_ratio, float *out) {
  V3 f = normalized(read_v3(look));
  V3 u0 = normalized(read_v3(up));
  V3 p = read_v3(pos);
  V3 s = cross(f, u0);
  V3 u = cross(s, f);
  float half = (float)M_PI * height_angle_deg / 360.f;
  double tan_h = std::tan((double)half);
  double tan_w = (double)width_height_ratio * tan_h;
  double sc[3] = {1.0 / tan_w, 1.0 / tan_h, 1.0};
  double rows[3][4] = {{s.x, s.y, s.z, -(double)dot(s, p)},
                       {u.x, u.y, u.z, -(double)dot(u, p)},
                       {-f.x, -f.y, -f.z, (double)dot(f, p)}};
  double r[3][3], t[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      r[i][j] = rows[i][j] * sc[i];
    }
    t[i] = rows[i][3] * sc[i];
  }
  // inverse of [r t; 0 1] = [r^-1, -r^-1 t], r^-1 by cofactors
  double det = r[0][0] * (r[1][1] * r[2][2] - r[1][2] * r[2][1]) -
               r[0][1] * (r[1][0] * r[2][2] - r[1][2] * r[2][0]) +
               r[0][2] * (r[1][0] * r[2][1] - r[1][1] * r[2][0]);
  double inv[3][3] = {
      {(r[1][1] * r[2][2] - r[1][2] * r[2][1]) / det, (r[0][2] * r[2][1] - r[0][1] * r[2][2]) / det,
       (r[0][1] * r[1][2] - r[0][2] * r[1][1]) / det},
      {(r[1][2] * r[2][0] - r[1][0] * r[2][2]) / det, (r[0][0] * r[2][2] - r[0][2] * r[2][0]) / det,
       (r[0][2] * r[1][0] - r[0][0] * r[1][2]) / det},
      {(r[1][0] * r[2][1] - r[1][1] * r[2][0]) / det, (r[0][1] * r[2][0] - r[0][0] * r[2][1]) / det,
       (r[0][0] * r[1][1] - r[0][1] * r[1][0]) / det}};
  for (int i = 0; i < 3; ++i) {
    double ti = -(inv[i][0] * t[0] + inv[i][1] * t[1] + inv[i][2] * t[2]);
    for (int j = 0; j < 3; ++j) {
      out[4 * i + j] = (float)inv[i][j];
    }
    out[4 * i + 3] = (float)ti;
  }
}

int oracle_debug_bsdf(const oracle_material *material, uint32_t op, const float *in,
                      uint32_t n, float *out) {
  Material m = make_material(*material);
  SobolTable draws;
  draws.dimension_bound = 4;
  draws.initial_dimension_bound = 4;
  for (uint32_t i = 0; i < n; ++i) {
    const float *a = in + (size_t)9 * i;
    if (op == 0) {
      RGB f = continuous_eval(m, read_v3(a), read_v3(a + 3), read_v3(a + 6));
      out[3 * i] = f.r;
      out[3 * i + 1] = f.g;
      out[3 * i + 2] = f.b;
    } else if (op == 1) {
      draws.vals.assign(a + 6, a + 9);
      draws.vals.push_back(0.f);
      RngState rng;
      rng.table = &draws;
      rng.sample = 0;
      rng.dim = 0;
      BSDFSample smp = continuous_sample(m, read_v3(a), read_v3(a + 3), rng);
      float *o = out + (size_t)6 * i;
      o[0] = smp.dir.x;
      o[1] = smp.dir.y;
      o[2] = smp.dir.z;
      o[3] = smp.mult.r;
      o[4] = smp.mult.g;
      o[5] = smp.mult.b;
    } else if (op == 2) {
      out[i] = ggx_d(a[0], a[1] * a[1]);
    } else {
      return 1;
    }
  }
  return 0;
}

void *oracle_prepare(const oracle_scene *scene, const oracle_settings *settings) {
  Prepared *p = new Prepared();
  prepare(*scene, *settings, *p);
  return p;
}

void oracle_prepared_free(void *p) { delete static_cast<Prepared *>(p); }

int oracle_render_prepared(void *prepared, const oracle_settings *settings,
                           uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                           const float *film_to_world, const oracle_render_options *opt,
                           float *out, double *out_f64, double *seconds) {
  const Prepared &pr = *static_cast<const Prepared *>(prepared);
  if (!settings_match_prepared(pr, *settings)) {
    return 2;
  }
  RowSet rows;
  rows.start = opt->row_start;
  rows.end = opt->row_end ? std::min(opt->row_end, y_dim) : y_dim;
  rows.stride = opt->row_stride ? opt->row_stride : 1;
  const unsigned off = opt->sample_offset;
  const unsigned spp = samples_per;
  if (spp == 0 || x_dim == 0 || y_dim == 0 || film_to_world == nullptr) {
    return 1;
  }
  if (opt->mode == 0) {
    RenderOut r;
    if (!render_prepared(pr, *settings, spp, x_dim, y_dim, film_to_world, rows, off, r,
                         seconds)) {
      return 1;
    }
    for (size_t i = 0; i < r.rgb.size(); ++i) {
      if (!rows.has((unsigned)(i / x_dim))) {
        continue;
      }
      out[3 * i] = r.rgb[i].r;
      out[3 * i + 1] = r.rgb[i].g;
      out[3 * i + 2] = r.rgb[i].b;
    }
    return 0;
  }
  if (opt->mode == 1) {
    // FP64 accumulation: each sample's radiance summed per pixel in double
    bool ok = for_pixels(pr, *settings, spp, x_dim, y_dim, film_to_world, rows, off, seconds,
                         [&](const RenderCtx &ctx, unsigned x, unsigned y, unsigned) {
                           double a = 0, b = 0, c = 0;
                           for (unsigned s = 0; s < spp; ++s) {
                             RGB v = integrate_sample(ctx, s, x, y);
                             a += (double)v.r;
                             b += (double)v.g;
                             c += (double)v.b;
                           }
                           size_t i = 3 * ((size_t)x + (size_t)y * x_dim);
                           out_f64[i] = a / spp;
                           out_f64[i + 1] = b / spp;
                           out_f64[i + 2] = c / spp;
                         });
    return ok ? 0 : 1;
  }
  if (opt->mode == 2) {
    // per-sample radiance [selected row][x][sample][3]
    bool ok = for_pixels(pr, *settings, spp, x_dim, y_dim, film_to_world, rows, off, seconds,
                         [&](const RenderCtx &ctx, unsigned x, unsigned y, unsigned r) {
                           float *o = out + 3 * (((size_t)r * x_dim + x) * spp);
                           for (unsigned s = 0; s < spp; ++s) {
                             RGB v = integrate_sample(ctx, s, x, y);
                             o[3 * s] = v.r;
                             o[3 * s + 1] = v.g;
                             o[3 * s + 2] = v.b;
                           }
                         });
    return ok ? 0 : 1;
  }
  return 1;
}

int oracle_render_samples(const oracle_scene *scene,
                          const oracle_settings *settings,
                          uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                          const float *film_to_world, uint32_t x, uint32_t y,
                          float *out) {
  FlatScene sc = flatten(*scene);
  if (settings->light_sampler != 0) {
    sc.light_tris.clear();
    sc.light_cdf.clear();
  }
  BVH bvh = build_bvh(sc.tris, settings->overlap_threshold,
                      settings->use_spatial_splits != 0,
                      settings->traversal_per_intersect_cost,
                      settings->target_objects);
  SobolTable sobol;
  if (!sobol_table(settings->max_sample_size, samples_per, sobol)) {
    return 1;
  }
  RenderCtx ctx{&sc, &bvh, settings, &sobol, read_affine(film_to_world),
                x_dim, y_dim};
  for (uint32_t s = 0; s < samples_per; ++s) {
    RGB v = integrate_sample(ctx, s, x, y);
    out[3 * s] = v.r;
    out[3 * s + 1] = v.g;
    out[3 * s + 2] = v.b;
  }
  return 0;
}

} // extern "C"
