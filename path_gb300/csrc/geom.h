// Vector, ray, box and triangle arithmetic shared by the host code and the
// kernels of the render path.
//
// Evaluation order is fixed (dot = (x x' + y y') + z z', affine rows
// ((m0 x + m1 y) + m2 z) + t) and no operation may be contracted into a fused
// multiply-add, so host and device produce the same bits.  The functions
// restate the arithmetic of include/intersect/triangle_impl.h,
// include/intersect/accel/aabb.h and Eigen's normalized().
#pragma once

#include "pmath.h"

#include <stdint.h>

namespace pg {

struct f3 {
  float x, y, z;
  PM_HDM float get(int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  PM_HDM void set(int i, float v) {
    if (i == 0) {
      x = v;
    } else if (i == 1) {
      y = v;
    } else {
      z = v;
    }
  }
};

PM_HD f3 mk(float x, float y, float z) {
  f3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
PM_HD f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
PM_HD f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
PM_HD f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
PM_HD f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
PM_HD f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
PM_HD f3 hmul(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
PM_HD float fmin2(float a, float b) { return b < a ? b : a; }
PM_HD float fmax2(float a, float b) { return a < b ? b : a; }
PM_HD f3 vmin(f3 a, f3 b) { return mk(fmin2(a.x, b.x), fmin2(a.y, b.y), fmin2(a.z, b.z)); }
PM_HD f3 vmax(f3 a, f3 b) { return mk(fmax2(a.x, b.x), fmax2(a.y, b.y), fmax2(a.z, b.z)); }
PM_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PM_HD f3 cross(f3 a, f3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
PM_HD float sqnorm(f3 a) { return dot(a, a); }
PM_HD float length(f3 a) { return pm::sqrt(sqnorm(a)); }
PM_HD f3 normalize(f3 a) {
  float n2 = sqnorm(a);
  if (n2 > 0.f) {
    return a / pm::sqrt(n2);
  }
  return a;
}

struct rgb {
  float r, g, b;
};
PM_HD rgb mkrgb(float r, float g, float b) {
  rgb o;
  o.r = r;
  o.g = g;
  o.b = b;
  return o;
}
PM_HD rgb operator+(rgb a, rgb b) { return mkrgb(a.r + b.r, a.g + b.g, a.b + b.b); }
PM_HD rgb operator-(rgb a, rgb b) { return mkrgb(a.r - b.r, a.g - b.g, a.b - b.b); }
PM_HD rgb operator*(rgb a, rgb b) { return mkrgb(a.r * b.r, a.g * b.g, a.b * b.b); }
PM_HD rgb operator*(rgb a, float s) { return mkrgb(a.r * s, a.g * s, a.b * s); }
PM_HD rgb operator/(rgb a, float s) { return mkrgb(a.r / s, a.g / s, a.b / s); }
PM_HD rgb zero_rgb() { return mkrgb(0.f, 0.f, 0.f); }
PM_HD float sum(rgb a) { return (a.r + a.g) + a.b; }

// 3x4 row-major affine transform
struct affine {
  float m[12];
  PM_HDM f3 point(f3 v) const {
    return mk(((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3],
              ((m[4] * v.x + m[5] * v.y) + m[6] * v.z) + m[7],
              ((m[8] * v.x + m[9] * v.y) + m[10] * v.z) + m[11]);
  }
  PM_HDM f3 vector(f3 v) const {
    return mk((m[0] * v.x + m[1] * v.y) + m[2] * v.z,
              (m[4] * v.x + m[5] * v.y) + m[6] * v.z,
              (m[8] * v.x + m[9] * v.y) + m[10] * v.z);
  }
  PM_HDM f3 translation() const { return mk(m[3], m[7], m[11]); }
};

struct ray {
  f3 o, d;
};

struct box {
  f3 lo, hi;
};

PM_HD box empty_box() {
  const float big = 3.40282347e+38f;
  box b;
  b.lo = mk(big, big, big);
  b.hi = mk(-big, -big, -big);
  return b;
}
PM_HD box merge(box a, box b) {
  box o;
  o.lo = vmin(a.lo, b.lo);
  o.hi = vmax(a.hi, b.hi);
  return o;
}
PM_HD box grow(box a, f3 p) {
  box o;
  o.lo = vmin(a.lo, p);
  o.hi = vmax(a.hi, p);
  return o;
}
PM_HD box overlap(box a, box b) {
  box o;
  o.lo = vmax(a.lo, b.lo);
  o.hi = vmin(a.hi, b.hi);
  return o;
}
PM_HD bool contains(box a, f3 p) {
  return a.lo.x <= p.x && a.lo.y <= p.y && a.lo.z <= p.z && a.hi.x >= p.x &&
         a.hi.y >= p.y && a.hi.z >= p.z;
}
// AABB::surface_area (aabb.h:93-103): zero for inverted boxes
PM_HD float area(box a) {
  f3 d = a.hi - a.lo;
  if (d.x < 0.f || d.y < 0.f || d.z < 0.f) {
    return 0.f;
  }
  return 2.f * (d.x * d.y + d.z * d.y + d.z * d.x);
}
PM_HD f3 centre(box a) { return (a.lo + a.hi) / 2.f; }

// get_inv_direction (aabb.h:16-28): zero components become 1e-20
PM_HD f3 inv_dir(f3 d) {
  float x = d.x == 0.f ? 1e-20f : d.x;
  float y = d.y == 0.f ? 1e-20f : d.y;
  float z = d.z == 0.f ? 1e-20f : d.z;
  return mk(1.0f / x, 1.0f / y, 1.0f / z);
}

// AABB::solve_bounding_intersection (aabb.h:112-131): no clamp at t = 0
PM_HD bool slab(box b, f3 o, f3 inv, float *tmin_out) {
  f3 t0 = hmul(b.lo - o, inv);
  f3 t1 = hmul(b.hi - o, inv);
  f3 near = vmin(t0, t1);
  f3 far = vmax(t0, t1);
  float tmin = fmax2(near.x, fmax2(near.y, near.z));
  float tmax = fmin2(far.x, fmin2(far.y, far.z));
  *tmin_out = tmin;
  return tmin <= tmax;
}

// Triangle::intersect (triangle_impl.h:9-39) on a triangle stored as
// (v0, e1 = v1 - v0, e2 = v2 - v0).  The reference's double-precision
// comparisons are written as the float comparisons they are equal to:
// |a| < 1e-7 (double) <=> |a| < 1e-7f, t > 1e-5 (double) <=> t > 1e-5f, and
// 1. / a computed in double then rounded equals the float division (53 >=
// 2 * 24 + 2, so the double rounding is innocuous).
PM_HD bool tri_hit(f3 v0, f3 e1, f3 e2, const ray &r, float *t_out,
                   bool *back_out) {
  f3 h = cross(r.d, e2);
  float a = dot(e1, h);
  if (pm::fabs(a) < 1e-7f) {
    return false;
  }
  float f = 1.0f / a;
  f3 s = r.o - v0;
  float u = f * dot(s, h);
  if (u < 0.f || u > 1.f) {
    return false;
  }
  f3 q = cross(s, e1);
  float v = f * dot(r.d, q);
  if (v < 0.f || u + v > 1.f) {
    return false;
  }
  float t = f * dot(e2, q);
  if (t > 1e-5f) {
    *t_out = t;
    *back_out = a < 0.f;
    return true;
  }
  return false;
}

// Triangle::interpolation_values (triangle_impl.h:55-72)
PM_HD void barycentric(f3 e1, f3 e2, f3 p_minus_v0, float w[3]) {
  float d00 = dot(e1, e1);
  float d01 = dot(e1, e2);
  float d11 = dot(e2, e2);
  float d20 = dot(p_minus_v0, e1);
  float d21 = dot(p_minus_v0, e2);
  float denom = d00 * d11 - d01 * d01;
  float v = (d11 * d20 - d01 * d21) / denom;
  float ww = (d00 * d21 - d01 * d20) / denom;
  // T u = 1. - v - w: evaluated in double, then rounded to float
  w[0] = (float)((1.0 - (double)v) - (double)ww);
  w[1] = v;
  w[2] = ww;
}

} // namespace pg
