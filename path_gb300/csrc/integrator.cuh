// Device side of the render path: BVH traversal (binary and compressed
// 8-wide), BSDFs, the RandomTriangle light sampler, the Sobol table RNG and
// the next-event-estimation integrator.
//
// Every function restates the reference's arithmetic in the same order
// (translation units including this header are compiled with --fmad=false):
//   integrate_sample  <- integrate::rendering_equation +
//                        rendering_equation_iteration
//                        (include/integrate/rendering_equation.h:27-129,
//                         rendering_equation_iteration.h:9-153)
//   sample_light      <- random_triangle.h:35-90
//   BSDFs             <- include/bsdf/*.h; GGX is new (Walter et al. 2007)
//   trace_binary      <- include/intersect/accel/detail/bvh/bvh_impl.h:12-89
#pragma once

#include "devtypes.h"
#include "geom.h"
#include "kernels.h"

#include <curand_kernel.h>

namespace pg {
namespace dev {
// internal linkage: every translation unit that includes this header gets
// its own copy of these device functions
namespace {

constexpr uint32_t kTag = 1u << 31;
#define PG_INF __int_as_float(0x7f800000)

struct Hit {
  float t;
  uint32_t idx; // BVH-order triangle index
  bool ok;
  bool back;
};

struct Counts {
  uint32_t rays, nodes, tris;
};

__device__ __forceinline__ Hit no_hit() {
  Hit h;
  h.t = PG_INF;
  h.idx = 0;
  h.ok = false;
  h.back = false;
  return h;
}

// optional_min fold (include/intersect/optional_min.h:10-26): a later
// candidate at equal distance replaces the current best
__device__ __forceinline__ void fold(Hit &best, float t, bool back,
                                     uint32_t idx) {
  if (!best.ok || !(best.t < t)) {
    best.ok = true;
    best.t = t;
    best.back = back;
    best.idx = idx;
  }
}

__device__ __forceinline__ void set_status(uint32_t *status, uint32_t code) {
  atomicCAS(status, 0u, code);
}

__device__ __forceinline__ void load_tri(const float4 *tris, uint32_t i, f3 &v0,
                                         f3 &e1, f3 &e2) {
  float4 a = __ldg(tris + 3 * i);
  float4 b = __ldg(tris + 3 * i + 1);
  float4 c = __ldg(tris + 3 * i + 2);
  v0 = mk(a.x, a.y, a.z);
  e1 = mk(a.w, b.x, b.y);
  e2 = mk(b.z, b.w, c.x);
}

// ---------------------------------------------------------------------------
// binary SBVH, the reference's traversal order: depth-first stack of 64,
// candidates gathered until target_objects are pending, then tested
template <bool kCount>
__device__ Hit trace_binary(const RenderParams &P, const ray &r, Counts &cnt) {
  Hit best = no_hit();
  if (P.n_bin_nodes == 0) {
    return best;
  }
  f3 inv = inv_dir(r.d);
  uint32_t stack[64];
  uint32_t sp = 0;
  stack[sp++] = 0;
  uint32_t objects[10];
  uint32_t n_obj = 0;
  const uint32_t target = P.target_objects;
  while (sp != 0) {
    while (n_obj < target && sp != 0) {
      uint32_t ni = stack[--sp];
      uint4 a = __ldg(P.bin_nodes + 2 * ni);
      uint4 b = __ldg(P.bin_nodes + 2 * ni + 1);
      if (kCount) {
        ++cnt.nodes;
      }
      box bx;
      bx.lo = mk(__uint_as_float(a.z), __uint_as_float(a.w), __uint_as_float(b.x));
      bx.hi = mk(__uint_as_float(b.y), __uint_as_float(b.z), __uint_as_float(b.w));
      float tmin;
      if (slab(bx, r.o, inv, &tmin) && (!best.ok || best.t > tmin)) {
        if (a.x & kTag) {
          if (sp + 2 > 64) {
            set_status(P.status, kStatusStackOverflow);
            return no_hit();
          }
          stack[sp++] = a.y;
          stack[sp++] = a.x & ~kTag;
        } else {
          uint32_t s = a.x;
          uint32_t e = a.y & ~kTag;
          bool extra = (a.y & kTag) != 0;
          if (e < s || n_obj + (e - s) > 10) {
            set_status(P.status, kStatusObjectsOverflow);
            return no_hit();
          }
          for (uint32_t i = s; i < e; ++i) {
            objects[n_obj++] = extra ? __ldg(P.extra_idxs + i) : i;
          }
        }
      }
    }
    if (n_obj == 0) {
      break;
    }
    for (uint32_t k = 0; k < n_obj; ++k) {
      uint32_t idx = objects[k];
      f3 v0, e1, e2;
      load_tri(P.tris, idx, v0, e1, e2);
      if (kCount) {
        ++cnt.tris;
      }
      float t;
      bool back;
      if (tri_hit(v0, e1, e2, r, &t, &back)) {
        fold(best, t, back, idx);
      }
    }
    n_obj = 0;
  }
  return best;
}

// ---------------------------------------------------------------------------
// compressed 8-wide BVH.  A node is five 128-bit loads.  Its eight child
// boxes are tested with one fused multiply-add per plane,
//   t = q a + b,  a = 2^e / d,  b = (p - o) / d,
// evaluated as m A + C with m = 1 + q 2^-15 (the byte placed in the float
// 1.0 by one byte permute), A = 2^15 a and C = b - A, and widened by a
// rounding margin of 2^-20 (|b| + 255 |a|), which covers the error of the
// fused form against the exact plane p + q 2^e (an exactly representable
// float, see wide.cpp), with 1 / d one ulp off (the hardware reciprocal),
// more than twice over, plus 2^-8 |a| + 2^-23 |b|, which
// covers the rounding of C (at most 2^-9 |a| + 2^-24 |b|).  Decoded boxes
// contain the binary SBVH's boxes, so every box the reference's slab test
// accepts is accepted here too.
__device__ __forceinline__ float exp2_byte(uint32_t e) {
  return __uint_as_float(e << 23);
}

// two-lane FP32 (one instruction on sm_100 and later; each lane rounds like
// the scalar operation)
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
  unsigned long long d;
  asm("{\n\t.reg .b64 ra, rb;\n\tmov.b64 ra, {%1, %2};\n\tmov.b64 rb, {%3, %4};\n\t"
      "add.rn.f32x2 %0, ra, rb;\n\t}"
      : "=l"(d)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return make_float2(__uint_as_float((uint32_t)d), __uint_as_float((uint32_t)(d >> 32)));
}

__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
  unsigned long long d;
  asm("{\n\t.reg .b64 ra, rb;\n\tmov.b64 ra, {%1, %2};\n\tmov.b64 rb, {%3, %4};\n\t"
      "sub.rn.f32x2 %0, ra, rb;\n\t}"
      : "=l"(d)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return make_float2(__uint_as_float((uint32_t)d), __uint_as_float((uint32_t)(d >> 32)));
}

__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
  unsigned long long d;
  asm("{\n\t.reg .b64 ra, rb;\n\tmov.b64 ra, {%1, %2};\n\tmov.b64 rb, {%3, %4};\n\t"
      "mul.rn.f32x2 %0, ra, rb;\n\t}"
      : "=l"(d)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return make_float2(__uint_as_float((uint32_t)d), __uint_as_float((uint32_t)(d >> 32)));
}

__device__ __forceinline__ float2 fma2_rn(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("{\n\t.reg .b64 ra, rb, rc;\n\tmov.b64 ra, {%1, %2};\n\tmov.b64 rb, {%3, %4};\n\t"
      "mov.b64 rc, {%5, %6};\n\tfma.rn.f32x2 %0, ra, rb, rc;\n\t}"
      : "=l"(d)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return make_float2(__uint_as_float((uint32_t)d), __uint_as_float((uint32_t)(d >> 32)));
}

// bytes i of (n, f) as the pair of plane distances m * A + (Cn, Cf) with
// m = 1 + q 2^-15 (the byte in the second byte of the float 1.0) and
// A = 2^15 a, C = b - A: q a + b in one fused multiply-add per plane
__device__ __forceinline__ float2 plane_pair(uint32_t nl, uint32_t nh, uint32_t fl,
                                               uint32_t fh, int i, float2 aa, float2 cc) {
  const uint32_t wn = i < 4 ? nl : nh, wf = i < 4 ? fl : fh;
  const uint32_t sel = 0x7604u | ((uint32_t)(i & 3) << 4);
  const float2 m = make_float2(__uint_as_float(__byte_perm(wn, 0x3F800000u, sel)),
                               __uint_as_float(__byte_perm(wf, 0x3F800000u, sel)));
  return fma2_rn(m, aa, cc);
}

constexpr int kWideStack = (int)kWideStackDepth;

// three-operand minimum / maximum (one instruction on sm_100 and later)
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// Order-independent closest hit of the wide traversal: the smallest
// distance wins and, at equal distance, the smallest BVH-order index, so the
// result does not depend on the order in which nodes are visited.  With
// best.ok false, best.t is the caller's distance limit (hits at or below it
// are taken).
__device__ __forceinline__ void fold_min(Hit &best, float t, bool back, uint32_t idx) {
  if (t < best.t || (t == best.t && (!best.ok || idx < best.idx))) {
    best.ok = true;
    best.t = t;
    best.back = back;
    best.idx = idx;
  }
}

// Traversal state of one ray through the wide BVH.  A node group is the set
// of a visited node's internal children the ray still has to enter: their
// first node index and the node's internal-slot mask (bits 0-7) plus the
// entered children as bits 8-15 in ray order (bit 8 + (slot ^ oct)).  The
// builder puts the child nearest the low corner of every axis in slot 0,
// the one on the high side of axis a in slots with bit a set, so the lowest
// ray-order bit is approximately the nearest child along the ray.
struct WideWalk {
  ray r;
  f3 inv;
  Hit best;   // best.t is the pruning distance: tlimit until the first hit
  float light_target; // shadow rays: the light point's distance, else -INF
  uint32_t oct;
  uint32_t ng_base, ng_bits;
  int sp;
  bool done;
};

// The inverse direction of the 8-wide walk: the reference's zero rule
// (aabb.h:16-28) with the hardware reciprocal (rcp.approx.f32, at most one
// ulp from 1 / x).  It only feeds the 8-wide box tests, whose rounding margin
// (2^-20 of the plane distance) covers an inverse one ulp off several times
// over; the triangle test and the binary traversal keep the exact division.
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ f3 inv_dir_wide(f3 d) {
  return mk(rcp_approx(d.x == 0.f ? 1e-20f : d.x), rcp_approx(d.y == 0.f ? 1e-20f : d.y),
            rcp_approx(d.z == 0.f ? 1e-20f : d.z));
}

// tlimit: hits beyond it are not wanted (shadow rays only need hits up to
// just past the light); INF for extension rays.  Within the limit the
// closest hit is the same as without it.
__device__ __forceinline__ void wide_begin(const RenderParams &P, WideWalk &w, const ray &r,
                                           float tlimit, float light_target,
                                           uint32_t root = 0) {
  w.r = r;
  w.inv = inv_dir_wide(r.d);
  w.best = no_hit();
  w.best.t = tlimit;
  w.light_target = light_target;
  w.oct = (w.inv.x < 0.f ? 1u : 0u) | (w.inv.y < 0.f ? 2u : 0u) | (w.inv.z < 0.f ? 4u : 0u);
  // the root as the only child of a pseudo node in slot 0
  w.ng_base = root;
  w.ng_bits = 1u | (1u << (8 + w.oct));
  w.sp = 0;
  w.done = P.n_wide_nodes == 0 || root == kEmptyRoot;
}

// A shadow ray only asks whether its closest hit lies within 1e-6 of the
// light point (rendering_equation_iteration.h:22-27, 44-55).  A hit with
// target - t > 1e-6 (in float, so every closer hit fails the same test)
// settles that it does not: the walk may stop there, and the hit it
// reports gives the same answer as the closest one.
__device__ __forceinline__ bool shadow_settled(const WideWalk &w) {
  return w.best.ok && w.light_target - w.best.t > 1e-6f;
}

// Enter the next child of the current node group and test its eight slots;
// the triangles of the leaf slots it hits are returned as a mask over the
// node's triangle block (tri_base + bit).  Its internal hits become the
// current group (the rest of the old group waits on the stack), or a group
// is taken from the stack, or the walk ends (w.done) once the returned
// triangles are tested.
// kStaged: nodes below n_top are read from `top`, the caller's shared-memory
// copy of the BVH's first nodes (one generic load serves both copies).
template <bool kCount, bool kStaged = false>
__device__ __forceinline__ void wide_node(const RenderParams &P, WideWalk &w,
                                          uint32_t *st_base, uint32_t *st_bits, Counts &cnt,
                                          uint32_t &tri_base, uint32_t &tmask,
                                          const uint4 *top = nullptr, uint32_t n_top = 0) {
  tmask = 0;
  tri_base = 0;
  const uint32_t j = __ffs(w.ng_bits >> 8) - 1;
  w.ng_bits &= ~(1u << (8 + j));
  const uint32_t slot = j ^ w.oct;
  const uint32_t node = w.ng_base + __popc(w.ng_bits & ((1u << slot) - 1u));
  if ((w.ng_bits >> 8) != 0) {
    if (w.sp >= kWideStack) {
      set_status(P.status, kStatusStackOverflow);
      w.best = no_hit();
      w.done = true;
      return;
    }
    st_base[w.sp] = w.ng_base;
    st_bits[w.sp] = w.ng_bits;
    ++w.sp;
  }
  uint4 n0, n1, n2, n3, n4;
  if constexpr (kStaged) {
    const uint4 *np = node < n_top ? top + 5 * node : P.wide_nodes + 5 * (size_t)node;
    n0 = np[0];
    n1 = np[1];
    n2 = np[2];
    n3 = np[3];
    n4 = np[4];
  } else {
    const uint4 *np = P.wide_nodes + 5 * (size_t)node;
    n0 = __ldg(np);
    n1 = __ldg(np + 1);
    n2 = __ldg(np + 2);
    n3 = __ldg(np + 3);
    n4 = __ldg(np + 4);
  }
  if (kCount) {
    ++cnt.nodes;
  }
  const f3 inv = w.inv;
  // per axis: t per quantum, offset of the node origin, rounding margin
  // (x and y as two-lane pairs: the same roundings as the scalar forms)
  const float2 inv_xy = make_float2(inv.x, inv.y);
  const float2 axy =
      mul2_rn(make_float2(exp2_byte(n0.w & 0xffu), exp2_byte((n0.w >> 8) & 0xffu)), inv_xy);
  const float2 bxy = mul2_rn(sub2_rn(make_float2(__uint_as_float(n0.x), __uint_as_float(n0.y)),
                                     make_float2(w.r.o.x, w.r.o.y)),
                             inv_xy);
  const float ax = axy.x, ay = axy.y, bx = bxy.x, by = bxy.y;
  const float az = exp2_byte((n0.w >> 16) & 0xffu) * inv.z;
  const float bz = (__uint_as_float(n0.z) - w.r.o.z) * inv.z;
  // 2^-20 (255 |a| + |b|), plus 2^-8 |a| + 2^-23 |b| for the rounding of
  // C = b - 2^15 a (at most 2^-9 |a| + 2^-24 |b|)
  const float ex = __fmul_rn(__fmaf_rn(4352.f, fabsf(ax), __fmul_rn(1.125f, fabsf(bx))), 0x1p-20f);
  const float ey = __fmul_rn(__fmaf_rn(4352.f, fabsf(ay), __fmul_rn(1.125f, fabsf(by))), 0x1p-20f);
  const float ez = __fmul_rn(__fmaf_rn(4352.f, fabsf(az), __fmul_rn(1.125f, fabsf(bz))), 0x1p-20f);
  const float bnx = bx - ex, bfx = bx + ex;
  const float bny = by - ey, bfy = by + ey;
  const float bnz = bz - ez, bfz = bz + ez;
  const uint32_t imask = n0.w >> 24;
  // near / far plane bytes per axis according to the direction's sign
  const bool sx = (w.oct & 1u) != 0, sy = (w.oct & 2u) != 0, sz = (w.oct & 4u) != 0;
  const uint32_t nxl = sx ? n3.z : n2.x, nxh = sx ? n3.w : n2.y;
  const uint32_t fxl = sx ? n2.x : n3.z, fxh = sx ? n2.y : n3.w;
  const uint32_t nyl = sy ? n4.x : n2.z, nyh = sy ? n4.y : n2.w;
  const uint32_t fyl = sy ? n2.z : n4.x, fyh = sy ? n2.w : n4.y;
  const uint32_t nzl = sz ? n4.z : n3.x, nzh = sz ? n4.w : n3.y;
  const uint32_t fzl = sz ? n3.x : n4.z, fzh = sz ? n3.y : n4.w;
  const float tcull = w.best.t;
  const float2 Axy = mul2_rn(axy, make_float2(32768.f, 32768.f));
  const float Ax = Axy.x, Ay = Axy.y, Az = __fmul_rn(az, 32768.f);
  const float2 aax = make_float2(Ax, Ax), aay = make_float2(Ay, Ay), aaz = make_float2(Az, Az);
  const float2 ccx = sub2_rn(make_float2(bnx, bfx), aax);
  const float2 ccy = sub2_rn(make_float2(bny, bfy), aay);
  const float2 ccz = sub2_rn(make_float2(bnz, bfz), aaz);
  // slot i's box test, a miss as the sign of tmax - tmin, tcull - tmin or
  // tmax (tmin <= tmax && tmin <= tcull && tmax >= 0; tcull >= 0; a box
  // holding a hit at t > 1e-5 has tmax > 0), shifted in from slot 7 down so
  // that slot i lands in bit i (empty slots never pass: lo > hi)
  uint32_t miss = 0;
#pragma unroll
  for (int i = 7; i >= 0; --i) {
    // (near, far) plane distance per axis
    const float2 tx = plane_pair(nxl, nxh, fxl, fxh, i, aax, ccx);
    const float2 ty = plane_pair(nyl, nyh, fyl, fyh, i, aay, ccy);
    const float2 tz = plane_pair(nzl, nzh, fzl, fzh, i, aaz, ccz);
    const float tmin = fmax3(tx.x, ty.x, tz.x);
    const float tmax = fmin3(tx.y, ty.y, tz.y);
    const uint32_t neg = __float_as_uint(__fsub_rn(tmax, tmin)) |
                         __float_as_uint(__fsub_rn(tcull, tmin)) | __float_as_uint(tmax);
    miss = __funnelshift_l(neg, miss, 1);
  }
  const uint32_t hm = ~miss & 0xffu;
  // internal children: slot i -> bit i ^ oct (ray order), by three swaps
  uint32_t hits = hm & imask;
  const uint32_t h1 = ((hits & 0x55u) << 1) | ((hits >> 1) & 0x55u);
  hits = (w.oct & 1u) ? h1 : hits;
  const uint32_t h2 = ((hits & 0x33u) << 2) | ((hits >> 2) & 0x33u);
  hits = (w.oct & 2u) ? h2 : hits;
  const uint32_t h4 = ((hits & 0x0fu) << 4) | (hits >> 4);
  hits = (w.oct & 4u) ? h4 : hits;
  // leaf children: meta = count << 5 | first triangle offset
  uint32_t tm = 0;
  for (uint32_t lh = hm & ~imask & 0xffu; lh != 0; lh &= lh - 1u) {
    const uint32_t i = __ffs(lh) - 1;
    const uint32_t meta = ((i < 4 ? n1.z : n1.w) >> (8 * (i & 3u))) & 0xffu;
    tm |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
  }
  tri_base = n1.y;
  tmask = tm;
  if (hits != 0) {
    w.ng_base = n1.x;
    w.ng_bits = imask | (hits << 8);
    return;
  }
  if (w.sp > 0) {
    // a waiting group keeps the children it had; the next step culls them
    --w.sp;
    w.ng_base = st_base[w.sp];
    w.ng_bits = st_bits[w.sp];
    return;
  }
  w.done = true;
}

// Moller-Trumbore on wide-leaf triangle k; folds a hit into best
__device__ __forceinline__ void wide_tri(const RenderParams &P, const ray &r, uint32_t k,
                                         Hit &best) {
  const float4 *tp = P.wide_tris + 3 * (size_t)k;
  const float4 a = __ldg(tp);
  const float4 b = __ldg(tp + 1);
  const float4 c = __ldg(tp + 2);
  float t;
  bool back;
  if (tri_hit(mk(a.x, a.y, a.z), mk(a.w, b.x, b.y), mk(b.z, b.w, c.x), r, &t, &back)) {
    fold_min(best, t, back, __float_as_uint(c.y));
  }
}

constexpr uint32_t kFull = 0xffffffffu;

// position of set bit r (0-based) of m; m has more than r set bits
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t r) {
  uint32_t pos = 0;
#pragma unroll
  for (uint32_t s = 16; s > 0; s >>= 1) {
    const uint32_t c = __popc(m & ((1u << s) - 1u));
    if (r >= c) {
      r -= c;
      m >>= s;
      pos += s;
    }
  }
  return pos;
}

// Per-warp shared-memory scratch of warp_triangles_shared: every lane's ray,
// written when the lane takes the ray (the w components are not read), and
// every lane's closest-hit key of the current step.
struct WarpTriScratch {
  float4 o[32];
  float4 d[32];
  unsigned long long key[32];
};

// The leaf triangles the warp's lanes took from their last nodes, tested by
// the whole warp: the work items (lane, triangle) are numbered lane-major
// (a shuffle scan) and dealt out 32 per round; an item finds its owner lane
// by a binary search over the lanes' inclusive counts, reads the owner's ray
// from shared memory and runs Moller-Trumbore.  The closest hit per lane is
// the minimum of 64-bit keys (distance bits, then BVH index, then the back
// flag; distances are positive, so the bit order is the numeric order),
// lowered by 64-bit shared-memory atomicMin from the items that hit and
// folded into the lane's walk: the same order-independent result the lane's
// own loop gives.  All 32 lanes call this; sh.o / sh.d hold the ray of every
// lane with triangles, or, with kStoreRay, each such lane writes its ray
// there first.
template <bool kCount, bool kStoreRay = false>
__device__ __forceinline__ void warp_triangles_shared(const RenderParams &P, WideWalk &w,
                                                      uint32_t tri_base, uint32_t tmask,
                                                      uint32_t lane, Counts &cnt,
                                                      WarpTriScratch &sh) {
  const uint32_t c = __popc(tmask);
  uint32_t incl = c;
#pragma unroll
  for (uint32_t off = 1; off < 32; off <<= 1) {
    const uint32_t v = __shfl_up_sync(kFull, incl, off);
    if (lane >= off) {
      incl += v;
    }
  }
  const uint32_t total = __shfl_sync(kFull, incl, 31);
  if (total == 0) {
    return;
  }
  const uint32_t excl = incl - c;
  sh.key[lane] = ~0ull;
  if (kStoreRay && c > 0) {
    sh.o[lane] = make_float4(w.r.o.x, w.r.o.y, w.r.o.z, 0.f);
    sh.d[lane] = make_float4(w.r.d.x, w.r.d.y, w.r.d.z, 0.f);
  }
  __syncwarp();
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t g = base + lane;
    // owner: the first lane whose inclusive count exceeds g
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t step = 16; step > 0; step >>= 1) {
      if (__shfl_sync(kFull, incl, pos + step - 1) <= g) {
        pos += step;
      }
    }
    const uint32_t o_excl = __shfl_sync(kFull, excl, pos);
    const uint32_t o_mask = __shfl_sync(kFull, tmask, pos);
    const uint32_t o_base = __shfl_sync(kFull, tri_base, pos);
    if (g < total) {
      const float4 o = sh.o[pos], d = sh.d[pos];
      ray r;
      r.o = mk(o.x, o.y, o.z);
      r.d = mk(d.x, d.y, d.z);
      const uint32_t k = o_base + nth_set_bit(o_mask, g - o_excl);
      Hit h = no_hit();
      wide_tri(P, r, k, h);
      if (h.ok) {
        atomicMin(&sh.key[pos], ((unsigned long long)__float_as_uint(h.t) << 32) |
                                    (unsigned long long)((h.idx << 1) | (h.back ? 1u : 0u)));
      }
      if (kCount) {
        ++cnt.tris;
      }
    }
  }
  __syncwarp();
  const unsigned long long mine = sh.key[lane];
  if (mine != ~0ull) {
    const uint32_t lo = (uint32_t)mine;
    fold_min(w.best, __uint_as_float((uint32_t)(mine >> 32)), (lo & 1u) != 0, lo >> 1);
    if (shadow_settled(w)) {
      w.done = true;
    }
  }
}

// one traversal step of a lone lane: a node and its triangles
template <bool kCount>
__device__ __forceinline__ void wide_step(const RenderParams &P, WideWalk &w,
                                          uint32_t *st_base, uint32_t *st_bits, Counts &cnt) {
  uint32_t tri_base, tmask;
  wide_node<kCount>(P, w, st_base, st_bits, cnt, tri_base, tmask);
  while (tmask != 0) {
    const uint32_t k = __ffs(tmask) - 1;
    tmask &= tmask - 1u;
    if (kCount) {
      ++cnt.tris;
    }
    wide_tri(P, w.r, tri_base + k, w.best);
  }
  if (shadow_settled(w)) {
    w.done = true;
  }
}

template <bool kCount>
__device__ Hit trace_wide(const RenderParams &P, const ray &r, Counts &cnt, float tlimit,
                          float light_target, uint32_t root = 0) {
  WideWalk w;
  wide_begin(P, w, r, tlimit, light_target, root);
  uint32_t st_base[kWideStack];
  uint32_t st_bits[kWideStack];
  while (!w.done) {
    wide_step<kCount>(P, w, st_base, st_bits, cnt);
  }
  return w.best;
}

// closest hit; the binary traversal keeps the reference's order and
// pruning exactly and ignores tlimit; root: the wide root node (a batch
// scene's)
template <uint32_t kTrav, bool kCount>
__device__ __forceinline__ Hit trace(const RenderParams &P, const ray &r, Counts &cnt,
                                     float tlimit, float light_target, uint32_t root = 0) {
  if (kCount) {
    ++cnt.rays;
  }
  if (kTrav == kTravWide) {
    return trace_wide<kCount>(P, r, cnt, tlimit, light_target, root);
  }
  return trace_binary<kCount>(P, r, cnt);
}

// A light sample is visible when the closest hit lies within 1e-6 of the
// light point's distance (rendering_equation_iteration.h:22-27); no hit
// beyond target + 1e-6 can pass, so shadow rays only need hits up to here.
__device__ __forceinline__ float light_bound(float target) {
  return target * 1.0000005f + 2e-6f;
}

// ---------------------------------------------------------------------------
// RNG.  Sobel: table-driven Sobol (include/rng/rng_from_sequence_gen.h:26-107).
// Uniform (include/rng/uniform/uniform.h:18-76, GPU execution model): a
// cuRAND XORWOW state per path, seeded with curand_init(seed, 0, 0) and
// drawn with curand_uniform, 1.0 mapped to 0.0
// (include/lib/cuda/curand_utils.h:58-66).  The state lives in memory (a
// slot of the streaming buffers or the thread's stack) as 32-bit words
// `stride` apart, so a path can stop in one kernel and go on in the next.
constexpr uint32_t kXorwowWords = sizeof(curandStateXORWOW) / 4;
static_assert(kXorwowWords == kRngStateWords, "Uniform RNG state size");

__device__ __noinline__ void uniform_seed(uint32_t seed, uint32_t *w, uint32_t stride) {
  curandStateXORWOW st;
  curand_init(seed, 0, 0, &st);
  const uint32_t *q = reinterpret_cast<const uint32_t *>(&st);
#pragma unroll
  for (uint32_t k = 0; k < kXorwowWords; ++k) {
    w[k * stride] = q[k];
  }
}

__device__ __forceinline__ float uniform_next(uint32_t *w, uint32_t stride) {
  curandStateXORWOW st;
  uint32_t *q = reinterpret_cast<uint32_t *>(&st);
#pragma unroll
  for (uint32_t k = 0; k < kXorwowWords; ++k) {
    q[k] = w[k * stride];
  }
  const float out = curand_uniform(&st);
#pragma unroll
  for (uint32_t k = 0; k < kXorwowWords; ++k) {
    w[k * stride] = q[k];
  }
  return out == 1.0f ? 0.0f : out;
}

// RngT<false>: Sobel, row = the sample's table row, dim = next dimension,
// bound = the dimension bound.  RngT<true>: Uniform, the state words `stride`
// apart from w.  The mode is a type so that the Sobel kernels carry no trace
// of the Uniform draw.
template <bool kUniform> struct RngT;

#if PG_SOBOL_DIRECT
// Sobel drawn from the direction vectors: x = scramble_d XOR the vectors
// v_{d,j} of the set bits j of the Gray code of the sample's Sobol index,
// XOR-ed in a register, mapped to (0, 1] and 1.0 to 0.0 -- the value the
// table holds (k_sobol), bit for bit.  vec = [bound][32] vectors followed
// by the [bound] scramble constants.
template <> struct RngT<false> {
  const uint32_t *vec;
  uint32_t gray;
  uint32_t dim;
  uint32_t bound;
  __device__ __forceinline__ float next() {
    uint32_t x = __ldg(vec + 32 * bound + dim);
    const uint32_t *v = vec + 32 * dim;
    for (uint32_t g = gray; g != 0; g &= g - 1) {
      x ^= __ldg(v + (__ffs(g) - 1));
    }
    const float f = __fadd_rn(__fmul_rn(__uint2float_rn(x), 0x1p-32f), 0x1p-33f);
    ++dim;
    dim = dim == bound ? 0u : dim;
    return f == 1.0f ? 0.0f : f;
  }
  __device__ __forceinline__ void begin(const RenderParams &P, uint32_t sobol_index) {
    vec = P.sobol_vec;
    gray = sobol_index ^ (sobol_index >> 1);
    bound = P.dim_bound;
  }
};
#else
template <> struct RngT<false> {
  const float *row;
  uint32_t dim;
  uint32_t bound;
  __device__ __forceinline__ float next() {
    float v = __ldg(row + dim);
    ++dim;
    dim = dim == bound ? 0u : dim;
    return v;
  }
  // the table row of Sobol index sobol_index
  __device__ __forceinline__ void begin(const RenderParams &P, uint32_t sobol_index) {
    row = P.sobol + (size_t)sobol_index * P.dim_bound;
    bound = P.dim_bound;
  }
};
#endif

template <> struct RngT<true> {
  uint32_t *w;
  uint32_t stride;
  __device__ __forceinline__ float next() { return uniform_next(w, stride); }
};

__device__ __forceinline__ uint32_t fnv_hash(uint32_t in) {
  uint32_t h = 2166136261u;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    h ^= (in >> (8 * i)) & 0xffu;
    h *= 16777619u;
  }
  return h;
}

// ---------------------------------------------------------------------------
// include/lib/projection.h:9-32, rotation by Rodrigues' formula
__device__ __forceinline__ f3 rotate(f3 v, float angle, f3 axis) {
  float s, c;
  pm::sincos(angle, &s, &c);
  f3 t0 = v * c;
  f3 t1 = cross(axis, v) * s;
  f3 t2 = axis * ((1.f - c) * dot(axis, v));
  return (t0 + t1) + t2;
}

__device__ __forceinline__ f3 relative_vec(f3 vec, float phi, float theta) {
  float st, ct, sp, cp;
  pm::sincos(theta, &st, &ct);
  pm::sincos(phi, &sp, &cp);
  f3 local = mk(st * cp, st * sp, ct);
  float angle = pm::acos(vec.z);
  f3 axis = normalize(cross(vec, mk(0.f, 0.f, 1.f)));
  return normalize(rotate(local, -angle, axis));
}

__device__ __forceinline__ f3 reflect(f3 v, f3 n) {
  float k = 2.0f * -dot(v, n);
  return normalize(v + n * k);
}

__device__ f3 refract(float ior, f3 v, f3 n) {
  float c = -dot(v, n);
  bool exiting = c < 0.f;
  float frac = exiting ? ior : 1.f / ior;
  float in_sqrt = 1.f - frac * frac * (1.f - c * c);
  f3 ne = exiting ? -n : n;
  if (in_sqrt > 0.f) {
    float angle = pm::acos(pm::sqrt(in_sqrt));
    f3 axis = normalize(cross(v, ne));
    return normalize(rotate(-ne, angle, axis));
  }
  return reflect(v, n);
}

// ---------------------------------------------------------------------------
// BSDFs
struct Mat {
  uint32_t type;
  rgb diffuse, specular, emission;
  float shininess, ior, w_d, roughness, glossy_norm, inv_shininess_p1, r0,
      cont_inclusive0;
};

__device__ __forceinline__ Mat load_mat(const DevMaterial *m) {
  Mat o;
  o.type = __ldg(&m->type);
  o.diffuse = mkrgb(__ldg(&m->diffuse[0]), __ldg(&m->diffuse[1]), __ldg(&m->diffuse[2]));
  o.specular = mkrgb(__ldg(&m->specular[0]), __ldg(&m->specular[1]), __ldg(&m->specular[2]));
  o.emission = mkrgb(__ldg(&m->emission[0]), __ldg(&m->emission[1]), __ldg(&m->emission[2]));
  o.shininess = __ldg(&m->shininess);
  o.ior = __ldg(&m->ior);
  o.w_d = __ldg(&m->w_d);
  o.roughness = __ldg(&m->roughness);
  o.glossy_norm = __ldg(&m->glossy_norm);
  o.inv_shininess_p1 = __ldg(&m->inv_shininess_p1);
  o.r0 = __ldg(&m->r0);
  o.cont_inclusive0 = __ldg(&m->cont_inclusive0);
  return o;
}

__device__ __forceinline__ rgb emission_of(const DevMaterial *m) {
  return mkrgb(__ldg(&m->emission[0]), __ldg(&m->emission[1]), __ldg(&m->emission[2]));
}

enum : uint32_t {
  kDiffuse = 0,
  kGlossy = 1,
  kDiffuseGlossy = 2,
  kDiffuseMirror = 3,
  kMirror = 4,
  kDielectric = 5,
  kGGX = 6,
};

// Compile-time feature set of a path kernel (kFeat* in devtypes.h): the
// cases of BSDF types outside F compile to nothing.
template <uint32_t F, uint32_t T> __device__ __forceinline__ constexpr bool has_mat() {
  return ((F >> T) & 1u) != 0;
}

__device__ __forceinline__ bool is_brdf(const Mat &m) { return m.type != kDielectric; }

template <uint32_t F = kFeatAll>
__device__ __forceinline__ float prob_continuous(const Mat &m) {
  switch (m.type) {
  case kDiffuse:
  case kGlossy:
  case kDiffuseGlossy:
  case kGGX:
    return 1.0f;
  case kMirror:
  case kDielectric:
    return 0.0f;
  default:
    return has_mat<F, kDiffuseMirror>() ? m.w_d : 1.0f;
  }
}

// (float)(1 / M_PI)
constexpr float kInvPi = 0x1.45f306p-2f;
constexpr double kTwoPi = 6.283185307179586;

__device__ __forceinline__ rgb glossy_eval(const Mat &m, f3 in, f3 out, f3 n) {
  float c = fmax2(dot(reflect(in, n), out), 0.0f);
  return (m.specular * m.glossy_norm) * pm::pow(c, m.shininess);
}

__device__ __forceinline__ float ggx_g1(float c, float a2) {
  return (2.f * c) / (c + pm::sqrt(a2 + (1.f - a2) * (c * c)));
}

__device__ __forceinline__ rgb schlick(rgb f0, float c) {
  float m = 1.f - c;
  float m2 = m * m;
  float m5 = (m2 * m2) * m;
  return mkrgb(f0.r + (1.f - f0.r) * m5, f0.g + (1.f - f0.g) * m5,
               f0.b + (1.f - f0.b) * m5);
}

// GGX normal distribution D(h) = a2 / (pi ((n.h)^2 (a2 - 1) + 1)^2)
// (Walter et al. 2007, eq. 33)
__device__ __forceinline__ float ggx_d(float ch, float a2) {
  float dd = (ch * ch) * (a2 - 1.f) + 1.f;
  return a2 / ((0x1.921fb6p+1f * dd) * dd); // (float)M_PI
}

// GGX microfacet reflection (Walter et al. 2007): D GGX, separable Smith G,
// Schlick Fresnel
__device__ rgb ggx_eval(const Mat &m, f3 in, f3 out, f3 n) {
  f3 wo = -in;
  if (dot(wo, n) < 0.f) {
    n = -n;
  }
  float co = dot(wo, n);
  float ci = dot(out, n);
  if (!(co > 0.f) || !(ci > 0.f)) {
    return zero_rgb();
  }
  float a2 = m.roughness * m.roughness;
  f3 h = normalize(wo + out);
  float ch = dot(h, n);
  float d = ggx_d(ch, a2);
  float g = ggx_g1(co, a2) * ggx_g1(ci, a2);
  rgb f = schlick(m.specular, dot(wo, h));
  float scale = (d * g) / ((4.f * ci) * co);
  return f * scale;
}

// d log f / d(parameter) of a differentiable BSDF at (in, out, n): per
// channel for the reflectance (Diffuse albedo, GGX F0) in `refl`, and for
// the GGX roughness alpha in `rough`.  d log D/d a2 = 1/a2 - 2 ch^2/dd;
// d log G1(c)/d a2 = -(1 - c^2) / (2 s (c + s)) with s = sqrt(a2 + (1-a2)c^2);
// d/d alpha = 2 alpha d/d a2.  False for materials without these parameters
// or directions where f vanishes.
__device__ bool bsdf_log_grad(const Mat &m, f3 in, f3 out, f3 n, rgb &refl, float &rough) {
  if (m.type == kDiffuse) {
    refl = mkrgb(m.diffuse.r > 0.f ? 1.f / m.diffuse.r : 0.f,
                 m.diffuse.g > 0.f ? 1.f / m.diffuse.g : 0.f,
                 m.diffuse.b > 0.f ? 1.f / m.diffuse.b : 0.f);
    rough = 0.f;
    return true;
  }
  if (m.type != kGGX) {
    return false;
  }
  f3 wo = -in;
  if (dot(wo, n) < 0.f) {
    n = -n;
  }
  float co = dot(wo, n);
  float ci = dot(out, n);
  if (!(co > 0.f) || !(ci > 0.f)) {
    return false;
  }
  float a = m.roughness;
  float a2 = a * a;
  f3 h = normalize(wo + out);
  float ch = dot(h, n);
  float dd = (ch * ch) * (a2 - 1.f) + 1.f;
  float dlog_d = 1.f / a2 - (2.f * (ch * ch)) / dd;
  float so = pm::sqrt(a2 + (1.f - a2) * (co * co));
  float si = pm::sqrt(a2 + (1.f - a2) * (ci * ci));
  float dlog_g = -(1.f - co * co) / ((2.f * so) * (co + so)) -
                 (1.f - ci * ci) / ((2.f * si) * (ci + si));
  rough = (2.f * a) * (dlog_d + dlog_g);
  float c = dot(wo, h);
  float mm = 1.f - c;
  float m5 = ((mm * mm) * (mm * mm)) * mm;
  rgb f = schlick(m.specular, c);
  refl = mkrgb(f.r > 0.f ? (1.f - m5) / f.r : 0.f, f.g > 0.f ? (1.f - m5) / f.g : 0.f,
               f.b > 0.f ? (1.f - m5) / f.b : 0.f);
  return true;
}

template <uint32_t F = kFeatAll>
__device__ rgb continuous_eval(const Mat &m, f3 in, f3 out, f3 n) {
  switch (m.type) {
  case kDiffuse:
    if constexpr (has_mat<F, kDiffuse>()) {
      return m.diffuse * kInvPi;
    }
    break;
  case kGlossy:
    if constexpr (has_mat<F, kGlossy>()) {
      return glossy_eval(m, in, out, n);
    }
    break;
  case kDiffuseGlossy:
    if constexpr (has_mat<F, kDiffuseGlossy>()) {
      float w0 = m.cont_inclusive0 - 0.f;
      float w1 = 1.f - m.cont_inclusive0;
      return (m.diffuse * kInvPi) * w0 + glossy_eval(m, in, out, n) * w1;
    }
    break;
  case kDiffuseMirror:
    if constexpr (has_mat<F, kDiffuseMirror>()) {
      return (m.diffuse * kInvPi) * (1.f - 0.f);
    }
    break;
  case kGGX:
    if constexpr (has_mat<F, kGGX>()) {
      return ggx_eval(m, in, out, n);
    }
    break;
  default:
    break;
  }
  return zero_rgb();
}

struct Sample {
  f3 dir;
  rgb mult;
};

template <class R>
__device__ __forceinline__ Sample diffuse_sample(rgb albedo, f3 in, f3 n, R &rng) {
  float v0 = rng.next();
  float v1 = rng.next();
  float phi = (float)(kTwoPi * (double)v0);
  float theta = pm::asin(pm::sqrt(v1));
  f3 aligned = dot(in, n) > 0.f ? -n : n;
  Sample s;
  s.dir = relative_vec(aligned, phi, theta);
  s.mult = albedo;
  return s;
}

template <class R>
__device__ Sample glossy_sample(const Mat &m, f3 in, f3 n, R &rng) {
  float v0 = rng.next();
  float v1 = rng.next();
  f3 refl = reflect(in, n);
  float phi = (float)(kTwoPi * (double)v0);
  float psi = pm::acos(pm::pow(v1, m.inv_shininess_p1));
  Sample s;
  s.dir = relative_vec(refl, phi, psi);
  s.mult = m.specular;
  return s;
}

// orthonormal basis (Duff et al. 2017, "Building an Orthonormal Basis,
// Revisited")
__device__ __forceinline__ void onb(f3 n, f3 &b1, f3 &b2) {
  float sign = n.z >= 0.f ? 1.f : -1.f;
  float a = -1.f / (sign + n.z);
  float b = n.x * n.y * a;
  b1 = mk(1.f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  b2 = mk(b, sign + n.y * n.y * a, -n.y);
}

template <class R>
__device__ Sample ggx_sample(const Mat &m, f3 in, f3 n, R &rng) {
  float u0 = rng.next();
  float u1 = rng.next();
  f3 wo = -in;
  if (dot(wo, n) < 0.f) {
    n = -n;
  }
  float a2 = m.roughness * m.roughness;
  float phi = (float)(kTwoPi * (double)u0);
  float tan2 = (a2 * u1) / (1.f - u1);
  float cos_t = 1.f / pm::sqrt(1.f + tan2);
  float sin_t = pm::sqrt(fmax2(0.f, 1.f - cos_t * cos_t));
  f3 b1, b2;
  onb(n, b1, b2);
  float sp, cp;
  pm::sincos(phi, &sp, &cp);
  f3 h = normalize((b1 * (sin_t * cp) + b2 * (sin_t * sp)) + n * cos_t);
  float k = 2.f * dot(wo, h);
  f3 wi = normalize(h * k - wo);
  float co = dot(wo, n);
  float ci = dot(wi, n);
  float ch = dot(h, n);
  float oh = dot(wo, h);
  Sample s;
  s.dir = wi;
  if (!(ci > 0.f) || !(co > 0.f) || !(ch > 0.f) || !(oh > 0.f)) {
    s.mult = zero_rgb();
    return s;
  }
  float g = ggx_g1(co, a2) * ggx_g1(ci, a2);
  rgb f = schlick(m.specular, oh);
  float w = (g * oh) / (co * ch);
  s.mult = f * w;
  return s;
}

template <uint32_t F = kFeatAll, class R>
__device__ Sample continuous_sample(const Mat &m, f3 in, f3 n, R &rng) {
  switch (m.type) {
  case kDiffuse:
    if constexpr (has_mat<F, kDiffuse>()) {
      return diffuse_sample(m.diffuse, in, n, rng);
    }
    break;
  case kGlossy:
    if constexpr (has_mat<F, kGlossy>()) {
      return glossy_sample(m, in, n, rng);
    }
    break;
  case kDiffuseGlossy:
    if constexpr (has_mat<F, kDiffuseGlossy>()) {
      float loc = rng.next();
      if (loc <= m.cont_inclusive0) {
        return diffuse_sample(m.diffuse, in, n, rng);
      }
      return glossy_sample(m, in, n, rng);
    }
    break;
  case kDiffuseMirror:
    if constexpr (has_mat<F, kDiffuseMirror>()) {
      (void)rng.next();
      return diffuse_sample(m.diffuse, in, n, rng);
    }
    break;
  case kGGX:
    if constexpr (has_mat<F, kGGX>()) {
      return ggx_sample(m, in, n, rng);
    }
    break;
  default:
    break;
  }
  Sample s;
  s.dir = in;
  s.mult = zero_rgb();
  return s;
}

template <uint32_t F = kFeatAll, class R>
__device__ Sample discrete_sample(const Mat &m, f3 in, f3 n, R &rng) {
  Sample s;
  s.mult = m.specular;
  switch (m.type) {
  case kMirror:
    if constexpr (has_mat<F, kMirror>()) {
      s.dir = reflect(in, n);
      return s;
    }
    break;
  case kDiffuseMirror:
    if constexpr (has_mat<F, kDiffuseMirror>()) {
      (void)rng.next();
      s.dir = reflect(in, n);
      return s;
    }
    break;
  case kDielectric:
    if constexpr (has_mat<F, kDielectric>()) {
    float c = pm::fabs(dot(in, n));
    double x = (double)(1.f - c);
    double x2 = x * x;
    double p5 = (x2 * x2) * x;
    float prop = (float)((double)m.r0 + (double)(1.f - m.r0) * p5);
    if (rng.next() < prop) {
      s.dir = reflect(in, n);
    } else {
      s.dir = refract(m.ior, in, n);
    }
    return s;
    }
    break;
  default:
    break;
  }
  s.dir = in;
  s.mult = zero_rgb();
  return s;
}

template <class R>
__device__ Sample uniform_dir_sample(const Mat &m, f3 in, f3 n, R &rng) {
  float v0 = rng.next();
  float v1 = rng.next();
  bool whole = !is_brdf(m);
  float phi = (float)(kTwoPi * (double)v0);
  float theta = pm::acos(whole ? 2.f * v1 - 1.f : v1);
  Sample s;
  s.dir = relative_vec(n, phi, theta);
  float inv_prob = whole ? 0x1.921fb6p+3f : 0x1.921fb6p+2f; // (float)(4 pi), (float)(2 pi)
  rgb f = continuous_eval(m, in, s.dir, n);
  s.mult = (f * dot(s.dir, n)) * inv_prob;
  return s;
}

// ---------------------------------------------------------------------------
// RandomTriangle light sample (random_triangle.h:35-90).  |n.d| |N_A.d| <
// 1e-8 in double equals <= 1e-8f in float for float operands.
struct LightSample {
  f3 dir;
  float mult;
  float target;
};

// the emissive triangles of one scene and their area x emission CDF
struct LightSet {
  const float4 *tris;
  const float *cdf;
  uint32_t n;
};

__device__ __forceinline__ LightSet lights_of(const RenderParams &P) {
  LightSet l;
  l.tris = P.light_tris;
  l.cdf = P.light_cdf;
  l.n = P.n_lights;
  return l;
}

// the lights of one scene of a batch
__device__ __forceinline__ LightSet lights_of(const RenderParams &P, const BatchScene &b) {
  LightSet l;
  l.tris = P.light_tris + 3 * (size_t)b.light_off;
  l.cdf = P.light_cdf + b.light_off;
  l.n = b.n_lights;
  return l;
}

// a position of a batch scene in the coordinates of the batch's radiance
// cache (BatchScene::cache_cell); clamped to the scene's box first, so that
// a hit point rounded just outside it stays in the scene's own cell
__device__ __forceinline__ f3 batch_cache_position(const BatchScene &b, f3 p) {
  const uint32_t c = b.cache_cell;
  const auto unit = [](float v) { return fminf(fmaxf(v, 0.f), 1.f); };
  return mk(unit((p.x - b.cache_lo[0]) * b.cache_inv[0]) + 2.f * (float)(c % kCacheCellsPerAxis),
            unit((p.y - b.cache_lo[1]) * b.cache_inv[1]) +
                2.f * (float)(c / kCacheCellsPerAxis % kCacheCellsPerAxis),
            unit((p.z - b.cache_lo[2]) * b.cache_inv[2]) +
                2.f * (float)(c / (kCacheCellsPerAxis * kCacheCellsPerAxis)));
}

template <class R>
__device__ bool sample_light(const LightSet &L, f3 pos, const Mat &m, f3 normal, R &rng,
                             LightSample &out) {
  if (L.n == 0) {
    return false;
  }
  float search = rng.next();
  uint32_t idx = 0;
  for (; idx < L.n; ++idx) {
    if (__ldg(L.cdf + idx) >= search) {
      break;
    }
  }
  if (idx >= L.n) {
    idx = L.n - 1; // unreachable for a normalised table
  }
  float4 a = __ldg(L.tris + 3 * idx);
  float4 b = __ldg(L.tris + 3 * idx + 1);
  float4 c = __ldg(L.tris + 3 * idx + 2);
  f3 v0 = mk(a.x, a.y, a.z), e0 = mk(a.w, b.x, b.y), e1 = mk(b.z, b.w, c.x);
  float s = rng.next();
  float t = rng.next();
  if (s + t > 1.f) {
    s = 1.f - s;
    t = 1.f - t;
  }
  f3 point = (e0 * s + e1 * t) + v0;
  f3 dir_un = point - pos;
  if (is_brdf(m) && dot(dir_un, normal) <= 0.f) {
    return false;
  }
  f3 dir = normalize(dir_un);
  f3 tn = cross(e0, e1) * 0.5f;
  float prob = __ldg(L.cdf + idx) - (idx == 0 ? 0.f : __ldg(L.cdf + idx - 1));
  float nw = pm::fabs(dot(normal, dir) * dot(tn, dir));
  if (nw <= 1e-8f) {
    return false;
  }
  float weight = nw / sqnorm(dir_un);
  out.dir = dir;
  out.mult = prob / weight;
  out.target = length(dir_un);
  return true;
}

// include/integrate/term_prob/*
template <uint32_t F = kFeatAll>
__device__ __forceinline__ float term_prob(const RenderParams &P, uint32_t iters,
                                           rgb mult) {
  if constexpr ((F & kFeatNIters) != 0) {
    return iters >= P.term_iters ? 1.0f : 0.0f;
  }
  switch (P.term_prob) {
  case 0:
    return P.term_prob_prob;
  case 1:
    return iters >= P.term_iters ? 1.0f : 0.0f;
  case 2: {
    rgb q = mkrgb(mult.r / (mult.r + 1.f), mult.g / (mult.g + 1.f),
                  mult.b / (mult.b + 1.f));
    q = q * 0.57f;
    float sq = (q.r * q.r + q.g * q.g) + q.b * q.b;
    sq = fmin2(fmax2(sq, 0.0f), 1.0f);
    float p = pm::fabs(pm::pow(1.f - sq, P.term_exp));
    return fmax2(p, P.term_min_prob);
  }
  default: {
    float p = 1.f - 1.f / (sum(mult) / 3.f);
    return fmin2(fmax2(p, P.term_min_prob), 1.f);
  }
  }
}

// camera ray (initial_ray_sample.h:16-56)
// film_to_world and image size of one camera
// the image a sample belongs to: camera, size and samples per location
struct Camera {
  const float *f2w;
  uint32_t x_dim, y_dim, spp;
  uint32_t sample_offset; // Sobol row of sample s: s + sample_offset
};

__device__ __forceinline__ Camera camera_of(const RenderParams &P) {
  Camera c;
  c.f2w = P.f2w;
  c.x_dim = P.x_dim;
  c.y_dim = P.y_dim;
  c.spp = P.spp;
  c.sample_offset = P.sample_offset;
  return c;
}

__device__ __forceinline__ ray camera_ray(const Camera &cam, float x, float y) {
  f3 film = mk((2.0f * x) / (float)cam.x_dim - 1.0f, (-2.0f * y) / (float)cam.y_dim + 1.0f,
               -1.0f);
  const float *m = cam.f2w;
  f3 world = mk(((m[0] * film.x + m[1] * film.y) + m[2] * film.z) + m[3],
                ((m[4] * film.x + m[5] * film.y) + m[6] * film.z) + m[7],
                ((m[8] * film.x + m[9] * film.y) + m[10] * film.z) + m[11]);
  ray r;
  r.o = mk(m[3], m[7], m[11]);
  r.d = normalize(world - r.o);
  return r;
}

__device__ __forceinline__ f3 shading_normal(const RenderParams &P, uint32_t idx,
                                             f3 point, uint32_t &material) {
  float4 a = __ldg(P.tri_data + 3 * idx);
  float4 b = __ldg(P.tri_data + 3 * idx + 1);
  float4 c = __ldg(P.tri_data + 3 * idx + 2);
  material = __float_as_uint(c.w);
  f3 n0 = mk(a.x, a.y, a.z), n1 = mk(a.w, b.x, b.y), n2 = mk(b.z, b.w, c.x);
  f3 v0, e1, e2;
  load_tri(P.tris, idx, v0, e1, e2);
  float w[3];
  barycentric(e1, e2, point - v0, w);
  return normalize((n0 * w[0] + n1 * w[1]) + n2 * w[2]);
}

// State of one camera sample between traces: the loop variables of
// rendering_equation (include/integrate/rendering_equation.h:41-124) and the
// RenderingEquationState (rendering_equation_state.h:14-52) with at most
// one light sample per vertex.  o is the current vertex, the origin of both
// the next extension ray (direction d) and the light ray (direction ld).
template <bool kUniform> struct PathStateT {
  f3 o, d, ld;
  float light_target;
  rgb multiplier, light_mult, total;
  uint32_t iters;
  bool count_emission, has_next, has_light;
  RngT<kUniform> rng;
};
using PathState = PathStateT<false>;

// camera ray of a sample (initial_ray_sample.h:36-56): 2 RNG draws for a
// square image, the caller's ray for an InitialRays spec.  A Uniform path's
// generator is seeded with sample + location x spp (uniform.h:63-66; the
// frame offset of a progressive render adds offset x locations) and keeps
// its state at rng_words (words rng_stride apart).
template <bool kUniform>
__device__ __forceinline__ void path_begin_cam(const RenderParams &P, const Camera &cam,
                                               uint32_t sample_idx, uint32_t x, uint32_t y,
                                               PathStateT<kUniform> &s, uint32_t *rng_words,
                                               uint32_t rng_stride) {
  const uint32_t location = x + y * cam.x_dim;
  if constexpr (kUniform) {
    uniform_seed(sample_idx + location * cam.spp + cam.sample_offset * (cam.x_dim * cam.y_dim),
                 rng_words, rng_stride);
    s.rng.w = rng_words;
    s.rng.stride = rng_stride;
  } else {
    s.rng.begin(P, sample_idx + cam.sample_offset);
    s.rng.dim = fnv_hash(location) % P.init_dim_bound;
  }
  ray r;
  if (P.initial_rays != nullptr) {
    // InitialRays: the caller's ray for this location, no RNG draw
    const float *q = P.initial_rays + 6 * (size_t)x;
    r.o = mk(q[0], q[1], q[2]);
    r.d = mk(q[3], q[4], q[5]);
  } else {
    float xo = s.rng.next();
    float yo = s.rng.next();
    r = camera_ray(cam, (float)x + xo, (float)y + yo);
  }
  s.o = r.o;
  s.d = r.d;
  s.ld = mk(0.f, 0.f, 0.f);
  s.light_target = 0.f;
  s.multiplier = mkrgb(1.f, 1.f, 1.f);
  s.light_mult = zero_rgb();
  s.total = zero_rgb();
  s.iters = 0;
  s.count_emission = true;
  s.has_next = true;
  s.has_light = false;
}

// rng_words: where a Uniform path keeps its XORWOW state (unused for Sobel)
template <bool kUniform>
__device__ __forceinline__ void path_begin(const RenderParams &P, uint32_t sample_idx,
                                           uint32_t x, uint32_t y, PathStateT<kUniform> &s,
                                           uint32_t *rng_words, uint32_t rng_stride) {
  path_begin_cam(P, camera_of(P), sample_idx, x, y, s, rng_words, rng_stride);
}

// One rendering_equation_iteration (rendering_equation_iteration.h:9-153)
// given the closest hits of the pending light ray (lh) and extension ray
// (nh).  Returns true while the path has rays left to trace; s.total is the
// sample's radiance once it returns false.
// What one path_step did, for the adjoint replay: the radiance its pending
// light ray and its hit's emission added (and from which materials), the
// shaded vertex, and the directions its light sample and continuation took.
struct StepTrace {
  bool light_added, emit_added, hit, nee, continuous, cache_query;
  uint32_t light_mat, mat;
  f3 in, normal, nee_dir, next_dir, point;
  rgb albedo;
};

// the reflectance a radiance-cache query carries for a material
__device__ __forceinline__ rgb albedo_of(const Mat &m) {
  switch (m.type) {
  case kGlossy:
  case kMirror:
  case kGGX:
    return m.specular;
  case kDielectric:
    return mkrgb(1.f, 1.f, 1.f);
  default:
    return m.diffuse;
  }
}

template <bool kUniform, uint32_t F = kFeatAll>
__device__ __forceinline__ bool path_step(const RenderParams &P, const LightSet &L,
                                       PathStateT<kUniform> &s,
                                       const Hit &lh, const Hit &nh,
                                       StepTrace *tr = nullptr) {
  const bool performs_samples = (F & kFeatLightTri) != 0 || P.light_sampler == 0;
  const bool cull = P.back_cull != 0;
  if (tr != nullptr) {
    tr->light_added = tr->emit_added = tr->hit = tr->nee = tr->continuous = false;
    tr->cache_query = false;
  }
  if (s.has_light && lh.ok && pm::fabs(s.light_target - lh.t) <= 1e-6f &&
      (!cull || !lh.back)) {
    float4 c = __ldg(P.tri_data + 3 * lh.idx + 2);
    s.total = s.total + emission_of(P.materials + __float_as_uint(c.w)) * s.light_mult;
    if (tr != nullptr) {
      tr->light_added = true;
      tr->light_mat = __float_as_uint(c.w);
    }
  }
  if (!s.has_next || !nh.ok) {
    return false;
  }
  f3 point = s.o + s.d * nh.t;
  uint32_t mi;
  f3 normal = shading_normal(P, nh.idx, point, mi);
  const Mat mat = load_mat(P.materials + mi);
  if ((!performs_samples || s.count_emission) && (!cull || !nh.back)) {
    s.total = s.total + s.multiplier * mat.emission;
    if (tr != nullptr) {
      tr->emit_added = true;
    }
  }
  if (tr != nullptr) {
    tr->hit = true;
    tr->mat = mi;
    tr->in = s.d;
    tr->normal = normal;
    tr->point = point;
    tr->albedo = albedo_of(mat);
    if (P.cache_depth != 0 && s.iters == P.cache_depth) {
      // the path ends into the radiance cache at this vertex
      tr->cache_query = true;
      s.o = point;
      s.has_next = false;
      s.has_light = false;
      return false;
    }
  }
  bool new_has_light = false;
  rgb new_light_mult = zero_rgb();
  float new_light_target = 0.f;
  f3 new_ld = s.ld;
  float pc = prob_continuous<F>(mat);
  if (pc > 0.f && performs_samples) {
    LightSample ls;
    if (sample_light(L, point, mat, normal, s.rng, ls)) {
      rgb f = continuous_eval<F>(mat, s.d, ls.dir, normal);
      new_light_mult = ((s.multiplier * f) * pc) / ls.mult;
      new_light_target = ls.target;
      new_ld = ls.dir;
      new_has_light = true;
      if (tr != nullptr) {
        tr->nee = true;
        tr->nee_dir = ls.dir;
      }
    }
  }
  bool take_discrete;
  if (pc == 0.f) {
    take_discrete = true;
  } else if (pc == 1.f) {
    take_discrete = false;
  } else {
    take_discrete = pc < s.rng.next();
  }
  Sample smp;
  if (take_discrete) {
    smp = discrete_sample<F>(mat, s.d, normal, s.rng);
  } else if ((F & kFeatBsdfDir) != 0 || P.dir_sampler == 0) {
    smp = continuous_sample<F>(mat, s.d, normal, s.rng);
  } else {
    smp = uniform_dir_sample(mat, s.d, normal, s.rng);
  }
  if (tr != nullptr) {
    tr->continuous = !take_discrete;
    tr->next_dir = smp.dir;
  }
  rgb new_multiplier = s.multiplier * smp.mult;
  float p = term_prob<F>(P, s.iters, new_multiplier);
  bool next = s.rng.next() > p;
  s.iters += 1;
  s.count_emission = take_discrete;
  s.has_light = new_has_light;
  s.light_mult = new_light_mult;
  s.light_target = new_light_target;
  s.ld = new_ld;
  s.o = point;
  if (next) {
    s.multiplier = new_multiplier / (1.0f - p);
    s.d = smp.dir;
    s.has_next = true;
  } else {
    s.has_next = false;
  }
  return s.has_next || s.has_light;
}

// the safety bound on path vertices (no counterpart in the reference)
template <class S>
__device__ __forceinline__ bool path_continues(const RenderParams &P, S &s, bool cont) {
  if (cont && s.iters >= kMaxPathVertices) {
    set_status(P.status, kStatusPathTooLong);
    return false;
  }
  return cont;
}

// closest hits of a path's pending light and extension rays.  The first
// step of an InitialIdxAndDir sample takes the caller's hit instead of
// tracing (initial_ray_sample.h:58-74: distance 1, front side).
template <uint32_t kTrav, bool kCount, class S>
__device__ __forceinline__ void step_hits(const RenderParams &P, const S &s,
                                          bool first, uint32_t x, Counts &cnt, Hit &lh,
                                          Hit &nh, uint32_t root = 0) {
  lh = no_hit();
  nh = no_hit();
  if (s.has_light) {
    ray lr;
    lr.o = s.o;
    lr.d = s.ld;
    lh = trace<kTrav, kCount>(P, lr, cnt, light_bound(s.light_target), s.light_target, root);
  }
  if (first && P.initial_idx != nullptr) {
    nh.t = 1.f;
    nh.idx = P.initial_idx[x];
    nh.ok = true;
    nh.back = false;
  } else if (s.has_next) {
    ray r;
    r.o = s.o;
    r.d = s.d;
    nh = trace<kTrav, kCount>(P, r, cnt, PG_INF, -PG_INF, root);
  }
}

// one camera sample of rendering_equation, traced in a loop
template <uint32_t kTrav, bool kCount, bool kUniform>
__device__ rgb integrate_sample(const RenderParams &P, uint32_t sample_idx,
                                uint32_t x, uint32_t y, Counts &cnt) {
  PathStateT<kUniform> s;
  uint32_t xw[kUniform ? kXorwowWords : 1]; // the Uniform generator's state
  path_begin(P, sample_idx, x, y, s, xw, 1);
  bool first = true;
  while (true) {
    Hit lh, nh;
    step_hits<kTrav, kCount>(P, s, first, x, cnt, lh, nh);
    first = false;
    if (!path_continues(P, s, path_step(P, lights_of(P), s, lh, nh))) {
      return s.total;
    }
  }
}

// OutputPerStep (rendering_equation.h:61-124): the radiance gathered in
// step k is added to steps[k]; a path stops after P.n_steps steps
template <uint32_t kTrav, bool kUniform>
__device__ void integrate_sample_steps(const RenderParams &P, uint32_t sample_idx,
                                       uint32_t x, uint32_t y, rgb *steps) {
  PathStateT<kUniform> s;
  uint32_t xw[kUniform ? kXorwowWords : 1];
  path_begin(P, sample_idx, x, y, s, xw, 1);
  Counts cnt = {0, 0, 0};
  for (uint32_t k = 0; k < P.n_steps; ++k) {
    Hit lh, nh;
    step_hits<kTrav, false>(P, s, k == 0, x, cnt, lh, nh);
    const bool cont = path_step(P, lights_of(P), s, lh, nh);
    steps[k] = steps[k] + s.total;
    s.total = zero_rgb();
    if (!cont) {
      return;
    }
  }
}

// ---------------------------------------------------------------------------
// WorkDivision thread info; threads of rows outside the rendered band exit
__device__ __forceinline__ ThreadWork band_work(const RenderParams &P, uint32_t block,
                                               uint32_t tid) {
  ThreadWork tw = thread_work(P.wd, block, tid);
  if (tw.y < P.row_lo || tw.y >= P.row_hi) {
    tw.exit = true;
  }
  return tw;
}

// reduction over sample_block_size lanes (include/lib/cuda/reduce.cuh:35-102)
__device__ __forceinline__ rgb warp_reduce(rgb v, uint32_t width) {
  for (uint32_t off = width / 2; off > 0; off /= 2) {
    float r = __shfl_down_sync(0xffffffffu, v.r, off, width);
    float g = __shfl_down_sync(0xffffffffu, v.g, off, width);
    float b = __shfl_down_sync(0xffffffffu, v.b, off, width);
    v = mkrgb(r + v.r, g + v.g, b + v.b);
  }
  return v;
}

__device__ __forceinline__ rgb sub_block_reduce(rgb v, uint32_t tid, uint32_t sbs) {
  v = warp_reduce(v, sbs < 32u ? sbs : 32u);
  if (sbs <= 32) {
    return v;
  }
  __shared__ float sh[32][3];
  uint32_t lane = tid % 32, warp = tid / 32;
  if (lane == 0) {
    sh[warp][0] = v.r;
    sh[warp][1] = v.g;
    sh[warp][2] = v.b;
  }
  __syncthreads();
  uint32_t per_group = sbs / 32;
  if (tid % sbs < per_group) {
    uint32_t k = lane + (tid / sbs) * per_group;
    v = mkrgb(sh[k][0], sh[k][1], sh[k][2]);
  }
  return warp_reduce(v, per_group);
}

// assign_output (include/render/detail/integrate_image/assign_output.h:11-24)
// and float_rgb_to_bgra_32 (include/lib/bgra_32.h:12-31)
__device__ __forceinline__ void write_pixel(float *out_rgb, uint8_t *out_bgra,
                                            bool bgra, size_t idx, rgb v) {
  if (bgra) {
    float tr = v.r / (v.r + 1.f), tg = v.g / (v.g + 1.f), tb = v.b / (v.b + 1.f);
    uchar4 o;
    o.x = (unsigned char)(tb * 255.0f);
    o.y = (unsigned char)(tg * 255.0f);
    o.z = (unsigned char)(tr * 255.0f);
    o.w = 0;
    reinterpret_cast<uchar4 *>(out_bgra)[idx] = o;
  } else {
    out_rgb[3 * idx] = v.r;
    out_rgb[3 * idx + 1] = v.g;
    out_rgb[3 * idx + 2] = v.b;
  }
}

} // namespace
} // namespace dev
} // namespace pg
