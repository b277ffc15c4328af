// 8-wide BVH built on the GPU: triangles sorted by the Morton codes of their
// centroids, clustered bottom-up into a binary BVH by PLOC (Meister and
// Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume
// Hierarchy Construction", IEEE TVCG 2018), then collapsed top-down into the
// 80-byte quantised nodes of the traversal, one tree level per launch.
//
// Any BVH over the triangles gives the traversal the same closest hits (the
// 8-wide traversal takes the smallest distance, then the smallest BVH-order
// index, whatever the visiting order), so images rendered through this BVH
// are those of the SBVH built on the host, up to which of two triangles at
// exactly the same distance is reported.
//
// Stages: Morton code of each centroid (10 bits per axis) -> radix sort of
// (code, triangle) pairs -> PLOC rounds (nearest neighbour by merged surface
// area within 16 clusters either side, mutual pairs merge, survivors
// compacted) with parent links -> boxes bottom-up (the second child to
// arrive at a node merges), together with the surface-area cost optimisation
// of the collapse (the host builder's: per binary node the cheapest forest
// of at most 1..8 slots -- a subtree of up to four triangles may be one leaf
// slot -- from its children's) -> collapse: every wide node takes the best
// forest of eight slots of its binary node's children, places them in
// octant slots (as the host builder does), quantises their boxes (the same
// exact-plane frame), and queues its internal children.
#include "geom.h"
#include "gpu_build.h"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>

namespace pg {
namespace dev {
namespace {

constexpr uint32_t kLeafBit = 1u << 31; // node ids: internal i, or leaf k | kLeafBit
// a wide-node slot holding every triangle of internal node i: i | kSlotBit
constexpr uint32_t kSlotBit = 1u << 30;
// most triangles of such a slot (eight slots of four stay within the 32
// triangles a wide node addresses)
constexpr uint32_t kSlotMaxTris = 4;

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__device__ __forceinline__ f3 vert(const float *t9, uint32_t i, int k) {
  const float *p = t9 + 9 * (size_t)i + 3 * k;
  return mk(p[0], p[1], p[2]);
}

__global__ void k_morton(const float *t9, uint32_t n, f3 lo, f3 inv_ext, uint32_t *keys,
                         uint32_t *vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  const f3 c = ((vert(t9, i, 0) + vert(t9, i, 1)) + vert(t9, i, 2)) * (1.f / 3.f);
  uint32_t q[3];
  for (int a = 0; a < 3; ++a) {
    const float u = (c.get(a) - lo.get(a)) * inv_ext.get(a) * 1024.f;
    q[a] = (uint32_t)fminf(fmaxf(u, 0.f), 1023.f);
  }
  keys[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
  vals[i] = i;
}

__device__ __forceinline__ box tri_box(const float *t9, uint32_t i) {
  box b = empty_box();
  b = grow(b, vert(t9, i, 0));
  b = grow(b, vert(t9, i, 1));
  b = grow(b, vert(t9, i, 2));
  return b;
}

// ---- PLOC: parallel locally-ordered clustering (Meister and Bittner,
// "Parallel Locally-Ordered Clustering for Bounding Volume Hierarchy
// Construction", IEEE TVCG 2018).  Clusters start as the triangles in
// Morton order; every round each cluster finds, among the kPlocRadius
// clusters on either side, the one whose merged box has the smallest
// surface area; pairs that chose each other merge into a new internal node,
// and the surviving clusters are compacted in order.  Internal node ids
// are handed out from n - 2 down, so the last merge, the root, is node 0.
constexpr int kPlocRadius = 16;

__global__ void k_ploc_init(const box *item_box, uint32_t n, uint32_t *clus, box *cbox) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) {
    return;
  }
  clus[k] = k | kLeafBit;
  cbox[k] = item_box[k];
}

// ---- items: the leaves the tree is built over.  Without splitting, item j
// is the j-th triangle in Morton order; with splitting (Karras and Aila,
// "Fast Parallel Construction of High-Quality Bounding Volume Hierarchies",
// HPG 2013, section 4.3), a triangle whose box is much larger than the
// triangle itself becomes several references, each with the box of the
// part of the triangle in one piece of its box (the triangle clipped to the
// piece: a spatial split made before the tree is built).  item_tri[j] is
// the triangle's position in Morton order, item_box[j] its box.

__global__ void k_items_plain(const float *t9, const uint32_t *perm, uint32_t n,
                              uint32_t *item_tri, box *item_box) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) {
    return;
  }
  item_tri[k] = k;
  item_box[k] = tri_box(t9, perm[k]);
}

// most references of one triangle
constexpr uint32_t kMaxRefs = 16;

// splitting priority: how much larger than the triangle its box is (the
// cube root evens out the budget between large and small excesses)
__global__ void k_split_priority(const float *t9, const uint32_t *perm, uint32_t n,
                                 float *prio) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) {
    return;
  }
  const uint32_t o = perm[k];
  const f3 a = vert(t9, o, 0), b = vert(t9, o, 1), c = vert(t9, o, 2);
  const float tri_area = 0.5f * length(cross(b - a, c - a));
  const float excess = area(tri_box(t9, o)) - 4.f * tri_area;
  prio[k] = excess > 0.f ? cbrtf(excess) : 0.f;
}

// references per triangle: 1 + its share of the split budget
__global__ void k_split_count(const float *prio, uint32_t n, float scale, uint32_t *count) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) {
    return;
  }
  const float extra = floorf(prio[k] * scale);
  count[k] = 1u + (uint32_t)fminf(fmaxf(extra, 0.f), (float)(kMaxRefs - 1));
}

struct Poly {
  double v[9][3];
  int n;
};

// the part of polygon p on one side of the plane x_axis = at
__device__ void clip_side(const Poly &p, int axis, double at, bool below, Poly &out) {
  out.n = 0;
  for (int i = 0; i < p.n; ++i) {
    const double *a = p.v[i];
    const double *b = p.v[(i + 1) % p.n];
    const bool ina = below ? a[axis] <= at : a[axis] >= at;
    const bool inb = below ? b[axis] <= at : b[axis] >= at;
    if (ina && out.n < 9) {
      for (int c = 0; c < 3; ++c) {
        out.v[out.n][c] = a[c];
      }
      ++out.n;
    }
    if (ina != inb && out.n < 9) {
      const double t = (at - a[axis]) / (b[axis] - a[axis]);
      for (int c = 0; c < 3; ++c) {
        out.v[out.n][c] = c == axis ? at : a[c] + t * (b[c] - a[c]);
      }
      ++out.n;
    }
  }
}

// polygon box rounded outward to float (empty polygon: `fallback`)
__device__ box poly_box(const Poly &p, const box &fallback) {
  if (p.n == 0) {
    return fallback;
  }
  double lo[3], hi[3];
  for (int c = 0; c < 3; ++c) {
    lo[c] = hi[c] = p.v[0][c];
  }
  for (int i = 1; i < p.n; ++i) {
    for (int c = 0; c < 3; ++c) {
      lo[c] = fmin(lo[c], p.v[i][c]);
      hi[c] = fmax(hi[c], p.v[i][c]);
    }
  }
  box b;
  b.lo = mk(__double2float_rd(lo[0]), __double2float_rd(lo[1]), __double2float_rd(lo[2]));
  b.hi = mk(__double2float_ru(hi[0]), __double2float_ru(hi[1]), __double2float_ru(hi[2]));
  return b;
}

// the count[k] references of triangle k: its polygon split in halves at
// the middle of the widest axis of the piece's box, recursively
__global__ void k_split_emit(const float *t9, const uint32_t *perm, uint32_t n,
                             const uint32_t *count, const uint32_t *offset, uint32_t *ref_tri,
                             box *ref_box) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) {
    return;
  }
  const uint32_t o = perm[k];
  uint32_t out = offset[k];
  const uint32_t end = out + count[k];
  struct Piece {
    Poly p;
    uint32_t refs;
  };
  Piece st[6];
  int sp = 0;
  Piece &root = st[sp++];
  root.p.n = 3;
  for (int i = 0; i < 3; ++i) {
    const f3 v = vert(t9, o, i);
    root.p.v[i][0] = v.x;
    root.p.v[i][1] = v.y;
    root.p.v[i][2] = v.z;
  }
  root.refs = count[k];
  const box whole = tri_box(t9, o);
  while (sp > 0 && out < end) {
    Piece cur = st[--sp];
    const box pb = poly_box(cur.p, whole);
    const f3 ext = pb.hi - pb.lo;
    const int axis = (ext.x >= ext.y && ext.x >= ext.z) ? 0 : (ext.y >= ext.z ? 1 : 2);
    if (cur.refs <= 1 || ext.get(axis) <= 0.f || sp + 2 > 6) {
      // one reference per remaining count (copies when it cannot split)
      for (uint32_t r = 0; r < cur.refs && out < end; ++r) {
        ref_tri[out] = k;
        ref_box[out] = pb;
        ++out;
      }
      continue;
    }
    const double at = 0.5 * ((double)pb.lo.get(axis) + (double)pb.hi.get(axis));
    Piece &a = st[sp++];
    Piece &b = st[sp++];
    clip_side(cur.p, axis, at, true, a.p);
    clip_side(cur.p, axis, at, false, b.p);
    a.refs = cur.refs / 2;
    b.refs = cur.refs - cur.refs / 2;
  }
  // (count[k] references were reserved; every path above writes them all)
  while (out < end) {
    ref_tri[out] = k;
    ref_box[out] = whole;
    ++out;
  }
}

// Morton code of a box's centre
__global__ void k_morton_box(const box *boxes, uint32_t n, f3 lo, f3 inv_ext, uint32_t *keys,
                             uint32_t *vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  const box b = boxes[i];
  uint32_t q[3];
  for (int a = 0; a < 3; ++a) {
    const float c = 0.5f * (b.lo.get(a) + b.hi.get(a));
    const float u = (c - lo.get(a)) * inv_ext.get(a) * 1024.f;
    q[a] = (uint32_t)fminf(fmaxf(u, 0.f), 1023.f);
  }
  keys[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
  vals[i] = i;
}

__global__ void k_items_refs(const uint32_t *order, const uint32_t *ref_tri, const box *ref_box,
                             uint32_t m, uint32_t *item_tri, box *item_box) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) {
    return;
  }
  item_tri[j] = ref_tri[order[j]];
  item_box[j] = ref_box[order[j]];
}

// nearest neighbour of every cluster: (merged area, index) smallest
__global__ void k_ploc_nn(const box *cbox, uint32_t m, uint32_t *nn) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= (int)m) {
    return;
  }
  const box bi = cbox[i];
  unsigned long long best = ~0ull;
  const int lo = max(0, i - kPlocRadius), hi = min((int)m - 1, i + kPlocRadius);
  for (int j = lo; j <= hi; ++j) {
    if (j == i) {
      continue;
    }
    const float d = area(merge(bi, cbox[j]));
    const unsigned long long key =
        ((unsigned long long)__float_as_uint(d) << 32) | (unsigned long long)(uint32_t)j;
    best = key < best ? key : best;
  }
  nn[i] = m > 1 ? (uint32_t)best : (uint32_t)i;
}

// keep[i]: 1 when cluster i survives the round (merged into its own slot,
// or not merged); mutual pairs (i < j) merge into slot i
__global__ void k_ploc_mark(const uint32_t *nn, uint32_t m, uint32_t *keep, uint32_t *merges) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) {
    return;
  }
  const uint32_t j = nn[i];
  const bool mutual = j != i && nn[j] == i;
  keep[i] = (!mutual || i < j) ? 1u : 0u;
  merges[i] = (mutual && i < j) ? 1u : 0u;
}

// with force (a round that found no mutual pair, possible only at exact
// ties): neighbours 2t, 2t + 1 merge instead
__global__ void k_ploc_force(uint32_t m, uint32_t *nn, uint32_t *keep, uint32_t *merges) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) {
    return;
  }
  const uint32_t j = (i & 1u) ? i - 1 : (i + 1 < m ? i + 1 : i);
  nn[i] = j;
  keep[i] = (j == i || i < j) ? 1u : 0u;
  merges[i] = (j != i && i < j) ? 1u : 0u;
}

// the merges of a round: the pair at rank r of the round (merge_pos[i] =
// exclusive prefix of merges) becomes internal node id_base - 1 - r; the
// survivors move to keep_pos[i] (exclusive prefix of keep)
__global__ void k_ploc_merge(const uint32_t *clus, const box *cbox, const uint32_t *nn,
                             const uint32_t *keep, const uint32_t *keep_pos,
                             const uint32_t *merges, const uint32_t *merge_pos, uint32_t m,
                             uint32_t n, uint32_t id_base, uint32_t *left, uint32_t *right,
                             uint32_t *parent, uint32_t *clus_out, box *cbox_out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m || !keep[i]) {
    return;
  }
  uint32_t id = clus[i];
  box b = cbox[i];
  if (merges[i]) {
    const uint32_t j = nn[i];
    const uint32_t a = clus[i], c = clus[j];
    id = id_base - 1 - merge_pos[i];
    left[id] = a;
    right[id] = c;
    parent[(a & kLeafBit) ? (n - 1) + (a & ~kLeafBit) : a] = id;
    parent[(c & kLeafBit) ? (n - 1) + (c & ~kLeafBit) : c] = id;
    b = merge(b, cbox[j]);
  }
  clus_out[keep_pos[i]] = id;
  cbox_out[keep_pos[i]] = b;
}

__device__ __forceinline__ box load_box_cg(const box *b) {
  const float *f = reinterpret_cast<const float *>(b);
  box o;
  o.lo = mk(__ldcg(f), __ldcg(f + 1), __ldcg(f + 2));
  o.hi = mk(__ldcg(f + 3), __ldcg(f + 4), __ldcg(f + 5));
  return o;
}

// collapse costs (as the host builder: a wide-node visit 1, a triangle test
// 0.3, per unit area); every leaf of the linear BVH is one triangle
constexpr float kCostNode = 1.0f;
constexpr float kCostTri = 0.3f;
// how the best forest of <= i slots represents a binary subtree: fewer
// slots, a wide node of its own, one leaf slot of all its triangles, or its
// two children's forests (kOpen + k: k slots to the left child)
constexpr uint8_t kFewer = 0, kWide = 1, kLeafSlot = 2, kOpen = 3;

// the cost of child c's best forest of <= i slots (i = 1..8)
__device__ __forceinline__ float child_cost(uint32_t c, const box &cb, const float *cost,
                                            int i) {
  return (c & kLeafBit) ? area(cb) * kCostTri : __ldcg(cost + 8 * (size_t)c + (i - 1));
}

// boxes [internal n-1 | leaves n] and the collapse costs of internal nodes
// ([n-1][8] cost and decision of the forests of 1..8 slots, the left share
// of a wide node's 8 slots), bottom-up; flags start at zero
__global__ void k_boxes(const box *item_box, uint32_t n, const uint32_t *left,
                        const uint32_t *right, const uint32_t *parent, box *boxes,
                        uint32_t *flags, float *cost, uint8_t *how, uint8_t *wide_k,
                        uint32_t *tri_count) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) {
    return;
  }
  boxes[(n - 1) + k] = item_box[k];
  if (n == 1) {
    return;
  }
  uint32_t node = parent[(n - 1) + k];
  while (true) {
    __threadfence();
    if (atomicAdd(&flags[node], 1u) == 0) {
      return; // the sibling's thread merges this node
    }
    __threadfence();
    const uint32_t l = left[node], r = right[node];
    // the sibling's box was written by another thread: read past L1
    const box bl = load_box_cg(boxes + ((l & kLeafBit) ? (n - 1) + (l & ~kLeafBit) : l));
    const box br = load_box_cg(boxes + ((r & kLeafBit) ? (n - 1) + (r & ~kLeafBit) : r));
    const box bn = merge(bl, br);
    boxes[node] = bn;
    const uint32_t cnt = ((l & kLeafBit) ? 1u : __ldcg(tri_count + l)) +
                         ((r & kLeafBit) ? 1u : __ldcg(tri_count + r));
    tri_count[node] = cnt;
    float cl[9], cr[9];
    for (int i = 1; i <= 8; ++i) {
      cl[i] = child_cost(l, bl, cost, i);
      cr[i] = child_cost(r, br, cost, i);
    }
    float best = INFINITY;
    uint8_t bk = 1;
    for (int k = 1; k < 8; ++k) {
      const float x = cl[k] + cr[8 - k];
      if (x < best) {
        best = x;
        bk = (uint8_t)k;
      }
    }
    wide_k[node] = bk;
    float c = area(bn) * kCostNode + best;
    uint8_t h1 = kWide;
    if (cnt <= kSlotMaxTris && area(bn) * (float)cnt * kCostTri < c) {
      // every triangle of the subtree in one leaf slot
      c = area(bn) * (float)cnt * kCostTri;
      h1 = kLeafSlot;
    }
    cost[8 * (size_t)node] = c;
    how[8 * (size_t)node] = h1;
    for (int i = 2; i <= 8; ++i) {
      uint8_t h = kFewer;
      for (int k = 1; k < i; ++k) {
        const float x = cl[k] + cr[i - k];
        if (x < c) {
          c = x;
          h = (uint8_t)(kOpen + k);
        }
      }
      cost[8 * (size_t)node + (i - 1)] = c;
      how[8 * (size_t)node + (i - 1)] = h;
    }
    if (node == 0) {
      return;
    }
    node = parent[node];
  }
}

// the exact-plane frame of one axis (as the host builder): origin a
// multiple of the power-of-two scale, every decoded plane representable
__device__ void axis_frame(float lo, float hi, float *p_out, uint8_t *e_out) {
  const double extent = (double)hi - (double)lo;
  int e = extent > 0.0 ? (int)ceil(log2(extent / 255.0)) : -126;
  if (e < -126) {
    e = -126;
  }
  for (int guard = 0; guard < 300; ++guard, ++e) {
    const double s = ldexp(1.0, e);
    const double k = floor((double)lo / s);
    const double q_hi = ceil(((double)hi - k * s) / s);
    if (q_hi <= 255.0 && fabs(k) + 256.0 < 16777216.0) {
      *p_out = (float)(k * s);
      *e_out = (uint8_t)(e + 127);
      return;
    }
  }
  *p_out = lo;
  *e_out = 254;
}

__device__ __forceinline__ float exp_scale(uint8_t e) { return __uint_as_float((uint32_t)e << 23); }

struct Entry {
  uint32_t bin;  // binary node id
  uint32_t wide; // its wide node
};

__global__ void k_collapse(const float *t9, const uint32_t *perm, const uint32_t *item_tri,
                           uint32_t n, const uint32_t *left,
                           const uint32_t *right, const box *boxes, const uint8_t *how,
                           const uint8_t *wide_k, const Entry *in, uint32_t n_in, Entry *out,
                           uint32_t *counters, WideNode *nodes, float *wide_tris) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_in) {
    return;
  }
  const Entry e = in[q];
  auto box_of = [&](uint32_t id) -> box {
    return boxes[(id & kLeafBit) ? (n - 1) + (id & ~kLeafBit) : (id & ~kSlotBit)];
  };
  // the sorted positions of the triangles under internal node v (at most
  // kSlotMaxTris), left to right
  auto slot_tris = [&](uint32_t v, uint32_t *tris) -> uint32_t {
    uint32_t st[2 * kSlotMaxTris], sp = 0, cnt = 0;
    st[sp++] = v;
    while (sp > 0 && cnt < kSlotMaxTris) {
      const uint32_t u = st[--sp];
      if (u & kLeafBit) {
        tris[cnt++] = u & ~kLeafBit;
      } else if (sp + 2 <= 2 * kSlotMaxTris) {
        st[sp++] = right[u];
        st[sp++] = left[u];
      }
    }
    return cnt;
  };
  uint32_t kids[8];
  uint32_t nk = 0;
  if (e.bin & kLeafBit) {
    kids[nk++] = e.bin;
  } else {
    // the best forest of eight slots: (subtree, slots) pairs still to decode
    uint32_t st_node[8], st_slots[8];
    uint32_t sp = 0;
    const uint32_t k = wide_k[e.bin];
    st_node[sp] = right[e.bin];
    st_slots[sp++] = 8 - k;
    st_node[sp] = left[e.bin];
    st_slots[sp++] = k;
    while (sp > 0 && nk < 8) {
      --sp;
      const uint32_t v = st_node[sp];
      uint32_t i = st_slots[sp];
      if (v & kLeafBit) {
        kids[nk++] = v; // a triangle
        continue;
      }
      while (i > 1 && how[8 * (size_t)v + (i - 1)] == kFewer) {
        --i;
      }
      const uint8_t h = how[8 * (size_t)v + (i - 1)];
      if (h == kLeafSlot) {
        kids[nk++] = v | kSlotBit; // one slot of all its triangles
      } else if (i == 1 || h == kWide) {
        kids[nk++] = v; // a wide node of its own
      } else {
        const uint32_t kk = h - kOpen; // 1 <= kk < i: both children get a slot
        st_node[sp] = right[v];
        st_slots[sp++] = i - kk;
        st_node[sp] = left[v];
        st_slots[sp++] = kk;
      }
    }
  }
  box all = empty_box();
  for (uint32_t i = 0; i < nk; ++i) {
    all = merge(all, box_of(kids[i]));
  }
  // octant slots: slot bit a set = high side of axis a, greedy by score
  int at[8];
  bool placed[8];
  for (int s = 0; s < 8; ++s) {
    at[s] = -1;
    placed[s] = false;
  }
  float cen[3];
  for (int a = 0; a < 3; ++a) {
    cen[a] = 0.5f * (all.lo.get(a) + all.hi.get(a));
  }
  for (uint32_t round = 0; round < nk; ++round) {
    float best = 0.f;
    int bk = -1, bs = -1;
    for (uint32_t k = 0; k < nk; ++k) {
      if (placed[k]) {
        continue;
      }
      const box bb = box_of(kids[k]);
      float c[3];
      for (int a = 0; a < 3; ++a) {
        c[a] = 0.5f * (bb.lo.get(a) + bb.hi.get(a)) - cen[a];
      }
      for (int s = 0; s < 8; ++s) {
        if (at[s] >= 0) {
          continue;
        }
        float v = 0.f;
        for (int a = 0; a < 3; ++a) {
          v += ((s >> a) & 1) ? c[a] : -c[a];
        }
        if (bk < 0 || v > best) {
          best = v;
          bk = (int)k;
          bs = s;
        }
      }
    }
    placed[bk] = true;
    at[bs] = bk;
  }
  uint32_t n_int = 0, n_leaf = 0;
  for (uint32_t i = 0; i < nk; ++i) {
    if (kids[i] & kLeafBit) {
      ++n_leaf;
    } else if (kids[i] & kSlotBit) {
      uint32_t tmp[kSlotMaxTris];
      n_leaf += slot_tris(kids[i] & ~kSlotBit, tmp);
    } else {
      ++n_int;
    }
  }
  const uint32_t child_base = n_int ? atomicAdd(&counters[0], n_int) : 0u;
  const uint32_t tri_base = n_leaf ? atomicAdd(&counters[1], n_leaf) : 0u;
  WideNode wn;
  uint8_t *raw = reinterpret_cast<uint8_t *>(&wn);
  for (size_t k = 0; k < sizeof(WideNode); ++k) {
    raw[k] = 0;
  }
  for (int a = 0; a < 3; ++a) {
    axis_frame(all.lo.get(a), all.hi.get(a), &wn.p[a], &wn.e[a]);
  }
  wn.child_base = child_base;
  wn.tri_base = tri_base;
  uint32_t rank = 0, tri_off = 0;
  for (int s = 0; s < 8; ++s) {
    if (at[s] < 0) {
      for (int a = 0; a < 3; ++a) {
        wn.qlo[a][s] = 255;
        wn.qhi[a][s] = 0;
      }
      continue;
    }
    const uint32_t id = kids[at[s]];
    const box cb = box_of(id);
    for (int a = 0; a < 3; ++a) {
      const double sc = (double)exp_scale(wn.e[a]);
      const double lo = floor(((double)cb.lo.get(a) - (double)wn.p[a]) / sc);
      const double hi = ceil(((double)cb.hi.get(a) - (double)wn.p[a]) / sc);
      wn.qlo[a][s] = (uint8_t)fmax(0.0, fmin(255.0, lo));
      wn.qhi[a][s] = (uint8_t)fmax(0.0, fmin(255.0, hi));
    }
    if (id & (kLeafBit | kSlotBit)) {
      // the slot's items; their triangles' Morton positions are the
      // BVH-order indices
      uint32_t ks[kSlotMaxTris];
      uint32_t cnt = 1;
      if (id & kLeafBit) {
        ks[0] = id & ~kLeafBit;
      } else {
        cnt = slot_tris(id & ~kSlotBit, ks);
      }
      for (uint32_t t = 0; t < cnt; ++t) {
        const uint32_t k = item_tri[ks[t]];
        const uint32_t o = perm[k];
        const f3 v0 = vert(t9, o, 0), v1 = vert(t9, o, 1), v2 = vert(t9, o, 2);
        const f3 e1 = v1 - v0, e2 = v2 - v0;
        float *dst = wide_tris + 12 * (size_t)(tri_base + tri_off + t);
        const float vals[12] = {v0.x, v0.y, v0.z, e1.x, e1.y, e1.z, e2.x, e2.y,
                                e2.z, __uint_as_float(k), 0.f, 0.f};
        for (int j = 0; j < 12; ++j) {
          dst[j] = vals[j];
        }
      }
      wn.meta[s] = (uint8_t)((cnt << 5) | tri_off);
      tri_off += cnt;
    } else {
      wn.imask |= (uint8_t)(1u << s);
      wn.meta[s] = (uint8_t)rank;
      const uint32_t slot = atomicAdd(&counters[2], 1u);
      out[slot].bin = id;
      out[slot].wide = child_base + rank;
      ++rank;
    }
  }
  nodes[e.wide] = wn;
}

} // namespace
} // namespace dev

namespace {

// the stream of the build this host thread is running (its scratch buffers
// are allocated and freed in that stream's order)
thread_local cudaStream_t t_build_stream = nullptr;

// Scratch device memory of one build: cudaMallocAsync / cudaFreeAsync in the
// build's stream, which, unlike cudaFree, do not synchronise the device, so
// builds run from several host threads on their own streams overlap.
class ScratchBuffer {
public:
  ScratchBuffer() = default;
  ScratchBuffer(const ScratchBuffer &) = delete;
  ScratchBuffer &operator=(const ScratchBuffer &) = delete;
  ~ScratchBuffer() { release(); }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= size_ && ptr_ != nullptr) {
      return cudaSuccess;
    }
    release();
    if (bytes == 0) {
      return cudaSuccess;
    }
    stream_ = t_build_stream;
    cudaError_t e = cudaMallocAsync(&ptr_, bytes, stream_);
    if (e != cudaSuccess) {
      ptr_ = nullptr;
      return e;
    }
    size_ = bytes;
    return cudaSuccess;
  }
  void release() {
    if (ptr_ != nullptr) {
      cudaFreeAsync(ptr_, stream_);
      ptr_ = nullptr;
      size_ = 0;
    }
  }
  void *get() const { return ptr_; }
  template <typename T> T *as() const { return static_cast<T *>(ptr_); }

private:
  void *ptr_ = nullptr;
  size_t size_ = 0;
  cudaStream_t stream_ = nullptr;
};

// the binary tree over the Morton-sorted triangles by PLOC (left, right:
// internal nodes 0..n-2, 0 the root; parent of every node)
Status ploc_tree(const box *item_box, uint32_t n, uint32_t *left, uint32_t *right,
                 uint32_t *parent, cudaStream_t s) {
#define PG_PL_TRY(expr, what)                                                  \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      return cuda_status(e_, what);                                            \
    }                                                                          \
  } while (0)
  const size_t nn = n;
  t_build_stream = s;
  ScratchBuffer clus[2], cbox[2], nbr, keep, keep_pos, merges, merge_pos, tmp, tail;
  for (int k = 0; k < 2; ++k) {
    PG_PL_TRY(clus[k].ensure(nn * 4), "ploc");
    PG_PL_TRY(cbox[k].ensure(nn * sizeof(box)), "ploc");
  }
  PG_PL_TRY(nbr.ensure(nn * 4), "ploc");
  PG_PL_TRY(keep.ensure(nn * 4), "ploc");
  PG_PL_TRY(keep_pos.ensure(nn * 4), "ploc");
  PG_PL_TRY(merges.ensure(nn * 4), "ploc");
  PG_PL_TRY(merge_pos.ensure(nn * 4), "ploc");
  PG_PL_TRY(tail.ensure(16), "ploc");
  size_t tmp_bytes = 0;
  PG_PL_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, keep.as<uint32_t>(),
                                          keep_pos.as<uint32_t>(), (int)n, s),
            "ploc scan");
  PG_PL_TRY(tmp.ensure(std::max<size_t>(tmp_bytes, 16)), "ploc");
  const uint32_t bs = 256;
  dev::k_ploc_init<<<(n + bs - 1) / bs, bs, 0, s>>>(item_box, n, clus[0].as<uint32_t>(),
                                                    cbox[0].as<box>());
  PG_PL_TRY(cudaGetLastError(), "ploc init");
  uint32_t m = n, id_base = n - 1, cur = 0;
  // every round merges at least one pair, so n - 1 rounds always suffice
  for (uint32_t round = 0; m > 1; ++round) {
    if (round > n) {
      return Status::err(PATH_ERR_DEVICE_TIMEOUT, "gpu build: clustering did not finish");
    }
    const uint32_t nb = (m + bs - 1) / bs;
    dev::k_ploc_nn<<<nb, bs, 0, s>>>(cbox[cur].as<box>(), m, nbr.as<uint32_t>());
    dev::k_ploc_mark<<<nb, bs, 0, s>>>(nbr.as<uint32_t>(), m, keep.as<uint32_t>(),
                                       merges.as<uint32_t>());
    PG_PL_TRY(cudaGetLastError(), "ploc neighbours");
    // merges in this round: last exclusive prefix + last flag
    PG_PL_TRY(cub::DeviceScan::ExclusiveSum(tmp.get(), tmp_bytes, merges.as<uint32_t>(),
                                            merge_pos.as<uint32_t>(), (int)m, s),
              "ploc scan");
    uint32_t h[2];
    PG_PL_TRY(cudaMemcpyAsync(&h[0], merge_pos.as<uint32_t>() + (m - 1), 4,
                              cudaMemcpyDeviceToHost, s),
              "ploc count");
    PG_PL_TRY(cudaMemcpyAsync(&h[1], merges.as<uint32_t>() + (m - 1), 4, cudaMemcpyDeviceToHost,
                              s),
              "ploc count");
    PG_PL_TRY(cudaStreamSynchronize(s), "ploc count");
    uint32_t n_merge = h[0] + h[1];
    if (n_merge == 0) {
      // no mutual pair (exact ties): merge neighbours pairwise this round
      dev::k_ploc_force<<<nb, bs, 0, s>>>(m, nbr.as<uint32_t>(), keep.as<uint32_t>(),
                                          merges.as<uint32_t>());
      PG_PL_TRY(cub::DeviceScan::ExclusiveSum(tmp.get(), tmp_bytes, merges.as<uint32_t>(),
                                              merge_pos.as<uint32_t>(), (int)m, s),
                "ploc scan");
      n_merge = m / 2;
    }
    PG_PL_TRY(cub::DeviceScan::ExclusiveSum(tmp.get(), tmp_bytes, keep.as<uint32_t>(),
                                            keep_pos.as<uint32_t>(), (int)m, s),
              "ploc scan");
    dev::k_ploc_merge<<<nb, bs, 0, s>>>(
        clus[cur].as<uint32_t>(), cbox[cur].as<box>(), nbr.as<uint32_t>(), keep.as<uint32_t>(),
        keep_pos.as<uint32_t>(), merges.as<uint32_t>(), merge_pos.as<uint32_t>(), m, n, id_base,
        left, right, parent, clus[cur ^ 1].as<uint32_t>(), cbox[cur ^ 1].as<box>());
    PG_PL_TRY(cudaGetLastError(), "ploc merge");
    id_base -= n_merge;
    m -= n_merge;
    cur ^= 1;
  }
  if (id_base != 0) {
    return Status::err(PATH_ERR_DEVICE_TIMEOUT, "gpu build: clustering left nodes unassigned");
  }
  return Status::ok();
#undef PG_PL_TRY
}

} // namespace

Status gpu_build_wide(const float *t9, uint32_t n, const float *lo, const float *hi,
                      bool split, cudaStream_t s, GpuWideBVH &out) {
  out.n_nodes = 0;
  out.n_wide_tris = 0;
  out.depth = 0;
  if (n == 0) {
    return Status::ok();
  }
#define PG_GB_TRY(expr, what)                                                  \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      return cuda_status(e_, what);                                            \
    }                                                                          \
  } while (0)
  const size_t nn = n;
  t_build_stream = s;
  ScratchBuffer keys, vals, keys2, tmp, left, right, parent, boxes, flags, qa, qb, counters, cost,
      how, wide_k, tri_count;
  PG_GB_TRY(keys.ensure(nn * 4), "gpu build");
  PG_GB_TRY(vals.ensure(nn * 4), "gpu build");
  PG_GB_TRY(keys2.ensure(nn * 4), "gpu build");
  PG_GB_TRY(out.perm.ensure(nn * 4), "gpu build");
  f3 flo = mk(lo[0], lo[1], lo[2]);
  f3 inv = mk(1.f / fmaxf(hi[0] - lo[0], 1e-20f), 1.f / fmaxf(hi[1] - lo[1], 1e-20f),
              1.f / fmaxf(hi[2] - lo[2], 1e-20f));
  const uint32_t bs = 256, nb = (n + bs - 1) / bs;
  dev::k_morton<<<nb, bs, 0, s>>>(t9, n, flo, inv, keys.as<uint32_t>(), vals.as<uint32_t>());
  PG_GB_TRY(cudaGetLastError(), "morton codes");
  size_t tmp_bytes = 0;
  PG_GB_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.as<uint32_t>(),
                                            keys2.as<uint32_t>(), vals.as<uint32_t>(),
                                            out.perm.as<uint32_t>(), (int)n, 0, 30, s),
            "radix sort");
  PG_GB_TRY(tmp.ensure(std::max<size_t>(tmp_bytes, 16)), "gpu build");
  PG_GB_TRY(cub::DeviceRadixSort::SortPairs(tmp.get(), tmp_bytes, keys.as<uint32_t>(),
                                            keys2.as<uint32_t>(), vals.as<uint32_t>(),
                                            out.perm.as<uint32_t>(), (int)n, 0, 30, s),
            "radix sort");
  // the items the tree is built over: triangles, or their references
  ScratchBuffer item_tri, item_box;
  uint32_t m = n;
  if (!split) {
    PG_GB_TRY(item_tri.ensure(nn * 4), "gpu build");
    PG_GB_TRY(item_box.ensure(nn * sizeof(box)), "gpu build");
    dev::k_items_plain<<<nb, bs, 0, s>>>(t9, out.perm.as<uint32_t>(), n,
                                         item_tri.as<uint32_t>(), item_box.as<box>());
    PG_GB_TRY(cudaGetLastError(), "items");
  } else {
    // budget: 30% more references than triangles, shared by priority
    ScratchBuffer prio, count, offset, sum, ref_tri, ref_box, rkeys, rvals, rkeys2, rorder;
    PG_GB_TRY(prio.ensure(nn * 4), "gpu build");
    PG_GB_TRY(count.ensure(nn * 4), "gpu build");
    PG_GB_TRY(offset.ensure(nn * 4), "gpu build");
    PG_GB_TRY(sum.ensure(16), "gpu build");
    dev::k_split_priority<<<nb, bs, 0, s>>>(t9, out.perm.as<uint32_t>(), n, prio.as<float>());
    PG_GB_TRY(cudaGetLastError(), "split priority");
    size_t rb = 0;
    PG_GB_TRY(cub::DeviceReduce::Sum(nullptr, rb, prio.as<float>(), sum.as<float>(), (int)n, s),
              "split budget");
    ScratchBuffer rtmp;
    PG_GB_TRY(rtmp.ensure(std::max<size_t>(rb, 16)), "gpu build");
    PG_GB_TRY(cub::DeviceReduce::Sum(rtmp.get(), rb, prio.as<float>(), sum.as<float>(), (int)n, s),
              "split budget");
    float total = 0.f;
    PG_GB_TRY(cudaMemcpyAsync(&total, sum.get(), 4, cudaMemcpyDeviceToHost, s), "split budget");
    PG_GB_TRY(cudaStreamSynchronize(s), "split budget");
    const float scale = total > 0.f ? 0.3f * (float)n / total : 0.f;
    dev::k_split_count<<<nb, bs, 0, s>>>(prio.as<float>(), n, scale, count.as<uint32_t>());
    PG_GB_TRY(cudaGetLastError(), "split count");
    size_t sb = 0;
    PG_GB_TRY(cub::DeviceScan::ExclusiveSum(nullptr, sb, count.as<uint32_t>(),
                                            offset.as<uint32_t>(), (int)n, s),
              "split offsets");
    PG_GB_TRY(rtmp.ensure(std::max<size_t>({rb, sb, 16})), "gpu build");
    PG_GB_TRY(cub::DeviceScan::ExclusiveSum(rtmp.get(), sb, count.as<uint32_t>(),
                                            offset.as<uint32_t>(), (int)n, s),
              "split offsets");
    uint32_t last[2] = {0, 0};
    PG_GB_TRY(cudaMemcpyAsync(&last[0], offset.as<uint32_t>() + (n - 1), 4,
                              cudaMemcpyDeviceToHost, s),
              "split offsets");
    PG_GB_TRY(cudaMemcpyAsync(&last[1], count.as<uint32_t>() + (n - 1), 4,
                              cudaMemcpyDeviceToHost, s),
              "split offsets");
    PG_GB_TRY(cudaStreamSynchronize(s), "split offsets");
    m = last[0] + last[1];
    const size_t mm = m;
    PG_GB_TRY(ref_tri.ensure(mm * 4), "gpu build");
    PG_GB_TRY(ref_box.ensure(mm * sizeof(box)), "gpu build");
    dev::k_split_emit<<<nb, bs, 0, s>>>(t9, out.perm.as<uint32_t>(), n, count.as<uint32_t>(),
                                        offset.as<uint32_t>(), ref_tri.as<uint32_t>(),
                                        ref_box.as<box>());
    PG_GB_TRY(cudaGetLastError(), "split references");
    // references in Morton order of their boxes' centres
    PG_GB_TRY(rkeys.ensure(mm * 4), "gpu build");
    PG_GB_TRY(rvals.ensure(mm * 4), "gpu build");
    PG_GB_TRY(rkeys2.ensure(mm * 4), "gpu build");
    PG_GB_TRY(rorder.ensure(mm * 4), "gpu build");
    const uint32_t mb = (m + bs - 1) / bs;
    dev::k_morton_box<<<mb, bs, 0, s>>>(ref_box.as<box>(), m, flo, inv, rkeys.as<uint32_t>(),
                                        rvals.as<uint32_t>());
    PG_GB_TRY(cudaGetLastError(), "reference codes");
    size_t ob = 0;
    PG_GB_TRY(cub::DeviceRadixSort::SortPairs(nullptr, ob, rkeys.as<uint32_t>(),
                                              rkeys2.as<uint32_t>(), rvals.as<uint32_t>(),
                                              rorder.as<uint32_t>(), (int)m, 0, 30, s),
              "reference sort");
    PG_GB_TRY(rtmp.ensure(std::max<size_t>({rb, sb, ob, 16})), "gpu build");
    PG_GB_TRY(cub::DeviceRadixSort::SortPairs(rtmp.get(), ob, rkeys.as<uint32_t>(),
                                              rkeys2.as<uint32_t>(), rvals.as<uint32_t>(),
                                              rorder.as<uint32_t>(), (int)m, 0, 30, s),
              "reference sort");
    PG_GB_TRY(item_tri.ensure(mm * 4), "gpu build");
    PG_GB_TRY(item_box.ensure(mm * sizeof(box)), "gpu build");
    dev::k_items_refs<<<mb, bs, 0, s>>>(rorder.as<uint32_t>(), ref_tri.as<uint32_t>(),
                                        ref_box.as<box>(), m, item_tri.as<uint32_t>(),
                                        item_box.as<box>());
    PG_GB_TRY(cudaGetLastError(), "items");
    PG_GB_TRY(cudaStreamSynchronize(s), "gpu build");
  }
  const size_t mm = m;
  const uint32_t mb = (m + bs - 1) / bs;
  const size_t n_int = mm > 1 ? mm - 1 : 0;
  PG_GB_TRY(left.ensure(std::max<size_t>(n_int, 1) * 4), "gpu build");
  PG_GB_TRY(right.ensure(std::max<size_t>(n_int, 1) * 4), "gpu build");
  PG_GB_TRY(parent.ensure((n_int + mm) * 4), "gpu build");
  PG_GB_TRY(boxes.ensure((n_int + mm) * sizeof(box)), "gpu build");
  PG_GB_TRY(flags.ensure(std::max<size_t>(n_int, 1) * 4), "gpu build");
  PG_GB_TRY(cudaMemsetAsync(flags.get(), 0, std::max<size_t>(n_int, 1) * 4, s), "gpu build");
  PG_GB_TRY(cost.ensure(std::max<size_t>(n_int, 1) * 32), "gpu build");
  PG_GB_TRY(how.ensure(std::max<size_t>(n_int, 1) * 8), "gpu build");
  PG_GB_TRY(wide_k.ensure(std::max<size_t>(n_int, 1)), "gpu build");
  PG_GB_TRY(tri_count.ensure(std::max<size_t>(n_int, 1) * 4), "gpu build");
  if (n_int > 0) {
    Status sp = ploc_tree(item_box.as<box>(), m, left.as<uint32_t>(), right.as<uint32_t>(),
                          parent.as<uint32_t>(), s);
    if (!sp.good()) {
      return sp;
    }
  }
  dev::k_boxes<<<mb, bs, 0, s>>>(item_box.as<box>(), m, left.as<uint32_t>(),
                                 right.as<uint32_t>(), parent.as<uint32_t>(), boxes.as<box>(),
                                 flags.as<uint32_t>(), cost.as<float>(), how.as<uint8_t>(),
                                 wide_k.as<uint8_t>(), tri_count.as<uint32_t>());
  PG_GB_TRY(cudaGetLastError(), "boxes");
  // collapse: a wide node has at most 8 children and at least 2 binary
  // nodes below it, so m wide nodes and m queue entries always suffice
  PG_GB_TRY(out.nodes.ensure(mm * sizeof(WideNode)), "gpu build");
  PG_GB_TRY(out.wide_tris.ensure(mm * 48), "gpu build");
  PG_GB_TRY(qa.ensure(mm * sizeof(dev::Entry)), "gpu build");
  PG_GB_TRY(qb.ensure(mm * sizeof(dev::Entry)), "gpu build");
  PG_GB_TRY(counters.ensure(16), "gpu build");
  // counters: [0] wide nodes allocated, [1] triangles placed, [2] next queue
  uint32_t h_init[4] = {1, 0, 0, 0};
  PG_GB_TRY(cudaMemcpyAsync(counters.get(), h_init, 16, cudaMemcpyHostToDevice, s),
            "gpu build");
  dev::Entry root{m > 1 ? 0u : (0u | dev::kLeafBit), 0u};
  PG_GB_TRY(cudaMemcpyAsync(qa.get(), &root, sizeof(root), cudaMemcpyHostToDevice, s),
            "gpu build");
  uint32_t n_in = 1, depth = 0;
  ScratchBuffer *cur = &qa, *nxt = &qb;
  while (n_in > 0) {
    PG_GB_TRY(cudaMemsetAsync(counters.as<uint32_t>() + 2, 0, 4, s), "gpu build");
    dev::k_collapse<<<(n_in + 127) / 128, 128, 0, s>>>(
        t9, out.perm.as<uint32_t>(), item_tri.as<uint32_t>(), m, left.as<uint32_t>(),
        right.as<uint32_t>(), boxes.as<box>(), how.as<uint8_t>(), wide_k.as<uint8_t>(),
        cur->as<dev::Entry>(), n_in, nxt->as<dev::Entry>(), counters.as<uint32_t>(),
        out.nodes.as<WideNode>(), out.wide_tris.as<float>());
    PG_GB_TRY(cudaGetLastError(), "collapse");
    uint32_t h[4];
    PG_GB_TRY(cudaMemcpyAsync(h, counters.get(), 16, cudaMemcpyDeviceToHost, s), "gpu build");
    PG_GB_TRY(cudaStreamSynchronize(s), "gpu build");
    n_in = h[2];
    out.n_nodes = h[0];
    out.n_wide_tris = h[1];
    ++depth;
    std::swap(cur, nxt);
    if (depth > 4096) {
      return Status::err(PATH_ERR_DEVICE_TIMEOUT, "gpu build did not finish");
    }
  }
  out.depth = depth - 1;
  return Status::ok();
#undef PG_GB_TRY
}

} // namespace pg
