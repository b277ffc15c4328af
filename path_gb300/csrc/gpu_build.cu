// 8-wide BVH built on the GPU: a linear BVH over Morton codes (Karras,
// "Maximizing Parallelism in the Construction of BVHs, Octrees, and k-d
// Trees", HPG 2012) collapsed top-down into the 80-byte quantised nodes of
// the traversal, one tree level per launch.
//
// Any BVH over the triangles gives the traversal the same closest hits (the
// 8-wide traversal takes the smallest distance, then the smallest BVH-order
// index, whatever the visiting order), so images rendered through this BVH
// are those of the SBVH built on the host, up to which of two triangles at
// exactly the same distance is reported.
//
// Stages: Morton code of each centroid (10 bits per axis) -> radix sort of
// (code, triangle) pairs -> internal nodes of the radix tree (longest common
// prefix, ties broken by position) with parent links -> boxes bottom-up (the
// second child to arrive at a node merges), together with the surface-area
// cost optimisation of the collapse (the host builder's: per binary node the
// cheapest forest of at most 1..8 slots, from its children's) -> collapse:
// every wide node takes the best forest of eight slots of its binary node's
// children, places them in octant slots (as the host builder does),
// quantises their boxes (the same exact-plane frame), and queues its
// internal children.
#include "geom.h"
#include "gpu_build.h"

#include <cub/device/device_radix_sort.cuh>

namespace pg {
namespace dev {
namespace {

constexpr uint32_t kLeafBit = 1u << 31; // node ids: internal i, or leaf k | kLeafBit

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

// common-prefix length of sorted positions i and j (-1 outside [0, n))
__device__ __forceinline__ int delta(const uint32_t *keys, uint32_t n, int i, int j) {
  if (j < 0 || j >= (int)n) {
    return -1;
  }
  const uint32_t a = keys[i], b = keys[j];
  if (a == b) {
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
  }
  return __clz(a ^ b);
}

__global__ void k_radix_tree(const uint32_t *keys, uint32_t n, uint32_t *left,
                             uint32_t *right, uint32_t *parent) {
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= (int)n - 1) {
    return;
  }
  const int d = delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1) >= 0 ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) {
    lmax *= 2;
  }
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2) {
    if (delta(keys, n, i, i + (l + t) * d) > dmin) {
      l += t;
    }
  }
  const int j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int s = 0;
  int t = l;
  do {
    t = (t + 1) / 2;
    if (delta(keys, n, i, i + (s + t) * d) > dnode) {
      s += t;
    }
  } while (t > 1);
  const int gamma = i + s * d + (d < 0 ? -1 : 0);
  const uint32_t lc = (min(i, j) == gamma) ? ((uint32_t)gamma | kLeafBit) : (uint32_t)gamma;
  const uint32_t rc =
      (max(i, j) == gamma + 1) ? ((uint32_t)(gamma + 1) | kLeafBit) : (uint32_t)(gamma + 1);
  left[i] = lc;
  right[i] = rc;
  parent[(lc & kLeafBit) ? (n - 1) + (lc & ~kLeafBit) : lc] = (uint32_t)i;
  parent[(rc & kLeafBit) ? (n - 1) + (rc & ~kLeafBit) : rc] = (uint32_t)i;
}

__device__ __forceinline__ box tri_box(const float *t9, uint32_t i) {
  box b = empty_box();
  b = grow(b, vert(t9, i, 0));
  b = grow(b, vert(t9, i, 1));
  b = grow(b, vert(t9, i, 2));
  return b;
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
// how the best forest of <= i slots represents a binary subtree
constexpr uint8_t kFewer = 0, kWide = 1, kOpen = 3; // kOpen + k: k slots left

// the cost of child c's best forest of <= i slots (i = 1..8)
__device__ __forceinline__ float child_cost(uint32_t c, const box &cb, const float *cost,
                                            int i) {
  return (c & kLeafBit) ? area(cb) * kCostTri : __ldcg(cost + 8 * (size_t)c + (i - 1));
}

// boxes [internal n-1 | leaves n] and the collapse costs of internal nodes
// ([n-1][8] cost and decision of the forests of 1..8 slots, the left share
// of a wide node's 8 slots), bottom-up; flags start at zero
__global__ void k_boxes(const float *t9, const uint32_t *perm, uint32_t n, const uint32_t *left,
                        const uint32_t *right, const uint32_t *parent, box *boxes,
                        uint32_t *flags, float *cost, uint8_t *how, uint8_t *wide_k) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) {
    return;
  }
  boxes[(n - 1) + k] = tri_box(t9, perm[k]);
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
    cost[8 * (size_t)node] = c;
    how[8 * (size_t)node] = kWide;
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

__global__ void k_collapse(const float *t9, const uint32_t *perm, uint32_t n, const uint32_t *left,
                           const uint32_t *right, const box *boxes, const uint8_t *how,
                           const uint8_t *wide_k, const Entry *in, uint32_t n_in, Entry *out,
                           uint32_t *counters, WideNode *nodes, float *wide_tris) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_in) {
    return;
  }
  const Entry e = in[q];
  auto box_of = [&](uint32_t id) -> box {
    return boxes[(id & kLeafBit) ? (n - 1) + (id & ~kLeafBit) : id];
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
      if (i == 1 || h == kWide) {
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
    if (id & kLeafBit) {
      const uint32_t k = id & ~kLeafBit; // sorted position = BVH-order index
      const uint32_t o = perm[k];
      const f3 v0 = vert(t9, o, 0), v1 = vert(t9, o, 1), v2 = vert(t9, o, 2);
      const f3 e1 = v1 - v0, e2 = v2 - v0;
      float *dst = wide_tris + 12 * (size_t)(tri_base + tri_off);
      const float vals[12] = {v0.x, v0.y, v0.z, e1.x, e1.y, e1.z, e2.x, e2.y,
                              e2.z, __uint_as_float(k), 0.f, 0.f};
      for (int j = 0; j < 12; ++j) {
        dst[j] = vals[j];
      }
      wn.meta[s] = (uint8_t)((1u << 5) | tri_off);
      ++tri_off;
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

Status gpu_build_wide(const float *t9, uint32_t n, const float *lo, const float *hi,
                      cudaStream_t s, GpuWideBVH &out) {
  out.n_nodes = 0;
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
  DeviceBuffer keys, vals, keys2, tmp, left, right, parent, boxes, flags, qa, qb, counters, cost,
      how, wide_k;
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
  const size_t n_int = nn > 1 ? nn - 1 : 0;
  PG_GB_TRY(left.ensure(std::max<size_t>(n_int, 1) * 4), "gpu build");
  PG_GB_TRY(right.ensure(std::max<size_t>(n_int, 1) * 4), "gpu build");
  PG_GB_TRY(parent.ensure((n_int + nn) * 4), "gpu build");
  PG_GB_TRY(boxes.ensure((n_int + nn) * sizeof(box)), "gpu build");
  PG_GB_TRY(flags.ensure(std::max<size_t>(n_int, 1) * 4), "gpu build");
  PG_GB_TRY(cudaMemsetAsync(flags.get(), 0, std::max<size_t>(n_int, 1) * 4, s), "gpu build");
  PG_GB_TRY(cost.ensure(std::max<size_t>(n_int, 1) * 32), "gpu build");
  PG_GB_TRY(how.ensure(std::max<size_t>(n_int, 1) * 8), "gpu build");
  PG_GB_TRY(wide_k.ensure(std::max<size_t>(n_int, 1)), "gpu build");
  if (n_int > 0) {
    dev::k_radix_tree<<<(uint32_t)((n_int + bs - 1) / bs), bs, 0, s>>>(
        keys2.as<uint32_t>(), n, left.as<uint32_t>(), right.as<uint32_t>(),
        parent.as<uint32_t>());
    PG_GB_TRY(cudaGetLastError(), "radix tree");
  }
  dev::k_boxes<<<nb, bs, 0, s>>>(t9, out.perm.as<uint32_t>(), n, left.as<uint32_t>(),
                                 right.as<uint32_t>(), parent.as<uint32_t>(), boxes.as<box>(),
                                 flags.as<uint32_t>(), cost.as<float>(), how.as<uint8_t>(),
                                 wide_k.as<uint8_t>());
  PG_GB_TRY(cudaGetLastError(), "boxes");
  // collapse: a wide node has at most 8 children and at least 2 binary
  // nodes below it, so n wide nodes and n queue entries always suffice
  PG_GB_TRY(out.nodes.ensure(nn * sizeof(WideNode)), "gpu build");
  PG_GB_TRY(out.wide_tris.ensure(nn * 48), "gpu build");
  PG_GB_TRY(qa.ensure(nn * sizeof(dev::Entry)), "gpu build");
  PG_GB_TRY(qb.ensure(nn * sizeof(dev::Entry)), "gpu build");
  PG_GB_TRY(counters.ensure(16), "gpu build");
  // counters: [0] wide nodes allocated, [1] triangles placed, [2] next queue
  uint32_t h_init[4] = {1, 0, 0, 0};
  PG_GB_TRY(cudaMemcpyAsync(counters.get(), h_init, 16, cudaMemcpyHostToDevice, s),
            "gpu build");
  dev::Entry root{n > 1 ? 0u : (0u | dev::kLeafBit), 0u};
  PG_GB_TRY(cudaMemcpyAsync(qa.get(), &root, sizeof(root), cudaMemcpyHostToDevice, s),
            "gpu build");
  uint32_t n_in = 1, depth = 0;
  DeviceBuffer *cur = &qa, *nxt = &qb;
  while (n_in > 0) {
    PG_GB_TRY(cudaMemsetAsync(counters.as<uint32_t>() + 2, 0, 4, s), "gpu build");
    dev::k_collapse<<<(n_in + 127) / 128, 128, 0, s>>>(
        t9, out.perm.as<uint32_t>(), n, left.as<uint32_t>(), right.as<uint32_t>(),
        boxes.as<box>(), how.as<uint8_t>(), wide_k.as<uint8_t>(), cur->as<dev::Entry>(), n_in,
        nxt->as<dev::Entry>(),
        counters.as<uint32_t>(), out.nodes.as<WideNode>(), out.wide_tris.as<float>());
    PG_GB_TRY(cudaGetLastError(), "collapse");
    uint32_t h[4];
    PG_GB_TRY(cudaMemcpyAsync(h, counters.get(), 16, cudaMemcpyDeviceToHost, s), "gpu build");
    PG_GB_TRY(cudaStreamSynchronize(s), "gpu build");
    n_in = h[2];
    out.n_nodes = h[0];
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
