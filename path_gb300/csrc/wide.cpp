// Compressed 8-wide BVH construction (see wide.h).
#include "wide.h"

#include <array>
#include <cmath>
#include <cstring>
#include <deque>

namespace pg {

namespace {

bool is_split(const BinaryNode &n) { return (n.w0 & kNodeTag) != 0; }

uint32_t leaf_count(const BinaryNode &n) { return (n.w1 & ~kNodeTag) - n.w0; }

// Origin and scale of one axis of a wide node: the origin is a multiple of
// the power-of-two scale, so every decoded plane p + q * 2^e (q < 256) is an
// exactly representable float.  Decoded boxes then contain the binary boxes
// exactly, and because float rounding is monotone the slab test on a
// decoded box passes whenever the reference's slab test on the contained
// box passes.
void axis_frame(float lo, float hi, float *p_out, uint8_t *e_out) {
  double extent = (double)hi - (double)lo;
  int e = extent > 0.0 ? (int)std::ceil(std::log2(extent / 255.0)) : -126;
  if (e < -126) {
    e = -126;
  }
  for (;; ++e) {
    double s = std::ldexp(1.0, e);
    double k = std::floor((double)lo / s);
    double q_hi = std::ceil(((double)hi - k * s) / s);
    if (q_hi <= 255.0 && std::fabs(k) + 256.0 < 16777216.0) {
      *p_out = (float)(k * s);
      *e_out = (uint8_t)(e + 127);
      return;
    }
  }
}

float exp_scale(uint8_t e) {
  uint32_t bits = (uint32_t)e << 23;
  float f;
  std::memcpy(&f, &bits, sizeof(f));
  return f;
}

// one slot of a wide node: an internal child, or (part of) a binary leaf
struct Slot {
  uint32_t bin;
  bool leaf;
  uint32_t first, count; // leaf: range in the binary leaf
};

// Places the (at most eight) slots so that slot bit a set means "on the high
// side of axis a": every slot direction d(s) = (+-1, +-1, +-1) takes the
// child whose centre lies furthest along d(s) from the node's centre,
// greedily by that score.  A ray with direction-sign octant o then meets
// the children roughly in the order of the slots o ^ 0, o ^ 1, ..., o ^ 7
// (nearest first), which the traversal uses instead of sorting.
std::array<int, 8> order_slots(const BinaryBVH &bvh, const std::vector<Slot> &slots,
                               const box &all) {
  std::array<int, 8> at;
  at.fill(-1);
  const size_t n = slots.size();
  double centre[3];
  for (int a = 0; a < 3; ++a) {
    centre[a] = 0.5 * ((double)all.lo.get(a) + (double)all.hi.get(a));
  }
  std::vector<std::array<double, 8>> score(n);
  for (size_t k = 0; k < n; ++k) {
    const box &b = bvh.nodes[slots[k].bin].aabb;
    double c[3];
    for (int a = 0; a < 3; ++a) {
      c[a] = 0.5 * ((double)b.lo.get(a) + (double)b.hi.get(a)) - centre[a];
    }
    for (int s = 0; s < 8; ++s) {
      double v = 0.0;
      for (int a = 0; a < 3; ++a) {
        v += ((s >> a) & 1) ? c[a] : -c[a];
      }
      score[k][(size_t)s] = v;
    }
  }
  std::vector<bool> placed(n, false);
  for (size_t round = 0; round < n; ++round) {
    double best = 0.0;
    int bk = -1, bs = -1;
    for (size_t k = 0; k < n; ++k) {
      if (placed[k]) {
        continue;
      }
      for (int s = 0; s < 8; ++s) {
        if (at[(size_t)s] >= 0) {
          continue;
        }
        if (bk < 0 || score[k][(size_t)s] > best) {
          best = score[k][(size_t)s];
          bk = (int)k;
          bs = s;
        }
      }
    }
    placed[(size_t)bk] = true;
    at[(size_t)bs] = bk;
  }
  return at;
}

} // namespace

box wide_child_box(const WideNode &n, int slot) {
  box b;
  for (int a = 0; a < 3; ++a) {
    float s = exp_scale(n.e[a]);
    b.lo.set(a, n.p[a] + (float)n.qlo[a][slot] * s);
    b.hi.set(a, n.p[a] + (float)n.qhi[a][slot] * s);
  }
  return b;
}

namespace {

// SAH weights of the collapse: a wide-node visit (eight box tests) against
// one triangle test, per unit of surface area
constexpr float kCostNode = 1.0f;
constexpr float kCostTri = 0.3f;
// triangles per leaf slot in the collapse: eight slots of at most four stay
// within the 32 triangles a node addresses
constexpr uint32_t kSlotTris = 4;

// how the best forest of <= i slots represents a binary subtree
enum How : uint8_t {
  kFewer = 0, // the forest of <= i - 1 slots
  kWide = 1,  // one wide node of its own
  kLeaf = 2,  // leaf slots (binary leaves only)
  kOpen = 3,  // kOpen + k: the left child's forest of <= k slots and the
              // right child's of <= i - k
};

struct Collapse {
  const BinaryBVH &bvh;
  std::vector<std::array<float, 9>> cost; // [node][i], i = 1..8 slots
  std::vector<std::array<uint8_t, 9>> how;
  std::vector<uint8_t> wide_k;            // left share of a wide node's 8 slots

  explicit Collapse(const BinaryBVH &b) : bvh(b) {}

  uint32_t left(uint32_t n) const { return bvh.nodes[n].w0 & ~kNodeTag; }
  uint32_t right(uint32_t n) const { return bvh.nodes[n].w1 & ~kNodeTag; }

  // Ylitie, Karras and Laine (HPG 2017), section 3.1: the cost of a subtree
  // as a forest of at most i slots of its parent wide node, minimised over
  // leaf slots, wide nodes and distributions of the slots between the two
  // children, bottom-up.
  void solve() {
    const size_t n = bvh.nodes.size();
    cost.assign(n, {});
    how.assign(n, {});
    wide_k.assign(n, 0);
    // post-order without recursion: a node after both of its children
    std::vector<uint32_t> order;
    order.reserve(n);
    std::vector<uint32_t> stack = {0};
    while (!stack.empty()) {
      const uint32_t v = stack.back();
      stack.pop_back();
      order.push_back(v);
      if (is_split(bvh.nodes[v])) {
        stack.push_back(left(v));
        stack.push_back(right(v));
      }
    }
    for (size_t o = order.size(); o-- > 0;) {
      const uint32_t v = order[o];
      const BinaryNode &b = bvh.nodes[v];
      const float a = area(b.aabb);
      std::array<float, 9> &c = cost[v];
      std::array<uint8_t, 9> &h = how[v];
      c[0] = INFINITY;
      if (!is_split(b)) {
        const uint32_t t = leaf_count(b);
        const uint32_t slots = std::max(1u, (t + kSlotTris - 1) / kSlotTris);
        const float tris = a * kCostTri * (float)t;
        for (uint32_t i = 1; i <= 8; ++i) {
          if (i >= slots) {
            c[i] = tris;
            h[i] = kLeaf;
          } else {
            c[i] = a * kCostNode + tris;
            h[i] = kWide;
          }
        }
        continue;
      }
      const std::array<float, 9> &cl = cost[left(v)], &cr = cost[right(v)];
      float best = INFINITY;
      uint8_t bk = 1;
      for (uint32_t k = 1; k < 8; ++k) {
        const float x = cl[k] + cr[8 - k];
        if (x < best) {
          best = x;
          bk = (uint8_t)k;
        }
      }
      wide_k[v] = bk;
      c[1] = a * kCostNode + best;
      h[1] = kWide;
      for (uint32_t i = 2; i <= 8; ++i) {
        c[i] = c[i - 1];
        h[i] = kFewer;
        for (uint32_t k = 1; k < i; ++k) {
          const float x = cl[k] + cr[i - k];
          if (x < c[i]) {
            c[i] = x;
            h[i] = (uint8_t)(kOpen + k);
          }
        }
      }
    }
  }

  // the slots of the best forest of <= i slots for subtree v
  void forest(uint32_t v, uint32_t i, std::vector<Slot> &out) const {
    while (how[v][i] == kFewer) {
      --i;
    }
    const uint8_t h = how[v][i];
    if (h == kWide) {
      out.push_back({v, false, 0, 0});
    } else if (h == kLeaf) {
      const uint32_t t = leaf_count(bvh.nodes[v]);
      if (t == 0) {
        out.push_back({v, true, 0, 0});
      }
      for (uint32_t f = 0; f < t; f += kSlotTris) {
        out.push_back({v, true, f, std::min(kSlotTris, t - f)});
      }
    } else {
      const uint32_t k = h - kOpen;
      forest(left(v), k, out);
      forest(right(v), i - k, out);
    }
  }
};

} // namespace

WideBVH build_wide(const BinaryBVH &bvh) {
  WideBVH out;
  if (bvh.nodes.empty()) {
    return out;
  }
  Collapse col(bvh);
  col.solve();
  // a wide node stands for binary node `bin`; for a binary leaf, for its
  // triangles from `first` on (a leaf of more than a node's 32 triangles
  // continues in a child node with the same box)
  struct Job {
    uint32_t wide;
    uint32_t bin;
    uint32_t first;
    uint32_t depth;
  };
  out.nodes.resize(1);
  // Nodes of depth < kBfsDepth are expanded breadth first, so the nodes of
  // depth <= kBfsDepth take the first indices level by level (a prefix of
  // them is what the trace kernel stages in shared memory); below that the
  // expansion is depth first, which keeps each subtree's nodes together.
  std::deque<Job> queue;
  std::vector<Job> stack;
  queue.push_back({0, 0, 0, 0});
  while (!queue.empty() || !stack.empty()) {
    Job job;
    if (!queue.empty()) {
      job = queue.front();
      queue.pop_front();
    } else {
      if (out.n_top == 0) {
        out.n_top = (uint32_t)out.nodes.size();
      }
      job = stack.back();
      stack.pop_back();
    }
    out.depth = std::max(out.depth, job.depth);
    std::vector<Slot> slots;
    const BinaryNode &root = bvh.nodes[job.bin];
    if (is_split(root)) {
      const uint32_t k = col.wide_k[job.bin];
      col.forest(col.left(job.bin), k, slots);
      col.forest(col.right(job.bin), 8 - k, slots);
    } else {
      const uint32_t t = leaf_count(root);
      uint32_t f = job.first, used = 0;
      if (t == 0) {
        slots.push_back({job.bin, true, 0, 0});
      }
      while (f < t && slots.size() < 7 && used + std::min(kMaxLeafTris, t - f) <= kMaxNodeTris) {
        const uint32_t c = std::min(kMaxLeafTris, t - f);
        slots.push_back({job.bin, true, f, c});
        f += c;
        used += c;
      }
      if (f < t) {
        slots.push_back({job.bin, false, f, 0}); // the rest of the leaf
      }
    }
    WideNode wn;
    std::memset(&wn, 0, sizeof(wn));
    box all = empty_box();
    for (const Slot &s : slots) {
      all = merge(all, bvh.nodes[s.bin].aabb);
    }
    for (int a = 0; a < 3; ++a) {
      axis_frame(all.lo.get(a), all.hi.get(a), &wn.p[a], &wn.e[a]);
    }
    uint32_t n_internal = 0;
    for (const Slot &s : slots) {
      n_internal += s.leaf ? 0u : 1u;
    }
    uint32_t child_base = (uint32_t)out.nodes.size();
    wn.child_base = child_base;
    wn.tri_base = (uint32_t)out.tri_index.size();
    // slot order: slot bit a set = high side of axis a (see order_slots)
    const std::array<int, 8> at = order_slots(bvh, slots, all);
    uint32_t rank = 0, tri_off = 0;
    std::vector<Job> children;
    for (size_t i = 0; i < 8; ++i) {
      if (at[i] < 0) {
        for (int a = 0; a < 3; ++a) {
          wn.qlo[a][i] = 255;
          wn.qhi[a][i] = 0;
        }
        continue;
      }
      const Slot &s = slots[(size_t)at[i]];
      const box &cb = bvh.nodes[s.bin].aabb;
      for (int a = 0; a < 3; ++a) {
        float sc = exp_scale(wn.e[a]);
        double lo = std::floor(((double)cb.lo.get(a) - (double)wn.p[a]) / sc);
        double hi = std::ceil(((double)cb.hi.get(a) - (double)wn.p[a]) / sc);
        int ql = (int)std::max(0.0, std::min(255.0, lo));
        int qh = (int)std::max(0.0, std::min(255.0, hi));
        wn.qlo[a][i] = (uint8_t)ql;
        wn.qhi[a][i] = (uint8_t)qh;
      }
      if (!s.leaf) {
        wn.imask |= (uint8_t)(1u << i);
        wn.meta[i] = (uint8_t)rank;
        children.push_back({child_base + rank, s.bin, s.first, job.depth + 1});
        ++rank;
      } else {
        const BinaryNode &ln = bvh.nodes[s.bin];
        bool extra = (ln.w1 & kNodeTag) != 0;
        for (uint32_t k = 0; k < s.count; ++k) {
          uint32_t pos = ln.w0 + s.first + k;
          out.tri_index.push_back(extra ? bvh.extra_idxs[pos] : pos);
        }
        wn.meta[i] = s.count == 0 ? 0 : (uint8_t)((s.count << 5) | tri_off);
        tri_off += s.count;
      }
    }
    out.nodes.resize(out.nodes.size() + n_internal);
    out.nodes[job.wide] = wn;
    if (job.depth + 1 < kBfsDepth) {
      queue.insert(queue.end(), children.begin(), children.end());
    } else {
      for (size_t k = children.size(); k-- > 0;) {
        stack.push_back(children[k]);
      }
    }
  }
  if (out.n_top == 0) {
    out.n_top = (uint32_t)out.nodes.size();
  }
  return out;
}

} // namespace pg
