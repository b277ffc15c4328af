// Compressed 8-wide BVH construction (see wide.h).
#include "wide.h"

#include <array>
#include <cmath>
#include <cstring>

namespace pg {

namespace {

struct Child {
  uint32_t bin; // binary node index
  bool leaf;
  uint32_t ntri;
  float area;
};

uint32_t leaf_count(const BinaryNode &n) {
  return (n.w1 & ~kNodeTag) - n.w0;
}

bool is_split(const BinaryNode &n) { return (n.w0 & kNodeTag) != 0; }

Child make_child(const BinaryBVH &b, uint32_t i) {
  const BinaryNode &n = b.nodes[i];
  Child c;
  c.bin = i;
  c.leaf = !is_split(n);
  c.ntri = c.leaf ? leaf_count(n) : 0;
  c.area = area(n.aabb);
  return c;
}

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

WideBVH build_wide(const BinaryBVH &bvh) {
  WideBVH out;
  if (bvh.nodes.empty()) {
    return out;
  }
  struct Job {
    uint32_t wide;
    uint32_t bin;
    uint32_t depth;
  };
  out.nodes.resize(1);
  std::vector<Job> stack;
  stack.push_back({0, 0, 0});
  while (!stack.empty()) {
    Job job = stack.back();
    stack.pop_back();
    out.depth = std::max(out.depth, job.depth);
    std::vector<Child> kids;
    const BinaryNode &root = bvh.nodes[job.bin];
    if (is_split(root)) {
      kids.push_back(make_child(bvh, root.w0 & ~kNodeTag));
      kids.push_back(make_child(bvh, root.w1 & ~kNodeTag));
    } else {
      kids.push_back(make_child(bvh, job.bin));
    }
    // greedy collapse: open the largest internal child while it fits
    while (kids.size() < 8) {
      int pick = -1;
      for (size_t i = 0; i < kids.size(); ++i) {
        if (kids[i].leaf) {
          continue;
        }
        const BinaryNode &n = bvh.nodes[kids[i].bin];
        Child l = make_child(bvh, n.w0 & ~kNodeTag);
        Child r = make_child(bvh, n.w1 & ~kNodeTag);
        uint32_t tris = l.ntri + r.ntri;
        for (size_t k = 0; k < kids.size(); ++k) {
          tris += kids[k].ntri;
        }
        if (tris > kMaxNodeTris) {
          continue;
        }
        if (pick < 0 || kids[i].area > kids[(size_t)pick].area) {
          pick = (int)i;
        }
      }
      if (pick < 0) {
        break;
      }
      const BinaryNode &n = bvh.nodes[kids[(size_t)pick].bin];
      Child l = make_child(bvh, n.w0 & ~kNodeTag);
      Child r = make_child(bvh, n.w1 & ~kNodeTag);
      kids[(size_t)pick] = l;
      kids.insert(kids.begin() + pick + 1, r);
    }
    // leaves larger than a slot can hold are split across slots with the
    // same box; leaves that no longer fit get a node of their own
    std::vector<Slot> slots;
    for (const Child &c : kids) {
      if (!c.leaf) {
        slots.push_back({c.bin, false, 0, 0});
        continue;
      }
      for (uint32_t f = 0; f < c.ntri; f += kMaxLeafTris) {
        slots.push_back({c.bin, true, f, std::min(kMaxLeafTris, c.ntri - f)});
      }
      if (c.ntri == 0) {
        slots.push_back({c.bin, true, 0, 0});
      }
    }
    if (slots.size() > 8) {
      // demote whole leaves into nodes of their own until the slots fit
      std::vector<Slot> merged;
      size_t excess = slots.size() - 8;
      for (size_t i = 0; i < slots.size(); ++i) {
        const Slot &s = slots[i];
        if (excess > 0 && s.leaf && s.first == 0 && leaf_count(bvh.nodes[s.bin]) > kMaxLeafTris) {
          uint32_t used = (leaf_count(bvh.nodes[s.bin]) + kMaxLeafTris - 1) / kMaxLeafTris;
          merged.push_back({s.bin, false, 0, 0});
          i += used - 1;
          excess -= std::min<size_t>(excess, used - 1);
          continue;
        }
        merged.push_back(s);
      }
      slots.swap(merged);
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
        children.push_back({child_base + rank, s.bin, job.depth + 1});
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
    for (size_t k = children.size(); k-- > 0;) {
      stack.push_back(children[k]);
    }
  }
  return out;
}

} // namespace pg
