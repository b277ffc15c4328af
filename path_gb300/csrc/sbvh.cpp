// Host SBVH builder (see sbvh.h).
#include "sbvh.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <iterator>
#include <limits>
#include <memory>
#include <unordered_map>
#include <unordered_set>
#include <utility>

namespace pg {

namespace {

constexpr uint32_t kNone = 0xffffffffu;
constexpr float kBig = std::numeric_limits<float>::max();
constexpr float kLowest = std::numeric_limits<float>::lowest();
constexpr size_t kTaskMin = 4096;    // subtrees smaller than this stay serial
constexpr size_t kAxisTaskMin = 65536; // nodes this large sort axes in parallel

struct Prim {
  f3 a, b, c;
  box bounds;
};

struct Tmp {
  box aabb;
  bool leaf = false;
  std::unique_ptr<Tmp> left, right;
  bool contiguous = true;
  uint32_t start = 0, count = 0;
  std::vector<uint32_t> list;
};

struct Split {
  float cost = kBig;
  bool spatial = false;
  std::vector<uint32_t> perm;
  uint32_t point = 0;
  float overlap_area = 0.f;
  std::vector<uint32_t> lt, rt;
  std::vector<box> lb, rb;
};

box tri_bounds(f3 a, f3 b, f3 c) {
  box o = empty_box();
  o = grow(o, a);
  o = grow(o, b);
  o = grow(o, c);
  return o;
}

struct Builder {
  SBVHSettings st;
  float root_area = 0.f;

  // object split on one axis: sort by box centre, sweep prefix / suffix
  // boxes (generator.cu:343-438)
  Split object_split(const Prim *p, size_t n, int axis) const {
    struct Key {
      float value;
      uint32_t idx;
    };
    std::vector<Key> keys(n);
    for (size_t i = 0; i < n; ++i) {
      keys[i] = {centre(p[i].bounds).get(axis), (uint32_t)i};
    }
    std::sort(keys.begin(), keys.end(),
              [](Key l, Key r) { return l.value < r.value; });
    Split s;
    s.perm.resize(n);
    for (size_t i = 0; i < n; ++i) {
      s.perm[i] = keys[i].idx;
    }
    std::vector<box> suffix(n);
    box run = empty_box();
    for (size_t i = n; i-- > 0;) {
      run = merge(run, p[s.perm[i]].bounds);
      suffix[i] = run;
    }
    box prefix = empty_box();
    for (size_t i = 0; i < n; ++i) {
      float ov = area(overlap(prefix, suffix[i]));
      float cost = (float)i * area(prefix) + (float)(n - i) * area(suffix[i]);
      if (cost < s.cost) {
        s.cost = cost;
        s.overlap_area = ov;
        s.point = (uint32_t)i;
      }
      prefix = merge(prefix, p[s.perm[i]].bounds);
    }
    return s;
  }

  // binned spatial split with unsplitting (generator.cu:440-713)
  Split spatial_split(const Prim *p, size_t n, int axis) const {
    box all = empty_box();
    for (size_t i = 0; i < n; ++i) {
      all = merge(all, p[i].bounds);
    }
    const uint32_t nd = (uint32_t)n * 2;
    const float lo = all.lo.get(axis);
    const float total = all.hi.get(axis) - lo;
    auto plane = [&](uint32_t loc) -> float {
      float frac = (float)loc / (float)nd;
      if (loc == nd) {
        return all.hi.get(axis);
      }
      return frac * total + lo;
    };
    struct Bin {
      box b = empty_box();
      uint32_t entries = 0, exits = 0;
    };
    std::vector<Bin> bins(nd);
    std::vector<std::vector<uint32_t>> crossing(nd - 1);
    for (uint32_t ti = 0; ti < n; ++ti) {
      const Prim &pr = p[ti];
      float mn = pr.bounds.lo.get(axis);
      float mx = pr.bounds.hi.get(axis);
      float min_prop = (mn - lo) / total;
      float max_prop = (mx - lo) / total;
      uint32_t a = std::min((uint32_t)std::floor(min_prop * (float)nd), nd - 1);
      uint32_t b = std::min((uint32_t)std::floor(max_prop * (float)nd), nd - 1);
      if (plane(a) > mn) {
        --a;
      }
      if (plane(b + 1) < mx) {
        ++b;
      }
      if (a != b) {
        if (plane(b) >= mx) {
          --b;
        }
        if (plane(a + 1) <= mn) {
          ++a;
        }
      }
      ++bins[a].entries;
      ++bins[b].exits;
      for (uint32_t loc = a; loc <= b; ++loc) {
        if (loc != b) {
          crossing[loc].push_back(ti);
        }
        bins[loc].b = merge(bins[loc].b, clipped_bounds(pr.a, pr.b, pr.c, pr.bounds,
                                                       plane(loc), plane(loc + 1), axis));
      }
    }
    std::vector<box> suffix(nd);
    box run = empty_box();
    for (size_t i = nd; i-- > 0;) {
      run = merge(run, bins[i].b);
      suffix[i] = run;
    }
    float best_cost = kBig;
    uint32_t best_edge = 0;
    std::unordered_set<uint32_t> best_l, best_r;
    uint32_t left_total = 0, right_total = (uint32_t)n;
    box prefix = empty_box();
    for (uint32_t e = 0; e + 1 < nd; ++e) {
      left_total += bins[e].entries;
      right_total -= bins[e].exits;
      uint32_t nl = left_total, nr = right_total;
      prefix = merge(prefix, bins[e].b);
      box lb = prefix, rb = suffix[e + 1];
      float al = area(lb), ar = area(rb);
      float cost = (float)nl * al + (float)nr * ar;
      std::unordered_set<uint32_t> lonly, ronly;
      for (uint32_t ti : crossing[e]) {
        box l2 = merge(lb, p[ti].bounds);
        box r2 = merge(rb, p[ti].bounds);
        float cl = (float)nl * area(l2) + (float)(nr - 1) * ar;
        float cr = (float)(nl - 1) * al + (float)nr * area(r2);
        if (std::min(cl, cr) < cost) {
          if (cl < cr) {
            nr -= 1;
            cost = cl;
            al = area(l2);
            lb = l2;
            lonly.insert(ti);
          } else {
            nl -= 1;
            cost = cr;
            ar = area(r2);
            rb = r2;
            ronly.insert(ti);
          }
        }
      }
      if (cost < best_cost) {
        best_cost = cost;
        best_edge = e;
        best_l = std::move(lonly);
        best_r = std::move(ronly);
      }
    }
    Split s;
    s.spatial = true;
    box lbox = empty_box(), rbox = empty_box();
    float sp = plane(best_edge + 1);
    for (uint32_t ti = 0; ti < n; ++ti) {
      const Prim &pr = p[ti];
      if (best_l.count(ti)) {
        lbox = merge(lbox, pr.bounds);
        s.lb.push_back(pr.bounds);
        s.lt.push_back(ti);
        continue;
      }
      if (best_r.count(ti)) {
        rbox = merge(rbox, pr.bounds);
        s.rb.push_back(pr.bounds);
        s.rt.push_back(ti);
        continue;
      }
      bool to_left = pr.bounds.lo.get(axis) < sp;
      bool to_right = pr.bounds.hi.get(axis) > sp;
      if (to_left || (!to_left && !to_right)) {
        box nb = clipped_bounds(pr.a, pr.b, pr.c, pr.bounds, kLowest, sp, axis);
        lbox = merge(lbox, nb);
        s.lb.push_back(nb);
        s.lt.push_back(ti);
      }
      if (to_right) {
        box nb = clipped_bounds(pr.a, pr.b, pr.c, pr.bounds, sp, kBig, axis);
        rbox = merge(rbox, nb);
        s.rb.push_back(nb);
        s.rt.push_back(ti);
      }
    }
    s.cost = (float)s.lt.size() * area(lbox) + (float)s.rt.size() * area(rbox);
    return s;
  }

  std::unique_ptr<Tmp> node(Prim *p, uint32_t *idx, uint32_t *fin, size_t n,
                            uint32_t start, bool is_root) {
    auto out = std::make_unique<Tmp>();
    box all = empty_box();
    for (size_t i = 0; i < n; ++i) {
      all = merge(all, p[i].bounds);
    }
    out->aabb = all;
    if (is_root) {
      root_area = area(all);
    }
    Split cand[3];
    if (n >= kAxisTaskMin) {
      for (int axis = 0; axis < 3; ++axis) {
#pragma omp task shared(cand) firstprivate(axis)
        cand[axis] = object_split(p, n, axis);
      }
#pragma omp taskwait
    } else {
      for (int axis = 0; axis < 3; ++axis) {
        cand[axis] = object_split(p, n, axis);
      }
    }
    Split best;
    for (int axis = 0; axis < 3; ++axis) {
      if (cand[axis].cost < best.cost) {
        best = std::move(cand[axis]);
      }
    }
    if (st.use_spatial_splits && best.overlap_area / root_area > st.overlap_threshold) {
      for (int axis = 0; axis < 3; ++axis) {
        Split c = spatial_split(p, n, axis);
        if (c.cost < best.cost) {
          best = std::move(c);
        }
      }
    }
    float leaf_cost = best.cost / area(all) + st.traversal_per_intersect_cost;
    if (leaf_cost >= (float)n) {
      out->leaf = true;
      std::vector<uint32_t> actual(n);
      uint32_t running = start;
      for (size_t i = 0; i < n; ++i) {
        actual[i] = fin[i] != kNone ? fin[i] : running++;
      }
      bool contiguous = true;
      for (size_t i = 0; i + 1 < n; ++i) {
        contiguous = contiguous && actual[i + 1] > actual[i] &&
                     actual[i + 1] - actual[i] == 1;
      }
      out->contiguous = contiguous;
      out->start = actual[0];
      out->count = (uint32_t)n;
      if (!contiguous) {
        out->list = std::move(actual);
      }
      return out;
    }

    std::vector<Prim> old_p(p, p + n);
    std::vector<uint32_t> old_idx(idx, idx + n);
    std::vector<uint32_t> old_fin(fin, fin + n);
    if (!best.spatial) {
      for (size_t i = 0; i < n; ++i) {
        uint32_t k = best.perm[i];
        p[i] = old_p[k];
        idx[i] = old_idx[k];
        fin[i] = old_fin[k];
      }
      uint32_t sp = best.point;
      uint32_t in_order = 0;
      for (uint32_t i = 0; i < sp; ++i) {
        in_order += fin[i] == kNone ? 1u : 0u;
      }
      old_p.clear();
      old_p.shrink_to_fit();
      if (n >= kTaskMin) {
        Tmp *o = out.get();
#pragma omp task firstprivate(o, p, idx, fin, sp, start)
        o->left = node(p, idx, fin, sp, start, false);
#pragma omp task firstprivate(o, p, idx, fin, sp, start, in_order, n)
        o->right = node(p + sp, idx + sp, fin + sp, n - sp, start + in_order, false);
#pragma omp taskwait
      } else {
        out->left = node(p, idx, fin, sp, start, false);
        out->right = node(p + sp, idx + sp, fin + sp, n - sp, start + in_order, false);
      }
      return out;
    }

    // spatial split: the right side is built after the left side because it
    // reads the left side's reordered indices (generator.cu:205-303)
    const auto &lt = best.lt;
    const auto &rt = best.rt;
    for (size_t i = 0; i < lt.size(); ++i) {
      p[i] = old_p[lt[i]];
      p[i].bounds = best.lb[i];
      idx[i] = old_idx[lt[i]];
      fin[i] = old_fin[lt[i]];
    }
    uint32_t sp = (uint32_t)lt.size();
    out->left = node(p, idx, fin, sp, start, false);
    std::unordered_set<uint32_t> dups;
    std::set_intersection(lt.begin(), lt.end(), rt.begin(), rt.end(),
                          std::inserter(dups, dups.begin()));
    std::unordered_map<uint32_t, uint32_t> dup_to_right;
    for (uint32_t i = 0; i < rt.size(); ++i) {
      if (dups.count(rt[i])) {
        dup_to_right.insert({old_idx[rt[i]], i});
      }
    }
    std::vector<Prim> rp(rt.size());
    std::vector<uint32_t> ridx(rt.size()), rfin(rt.size());
    for (uint32_t i = 0; i < rt.size(); ++i) {
      rp[i] = old_p[rt[i]];
      rp[i].bounds = best.rb[i];
      ridx[i] = i;
      rfin[i] = old_fin[rt[i]];
    }
    uint32_t in_order = 0;
    for (uint32_t i = 0; i < lt.size(); ++i) {
      auto it = dup_to_right.find(idx[i]);
      if (it != dup_to_right.end() && rfin[it->second] == kNone) {
        rfin[it->second] = start + in_order;
      }
      in_order += fin[i] == kNone ? 1u : 0u;
    }
    out->right = node(rp.data(), ridx.data(), rfin.data(), rt.size(),
                      start + in_order, false);
    uint32_t pos = (uint32_t)lt.size();
    for (uint32_t i = 0; i < rt.size(); ++i) {
      uint32_t prev = ridx[i];
      if (dups.count(rt[prev])) {
        continue;
      }
      idx[pos] = old_idx[rt[prev]];
      fin[pos] = old_fin[rt[prev]];
      ++pos;
    }
    return out;
  }
};

void layout(const Tmp *t, uint32_t slot, uint32_t depth, BinaryBVH &out) {
  out.depth = std::max(out.depth, depth);
  if (t->leaf) {
    out.max_leaf_size = std::max(out.max_leaf_size, t->count);
    if (t->contiguous) {
      out.nodes[slot] = {t->start, t->start + t->count, t->aabb};
    } else {
      uint32_t s = (uint32_t)out.extra_idxs.size();
      out.extra_idxs.insert(out.extra_idxs.end(), t->list.begin(), t->list.end());
      out.nodes[slot] = {s, (uint32_t)out.extra_idxs.size() | kNodeTag, t->aabb};
    }
    return;
  }
  uint32_t l = (uint32_t)out.nodes.size();
  out.nodes.resize(l + 2);
  out.nodes[slot] = {l | kNodeTag, l + 1, t->aabb};
  layout(t->left.get(), l, depth + 1, out);
  layout(t->right.get(), l + 1, depth + 1, out);
}

} // namespace

box clipped_bounds(f3 a, f3 b, f3 c, box bounds, float left, float right,
                   int axis) {
  const f3 v[3] = {a, b, c};
  box nb = bounds;
  nb.lo.set(axis, fmax2(nb.lo.get(axis), left));
  nb.hi.set(axis, fmin2(nb.hi.get(axis), right));
  for (int ax = 0; ax < 3; ++ax) {
    if (nb.lo.get(ax) == nb.hi.get(ax)) {
      // flat axis widened by one on each side (clipped_triangle_impl.h:33-45)
      nb.lo.set(ax, nb.lo.get(ax) - 1.f);
      nb.hi.set(ax, nb.hi.get(ax) + 1.f);
    }
  }
  box out = empty_box();
  for (int k = 0; k < 3; ++k) {
    if (contains(nb, v[k])) {
      out = grow(out, v[k]);
    }
  }
  const int edges[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int e = 0; e < 3; ++e) {
    f3 dir = v[edges[e][1]] - v[edges[e][0]];
    for (int sg = 0; sg < 2; ++sg) {
      f3 ds = dir * (sg == 0 ? -1.f : 1.f);
      float tmin;
      f3 inv = inv_dir(ds);
      if (slab(nb, v[edges[e][0]], inv, &tmin)) {
        out = grow(out, ds * tmin + v[edges[e][0]]);
      }
    }
  }
  for (int pd = 0; pd < 3; ++pd) {
    for (int mn = 0; mn < 2; ++mn) {
      for (int mnn = 0; mnn < 2; ++mnn) {
        int na = (pd + 1) % 3, nna = (pd + 2) % 3;
        float px = (mn ? nb.lo : nb.hi).get(na);
        float py = (mnn ? nb.lo : nb.hi).get(nna);
        f3 d01 = v[1] - v[0], d02 = v[2] - v[0];
        float x0 = v[0].get(na), y0 = v[0].get(nna);
        float x1 = v[1].get(na), y1 = v[1].get(nna);
        float x2 = v[2].get(na), y2 = v[2].get(nna);
        float inner = (((-y1) * x2 + y0 * ((-x1) + x2)) + x0 * (y1 - y2)) + x1 * y2;
        float ar = 0.5f * inner;
        float inv2a = 1 / (2 * ar);
        float s = inv2a * (((y0 * x2 - x0 * y2) + (y2 - y0) * px) + (x0 - x2) * py);
        float t = inv2a * (((x0 * y1 - y0 * x1) + (y0 - y1) * px) + (x1 - x0) * py);
        if (s >= 0 && t >= 0 && (1 - s - t) > 0) {
          out = grow(out, (d01 * s + d02 * t) + v[0]);
        }
      }
    }
  }
  return out;
}

BinaryBVH build_sbvh(const f3 *v0, const f3 *v1, const f3 *v2, size_t n,
                     const SBVHSettings &settings) {
  BinaryBVH out;
  if (n == 0) {
    return out;
  }
  std::vector<Prim> prims(n);
  std::vector<uint32_t> idx(n), fin(n, kNone);
  for (size_t i = 0; i < n; ++i) {
    prims[i] = {v0[i], v1[i], v2[i], tri_bounds(v0[i], v1[i], v2[i])};
    idx[i] = (uint32_t)i;
  }
  Builder b;
  b.st = settings;
  std::unique_ptr<Tmp> root;
#pragma omp parallel
#pragma omp single
  root = b.node(prims.data(), idx.data(), fin.data(), n, 0, true);
  out.nodes.resize(1);
  layout(root.get(), 0, 0, out);
  out.permutation = std::move(idx);
  // free the temporary tree iteratively deep trees do not recurse too far
  std::vector<std::unique_ptr<Tmp>> pending;
  pending.push_back(std::move(root));
  while (!pending.empty()) {
    std::unique_ptr<Tmp> t = std::move(pending.back());
    pending.pop_back();
    if (t->left) {
      pending.push_back(std::move(t->left));
    }
    if (t->right) {
      pending.push_back(std::move(t->right));
    }
  }
  return out;
}

} // namespace pg
