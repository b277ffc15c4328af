"""Host-side checks of the 8-wide BVH and of the traversal order the CUDA
kernels use (no GPU needed).

The traversal is mirrored here step by step (node groups of internal
children in ray order, one waiting group per level, leaf triangles as a
32-bit mask) with exact decoded boxes, and must find the order-independent
closest hit: the smallest distance, then the smallest BVH-order index.
"""

import numpy as np
import pytest

from path_gb300 import api, scenes
from oracle import oracle_lib as ol


def _decoded_boxes(node):
    scale = np.array([np.ldexp(1.0, int(e) - 127) for e in node["e"]])
    p = node["p"].astype(np.float64)
    lo = p[:, None] + node["qlo"].astype(np.float64) * scale[:, None]
    hi = p[:, None] + node["qhi"].astype(np.float64) * scale[:, None]
    return lo.T, hi.T  # [8, 3]


def _slot_triangles(node, slot):
    meta = int(node["meta"][slot])
    cnt, off = meta >> 5, meta & 31
    return [int(node["tri_base"]) + off + k for k in range(cnt)]


def _walk(w, o, d, tri_t, tlimit=np.inf):
    """Mirror of wide_step: returns (bvh idx or -1, t, max stack depth)."""
    nodes, refs = w["nodes"], w["leaf_refs"]
    inv = 1.0 / np.where(d == 0.0, 1e-20, d)  # get_inv_direction
    oct_ = int(inv[0] < 0) | (int(inv[1] < 0) << 1) | (int(inv[2] < 0) << 2)
    best_t, best_i = tlimit, -1
    ng_base, ng_bits = 0, 1 | (1 << (8 + oct_))
    stack, max_sp = [], 0
    while True:
        hits8 = ng_bits >> 8
        j = (hits8 & -hits8).bit_length() - 1
        ng_bits &= ~(1 << (8 + j))
        slot = j ^ oct_
        node_i = ng_base + bin(ng_bits & 0xFF & ((1 << slot) - 1)).count("1")
        if ng_bits >> 8:
            stack.append((ng_base, ng_bits))
            max_sp = max(max_sp, len(stack))
        node = nodes[node_i]
        lo, hi = _decoded_boxes(node)
        # the kernel's rounding margin 2^-20 (|(p - o) / d| + 255 |2^e / d|)
        scale = np.array([np.ldexp(1.0, int(e) - 127) for e in node["e"]])
        margin = 2.0 ** -20 * (np.abs((node["p"] - o) * inv) + 255 * np.abs(scale * inv))
        t0 = (lo - o) * inv
        t1 = (hi - o) * inv
        tmin = (np.minimum(t0, t1) - margin).max(1)
        tmax = (np.maximum(t0, t1) + margin).min(1)
        imask = int(node["imask"])
        hits, tris = 0, []
        for i in range(8):
            hit = tmin[i] <= tmax[i] and tmax[i] >= 0 and tmin[i] <= best_t
            if (imask >> i) & 1:
                hits |= int(hit) << (i ^ oct_)
            elif hit:
                tris += _slot_triangles(node, i)
        for k in sorted(set(tris)):
            b = int(refs[k])
            t = tri_t[b]
            if np.isfinite(t) and (t < best_t or (t == best_t and (best_i < 0 or b < best_i))):
                best_t, best_i = t, b
        if hits:
            ng_base, ng_bits = int(node["child_base"]), imask | (hits << 8)
        elif stack:
            ng_base, ng_bits = stack.pop()
        else:
            return best_i, best_t, max_sp


def test_wide_bvh_covers_every_triangle_and_children_contain_their_subtrees():
    tris, _ = scenes.displaced_icosphere(3)
    w = api.wide_build(tris, api.Settings())
    n = len(tris)
    assert set(w["leaf_refs"].tolist()) == set(range(n))
    perm = w["permutation"]
    bvh_tris = np.asarray(tris, np.float64).reshape(-1, 3, 3)[perm]
    nodes = w["nodes"]

    def subtree_box(i):
        node = nodes[i]
        lo, hi = _decoded_boxes(node)
        out_lo, out_hi = np.full(3, np.inf), np.full(3, -np.inf)
        rank = 0
        for s in range(8):
            if (int(node["imask"]) >> s) & 1:
                clo, chi = subtree_box(int(node["child_base"]) + rank)
                rank += 1
            else:
                ts = _slot_triangles(node, s)
                if not ts:
                    continue
                pts = bvh_tris[[int(w["leaf_refs"][k]) for k in ts]].reshape(-1, 3)
                clo, chi = pts.min(0), pts.max(0)
            assert np.all(lo[s] <= clo) and np.all(chi <= hi[s])
            out_lo, out_hi = np.minimum(out_lo, clo), np.maximum(out_hi, chi)
        return out_lo, out_hi

    subtree_box(0)


def test_wide_bvh_top_levels_are_breadth_first():
    # the nodes of depth <= 3 take the first indices, level by level, so a
    # prefix of the node array is the top of the tree (the part the trace
    # kernel keeps in shared memory)
    tris, _ = scenes.displaced_icosphere(6)
    nodes = api.wide_build(tris, api.Settings())["nodes"]
    depth = np.full(len(nodes), -1)
    depth[0] = 0
    order = [0]
    for i in order:
        node = nodes[i]
        rank = 0
        for s in range(8):
            if (int(node["imask"]) >> s) & 1:
                c = int(node["child_base"]) + rank
                rank += 1
                depth[c] = depth[i] + 1
                order.append(c)
    assert np.all(depth >= 0)
    top = int(np.sum(depth <= 3))
    assert top > 73 and np.all(depth[:top] <= 3) and np.all(depth[top:] > 3)
    assert np.all(np.diff(depth[:top]) >= 0)


def _big_leaf_scene(rng):
    """90 copies of one triangle (the SBVH cannot split them: one binary leaf
    of 90, more than the 32 triangles a wide node addresses) among random
    triangles."""
    one = np.array([[-0.5, -0.5, 0.2, 0.5, -0.5, 0.2, 0.0, 0.5, 0.2]], np.float32)
    return np.concatenate([rng.uniform(-1, 1, (60, 9)).astype(np.float32),
                           np.repeat(one, 90, 0)])


def test_wide_bvh_splits_a_leaf_larger_than_a_node():
    tris = _big_leaf_scene(np.random.default_rng(5))
    w = api.wide_build(tris, api.Settings())
    assert sorted(w["leaf_refs"].tolist()) == list(range(len(tris)))
    for node in w["nodes"]:
        used = sum(int(m) >> 5 for s, m in enumerate(node["meta"])
                   if not (int(node["imask"]) >> s) & 1)
        assert used <= 32


@pytest.mark.parametrize("case", ["random", "sphere", "grid_ties", "big_leaf"])
def test_wide_traversal_mirror_finds_the_order_independent_closest_hit(case):
    rng = np.random.default_rng(3)
    if case == "big_leaf":
        tris = _big_leaf_scene(rng)
        o = np.concatenate([rng.uniform(-0.3, 0.3, (100, 2)), np.ones((100, 1))], 1)
        d = rng.normal(size=(100, 3)) * [0.1, 0.1, 0.0] + [0.0, 0.0, -1.0]
    elif case == "random":
        tris = rng.uniform(-1, 1, (300, 9)).astype(np.float32)
        o = rng.uniform(-1, 1, (200, 3))
        d = rng.normal(size=(200, 3))
    elif case == "sphere":
        tris, _ = scenes.displaced_icosphere(3)
        o = np.tile([0.0, 0.0, 3.5], (200, 1))
        d = rng.normal(size=(200, 3)) * [0.2, 0.2, 0.0] + [0.35, -0.4, -3.75]
    else:
        # unit grid in z = 0; rays straight down onto shared vertices and
        # edges hit several triangles at exactly the same distance
        quads = []
        for i in range(8):
            for j in range(8):
                a, b, c, e = (i, j, 0), (i + 1, j, 0), (i + 1, j + 1, 0), (i, j + 1, 0)
                quads += [a + b + c, a + c + e]
        tris = np.array(quads, np.float32)
        pts = np.stack(np.meshgrid(np.arange(1, 8) * 1.0, np.arange(1, 8) * 0.5), -1)
        o = np.concatenate([pts.reshape(-1, 2), np.ones((49, 1))], 1)
        d = np.tile([0.0, 0.0, -1.0], (49, 1))
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    w = api.wide_build(tris, api.Settings())
    perm = w["permutation"]
    nt, nr = len(tris), len(rays)
    bvh_tris = np.asarray(tris, np.float32).reshape(-1, 9)[perm]
    t_all, _ = ol.triangle_intersect(np.repeat(bvh_tris, nr, 0), np.tile(rays, (nt, 1)))
    t_all = t_all.reshape(nt, nr).astype(np.float64)
    ties = 0
    for r in range(nr):
        col = t_all[:, r]
        ok = np.isfinite(col)
        want_i, want_t = -1, np.inf
        if ok.any():
            want_t = col[ok].min()
            want_i = int(np.flatnonzero(col == want_t).min())
            ties += int((col == want_t).sum() > 1)
        got_i, got_t, max_sp = _walk(w, rays[r, :3].astype(np.float64),
                                     rays[r, 3:].astype(np.float64), col)
        assert (got_i, got_t) == (want_i, want_t)
        assert max_sp <= w["depth"] + 1
    if case == "grid_ties":
        assert ties > 10
