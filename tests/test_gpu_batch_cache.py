"""Batched render with one radiance cache for the whole batch
(path_render_batch_cached): the cache's batch-cell coordinates against the
NumPy restatement of the network, every item's image against the same item
rendered in the same cell without the others, the plain batch when no path
reaches the cache vertex, and training frames that lower the error of the
batch's images."""

import numpy as np
import pytest

from path_gb300 import api, scenes

import nrc_reference as ref
from test_gpu_batch import _small_batch, bits

pytestmark = pytest.mark.gpu


def _cell_queries(rng, cells):
    n = len(cells)
    off = 2 * np.stack([cells % 16, cells // 16 % 16, cells // 256], 1)
    pos = rng.uniform(0, 1, (n, 3)) + off
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    alb = rng.uniform(0, 1, (n, 3))
    return np.concatenate([pos, d, nrm, alb], 1).astype(np.float32)


def _random_table_cache(seed):
    c = api.RadianceCache(seed=seed)
    w, t = c.get()
    rng = np.random.default_rng(seed)
    t = rng.uniform(-0.5, 0.5, t.shape).astype(np.float32)
    c.set(table=t)
    return c, w, t


def test_batch_cell_inference_matches_numpy(lib):
    rng = np.random.default_rng(6)
    c, w, t = _random_table_cache(3)
    c.use_batch_cells()
    cells = rng.choice(np.array([0, 1, 17, 300, 4095]), 1500)
    q = _cell_queries(rng, cells)
    got = c.query(q)
    want = ref.forward(q, w, t, None, None)[0]
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    print(f"batch-cell inference rel err {err:.2e}")
    assert err < 1e-2
    # one position in two cells reads different table entries
    q2 = q[:200].copy()
    q2[:, :3] = q2[:, :3] - 2 * np.floor(q2[:, :3] / 2) + np.array([2, 0, 0], np.float32)
    q1 = q2.copy()
    q1[:, 0] -= 2
    assert not np.array_equal(c.query(q1), c.query(q2))


def _run(cache, raw, sel, settings, depth=2, train_paths=0, train_steps=0):
    outs, batch = [], []
    for k in sel:
        sc, w, h, spp = raw[k]
        out = np.zeros((h, w, 3), np.float32)
        outs.append(out)
        batch.append((sc, api.SquareImage(w, h, scenes.cornell_camera(w, h)), out, spp))
    r = api.Renderer()
    r.render_batch_cached(cache, batch, settings, cache_depth=depth, train_paths=train_paths,
                          train_steps=train_steps)
    assert r.stats()["device_status"] == 0
    return outs


def test_batch_cached_items_equal_the_item_alone(lib):
    """Item i takes cell i: its image is the same bit for bit whatever else
    is in the batch, with the same cache."""
    s = scenes.path_settings(6, "wide")
    raw = _small_batch(21, 3)
    c, _, _ = _random_table_cache(9)
    full = _run(c, raw, [0, 1, 2], s)
    alone = _run(c, raw, [0], s)
    assert np.array_equal(bits(full[0]), bits(alone[0]))
    other = _run(c, raw, [2, 1], s)
    assert np.array_equal(bits(full[1]), bits(other[1]))
    # the cache's predictions are in the images: they differ from the plain batch
    plain = []
    batch = []
    for sc, w, h, spp in raw:
        out = np.zeros((h, w, 3), np.float32)
        plain.append(out)
        batch.append((sc, api.SquareImage(w, h, scenes.cornell_camera(w, h)), out, spp))
    api.Renderer().render_batch(batch, s)
    assert not np.array_equal(bits(full[0]), bits(plain[0]))


def test_batch_cached_without_cache_vertices_equals_the_plain_batch(lib):
    """Paths of at most 5 bounces never reach vertex 40: no query, and every
    image equals the plain batch's bit for bit."""
    s = scenes.path_settings(6, "wide")
    raw = _small_batch(23, 4)
    c, _, _ = _random_table_cache(4)
    cached = _run(c, raw, range(4), s, depth=40, train_paths=1 << 10, train_steps=1)
    plain, batch = [], []
    for sc, w, h, spp in raw:
        out = np.zeros((h, w, 3), np.float32)
        plain.append(out)
        batch.append((sc, api.SquareImage(w, h, scenes.cornell_camera(w, h)), out, spp))
    api.Renderer().render_batch(batch, s)
    for a, b in zip(cached, plain):
        assert np.array_equal(bits(a), bits(b))


def test_batch_cached_frame_queries_lie_in_their_cells(lib):
    s = scenes.path_settings(6, "wide")
    raw = _small_batch(25, 3)
    c, _, _ = _random_table_cache(5)
    outs, batch = [], []
    for sc, w, h, spp in raw:
        out = np.zeros((h, w, 3), np.float32)
        outs.append(out)
        batch.append((sc, api.SquareImage(w, h, scenes.cornell_camera(w, h)), out, spp))
    r = api.Renderer()
    r.render_batch_cached(c, batch, s, cache_depth=2, train_paths=0, train_steps=0)
    q, beta = r.cached_frame_queries(max_n=1 << 16, stride=1)
    assert len(q) > 0
    cell = np.floor(q[:, :3] / 2)
    assert set(np.unique(cell[:, 0]).astype(int)) <= {0, 1, 2}
    assert np.all(cell[:, 1:] == 0)
    frac = q[:, :3] - 2 * cell
    assert frac.min() >= 0 and frac.max() <= 1


def test_trained_batch_cache_lowers_the_error_of_the_frames(lib):
    """After training frames, the batch's 4-spp cached frame is closer to a
    1024-spp render of each item than the plain 4-spp frame."""
    s = scenes.path_settings(8, "wide")
    raw = [(sc, 48, 48, 4) for sc, _, _, _ in _small_batch(27, 3)]
    refs, batch = [], []
    for sc, w, h, _ in raw:
        out = np.zeros((h, w, 3), np.float32)
        refs.append(out)
        batch.append((sc, api.SquareImage(w, h, scenes.cornell_camera(w, h)), out, 1024))
    api.Renderer().render_batch(batch, s)
    cache = api.RadianceCache(seed=11)
    r = api.Renderer()
    for _ in range(40):
        _run_with(r, cache, raw, s, train_paths=1 << 14, train_steps=4)
    cached = _run_with(r, cache, raw, s, train_paths=0, train_steps=0)
    plain, batch = [], []
    for sc, w, h, spp in raw:
        out = np.zeros((h, w, 3), np.float32)
        plain.append(out)
        batch.append((sc, api.SquareImage(w, h, scenes.cornell_camera(w, h)), out, spp))
    r.render_batch(batch, s)

    def rel(imgs):
        return float(np.mean([np.linalg.norm(a - b) / np.linalg.norm(b)
                              for a, b in zip(imgs, refs)]))

    e_plain, e_cached = rel(plain), rel(cached)
    print(f"batch 4-spp frames, mean rel RMSE: plain {e_plain:.4f}, "
          f"with trained cache {e_cached:.4f}")
    assert all(np.isfinite(a).all() for a in cached)
    assert e_cached < e_plain


def _run_with(r, cache, raw, s, train_paths, train_steps):
    outs, batch = [], []
    for sc, w, h, spp in raw:
        out = np.zeros((h, w, 3), np.float32)
        outs.append(out)
        batch.append((sc, api.SquareImage(w, h, scenes.cornell_camera(w, h)), out, spp))
    r.render_batch_cached(cache, batch, s, cache_depth=2, train_paths=train_paths,
                          train_steps=train_steps)
    return outs


def test_batch_cached_with_an_empty_scene_and_bgra_output(lib):
    """An item without triangles and an item written as BGRA in a cached
    batch: the empty item stays black, the BGRA item equals the same item's
    FloatRGB image tone-mapped by the plain batch's BGRA path."""
    s = scenes.path_settings(6, "wide")
    empty = api.Scene()
    empty.add_material(api.material("Diffuse", diffuse=(0.5, 0.5, 0.5)))
    sc = scenes.cornell_box()
    c, _, _ = _random_table_cache(12)
    w = h = 16
    f2w = scenes.cornell_camera(w, h)
    e_out = np.zeros((h, w, 3), np.float32)
    rgb = np.zeros((h, w, 3), np.float32)
    bgra = np.zeros((h, w, 4), np.uint8)
    r = api.Renderer()
    r.render_batch_cached(c, [(empty, api.SquareImage(w, h, f2w), e_out, 4),
                              (sc, api.SquareImage(w, h, f2w), rgb, 4)], s,
                          cache_depth=2, train_paths=0, train_steps=0)
    assert r.stats()["device_status"] == 0
    assert not e_out.any()
    e2 = np.zeros((h, w, 3), np.float32)
    r.render_batch_cached(c, [(empty, api.SquareImage(w, h, f2w), e2, 4),
                              (sc, api.SquareImage(w, h, f2w), bgra, 4)], s,
                          cache_depth=2, train_paths=0, train_steps=0)
    v = np.maximum(rgb.astype(np.float32), 0)
    want = np.clip((v / (v + 1)) * 255, 0, 255).astype(np.uint8)
    assert np.abs(bgra[..., 2::-1].astype(int) - want.astype(int)).max() <= 1


def test_single_cached_frame_after_a_batch_uses_the_scene_box(lib):
    """One cache used for a batch (cell coordinates) and then for a single
    scene renders that scene's cached frame exactly as a cache that never
    served a batch (the scene's box is set before the frame's queries)."""
    s = scenes.path_settings(6, "wide")
    s.kernel_approach = 1
    sc = scenes.cornell_box()
    w = h = 16
    f2w = scenes.cornell_camera(w, h)
    a, _, _ = _random_table_cache(21)
    b, _, _ = _random_table_cache(21)
    junk = np.zeros((h, w, 3), np.float32)
    api.Renderer().render_batch_cached(a, [(sc, api.SquareImage(w, h, f2w), junk, 4)], s,
                                       cache_depth=2, train_paths=0, train_steps=0)
    ia = np.zeros((h, w, 3), np.float32)
    ib = np.zeros((h, w, 3), np.float32)
    api.Renderer().render_cached(a, api.SquareImage(w, h, f2w), ia, sc, 4, s, cache_depth=2,
                                 train_paths=0, train_steps=0)
    api.Renderer().render_cached(b, api.SquareImage(w, h, f2w), ib, sc, 4, s, cache_depth=2,
                                 train_paths=0, train_steps=0)
    assert np.array_equal(bits(ia), bits(ib))
