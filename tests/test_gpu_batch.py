"""Batched render (path_render_batch): every image of a batch equals the
single-scene streaming render of the same item, bit for bit, whatever the
launch shape."""

import numpy as np
import pytest

from path_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32 if a.dtype == np.float32 else np.uint8)


def _single(scene, settings, spp, w, h, f2w, bgra=False):
    out = np.zeros((h, w, 4), np.uint8) if bgra else np.zeros((h, w, 3), np.float32)
    s = settings.copy()
    s.kernel_approach = 1
    api.Renderer().render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w), out, scene, spp, s)
    return out


def _small_batch(seed, n):
    rng = np.random.default_rng(seed)
    items = []
    for k in range(n):
        if k % 3 == 0:
            sc = scenes.cornell_box()
        else:
            sc = api.Scene()
            white = sc.add_material(api.material("Diffuse", diffuse=(0.7, 0.7, 0.7)))
            light = sc.add_material(api.material("Diffuse", diffuse=(0.5, 0.5, 0.5),
                                                 emission=(8, 8, 8)))
            walls, lt = scenes.room_triangles()
            tris = [t for ts in walls.values() for t in ts]
            sc.add_mesh(np.stack(tris).reshape(-1, 9), np.full(len(tris), white, np.uint32))
            sc.add_mesh(np.stack(lt).reshape(-1, 9), np.full(len(lt), light, np.uint32))
            ggx = sc.add_material(api.material("GGX", specular=(0.04, 0.04, 0.04),
                                               roughness=float(rng.uniform(0.1, 0.6))))
            glass = sc.add_material(api.material("DielectricRefractive", specular=(1, 1, 1),
                                                 ior=1.5))
            t, n_ = scenes._sphere_grid(int(rng.integers(6, 20)), 0.3, (0.2, -0.5, 0.0))
            sc.add_mesh(t, np.full(len(t), ggx, np.uint32), normals=n_)
            t, n_ = scenes._sphere_grid(8, 0.2, (-0.4, -0.6, 0.3))
            sc.add_mesh(t, np.full(len(t), glass, np.uint32), normals=n_)
        w = int(rng.choice([16, 24, 40]))
        h = int(rng.choice([16, 32]))
        spp = int(rng.choice([4, 8, 13]))
        items.append((sc, w, h, spp))
    return items


@pytest.mark.parametrize("tuning,rng", [(None, 0),
                                        ({"slots_log2": 10, "trace_min_blocks": 3,
                                          "shade_ctas_per_sm": 2, "iterations_per_graph": 2}, 0),
                                        ({"slots_log2": 10}, 1)])
def test_batch_images_equal_single_renders(lib, tuning, rng):
    s = scenes.path_settings(6, "wide")
    s.rng = rng
    items = _small_batch(3, 7)
    outs, refs, batch = [], [], []
    for k, (sc, w, h, spp) in enumerate(items):
        f2w = scenes.cornell_camera(w, h)
        bgra = k == 2
        out = np.zeros((h, w, 4), np.uint8) if bgra else np.zeros((h, w, 3), np.float32)
        outs.append(out)
        refs.append(_single(sc, s, spp, w, h, f2w, bgra))
        batch.append((sc, api.SquareImage(w, h, f2w), out, spp))
    r = api.Renderer()
    r.render_batch(batch, s, tuning)
    assert r.stats()["device_status"] == 0
    for out, ref in zip(outs, refs):
        assert np.array_equal(bits(out), bits(ref))


def test_batch_with_repeated_scene_sample_blocks_and_device_output(lib):
    import torch
    s = scenes.path_settings(5, "wide")
    s.render_work_division.block_size = 32
    s.render_work_division.force_target_samples = 1
    s.render_work_division.forced_target_samples_per_thread = 1
    sc = scenes.cornell_box()
    f2w = scenes.cornell_camera(16, 16)
    ref = _single(sc, s, 64, 16, 16, f2w)
    dev = torch.zeros((16, 16, 3), dtype=torch.float32, device="cuda")
    host = np.zeros((16, 16, 3), np.float32)
    r = api.Renderer()
    r.render_batch([(sc, api.SquareImage(16, 16, f2w), host, 64),
                    (sc, api.SquareImage(16, 16, f2w), dev, 64)], s)
    torch.cuda.synchronize()
    assert np.array_equal(bits(host), bits(ref))
    assert np.array_equal(bits(dev.cpu().numpy()), bits(ref))


def test_batch_autotune_returns_a_shape_that_renders_the_same(lib):
    s = scenes.path_settings(6, "wide")
    items = _small_batch(5, 4)
    batch, outs, refs = [], [], []
    for sc, w, h, spp in items:
        f2w = scenes.cornell_camera(w, h)
        out = np.zeros((h, w, 3), np.float32)
        outs.append(out)
        refs.append(_single(sc, s, spp, w, h, f2w))
        batch.append((sc, api.SquareImage(w, h, f2w), out, spp))
    r = api.Renderer()
    t = r.autotune_batch(batch, s, sample_budget=1 << 16)
    assert 23 <= t["slots_log2"] <= 26 and 3 <= t["trace_min_blocks"] <= 5
    r.render_batch(batch, s, t)
    for out, ref in zip(outs, refs):
        assert np.array_equal(bits(out), bits(ref))


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_with_gpu_built_bvhs_renders_the_same_images(lib, mode):
    s = scenes.path_settings(6, "wide")
    items = _small_batch(11, 5)
    batch, outs, refs = [], [], []
    for sc, w, h, spp in items:
        f2w = scenes.cornell_camera(w, h)
        out = np.zeros((h, w, 3), np.float32)
        outs.append(out)
        refs.append(_single(sc, s, spp, w, h, f2w))
        batch.append((sc, api.SquareImage(w, h, f2w), out, spp))
    g = s.copy()
    g.gpu_build = mode
    api.Renderer().render_batch(batch, g)
    # the same closest hits up to exact-distance ties, which the two BVHs
    # may break with different triangles
    for out, ref in zip(outs, refs):
        err = np.linalg.norm(out.astype(np.float64) - ref) / np.linalg.norm(ref)
        assert err <= 1e-4


def test_batch_sample_offsets_equal_single_renders(lib):
    """An item's sample_offset picks the same Sobol samples as the
    single-scene render's (progressive frames of a batch)."""
    s = scenes.path_settings(6, "wide")
    items = _small_batch(13, 3)
    batch, outs, refs = [], [], []
    for k, (sc, w, h, spp) in enumerate(items):
        f2w = scenes.cornell_camera(w, h)
        off = 7 + 100 * k
        out = np.zeros((h, w, 3), np.float32)
        outs.append(out)
        ref = np.zeros((h, w, 3), np.float32)
        s1 = s.copy()
        s1.kernel_approach = 1
        api.Renderer().render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w, sample_offset=off),
                              ref, sc, spp, s1)
        refs.append(ref)
        batch.append((sc, api.SquareImage(w, h, f2w, sample_offset=off), out, spp))
    api.Renderer().render_batch(batch, s)
    for out, ref in zip(outs, refs):
        assert np.array_equal(bits(out), bits(ref))


@pytest.mark.parametrize("gpu_build", [0, 1, 2])
def test_batch_with_empty_and_light_only_scenes(lib, gpu_build):
    """Degenerate items in a batch (no triangles; nothing but the light)
    render as they do alone, with host-built and GPU-built BVHs."""
    s = scenes.path_settings(5, "wide")
    s.gpu_build = gpu_build
    empty = api.Scene()
    empty.add_material(api.material("Diffuse", diffuse=(0.5, 0.5, 0.5)))
    light_only = api.Scene()
    m = light_only.add_material(api.material("Diffuse", diffuse=(0.5, 0.5, 0.5),
                                             emission=(4, 4, 4)))
    _, lt = scenes.room_triangles()
    light_only.add_mesh(np.stack(lt).reshape(-1, 9), np.full(2, m, np.uint32))
    items = [(empty, 16, 16, 4), (scenes.cornell_box(), 24, 16, 4), (light_only, 16, 24, 8)]
    batch, outs, refs = [], [], []
    for sc, w, h, spp in items:
        f2w = scenes.cornell_camera(w, h)
        out = np.zeros((h, w, 3), np.float32)
        outs.append(out)
        refs.append(_single(sc, s, spp, w, h, f2w))
        batch.append((sc, api.SquareImage(w, h, f2w), out, spp))
    r = api.Renderer()
    r.render_batch(batch, s)
    assert r.stats()["device_status"] == 0
    assert not outs[0].any()
    for out, ref in zip(outs, refs):
        assert np.array_equal(bits(out), bits(ref))
