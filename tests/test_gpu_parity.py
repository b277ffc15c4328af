"""Parity of the CUDA render path with the CPU oracle (GPU tests).

Tolerances: Sobol values, transcendental functions, closest-hit ids (except
exact-distance ties) and images rendered with the binary traversal are
compared bit for bit; images through the 8-wide traversal may differ only
where two triangles are hit at exactly the same distance, and must stay
within 1e-4 relative RMSE (||gpu - oracle||_2 / ||oracle||_2 over all
pixel channels), the bar the render path is held to.
"""

import numpy as np
import pytest

from path_gb300 import api, scenes
from oracle import oracle_lib as ol

pytestmark = pytest.mark.gpu

RMSE_TOL = 1e-4


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("count", [16, 64, 1024, 4096])
def test_sobol_bit_exact_against_curand_and_oracle(lib, oracle, count):
    ours = api.sobol_table(256, count)
    curand = api.sobol_table(256, count, use_curand=True)
    host = ol.sobol_table(256, count)
    assert np.array_equal(bits(ours), bits(curand))
    assert np.array_equal(bits(ours), bits(host))


def test_pmath_gpu_equals_host(lib, oracle):
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.uniform(-7, 7, 200000), [0.0, -0.0, np.pi, -np.pi, 1e-30]]).astype(np.float32)
    a = np.concatenate([rng.uniform(-1, 1, 200000), [1.0, -1.0, 0.5, -0.5, 0.0]]).astype(np.float32)
    b = rng.uniform(0, 1, a.size).astype(np.float32)
    e = rng.uniform(0, 100, a.size).astype(np.float32)
    for fn in (0, 1):
        assert np.array_equal(bits(api.debug_pmath(fn, x)), bits(ol.pmath(fn, x)))
    for fn in (2, 3):
        assert np.array_equal(bits(api.debug_pmath(fn, a)), bits(ol.pmath(fn, a)))
    assert np.array_equal(bits(api.debug_pmath(4, b, e)), bits(ol.pmath(4, b, e)))


def _random_rays(rng, lo, hi, n):
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.uniform(lo, hi, (n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


@pytest.mark.parametrize("traversal,spatial", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_closest_hit_matches_oracle(lib, oracle, traversal, spatial):
    """Closest hits through the SBVH (with spatial splits: duplicated
    triangle references and clipped bounds) against testing every triangle."""
    rng = np.random.default_rng(21)
    r = api.Renderer()
    s = api.Settings()
    s.traversal = traversal
    s.use_spatial_splits = spatial
    cases = []
    for n in (1, 4, 37, 100, 300 if spatial else 5000):
        cases.append((rng.uniform(-1, 1, (n, 9)).astype(np.float32),
                      _random_rays(rng, -1, 1, 4096)))
    tris, _ = scenes.displaced_icosphere(3 if spatial else 5)
    o = np.tile([0.0, 0.0, 3.5], (20000, 1))
    d = rng.normal(size=(20000, 3)) * [0.3, 0.3, 0.0] + [0.35, -0.4, -3.75]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    cases.append((tris, np.concatenate([o, d], 1).astype(np.float32)))
    for tris, rays in cases:
        want, wt = ol.loop_all(tris, rays)
        got, gt = r.intersect(tris, rays, s)
        assert np.array_equal(want >= 0, got >= 0)
        hit = want >= 0
        tie = np.abs(wt - gt) <= 1e-6
        assert np.all((want == got) | (hit & tie))
        assert np.array_equal(bits(wt[hit]), bits(gt[hit]))


def _render_gpu(scene, settings, spp, w, h, f2w, bgra=False):
    out = np.zeros((h, w, 4), np.uint8) if bgra else np.zeros((h, w, 3), np.float32)
    r = api.Renderer()
    r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w), out, scene, spp, settings)
    assert r.stats()["device_status"] == 0
    return out


def _render_oracle(scene, settings, spp, w, h, f2w, rows=None):
    arr = ol.SceneArrays(scene.export())
    img, _ = ol.render(arr, ol.settings_from(settings, reduce_order=1), spp, w, h, f2w, rows)
    return img


@pytest.mark.parametrize("traversal", [0, 1])
def test_cornell_bit_exact(lib, oracle, traversal):
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "wide" if traversal else "binary")
    f2w = scenes.cornell_camera(64, 64)
    gpu = _render_gpu(sc, s, 16, 64, 64, f2w)
    ref = _render_oracle(sc, s, 16, 64, 64, f2w)
    assert rel_rmse(gpu, ref) <= RMSE_TOL
    if traversal == 0:
        assert np.array_equal(bits(gpu), bits(ref))


@pytest.mark.parametrize("traversal", [0, 1])
def test_cornell_full_size(lib, oracle, traversal):
    # the small-Cornell workload: 256 x 256, 16 spp, max depth 5
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "wide" if traversal else "binary")
    f2w = scenes.cornell_camera(256, 256)
    gpu = _render_gpu(sc, s, 16, 256, 256, f2w)
    ref = _render_oracle(sc, s, 16, 256, 256, f2w)
    err = rel_rmse(gpu, ref)
    print(f"cornell 256x256x16 traversal={traversal} rel RMSE vs oracle {err:.3e}")
    assert err <= RMSE_TOL
    assert 0.15 < float(gpu.mean()) < 0.6


@pytest.mark.parametrize("traversal", ["binary", "wide"])
def test_cornell_bgra(lib, oracle, traversal):
    """BGRA output (tone map v / (v + 1), x 255 truncated) of the per-thread
    (binary) and warp-cooperative (8-wide) megakernels."""
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, traversal)
    f2w = scenes.cornell_camera(48, 40)
    gpu = _render_gpu(sc, s, 8, 48, 40, f2w, bgra=True)
    arr = ol.SceneArrays(sc.export())
    ref = ol.render_bgra(arr, ol.settings_from(s, reduce_order=1), 8, 48, 40, f2w)
    assert np.array_equal(gpu, ref)


def _settings_variants():
    out = []
    s = scenes.path_settings(5, "binary")
    s.set_term_prob("MultiplierFunc", exp=50.0, min_prob=0.1)
    out.append(("multiplier_func", s))
    s = scenes.path_settings(4, "binary")
    s.set_term_prob("Normalize", min_prob=0.1)
    out.append(("normalize", s))
    s = scenes.path_settings(4, "binary")
    s.set_term_prob("Constant", prob=0.3)
    out.append(("constant", s))
    s = scenes.path_settings(5, "binary")
    s.light_sampler = 1
    out.append(("no_light_sampling", s))
    s = scenes.path_settings(5, "binary")
    s.dir_sampler = 1
    out.append(("uniform_dir", s))
    s = scenes.path_settings(5, "binary")
    s.back_cull_emission = 0
    out.append(("no_back_cull", s))
    # several sample blocks per pixel: exercises the second reduction stage
    s = scenes.path_settings(5, "binary")
    s.render_work_division.block_size = 32
    s.render_work_division.force_target_samples = 1
    s.render_work_division.forced_target_samples_per_thread = 1
    out.append(("sample_blocks", s))
    # SBVH spatial splits (duplicated triangle references, ClippedTriangle
    # bounds), through both traversals
    s = scenes.path_settings(5, "binary")
    s.use_spatial_splits = 1
    s.overlap_threshold = 0.0
    out.append(("spatial_splits", s))
    s = scenes.path_settings(5, "wide")
    s.use_spatial_splits = 1
    s.overlap_threshold = 0.0
    out.append(("spatial_splits_wide", s))
    return out


@pytest.mark.parametrize("name,settings", _settings_variants())
def test_settings_variants_match(lib, oracle, name, settings):
    sc = scenes.cornell_box()
    f2w = scenes.cornell_camera(32, 32)
    spp = 128 if name == "sample_blocks" else 16
    gpu = _render_gpu(sc, settings, spp, 32, 32, f2w)
    ref = _render_oracle(sc, settings, spp, 32, 32, f2w)
    if name.endswith("_wide"):
        assert rel_rmse(gpu, ref) <= RMSE_TOL
    else:
        assert np.array_equal(bits(gpu), bits(ref)), (name, rel_rmse(gpu, ref))


def _material_zoo_scene():
    sc = api.Scene()
    mats = [
        api.material("Diffuse", diffuse=(0.7, 0.7, 0.7)),
        api.material("Glossy", specular=(0.8, 0.6, 0.4), shininess=40.0),
        api.material("DiffuseGlossy", diffuse=(0.5, 0.3, 0.3), specular=(0.4, 0.4, 0.4),
                     shininess=20.0, diffuse_weight=0.6, glossy_weight=0.4),
        api.material("DiffuseMirror", diffuse=(0.3, 0.5, 0.3), specular=(0.9, 0.9, 0.9),
                     diffuse_weight=0.5, glossy_weight=0.5),
        api.material("Mirror", specular=(0.9, 0.9, 0.9)),
        api.material("DielectricRefractive", specular=(1, 1, 1), ior=1.5),
        api.material("GGX", specular=(0.9, 0.6, 0.3), roughness=0.3),
        api.material("Diffuse", diffuse=(0.78, 0.78, 0.78), emission=(12, 12, 12)),
    ]
    ids = [sc.add_material(m) for m in mats]
    walls, light = scenes.room_triangles()
    tris = np.stack([t for ts in walls.values() for t in ts] + light).reshape(-1, 9)
    mat = np.array([ids[0]] * 10 + [ids[7]] * 2, np.uint32)
    sc.add_mesh(tris, mat)
    for k, m in enumerate(ids[1:7]):
        cx = -0.6 + 0.4 * (k % 4)
        cz = -0.4 + 0.6 * (k // 4)
        gt, gn = scenes.uv_sphere(12, 16, radius=0.17, centre=(cx, -0.8, cz))
        sc.add_mesh(gt, np.full(len(gt), m, np.uint32), normals=gn)
    return sc


@pytest.mark.parametrize("traversal", [0, 1])
def test_material_zoo_matches(lib, oracle, traversal):
    sc = _material_zoo_scene()
    s = scenes.path_settings(6, "wide" if traversal else "binary")
    f2w = scenes.cornell_camera(48, 48)
    gpu = _render_gpu(sc, s, 16, 48, 48, f2w)
    ref = _render_oracle(sc, s, 16, 48, 48, f2w)
    assert rel_rmse(gpu, ref) <= RMSE_TOL
    if traversal == 0:
        assert np.array_equal(bits(gpu), bits(ref))


@pytest.mark.parametrize("traversal", [0, 1])
def test_large_mesh_small_case(lib, oracle, traversal):
    sc = scenes.large_mesh_room(subdivisions=5, glass_lat=40, glass_lon=40)
    s = scenes.path_settings(8, "wide" if traversal else "binary")
    f2w = scenes.cornell_camera(64, 64)
    gpu = _render_gpu(sc, s, 8, 64, 64, f2w)
    ref = _render_oracle(sc, s, 8, 64, 64, f2w)
    err = rel_rmse(gpu, ref)
    print(f"large mesh (20480 tris) traversal={traversal} rel RMSE {err:.3e}")
    assert err <= RMSE_TOL


def test_device_output_equals_host_output(lib):
    torch = pytest.importorskip("torch")
    sc = scenes.cornell_box()
    s = scenes.path_settings(5)
    f2w = scenes.cornell_camera(64, 64)
    host = _render_gpu(sc, s, 16, 64, 64, f2w)
    dev = torch.zeros((64, 64, 3), dtype=torch.float32, device="cuda")
    r = api.Renderer()
    r.render(api.ExecutionModel.GPU, api.SquareImage(64, 64, f2w), dev, sc, 16, s)
    torch.cuda.synchronize()
    assert np.array_equal(bits(dev.cpu().numpy()), bits(host))


@pytest.mark.parametrize("case", ["cornell", "zoo", "large_mesh", "sample_blocks"])
def test_streaming_matches_oracle(lib, oracle, case):
    """The wavefront (streaming) render: per-sample radiance from queued
    trace / shade passes, summed per pixel in the reference's order."""
    spp = 16
    if case == "cornell":
        sc, w, h, depth = scenes.cornell_box(), 64, 64, 5
    elif case == "zoo":
        sc, w, h, depth = _material_zoo_scene(), 48, 48, 6
    elif case == "large_mesh":
        sc, w, h, depth = scenes.large_mesh_room(5, 40, 40), 64, 64, 8
        spp = 8
    else:
        sc, w, h, depth = scenes.cornell_box(), 32, 32, 5
        spp = 128
    s = scenes.path_settings(depth, "wide")
    s.kernel_approach = 1
    if case == "sample_blocks":
        s.render_work_division.block_size = 32
        s.render_work_division.force_target_samples = 1
        s.render_work_division.forced_target_samples_per_thread = 1
    f2w = scenes.cornell_camera(w, h)
    gpu = _render_gpu(sc, s, spp, w, h, f2w)
    ref = _render_oracle(sc, s, spp, w, h, f2w)
    err = rel_rmse(gpu, ref)
    print(f"streaming {case} rel RMSE {err:.3e}")
    assert err <= RMSE_TOL


def test_streaming_equals_megakernel_full_cornell(lib):
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "wide")
    f2w = scenes.cornell_camera(256, 256)
    mega = _render_gpu(sc, s, 16, 256, 256, f2w)
    s.kernel_approach = 1
    wave = _render_gpu(sc, s, 16, 256, 256, f2w)
    assert np.array_equal(bits(mega), bits(wave))


@pytest.mark.parametrize("slots_log2", [10, 13])
def test_streaming_refill_equals_megakernel(lib, slots_log2):
    """Fewer paths in flight than samples: slots are refilled with new
    samples as paths end, and the image stays the megakernel's bit for bit."""
    sc = scenes.large_mesh_room(5, 40, 40)
    s = scenes.path_settings(8, "wide")
    f2w = scenes.cornell_camera(96, 96)
    mega = _render_gpu(sc, s, 8, 96, 96, f2w)
    s.kernel_approach = 1
    s.wavefront_slots_log2 = slots_log2
    wave = _render_gpu(sc, s, 8, 96, 96, f2w)
    assert np.array_equal(bits(mega), bits(wave))


@pytest.mark.parametrize("depth", [1, 2, 3, 63, 64])
def test_streaming_pass_kinds_equal_megakernel(lib, depth):
    """Every sample in flight under NIters{depth - 1}: the first pass stages
    fresh slots only, and the pass after the last vertex is the light-only
    finishing pass when it falls in the first round of passes (depth + 1 <=
    64; at depth 64 it falls in the second round and the shade kernel runs
    it).  The image is the megakernel's bit for bit, and no light-only pass
    meets a path with an extension ray (device status 0)."""
    sc = scenes.cornell_box()
    s = scenes.path_settings(depth, "wide")
    f2w = scenes.cornell_camera(32, 32)
    mega = _render_gpu(sc, s, 4, 32, 32, f2w)
    s.kernel_approach = 1
    wave = _render_gpu(sc, s, 4, 32, 32, f2w)
    assert np.array_equal(bits(mega), bits(wave))


def _camera_rays(rng, n, f2w):
    """Rays through random film points of the Cornell camera."""
    m = np.asarray(f2w, np.float64).reshape(3, 4)
    film = np.stack([rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), -np.ones(n)], 1)
    world = film @ m[:, :3].T + m[:, 3]
    d = world - m[:, 3]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([np.tile(m[:, 3], (n, 1)), d], 1).astype(np.float32)


@pytest.mark.parametrize("approach", ["mega_binary", "mega_wide", "streaming"])
def test_initial_rays_match_oracle(lib, oracle, approach):
    """SampleSpecType::InitialRays: one output per caller ray, location x =
    ray index, no camera draws from the RNG."""
    rng = np.random.default_rng(5)
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "binary" if approach == "mega_binary" else "wide")
    if approach == "streaming":
        s.kernel_approach = 1
    rays = _camera_rays(rng, 3001, scenes.cornell_camera(64, 64))
    out = np.zeros((len(rays), 3), np.float32)
    r = api.Renderer()
    r.render(api.ExecutionModel.GPU, api.InitialRays(rays), out, sc, 8, s)
    assert r.stats()["device_status"] == 0
    ref = ol.render_rays(ol.SceneArrays(sc.export()), ol.settings_from(s, reduce_order=1), 8,
                         rays)
    assert rel_rmse(out, ref) <= RMSE_TOL
    if approach == "mega_binary":
        assert np.array_equal(bits(out), bits(ref))


@pytest.mark.parametrize("case", ["binary", "wide", "sample_blocks"])
def test_output_per_step_matches_oracle(lib, oracle, case):
    """OutputType::OutputPerStep: step k's radiance per pixel, paths cut
    after n_steps steps (rendering_equation.h:61-124)."""
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "wide" if case == "wide" else "binary")
    spp, w, h, n_steps = 16, 48, 40, 4
    if case == "sample_blocks":
        s.render_work_division.block_size = 32
        s.render_work_division.force_target_samples = 1
        s.render_work_division.forced_target_samples_per_thread = 1
        spp, w, h = 64, 16, 16
    f2w = scenes.cornell_camera(w, h)
    out = np.zeros((n_steps, h, w, 3), np.float32)
    r = api.Renderer()
    r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w), api.OutputPerStep(out), sc,
             spp, s)
    assert r.stats()["device_status"] == 0
    ref = ol.render_steps(ol.SceneArrays(sc.export()), ol.settings_from(s, reduce_order=1), spp,
                          w, h, f2w, n_steps)
    assert rel_rmse(out, ref) <= RMSE_TOL
    if case != "wide":
        assert np.array_equal(bits(out), bits(ref))


def test_output_per_step_device_output(lib):
    import torch
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "binary")
    f2w = scenes.cornell_camera(32, 32)
    host = np.zeros((3, 32, 32, 3), np.float32)
    api.Renderer().render(api.ExecutionModel.GPU, api.SquareImage(32, 32, f2w),
                          api.OutputPerStep(host), sc, 8, s)
    dev = torch.zeros((3, 32, 32, 3), dtype=torch.float32, device="cuda")
    api.Renderer().render(api.ExecutionModel.GPU, api.SquareImage(32, 32, f2w),
                          api.OutputPerStep(dev), sc, 8, s)
    torch.cuda.synchronize()
    assert np.array_equal(bits(dev.cpu().numpy()), bits(host))


def _idx_and_dir_case(rng, sc, n):
    tris = sc.export()["triangles"].reshape(-1, 3, 3).astype(np.float64)
    ti = rng.integers(0, len(tris), n)
    bary = rng.dirichlet([1, 1, 1], n)
    p = np.einsum("nk,nkj->nj", bary, tris[ti])
    nrm = np.cross(tris[ti, 1] - tris[ti, 0], tris[ti, 2] - tris[ti, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = -nrm + 0.3 * rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return ti.astype(np.uint32), np.concatenate([p - d, d], 1).astype(np.float32)


@pytest.mark.parametrize("traversal", ["binary", "wide"])
def test_initial_idx_and_dir_matches_oracle(lib, oracle, traversal):
    """SampleSpecType::InitialIdxAndDir: each path starts at the caller's
    triangle hit (distance 1, front side) without tracing the first ray."""
    rng = np.random.default_rng(8)
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, traversal)
    idxs, rays = _idx_and_dir_case(rng, sc, 2000)
    out = np.zeros((len(rays), 3), np.float32)
    r = api.Renderer()
    r.render(api.ExecutionModel.GPU, api.InitialIdxAndDir(idxs, rays), out, sc, 8, s)
    assert r.stats()["device_status"] == 0
    ref = ol.render_rays(ol.SceneArrays(sc.export()), ol.settings_from(s, reduce_order=1), 8,
                         rays, idxs=idxs)
    assert rel_rmse(out, ref) <= RMSE_TOL
    if traversal == "binary":
        assert np.array_equal(bits(out), bits(ref))
    # the same spec with OutputPerStep
    steps = np.zeros((3, len(rays), 3), np.float32)
    r.render(api.ExecutionModel.GPU, api.InitialIdxAndDir(idxs, rays), api.OutputPerStep(steps),
             sc, 8, s)
    ref_steps = ol.render_rays(ol.SceneArrays(sc.export()), ol.settings_from(s, reduce_order=1),
                               8, rays, idxs=idxs, n_steps=3)
    assert rel_rmse(steps, ref_steps) <= RMSE_TOL


def test_wide_closest_hit_is_order_independent(lib, oracle):
    """The 8-wide traversal returns the smallest distance and, among equal
    distances, the smallest BVH-order index: rays onto the shared vertices
    and edges of a grid meet several triangles at exactly the same t."""
    quads = []
    for i in range(8):
        for j in range(8):
            a, b, c, e = (i, j, 0), (i + 1, j, 0), (i + 1, j + 1, 0), (i, j + 1, 0)
            quads += [a + b + c, a + c + e]
    tris = np.array(quads, np.float32)
    pts = np.stack(np.meshgrid(np.arange(1, 8) * 1.0, np.arange(1, 8) * 0.5), -1).reshape(-1, 2)
    rays = np.concatenate([pts, np.ones((len(pts), 1)), np.tile([0.0, 0.0, -1.0], (len(pts), 1))],
                          1).astype(np.float32)
    s = api.Settings()
    s.traversal = 1
    w = api.wide_build(tris, s)
    perm = w["permutation"]
    nt, nr = len(tris), len(rays)
    t_all, _ = ol.triangle_intersect(np.repeat(tris[perm], nr, 0), np.tile(rays, (nt, 1)))
    t_all = t_all.reshape(nt, nr)
    got, gt = api.Renderer().intersect(tris, rays, s)
    ties = 0
    for r in range(nr):
        col = t_all[:, r]
        ok = np.isfinite(col)
        assert ok.any()
        tmin = col[ok].min()
        ties += int((col == tmin).sum() > 1)
        assert got[r] == perm[np.flatnonzero(col == tmin).min()]
        assert gt[r] == tmin
    assert ties > 10


@pytest.mark.parametrize("case", ["mega_binary", "mega_wide", "streaming", "sample_blocks",
                                  "bgra"])
def test_row_band_equals_the_same_rows_of_the_whole_render(lib, case):
    """SquareImage(rows=...) computes a band exactly as the whole-image render
    does (the unit of sharding one image over GPUs) and leaves other rows."""
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, "binary" if case == "mega_binary" else "wide")
    spp, w, h = 8, 40, 36
    if case == "streaming":
        s.kernel_approach = 1
    if case == "sample_blocks":
        s.render_work_division.block_size = 32
        s.render_work_division.force_target_samples = 1
        s.render_work_division.forced_target_samples_per_thread = 1
        spp = 64
    f2w = scenes.cornell_camera(w, h)
    bgra = case == "bgra"
    whole = _render_gpu(sc, s, spp, w, h, f2w, bgra=bgra)
    for lo, hi in [(0, 5), (5, 17), (17, 36), (3, 4)]:
        band = np.full_like(whole, 7)
        r = api.Renderer()
        r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w, rows=(lo, hi)), band, sc,
                 spp, s)
        assert r.stats()["device_status"] == 0
        assert np.array_equal(band[lo:hi], whole[lo:hi])
        assert np.all(band[:lo] == 7) and np.all(band[hi:] == 7)


@pytest.mark.parametrize("case", ["empty_scene", "light_only", "one_pixel", "ragged",
                                  "spp1", "few_dims"])
def test_edge_cases_match_oracle(lib, oracle, case):
    """Empty and degenerate inputs: no triangles, nothing but the light, a
    1 x 1 image, image sizes that divide no block, one sample, and a Sobol
    dimension bound small enough that every path wraps around it."""
    s = scenes.path_settings(5, "binary")
    sc = scenes.cornell_box()
    w, h, spp = 32, 32, 8
    if case == "empty_scene":
        sc = api.Scene()
        sc.add_material(api.material("Diffuse", diffuse=(0.5, 0.5, 0.5)))
    elif case == "light_only":
        sc = api.Scene()
        m = sc.add_material(api.material("Diffuse", diffuse=(0.5, 0.5, 0.5),
                                         emission=(4, 4, 4)))
        _, lt = scenes.room_triangles()
        sc.add_mesh(np.stack(lt).reshape(-1, 9), np.full(2, m, np.uint32))
    elif case == "one_pixel":
        w = h = 1
        spp = 33
    elif case == "ragged":
        w, h, spp = 257, 131, 3
    elif case == "spp1":
        spp = 1
    else:
        s.max_sample_size = 8
    f2w = scenes.cornell_camera(w, h)
    gpu = _render_gpu(sc, s, spp, w, h, f2w)
    ref = _render_oracle(sc, s, spp, w, h, f2w)
    assert np.array_equal(bits(gpu), bits(ref))
    s.kernel_approach = 1
    s.traversal = 1
    wave = _render_gpu(sc, s, spp, w, h, f2w)
    assert rel_rmse(wave, ref) <= RMSE_TOL if np.linalg.norm(ref) > 0 else not wave.any()


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("n", [1, 2, 3, 37, 5000])
def test_gpu_built_wide_bvh_finds_the_order_independent_closest_hit(lib, oracle, n, mode):
    """The GPU builder (PLOC collapsed to 8-wide; mode 2 after splitting the
    long thin triangles of this soup into clipped references): the same
    closest hit as a brute-force search, ties by smallest BVH-order index."""
    rng = np.random.default_rng(n)
    tris = rng.uniform(-1, 1, (n, 9)).astype(np.float32)
    rays = _random_rays(rng, -1, 1, 3000)
    s = api.Settings()
    s.traversal = 1
    s.gpu_build = mode
    got, gt = api.Renderer().intersect(tris, rays, s)
    want, wt = ol.loop_all(tris, rays)
    hit = want >= 0
    assert np.array_equal(hit, got >= 0)
    assert np.array_equal(bits(wt[hit]), bits(gt[hit]))
    tie = np.abs(wt - gt) <= 1e-6
    assert np.all((want == got) | (hit & tie))


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("case", ["cornell", "large_mesh"])
def test_gpu_built_bvh_renders_the_same_image(lib, case, mode):
    """Images through the GPU-built BVH equal those through the host SBVH
    (both through the order-independent 8-wide traversal)."""
    if case == "cornell":
        sc, w, h, depth, spp = scenes.cornell_box(), 64, 64, 5, 16
    else:
        sc, w, h, depth, spp = scenes.large_mesh_room(6, 40, 40), 64, 64, 8, 4
    s = scenes.path_settings(depth, "wide")
    s.kernel_approach = 1
    f2w = scenes.cornell_camera(w, h)
    host_built = _render_gpu(sc, s, spp, w, h, f2w)
    s.gpu_build = mode
    r = api.Renderer()
    out = np.zeros((h, w, 3), np.float32)
    r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w), out, sc, spp, s)
    st = r.stats()
    assert st["device_status"] == 0
    print(f"{case} mode {mode}: gpu build {1e3 * st['bvh_build_seconds']:.1f} ms, "
          f"{st['num_wide_nodes']} wide nodes, rel RMSE {rel_rmse(out, host_built):.2e}")
    assert rel_rmse(out, host_built) <= RMSE_TOL


def _adversarial_rays(rng, tris):
    """Rays that stress the 8-wide box test's margin: axis-parallel rays
    (zero direction components, the 1e-20 rule) with origins on the
    triangles' own vertex coordinates (on node planes), directions with
    components of 1e-30 and 1e-40 (a subnormal), rays grazing the axis
    planes of the room's walls, and rays from vertices towards vertices."""
    v = tris.reshape(-1, 3)
    rays = []
    axes = np.eye(3)
    for k in range(600):
        o = v[rng.integers(len(v))].astype(np.float64).copy()
        a = rng.integers(3)
        o[(a + 1) % 3] += rng.choice([0.0, 1e-7, -1e-7, 0.01])
        d = axes[a] * rng.choice([-1.0, 1.0])
        rays.append(np.concatenate([o - 3 * d, d]))
    for tiny in (1e-30, -1e-30, 1e-40, -1e-40):
        for k in range(200):
            o = rng.uniform(-0.9, 0.9, 3)
            d = np.zeros(3)
            a = rng.integers(3)
            d[a] = rng.choice([-1.0, 1.0])
            d[(a + 1) % 3] = tiny
            d[(a + 2) % 3] = rng.choice([0.0, tiny, 0.3])
            rays.append(np.concatenate([o, d]))
    for k in range(400):
        # grazing the walls: origin on a wall plane, direction in it
        o = rng.uniform(-1, 1, 3)
        a = rng.integers(3)
        o[a] = rng.choice([-1.0, 1.0])
        d = rng.normal(size=3)
        d[a] = rng.choice([0.0, 1e-7, -1e-7])
        rays.append(np.concatenate([o, d / np.linalg.norm(d)]))
    for k in range(800):
        p, q = v[rng.integers(len(v))], v[rng.integers(len(v))]
        d = q.astype(np.float64) - p
        n = np.linalg.norm(d)
        if n == 0:
            continue
        rays.append(np.concatenate([p, d / n]))
    return np.array(rays, np.float32)


def test_wide_traversal_on_adversarial_rays(lib, oracle):
    """The 8-wide walk (quantised boxes, rounding margin, hardware
    reciprocal) finds every closest hit that testing every triangle finds,
    on rays built to sit on its box planes and to have zero, tiny and
    subnormal direction components."""
    rng = np.random.default_rng(33)
    walls, light = scenes.room_triangles()
    room = [t for ts in walls.values() for t in ts] + list(light)
    for k in range(12):
        room.extend(scenes._box(rng.uniform(0.05, 0.6), rng.uniform(0.05, 1.2),
                                rng.uniform(0.05, 0.6),
                                float(rng.choice([0.0, 90.0, rng.uniform(0, 90)])),
                                tuple(rng.uniform(-0.7, 0.7, 2))))
    room = np.stack(room).reshape(-1, 9).astype(np.float32)
    ico, _ = scenes.displaced_icosphere(4)
    s = api.Settings()
    s.traversal = 1
    r = api.Renderer()
    for tris in (room, np.concatenate([room, ico]).astype(np.float32)):
        rays = _adversarial_rays(rng, tris)
        want, wt = ol.loop_all(tris, rays)
        got, gt = r.intersect(tris, rays, s)
        hit = want >= 0
        assert np.array_equal(hit, got >= 0)
        assert np.array_equal(bits(wt[hit]), bits(gt[hit]))
        # equal distances may name another triangle (the tie rules differ)
        assert np.all((want == got) | hit)


@pytest.mark.parametrize("traversal", ["binary", "wide"])
def test_scene_reupload_renders_the_same_image(lib, traversal):
    """upload_scene_every_render (the bench's end-to-end leg) re-copies the
    arrays the traversal reads and renders the same image bit for bit."""
    sc = scenes.cornell_box()
    s = scenes.path_settings(5, traversal)
    w = h = 24
    f2w = scenes.cornell_camera(w, h)
    r = api.Renderer()
    a = np.zeros((h, w, 3), np.float32)
    r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w), a, sc, 8, s)
    e = s.copy()
    e.upload_scene_every_render = 1
    b = np.zeros((h, w, 3), np.float32)
    r.render(api.ExecutionModel.GPU, api.SquareImage(w, h, f2w), b, sc, 8, e)
    assert r.stats()["h2d_bytes"] > 0
    assert np.array_equal(bits(a), bits(b))
