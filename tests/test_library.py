"""Host-side checks of the C-ABI library (no GPU needed)."""

import ctypes
import os
import re

import numpy as np
import pytest

from path_gb300 import api, capi, scenes
from oracle import oracle_lib as ol

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(lib):
    header = open(os.path.join(ROOT, "include", "path_gb300.h")).read()
    declared = set(re.findall(r"\b(path_[a-z0-9_]+)\s*\(", header))
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    assert set(capi.SIGNATURES) == declared


def test_settings_defaults_match_reference(lib):
    s = api.Settings()
    # include/render/settings.h:27-45 and the structs it names
    assert s.kernel_approach == 0 and s.max_blocks_per_launch_gpu == 4096
    assert s.max_blocks_per_launch_cpu == 128
    assert s.render_work_division.block_size == 256
    assert s.render_work_division.target_x_block_size == 32
    assert s.render_work_division.base_num_threads == 16384
    assert s.render_work_division.max_samples_per_thread == 32
    assert s.reduce_work_division.target_x_block_size == 256
    assert abs(s.overlap_threshold - 1e-5) < 1e-12 and s.use_spatial_splits == 0
    assert s.traversal_per_intersect_cost == 0.5 and s.target_objects == 4
    assert s.term_prob == capi.TERM["MultiplierFunc"]
    assert s.term_prob_exp == 50.0 and abs(s.term_prob_min_prob - 0.1) < 1e-7
    assert s.rng == 0 and s.max_sample_size == 256 and s.back_cull_emission == 1


def test_settings_yaml(lib, tmp_path):
    text = """
settings:
  kernel_approach:
    type: MegaKernel
    value:
      computation_settings:
        max_blocks_per_launch_gpu: 1024
        render_work_division:
          block_size: 128
          target_x_block_size: 16
          force_target_samples: true
          forced_target_samples_per_thread: 4
      individually_intersectable_settings:
        accel:
          type: SBVH
          value:
            overlap_threshold: 1e-4
            use_spatial_splits: true
            bvh_settings: {traversal_per_intersect_cost: 0.75, target_objects: 3}
  light_sampler:
    type: RandomTriangle
    value: {binary_search_threshold: 100}
  dir_sampler: {type: BSDF, value: {}}
  term_prob:
    type: NIters   # max depth 5
    value:
      iters: 4
  rng:
    type: Sobel
    value: {sequence_settings: {}, max_sample_size: 128}
  rendering_equation_settings:
    back_cull_emission: false
  gb300:
    traversal: Wide8
    trace_min_blocks: 5
    gpu_build: true
    wavefront_slots_log2: 22
"""
    p = tmp_path / "cfg.yaml"
    p.write_text(text)
    s = api.Settings.from_yaml(p)
    assert s.max_blocks_per_launch_gpu == 1024
    assert s.render_work_division.block_size == 128
    assert s.render_work_division.force_target_samples == 1
    assert s.render_work_division.forced_target_samples_per_thread == 4
    assert abs(s.overlap_threshold - 1e-4) < 1e-10 and s.use_spatial_splits == 1
    assert s.traversal_per_intersect_cost == 0.75 and s.target_objects == 3
    assert s.binary_search_threshold == 100
    assert s.term_prob == capi.TERM["NIters"] and s.term_prob_iters == 4
    assert s.max_sample_size == 128 and s.back_cull_emission == 0
    assert s.traversal == 1 and s.trace_min_blocks == 5 and s.gpu_build == 1
    assert s.wavefront_slots_log2 == 22
    bad = tmp_path / "bad.yaml"
    bad.write_text("settings:\n  term_prob:\n    type: Nope\n")
    with pytest.raises(capi.PathError) as e:
        api.Settings.from_yaml(bad)
    assert e.value.status == 2
    with pytest.raises(capi.PathError) as e:
        api.Settings.from_yaml(tmp_path / "missing.yaml")
    assert e.value.status == 7


def test_work_division_matches_oracle(lib, oracle):
    names = ["block_size", "base_samples_per_thread", "n_threads_per_unit_extra",
             "sample_block_size", "x_block_size", "y_block_size", "num_sample_blocks",
             "num_x_blocks", "num_y_blocks", "x_dim", "y_dim"]
    for force, target in ((False, 8), (True, 2), (True, 3)):
        for bs in (32, 256, 1024):
            for spp in (1, 3, 16, 64, 100, 2048):
                for dims in ((1, 1), (17, 3), (256, 256), (1024, 1024)):
                    wds = capi.WorkDivisionSettings(bs, 32, int(force), target, 16384, 0.5, 32)
                    got = api.work_division(wds, spp, *dims)
                    want = ol.work_division(ol.wd_settings(bs, 32, force, target), spp, *dims)
                    assert [got[n] for n in names] == [getattr(want, n) for n in names]


@pytest.mark.parametrize("spatial", [False, True])
def test_sbvh_matches_oracle(lib, oracle, spatial):
    rng = np.random.default_rng(11)
    soups = [rng.uniform(-1, 1, (n, 9)).astype(np.float32) for n in (1, 2, 7, 100, 2000)]
    soups.append(scenes.cornell_box().export()["triangles"])
    tris, _ = scenes.displaced_icosphere(3)
    soups.append(tris)
    s = api.Settings()
    s.use_spatial_splits = int(spatial)
    for tris in soups:
        got = api.sbvh_build(tris, s)
        want = ol.SBVH(tris, use_spatial_splits=spatial).export()
        for k in ("node_words", "node_aabbs", "extra_idxs", "permutation"):
            assert np.array_equal(got[k], want[k]), k


def test_cornell_scene_layout(lib):
    sc = scenes.cornell_box()
    z = sc.sizes()
    assert z["triangles"] == 36 and z["materials"] == 4 and z["clusters"] == 2
    ex = sc.export()
    tris = ex["triangles"].reshape(-1, 3, 3)
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    centre = tris.mean(1)
    walls = n[:10]
    # walls face the room's centre; the light faces down
    assert np.all(np.einsum("ij,ij->i", walls, -centre[:10]) > 0)
    assert np.all(n[10:12, 1] < 0)
    np.testing.assert_allclose(ex["materials"][3].emission[:], [15, 15, 15])


def test_icosphere_counts_and_winding():
    verts, faces = scenes.icosphere(3)
    assert len(faces) == 20 * 4 ** 3
    tris, nrm = scenes.displaced_icosphere(3)
    c = tris.reshape(-1, 3, 3)
    fn = np.cross(c[:, 1] - c[:, 0], c[:, 2] - c[:, 0])
    cen = c.mean(1) - np.array([0.35, -0.4, -0.25])
    assert np.all(np.einsum("ij,ij->i", fn, cen) > 0)
    g, gn = scenes.uv_sphere()
    assert 19000 <= len(g) <= 21000


def test_camera_transform(lib):
    f2w = api.camera_transform((0, 0, -1), (0, 1, 0), (0, 0, 3.5), 40.0, 1.0)
    m = f2w.reshape(3, 4)
    t = np.tan(np.radians(20.0))
    np.testing.assert_allclose(m[:, :3], np.diag([t, t, 1.0]), atol=1e-6)
    np.testing.assert_allclose(m[:, 3], [0, 0, 3.5], atol=1e-6)


def test_render_rejects_bad_requests_before_touching_the_gpu(lib):
    sc = scenes.cornell_box()
    r = api.Renderer()
    spec = api.SquareImage(8, 8, scenes.cornell_camera(8, 8))
    out = np.zeros((8, 8, 3), np.float32)
    s = api.Settings()
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.CPU, spec, out, sc, 4, s)
    assert e.value.status == 5
    s.rng = 2
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.GPU, spec, out, sc, 4, s)
    assert e.value.status == 1
    s = api.Settings()
    s.target_objects = 11
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.GPU, spec, out, sc, 4, s)
    assert e.value.status == 1
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.GPU, spec, out, sc, 0, api.Settings())
    assert e.value.status == 1
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.GPU, api.InitialRays(np.zeros((0, 6))), out, sc, 4,
                 api.Settings())
    assert e.value.status == 1
    steps = np.zeros((65, 8, 8, 3), np.float32)
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.GPU, spec, api.OutputPerStep(steps), sc, 4, api.Settings())
    assert e.value.status == 1
    # OutputPerStep and InitialIdxAndDir are MegaKernel-only, as in the reference
    s = api.Settings()
    s.kernel_approach = 1
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.GPU, spec, api.OutputPerStep(steps[:2]), sc, 4, s)
    assert e.value.status == 5
    idx_spec = api.InitialIdxAndDir(np.zeros(2, np.uint32), np.zeros((2, 6), np.float32))
    with pytest.raises(capi.PathError) as e:
        r.render(api.ExecutionModel.GPU, idx_spec, out, sc, 4, s)
    assert e.value.status == 5


def test_scene_rejects_bad_material_index(lib):
    sc = api.Scene()
    sc.add_material(api.material("Diffuse", diffuse=(0.5, 0.5, 0.5)))
    with pytest.raises(capi.PathError) as e:
        sc.add_mesh(np.zeros((1, 9), np.float32), np.array([3], np.uint32))
    assert e.value.status == 1
    bad = capi.PathMaterial()
    bad.type = 99
    with pytest.raises(capi.PathError):
        sc.add_material(bad)
